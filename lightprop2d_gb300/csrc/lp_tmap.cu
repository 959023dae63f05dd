// Tensor maps for the TMA-staged pass kernels: one 2-D map per (grid
// address, size, box), encoded on the host with the driver's
// cuTensorMapEncodeTiled (reached through the runtime's entry-point query, so
// the library links no driver library) and cached.
#include <cuda.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <mutex>

#include "lp_internal.h"

namespace lp {
namespace {

std::mutex g_tmap_mu;
PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
bool g_encode_tried = false;

struct Entry {
  const void* base;
  int n, bx, by;
  CUtensorMap map;
};
constexpr int kCache = 16;
Entry g_cache[kCache];
int g_used = 0, g_next = 0;

}  // namespace

bool grid_tensor_map(CUtensorMap* out, const void* base, int n, int bx, int by) {
  std::lock_guard<std::mutex> lk(g_tmap_mu);
  for (int i = 0; i < g_used; ++i) {
    const Entry& e = g_cache[i];
    if (e.base == base && e.n == n && e.bx == bx && e.by == by) {
      *out = e.map;
      return true;
    }
  }
  if (!g_encode_tried) {
    g_encode_tried = true;
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  }
  if (!g_encode) return false;
  // complex64 elements as 8-byte words; dims {x, y}, row stride n*8 bytes
  const cuuint64_t dims[2] = {(cuuint64_t)n, (cuuint64_t)n};
  const cuuint64_t strides[1] = {(cuuint64_t)n * 8};
  const cuuint32_t box[2] = {(cuuint32_t)bx, (cuuint32_t)by};
  const cuuint32_t estr[2] = {1, 1};
  CUtensorMap m;
  const CUresult r =
      g_encode(&m, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 2, const_cast<void*>(base), dims, strides, box,
               estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
               CU_TENSOR_MAP_L2_PROMOTION_NONE, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return false;
  Entry& e = g_cache[g_next];
  e = Entry{base, n, bx, by, m};
  g_next = (g_next + 1) % kCache;
  if (g_used < kCache) ++g_used;
  *out = m;
  return true;
}

}  // namespace lp
