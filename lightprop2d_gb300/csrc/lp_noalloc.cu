// lp_plain_propagate_field_noalloc: the unfused FFT -> multiply -> IFFT
// propagate with its transfer-function grid in a fixed device array.
//
// Who this is for: callers that must not call cudaMalloc once they are
// running.  Two common cases: a host application that reserves (nearly) all
// device memory for its own pool at start-up, so that any further cudaMalloc
// fails; and a real-time loop (for example a camera or spatial-light-modulator
// feedback loop) that forbids device allocation after start-up because
// cudaMalloc can block and synchronise the whole device.
// lp_plain_propagate_field allocates its H grid with cudaMalloc on the first
// call for each stream; this variant uses the static array below instead,
// which is reserved when the library is loaded and held by every device that
// loads the library until the process exits.
//
// Limits and sharing rules:
//   * grids up to kMaxN x kMaxN (1024 x 1024; the array is 8 MiB of complex64);
//     larger N is rejected with LP_ERR_UNSUPPORTED_SIZE.
//   * every call on a device uses the same array.  Each call writes every H
//     element it later reads, so nothing needs clearing between calls, but
//     calls that overlap on the GPU (different streams, or different host
//     threads) race on the array: serialise them.
//   * the first call on a device does the one-time set-up (twiddle tables via
//     lp_init, and the device address of the array via cudaGetSymbolAddress);
//     make that first call before any stream capture (a first call made
//     while its stream is capturing returns LP_ERR_NOT_INITIALIZED).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <mutex>

#include "lightprop2d_gb300.h"
#include "lp_internal.h"

using namespace lp;

namespace {

constexpr int kMaxN = 1024;
constexpr int kMaxDevices = 64;

// Transfer-function grid shared by every call (see the file comment).
static __device__ __align__(256) float2 g_noalloc_h[kMaxN * kMaxN];

std::mutex g_setup_mu;
float2* g_h_addr[kMaxDevices] = {};  // device address of g_noalloc_h, per device

lp_status noalloc_fail(lp_status s, const char* msg) {
  return (lp_status)set_last_error((int)s, msg);
}

// Once per device, with that device current: library set-up and the device
// address of the static H grid (host code must not pass &g_noalloc_h itself:
// on the host that name is only a stand-in, not a device address).
// A first call inside stream capture is refused (the set-up copies tables and
// sets kernel attributes, which would invalidate the caller's capture).
lp_status setup_device(int dev, cudaStream_t st, float2** h_out) {
  std::lock_guard<std::mutex> lk(g_setup_mu);
  if (g_h_addr[dev]) {
    *h_out = g_h_addr[dev];
    return LP_OK;
  }
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(st, &cs) != cudaSuccess)
    return noalloc_fail(LP_ERR_CUDA, "cudaStreamIsCapturing failed");
  if (cs != cudaStreamCaptureStatusNone)
    return noalloc_fail(LP_ERR_NOT_INITIALIZED,
                        "lp_plain_propagate_field_noalloc: first call on this device inside "
                        "stream capture; make one call (or lp_init) before capturing");
  lp_status s = lp_init(dev);
  if (s != LP_OK) return s;
  void* p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_h);
  if (e != cudaSuccess) {
    char msg[256];
    snprintf(msg, sizeof(msg), "cudaGetSymbolAddress(H grid): %s", cudaGetErrorString(e));
    return noalloc_fail(LP_ERR_CUDA, msg);
  }
  g_h_addr[dev] = reinterpret_cast<float2*>(p);
  *h_out = g_h_addr[dev];
  return LP_OK;
}

// H at every point of the N x N spectrum (float-float phase, as the fused
// path computes it).
__global__ void noalloc_build_h(float2* __restrict__ h, int n, KParams kp) {
  const size_t n2 = (size_t)n * n;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n2;
       i += (size_t)gridDim.x * blockDim.x) {
    const int ky = (int)(i / n), kx = (int)(i % n);
    const int sx = kx < n / 2 ? kx : kx - n, sy = ky < n / 2 ? ky : ky - n;
    float a_hi, a_lo;
    column_constant(kp, (float)(sx * sx), a_hi, a_lo);
    bool evan;
    float sv;
    const float f = kz_phase_ff(kp, a_hi, a_lo, (float)(sy * sy), evan, sv);
    h[i] = evan ? make_float2(1.0f, 0.0f) : cis_cycles(f, -1.0f);
  }
}

__global__ void noalloc_cmul(float2* __restrict__ a, const float2* __restrict__ b, size_t n2) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n2;
       i += (size_t)gridDim.x * blockDim.x)
    a[i] = cmul(a[i], b[i]);
}

}  // namespace

extern "C" lp_status lp_plain_propagate_field_noalloc(const lp_cfloat* field_in,
                                                      lp_cfloat* field_out, int n,
                                                      double area_size, double wl, double z,
                                                      uint32_t flags, void* stream) {
  if (!size_ops(n) || n > kMaxN) {
    char msg[160];
    snprintf(msg, sizeof(msg),
             "lp_plain_propagate_field_noalloc: npoints=%d unsupported (powers of two "
             "from 16 to %d, the size of its fixed H grid)", n, kMaxN);
    return noalloc_fail(LP_ERR_UNSUPPORTED_SIZE, msg);
  }
  if (!field_in || !field_out)
    return noalloc_fail(LP_ERR_INVALID_ARGUMENT, "field_in and field_out are required");
  if ((reinterpret_cast<uintptr_t>(field_in) | reinterpret_cast<uintptr_t>(field_out)) & 7u)
    return noalloc_fail(LP_ERR_MISALIGNED, "field pointers must be 8-byte aligned");
  if (!(std::isfinite(area_size) && area_size > 0 && std::isfinite(wl) && wl > 0 &&
        std::isfinite(z)))
    return noalloc_fail(LP_ERR_INVALID_ARGUMENT, "area_size, wl must be finite and > 0, z finite");
  if (flags != 0u)
    return noalloc_fail(LP_ERR_INVALID_ARGUMENT,
                        "lp_plain_propagate_field_noalloc takes no flags (pass 0)");
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= kMaxDevices)
    return noalloc_fail(LP_ERR_CUDA, "cudaGetDevice failed");
  cudaStream_t st = (cudaStream_t)stream;
  float2* h = nullptr;
  lp_status s = setup_device(dev, st, &h);
  if (s != LP_OK) return s;

  const SizeOps* so = size_ops(n);
  float2* out = reinterpret_cast<float2*>(field_out);
  const size_t n2 = (size_t)n * n;
  const int grid = (int)((n2 + 255) / 256 < 2432 ? (n2 + 255) / 256 : 2432);

  // Transfer-function constants (the same function the fused path uses).
  const KParams kp = make_kparams(n, area_size, wl, z);

  ColOps inv = col_ops_none();
  inv.scale = 1.0f / ((float)n * (float)n);
  e = so->row(0, reinterpret_cast<const float2*>(field_in), out, row_ops_none(), st);
  if (e == cudaSuccess) e = so->col(COL_FWD, out, out, col_ops_none(), st);
  if (e == cudaSuccess) {
    noalloc_build_h<<<grid, 256, 0, st>>>(h, n, kp);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) {
    noalloc_cmul<<<grid, 256, 0, st>>>(out, h, n2);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = so->col(COL_INV, out, out, inv, st);
  if (e == cudaSuccess) e = so->row(1, out, out, row_ops_none(), st);
  if (e != cudaSuccess) {
    char msg[256];
    snprintf(msg, sizeof(msg), "lp_plain_propagate_field_noalloc: %s", cudaGetErrorString(e));
    return noalloc_fail(LP_ERR_CUDA, msg);
  }
  return LP_OK;
}
