// complex128 line passes of npoints 1024, 2048 (lp_c128_lines.cuh).
#include "lp_c128_lines.cuh"

namespace lp {

cudaError_t zline_g1024_2048(int n, int mode, bool in_d, bool out_d, bool cols, const void* in,
                    void* out, const ZOps& o, const float4* tw, cudaStream_t st) {
  switch (n) {
    case 1024: return zline<1024>(mode, in_d, out_d, cols, in, out, o, tw, st);
    case 2048: return zline<2048>(mode, in_d, out_d, cols, in, out, o, tw, st);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t zsmem_g1024_2048(int n) {
  switch (n) {
    case 1024: return set_smem<1024>();
    case 2048: return set_smem<2048>();
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace lp
