// complex128 line passes of npoints 8192 (lp_c128_lines.cuh).
#include "lp_c128_lines.cuh"

namespace lp {

cudaError_t zline_g8192(int n, int mode, bool in_d, bool out_d, bool cols, const void* in,
                    void* out, const ZOps& o, const float4* tw, cudaStream_t st) {
  switch (n) {
    case 8192: return zline<8192>(mode, in_d, out_d, cols, in, out, o, tw, st);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t zsmem_g8192(int n) {
  switch (n) {
    case 8192: return set_smem<8192>();
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace lp
