// complex128 line passes of npoints 4096 (lp_c128_lines.cuh).
#include "lp_c128_lines.cuh"

namespace lp {

cudaError_t zline_g4096(int n, int mode, bool in_d, bool out_d, bool cols, const void* in,
                    void* out, const ZOps& o, const float4* tw, cudaStream_t st) {
  switch (n) {
    case 4096: return zline<4096>(mode, in_d, out_d, cols, in, out, o, tw, st);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t zsmem_g4096(int n) {
  switch (n) {
    case 4096: return set_smem<4096>();
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace lp
