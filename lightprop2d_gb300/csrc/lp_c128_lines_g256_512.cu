// complex128 line passes of npoints 256, 512 (lp_c128_lines.cuh).
#include "lp_c128_lines.cuh"

namespace lp {

cudaError_t zline_g256_512(int n, int mode, bool in_d, bool out_d, bool cols, const void* in,
                    void* out, const ZOps& o, const float4* tw, cudaStream_t st) {
  switch (n) {
    case 256: return zline<256>(mode, in_d, out_d, cols, in, out, o, tw, st);
    case 512: return zline<512>(mode, in_d, out_d, cols, in, out, o, tw, st);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t zsmem_g256_512(int n) {
  switch (n) {
    case 256: return set_smem<256>();
    case 512: return set_smem<512>();
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace lp
