// complex128 line passes of npoints 16, 32, 64, 128 (lp_c128_lines.cuh).
#include "lp_c128_lines.cuh"

namespace lp {

cudaError_t zline_g16_128(int n, int mode, bool in_d, bool out_d, bool cols, const void* in,
                    void* out, const ZOps& o, const float4* tw, cudaStream_t st) {
  switch (n) {
    case 16: return zline<16>(mode, in_d, out_d, cols, in, out, o, tw, st);
    case 32: return zline<32>(mode, in_d, out_d, cols, in, out, o, tw, st);
    case 64: return zline<64>(mode, in_d, out_d, cols, in, out, o, tw, st);
    case 128: return zline<128>(mode, in_d, out_d, cols, in, out, o, tw, st);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t zsmem_g16_128(int n) {
  switch (n) {
    case 16: return set_smem<16>();
    case 32: return set_smem<32>();
    case 64: return set_smem<64>();
    case 128: return set_smem<128>();
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace lp
