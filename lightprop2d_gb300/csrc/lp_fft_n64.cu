// 2-D FFT passes for 64x64 grids (kernel templates in lp_fft_impl.cuh).
#define LP_N 64
#include "lp_fft_impl.cuh"
