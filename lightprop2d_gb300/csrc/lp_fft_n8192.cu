// 2-D FFT passes for 8192x8192 grids (kernel templates in lp_fft_impl.cuh).
#define LP_N 8192
#include "lp_fft_impl.cuh"
