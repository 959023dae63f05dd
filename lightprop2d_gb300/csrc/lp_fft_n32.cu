// 2-D FFT passes for 32x32 grids (kernel templates in lp_fft_impl.cuh).
#define LP_N 32
#include "lp_fft_impl.cuh"
