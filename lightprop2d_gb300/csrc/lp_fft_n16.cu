// 2-D FFT passes for 16x16 grids (kernel templates in lp_fft_impl.cuh).
#define LP_N 16
#include "lp_fft_impl.cuh"
