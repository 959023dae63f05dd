// 2-D FFT passes for 2048x2048 grids (kernel templates in lp_fft_impl.cuh).
#define LP_N 2048
#include "lp_fft_impl.cuh"
