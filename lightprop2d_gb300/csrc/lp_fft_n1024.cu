// 2-D FFT passes for 1024x1024 grids (kernel templates in lp_fft_impl.cuh).
#define LP_N 1024
#include "lp_fft_impl.cuh"
