// 2-D FFT passes for 512x512 grids (kernel templates in lp_fft_impl.cuh).
#define LP_N 512
#include "lp_fft_impl.cuh"
