// 2-D FFT passes for 128x128 grids (kernel templates in lp_fft_impl.cuh).
#define LP_N 128
#include "lp_fft_impl.cuh"
