// 2-D FFT passes for 256x256 grids (kernel templates in lp_fft_impl.cuh).
#define LP_N 256
#include "lp_fft_impl.cuh"
