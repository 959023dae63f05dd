// 2-D FFT passes for 4096x4096 grids (kernel templates in lp_fft_impl.cuh).
#define LP_N 4096
#include "lp_fft_impl.cuh"
