// Mode decomposition of Beam2D (beam2d.py:539-667): projection of the central
// nb x nb window of a field onto a mode basis and the inverse synthesis.
//
//   project:  c[m] = sum_p modes[m][p] * w[p]      (deconstruct_by_modes,
//             w = field window, row-major)        "scalar": modes @ field)
//   combine:  field = sum_m c[m] * modes[m] inside the window, 0 outside
//             (construct_by_modes with _expand_basis' zero padding)
//
// Both are matrix-vector products over an M x P complex64 basis (P = nb^2):
// HBM-bound (every basis element is read once, 8 B, for 8 flops), so they are
// CUDA-core kernels reading the basis with coalesced loads, several in flight
// per thread, not tensor-core GEMMs.  Sums run in FP32 over short runs (4
// terms in the projection, 16 in the synthesis) and in FP64 across runs, so
// results carry FP32 rounding of the inputs only.
#include <cuda_runtime.h>

#include <cstdint>

#include "lightprop2d_gb300.h"
#include "lp_internal.h"

using namespace lp;

namespace {

constexpr int kThreads = 256;
constexpr int kChunk = 1 << 16;  // basis points per CTA of the projection

lp_status fail(lp_status s, const char* msg) { return (lp_status)set_last_error((int)s, msg); }

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// grid (chunks, modes): CTA (ck, m) adds sum over points [ck*kChunk, ...) of
// modes[m][p] * w[p] into c[m] (FP64 pair).
__global__ void __launch_bounds__(kThreads) project_kernel(const float2* __restrict__ modes,
                                                           long long P, int nb,
                                                           const float2* __restrict__ field,
                                                           int n, int first,
                                                           double* __restrict__ c) {
  const int m = blockIdx.y;
  const long long p0 = (long long)blockIdx.x * kChunk;
  const long long p1 = p0 + kChunk < P ? p0 + kChunk : P;
  const float2* row = modes + (size_t)m * P;
  double ar = 0.0, ai = 0.0;
  // (r, q) of point p tracked incrementally (no division in the loop)
  long long p = p0 + threadIdx.x;
  int r = (int)(p / nb), q = (int)(p - (long long)r * nb);
  while (p < p1) {
    float fr = 0.0f, fi = 0.0f;
    float2 a[4], w[4];
    bool ok[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {  // four independent pairs of loads in flight
      ok[u] = p < p1;
      a[u] = ok[u] ? __ldg(row + p) : make_float2(0.0f, 0.0f);
      w[u] = ok[u] ? __ldg(field + (size_t)(first + r) * n + first + q) : make_float2(0.0f, 0.0f);
      p += kThreads;
      q += kThreads;
      while (q >= nb) {
        q -= nb;
        ++r;
      }
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      fr = fmaf(a[u].x, w[u].x, fmaf(-a[u].y, w[u].y, fr));
      fi = fmaf(a[u].x, w[u].y, fmaf(a[u].y, w[u].x, fi));
    }
    ar += fr;
    ai += fi;
  }
  __shared__ double part[2][kThreads / 32];
  const int lane = threadIdx.x & 31, wi = threadIdx.x >> 5;
  ar = warp_sum(ar);
  ai = warp_sum(ai);
  if (lane == 0) {
    part[0][wi] = ar;
    part[1][wi] = ai;
  }
  __syncthreads();
  if (threadIdx.x < 32) {
    double sr = threadIdx.x < kThreads / 32 ? part[0][threadIdx.x] : 0.0;
    double si = threadIdx.x < kThreads / 32 ? part[1][threadIdx.x] : 0.0;
    sr = warp_sum(sr);
    si = warp_sum(si);
    if (threadIdx.x == 0) {
      atomicAdd(c + 2 * m, sr);
      atomicAdd(c + 2 * m + 1, si);
    }
  }
}

// One thread per field point: inside the window sum_m c[m]*modes[m][p], else 0.
// The coefficients are staged through shared memory in blocks of kCoef.
constexpr int kCoef = 512;

__global__ void __launch_bounds__(kThreads) combine_kernel(const float2* __restrict__ modes,
                                                           int M, long long P, int nb,
                                                           const double* __restrict__ c,
                                                           float2* __restrict__ field, int n,
                                                           int first) {
  __shared__ float2 cs[kCoef];
  const size_t total = (size_t)n * n;
  for (size_t base = (size_t)blockIdx.x * kThreads; base < total;
       base += (size_t)gridDim.x * kThreads) {
    const size_t i = base + threadIdx.x;
    const int y = (int)(i / n), x = (int)(i % n);
    const int r = y - first, q = x - first;
    const bool in = i < total && r >= 0 && r < nb && q >= 0 && q < nb;
    const long long p = (long long)r * nb + q;
    double sr = 0.0, si = 0.0;
    for (int m0 = 0; m0 < M; m0 += kCoef) {
      const int mc = M - m0 < kCoef ? M - m0 : kCoef;
      __syncthreads();
      for (int j = threadIdx.x; j < mc; j += kThreads)
        cs[j] = make_float2((float)c[2 * (m0 + j)], (float)c[2 * (m0 + j) + 1]);
      __syncthreads();
      if (in) {
        float fr = 0.0f, fi = 0.0f;
        for (int j = 0; j < mc; ++j) {
          const float2 a = __ldg(modes + (size_t)(m0 + j) * P + p);
          const float2 w = cs[j];
          fr = fmaf(a.x, w.x, fmaf(-a.y, w.y, fr));
          fi = fmaf(a.x, w.y, fmaf(a.y, w.x, fi));
          if ((j & 15) == 15) {
            sr += fr;
            si += fi;
            fr = fi = 0.0f;
          }
        }
        sr += fr;
        si += fi;
      }
    }
    if (i < total) field[i] = make_float2((float)sr, (float)si);
  }
}

bool aligned(const void* p, unsigned a) { return (reinterpret_cast<uintptr_t>(p) % a) == 0; }

lp_status check_common(const void* modes, int n_modes, int nb, const void* field, int n,
                       const void* c) {
  if (!modes || !field || !c) return fail(LP_ERR_INVALID_ARGUMENT, "mode basis: NULL pointer");
  if (n_modes < 1 || nb < 1 || n < 1 || nb > n || ((n - nb) & 1))
    return fail(LP_ERR_INVALID_ARGUMENT,
                "mode basis: need n_modes >= 1 and 1 <= nb <= n with n - nb even");
  if (!aligned(modes, 8) || !aligned(field, 8) || !aligned(c, 8))
    return fail(LP_ERR_MISALIGNED, "mode basis: 8-byte alignment");
  if (n_modes > 65535) return fail(LP_ERR_INVALID_ARGUMENT, "mode basis: at most 65535 modes");
  return LP_OK;
}

}  // namespace

extern "C" {

lp_status lp_modes_project(const lp_cfloat* modes, int n_modes, int nb, const lp_cfloat* field,
                           int n, double* coeffs, void* stream) {
  lp_status s = check_common(modes, n_modes, nb, field, n, coeffs);
  if (s != LP_OK) return s;
  cudaStream_t st = (cudaStream_t)stream;
  const long long P = (long long)nb * nb;
  cudaError_t e = cudaMemsetAsync(coeffs, 0, sizeof(double) * 2 * (size_t)n_modes, st);
  if (e != cudaSuccess) return fail(LP_ERR_CUDA, cudaGetErrorString(e));
  const dim3 grid((unsigned)((P + kChunk - 1) / kChunk), (unsigned)n_modes);
  project_kernel<<<grid, kThreads, 0, st>>>(reinterpret_cast<const float2*>(modes), P, nb,
                                            reinterpret_cast<const float2*>(field), n,
                                            (n - nb) / 2, coeffs);
  e = cudaGetLastError();
  return e == cudaSuccess ? LP_OK : fail(LP_ERR_CUDA, cudaGetErrorString(e));
}

lp_status lp_modes_combine(const lp_cfloat* modes, int n_modes, int nb, const double* coeffs,
                           lp_cfloat* field, int n, void* stream) {
  lp_status s = check_common(modes, n_modes, nb, field, n, coeffs);
  if (s != LP_OK) return s;
  const size_t total = (size_t)n * n;
  const size_t blocks = (total + kThreads - 1) / kThreads;
  const int grid = (int)(blocks < 65535u * 16u ? blocks : 65535u * 16u);
  combine_kernel<<<grid, kThreads, 0, (cudaStream_t)stream>>>(
      reinterpret_cast<const float2*>(modes), n_modes, (long long)nb * nb, nb, coeffs,
      reinterpret_cast<float2*>(field), n, (n - nb) / 2);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? LP_OK : fail(LP_ERR_CUDA, cudaGetErrorString(e));
}

}  // extern "C"
