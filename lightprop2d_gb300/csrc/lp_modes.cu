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
// CUDA-core kernels streaming the basis with coalesced loads, many in flight
// per thread, not tensor-core GEMMs.  Products are summed in FP32 over runs of
// 16 terms and the runs in FP64, so results carry FP32 rounding of the
// inputs only (GB300's FP64 rate is far too low for one FP64 add per term).
#include <cuda_runtime.h>

#include <cstdint>

#include "lightprop2d_gb300.h"
#include "lp_internal.h"

using namespace lp;

namespace {

constexpr int kThreads = 256;
// Projection tiling: kModes modes per CTA, kPts window points per thread per
// step (kModes * kPts basis loads in flight), kChunk window points per CTA,
// FP32 runs of kRun steps.  Measured on GB300 (256 modes x 1024^2): 4 x 4 at
// 80 registers 356 us, 8 x 2 427 us, 8 x 4 493 us, 2 x 8 369 us.
#ifndef LP_MODES_MB
#define LP_MODES_MB 4
#endif
#ifndef LP_MODES_PT
#define LP_MODES_PT 4
#endif
constexpr int kModes = LP_MODES_MB;
constexpr int kPts = LP_MODES_PT;
constexpr int kChunk = 1 << 14;
constexpr int kRun = 16 / kPts;

lp_status fail(lp_status s, const char* msg) { return (lp_status)set_last_error((int)s, msg); }

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// grid (chunks, ceil(M / kModes)): CTA (ck, g) adds, for modes
// m = g*kModes .. +kModes-1, the sum over window points [ck*kChunk, ...) of
// modes[m][p] * w[p] into c[m] (FP64 pair).  Each thread reads a field value
// once for all kModes modes; window point p = r*nb + q is field element
// (first + r, first + q), with (r, q) advanced incrementally (P < 2^31).
__global__ void __launch_bounds__(kThreads) project_kernel(const float2* __restrict__ modes,
                                                           int M, int P, int nb,
                                                           const float2* __restrict__ field,
                                                           int n, int first,
                                                           double* __restrict__ c) {
  const int m0 = blockIdx.y * kModes;
  const int mc = M - m0 < kModes ? M - m0 : kModes;
  const int p0 = blockIdx.x * kChunk;
  const int p1 = P - p0 > kChunk ? p0 + kChunk : P;
  const float2* base = modes + (size_t)m0 * P;
  const float2* frow = field + (size_t)first * n + first;
  double tr[kModes], ti[kModes];
#pragma unroll
  for (int k = 0; k < kModes; ++k) tr[k] = ti[k] = 0.0;
  int p = p0 + threadIdx.x;
  int r = p / nb, q = p - r * nb;
  while (p < p1) {
    float fr[kModes], fi[kModes];
#pragma unroll
    for (int k = 0; k < kModes; ++k) fr[k] = fi[k] = 0.0f;
#pragma unroll 1
    for (int it = 0; it < kRun && p < p1; ++it) {
      float2 w[kPts], a[kPts][kModes];
#pragma unroll
      for (int u = 0; u < kPts; ++u) {
        const int pu = p + u * kThreads;
        const bool ok = pu < p1;
        w[u] = ok ? __ldg(frow + (size_t)r * n + q) : make_float2(0.0f, 0.0f);
#pragma unroll
        for (int k = 0; k < kModes; ++k)
          a[u][k] = ok && k < mc ? __ldg(base + (size_t)k * P + pu) : make_float2(0.0f, 0.0f);
        q += kThreads;
        while (q >= nb) {
          q -= nb;
          ++r;
        }
      }
      p += kPts * kThreads;
#pragma unroll
      for (int u = 0; u < kPts; ++u) {
#pragma unroll
        for (int k = 0; k < kModes; ++k) {
          fr[k] = fmaf(a[u][k].x, w[u].x, fmaf(-a[u][k].y, w[u].y, fr[k]));
          fi[k] = fmaf(a[u][k].x, w[u].y, fmaf(a[u][k].y, w[u].x, fi[k]));
        }
      }
    }
#pragma unroll
    for (int k = 0; k < kModes; ++k) {
      tr[k] += fr[k];
      ti[k] += fi[k];
    }
  }
  __shared__ double part[2 * kModes][kThreads / 32];
  const int lane = threadIdx.x & 31, wi = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < kModes; ++k) {
    const double sr = warp_sum(tr[k]), si = warp_sum(ti[k]);
    if (lane == 0) {
      part[2 * k][wi] = sr;
      part[2 * k + 1][wi] = si;
    }
  }
  __syncthreads();
  if (threadIdx.x < 2 * mc) {
    double acc = 0.0;
#pragma unroll
    for (int w = 0; w < kThreads / 32; ++w) acc += part[threadIdx.x][w];
    atomicAdd(c + 2 * m0 + threadIdx.x, acc);
  }
}

// One thread per window point: sum_m c[m] * modes[m][p], with 16 basis loads
// issued before they are used; the coefficients are staged through shared
// memory in blocks of kCoef.  Points outside the window were zeroed by the
// caller.
constexpr int kCoef = 512;
constexpr int kBlk = 16;

__global__ void __launch_bounds__(kThreads) combine_kernel(const float2* __restrict__ modes,
                                                           int M, long long P, int nb,
                                                           const double* __restrict__ c,
                                                           float2* __restrict__ field, int n,
                                                           int first) {
  __shared__ float2 cs[kCoef];
  for (long long base = (long long)blockIdx.x * kThreads; base < P;
       base += (long long)gridDim.x * kThreads) {
    const long long p = base + threadIdx.x;
    const bool in = p < P;
    double sr = 0.0, si = 0.0;
    for (int m0 = 0; m0 < M; m0 += kCoef) {
      const int mc = M - m0 < kCoef ? M - m0 : kCoef;
      __syncthreads();
      for (int j = threadIdx.x; j < mc; j += kThreads)
        cs[j] = make_float2((float)c[2 * (m0 + j)], (float)c[2 * (m0 + j) + 1]);
      __syncthreads();
      if (in) {
        const float2* col = modes + (size_t)m0 * P + p;
#pragma unroll 1
        for (int j0 = 0; j0 < mc; j0 += kBlk) {
          float2 a[kBlk];
          if (j0 + kBlk <= mc) {
#pragma unroll
            for (int u = 0; u < kBlk; ++u) a[u] = __ldg(col + (size_t)(j0 + u) * P);
          } else {
#pragma unroll
            for (int u = 0; u < kBlk; ++u)
              a[u] = j0 + u < mc ? __ldg(col + (size_t)(j0 + u) * P) : make_float2(0.0f, 0.0f);
          }
          float fr = 0.0f, fi = 0.0f;
#pragma unroll
          for (int u = 0; u < kBlk; ++u) {
            const float2 w = cs[j0 + u < mc ? j0 + u : 0];
            fr = fmaf(a[u].x, w.x, fmaf(-a[u].y, w.y, fr));
            fi = fmaf(a[u].x, w.y, fmaf(a[u].y, w.x, fi));
          }
          sr += fr;
          si += fi;
        }
      }
    }
    if (in) {
      const int r = (int)(p / nb), q = (int)(p - (long long)r * nb);
      field[(size_t)(first + r) * n + first + q] = make_float2((float)sr, (float)si);
    }
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
  if (nb > 46340) return fail(LP_ERR_INVALID_ARGUMENT, "mode basis: window side at most 46340");
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
  const dim3 grid((unsigned)((P + kChunk - 1) / kChunk), (unsigned)((n_modes + kModes - 1) / kModes));
  project_kernel<<<grid, kThreads, 0, st>>>(reinterpret_cast<const float2*>(modes), n_modes,
                                            (int)P, nb, reinterpret_cast<const float2*>(field),
                                            n, (n - nb) / 2, coeffs);
  e = cudaGetLastError();
  return e == cudaSuccess ? LP_OK : fail(LP_ERR_CUDA, cudaGetErrorString(e));
}

lp_status lp_modes_combine(const lp_cfloat* modes, int n_modes, int nb, const double* coeffs,
                           lp_cfloat* field, int n, void* stream) {
  lp_status s = check_common(modes, n_modes, nb, field, n, coeffs);
  if (s != LP_OK) return s;
  cudaStream_t st = (cudaStream_t)stream;
  if (nb < n) {  // zero the field outside the window
    cudaError_t e = cudaMemsetAsync(field, 0, sizeof(lp_cfloat) * (size_t)n * n, st);
    if (e != cudaSuccess) return fail(LP_ERR_CUDA, cudaGetErrorString(e));
  }
  const long long P = (long long)nb * nb;
  const long long blocks = (P + kThreads - 1) / kThreads;
  const int grid = (int)(blocks < 65535LL * 16 ? blocks : 65535LL * 16);
  combine_kernel<<<grid, kThreads, 0, st>>>(reinterpret_cast<const float2*>(modes), n_modes, P,
                                            nb, coeffs, reinterpret_cast<float2*>(field), n,
                                            (n - nb) / 2);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? LP_OK : fail(LP_ERR_CUDA, cudaGetErrorString(e));
}

}  // extern "C"
