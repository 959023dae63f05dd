// Intensity moments of a field for Beam2D.centroid / D4sigma /
// centroid_intensity (beam2d.py:669-752): one read pass over the grid and a
// one-thread finish.
//
//   out = m0 = sum I, m1 = sum jx*I, m2 = sum jy*I,
//         m3 = sum (jx - xc)^2 I, m4 = sum (jy - yc)^2 I,  xc = m1/m0, yc = m2/m0
//
// with I = |field|^2 and jx = ix - n/2, jy = iy - n/2 (n even; grid-index
// offsets from the centre; the caller scales by dL).  A thread owns one
// column and a run of contiguous rows starting at row r0, and accumulates
// in FP32 about r0 (offsets below the run length, so the products stay
// exact to FP32 rounding).  A warp adds its lanes' sums in FP32 about the
// warp's first column (lane offsets 0..31), and lane 0 moves the warp's five
// sums to the grid centre in float-float (sum (r-c)^2 I = S2 + 2 (r0-c) S1 +
// (r0-c)^2 S0 with exact products, likewise in x); a CTA adds its warps'
// pairs in float-float and adds the five sums to out in FP64 (one atomicAdd
// per value per CTA).  The finish
// turns the raw second moments into moments about the centroid in FP64, so
// an off-centre beam keeps its precision without a second read pass (the
// cancellation costs ~1e-16 (offset/width)^2).
#include <cuda_runtime.h>

#include <cstdint>

#include "lightprop2d_gb300.h"
#include "lp_device.cuh"
#include "lp_internal.h"

namespace {

using lp::FF;
using lp::ff_add;
using lp::ff_fma;

// 512-thread CTAs, four per SM (32 registers a thread); a thread owns two
// adjacent columns (one 16-byte load per row) and keeps four rows of loads
// in flight: 128 KB of reads in flight per SM.
constexpr int kThreads = 512;
constexpr int kCols = 2 * kThreads;  // columns per CTA
constexpr int kUnroll = 4;
constexpr int kCtasPerSm = 4;

// One pass.  CTA (bx, by): columns bx*kCols + 2*tx and the next one, rows
// by*rows .. by*rows + rows - 1 (lanes run along a row: coalesced).  V4:
// the field is 16-byte aligned (one float4 load per row and thread).
template <bool V4>
__global__ void __launch_bounds__(kThreads, kCtasPerSm) moments_kernel(
    const float2* __restrict__ f, int n, int rows, double* out) {
  asm volatile("griddepcontrol.launch_dependents;");
  const int x = blockIdx.x * kCols + 2 * threadIdx.x;  // n is even: both columns or neither
  const int r0 = blockIdx.y * rows, r1 = min(n, r0 + rows);
  // s*: both columns about row r0; b0: the second column's sum I
  float s0 = 0.0f, s1 = 0.0f, s2 = 0.0f, b0 = 0.0f;
  if (x < n) {
    const float2* col = f + x;
    for (int r = r0; r < r1; r += kUnroll) {
      // unconditional loads (rows past the run re-read its last row, an L1
      // hit, and count zero), so all kUnroll are in flight at once
      float4 v[kUnroll];
#pragma unroll
      for (int u = 0; u < kUnroll; ++u) {
        const float2* p = col + (size_t)min(r + u, r1 - 1) * n;
        if constexpr (V4) {
          v[u] = __ldg(reinterpret_cast<const float4*>(p));
        } else {
          const float2 lo = __ldg(p), hi = __ldg(p + 1);
          v[u] = make_float4(lo.x, lo.y, hi.x, hi.y);
        }
      }
      const float d0 = (float)(r - r0);
#pragma unroll
      for (int u = 0; u < kUnroll; ++u) {
        const bool in = r + u < r1;
        const float Ia = in ? fmaf(v[u].x, v[u].x, v[u].y * v[u].y) : 0.0f;
        const float Ib = in ? fmaf(v[u].z, v[u].z, v[u].w * v[u].w) : 0.0f;
        const float I = Ia + Ib, d = d0 + (float)u;
        s0 += I;
        s1 = fmaf(d, I, s1);
        s2 = fmaf(d * d, I, s2);
        b0 += Ib;
      }
    }
  }
  // Warp: FP32 sums about the warp's first column (the thread's columns sit
  // at offsets 2l and 2l+1, l = lane: sum c I = 2l s0 + b0, sum c^2 I =
  // 4l^2 s0 + (4l+1) b0).  Every term is non-negative, so each sum is
  // accurate to FP32 rounding.
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const float l2 = (float)(2 * lane);
  float t[5] = {s0, fmaf(l2, s0, b0), fmaf(l2 * l2, s0, (2.0f * l2 + 1.0f) * b0), s1, s2};
#pragma unroll
  for (int k = 0; k < 5; ++k) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t[k] += __shfl_down_sync(0xffffffffu, t[k], o);
  }
  // Lane 0 moves the warp's sums to the grid centre in float-float (integer
  // offsets |X|, |Y| <= 4096, so X^2 and 2X are exact and every product is
  // exact by two_prod): sum jx I = X A0 + AX1, sum jx^2 I = X^2 A0 + 2X AX1
  // + AX2, likewise in y.  FP64 runs at a small fraction of the FP32 rate on
  // this part, so it appears only in the five lanes that convert the CTA's
  // sums for the atomics.
  __shared__ FF part[5][kThreads / 32];
  if (lane == 0) {
    const int h = n >> 1;
    const float X = (float)((int)(blockIdx.x * kCols + 2 * threadIdx.x) - h);
    const float Y = (float)(r0 - h);
    part[0][w] = FF{t[0], 0.0f};
    part[1][w] = ff_fma(X, t[0], FF{t[1], 0.0f});
    part[2][w] = ff_fma(Y, t[0], FF{t[3], 0.0f});
    part[3][w] = ff_fma(X * X, t[0], ff_fma(2.0f * X, t[1], FF{t[2], 0.0f}));
    part[4][w] = ff_fma(Y * Y, t[0], ff_fma(2.0f * Y, t[3], FF{t[4], 0.0f}));
  }
  __syncthreads();
  if (threadIdx.x < 32) {
    __shared__ FF fin[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) {
      FF a = threadIdx.x < kThreads / 32 ? part[k][threadIdx.x] : FF{0.0f, 0.0f};
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const FF b = {__shfl_down_sync(0xffffffffu, a.hi, o),
                      __shfl_down_sync(0xffffffffu, a.lo, o)};
        a = ff_add(a, b);
      }
      if (threadIdx.x == 0) fin[k] = a;
    }
    __syncwarp();
    if (threadIdx.x < 5)
      atomicAdd(out + threadIdx.x, (double)fin[threadIdx.x].hi + (double)fin[threadIdx.x].lo);
  }
}

// Raw second moments about the grid centre -> about the centroid.
__global__ void moments_finish_kernel(double* out) {
  asm volatile("griddepcontrol.wait;" ::: "memory");
  const double m0 = out[0];
  if (m0 > 0.0) {
    out[3] -= out[1] * out[1] / m0;
    out[4] -= out[2] * out[2] / m0;
  }
}

int g_sms_metrics = 0;

}  // namespace

extern "C" lp_status lp_beam_moments(const lp_cfloat* field, int n, double* moments,
                                     void* stream) {
  using namespace lp;
  if (!lp_is_supported_n(n) || (n & 1))
    return (lp_status)set_last_error(
        LP_ERR_UNSUPPORTED_SIZE,
        "lp_beam_moments: npoints must be even and supported (the reference's index grid "
        "mgrid[-n//2:n//2] does not match an odd npoints)");
  if (!field || !moments)
    return (lp_status)set_last_error(LP_ERR_INVALID_ARGUMENT, "lp_beam_moments: NULL pointer");
  if ((reinterpret_cast<uintptr_t>(field) & 7u) || (reinterpret_cast<uintptr_t>(moments) & 7u))
    return (lp_status)set_last_error(LP_ERR_MISALIGNED, "lp_beam_moments: 8-byte alignment");
  if (!g_sms_metrics) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&g_sms_metrics, cudaDevAttrMultiProcessorCount, dev);
    if (g_sms_metrics <= 0) g_sms_metrics = 1;
  }
  // grid: column blocks of kCols x row runs, one wave of kCtasPerSm CTAs per
  // SM (the five FP64 atomics per CTA all land on the same 40 bytes, so few
  // CTAs)
  const int cb = (n + kCols - 1) / kCols;
  int rb = (kCtasPerSm * g_sms_metrics + cb - 1) / cb;
  if (rb > n) rb = n;
  const int rows = (n + rb - 1) / rb;
  rb = (n + rows - 1) / rows;
  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e = cudaMemsetAsync(moments, 0, 5 * sizeof(double), st);
  if (e == cudaSuccess) {
    const float2* f = reinterpret_cast<const float2*>(field);
    if ((reinterpret_cast<uintptr_t>(field) & 15u) == 0)
      moments_kernel<true><<<dim3(cb, rb), kThreads, 0, st>>>(f, n, rows, moments);
    else
      moments_kernel<false><<<dim3(cb, rb), kThreads, 0, st>>>(f, n, rows, moments);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(1);
    cfg.blockDim = dim3(1);
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    e = cudaLaunchKernelEx(&cfg, moments_finish_kernel, moments);
  }
  if (e != cudaSuccess)
    return (lp_status)set_last_error(LP_ERR_CUDA, cudaGetErrorString(e));
  return LP_OK;
}

// ------------------------------------------------------- intensity loss --
namespace {

constexpr int kLossThreads = 256;

__global__ void __launch_bounds__(kLossThreads) mse_sum_kernel(const float2* __restrict__ y,
                                                               const float* __restrict__ tg,
                                                               long long count, double* out) {
  float s = 0.0f;
  const long long stride = (long long)gridDim.x * kLossThreads;
  for (long long i = (long long)blockIdx.x * kLossThreads + threadIdx.x; i < count;
       i += 4 * stride) {
    float2 v[4];
    float t[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {  // four independent loads in flight
      const long long k = i + u * stride;
      v[u] = k < count ? __ldg(y + k) : make_float2(0.0f, 0.0f);
      t[u] = k < count ? __ldg(tg + k) : 0.0f;
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const float d = fmaf(v[u].x, v[u].x, fmaf(v[u].y, v[u].y, -t[u]));
      s = fmaf(d, d, s);
    }
  }
  // non-negative terms: FP32 warp sums, the CTA's warps in float-float, one
  // FP64 conversion for the atomic (FP64 runs at a small fraction of the
  // FP32 rate on this part)
  __shared__ float part[kLossThreads / 32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    FF a = {0.0f, 0.0f};
#pragma unroll
    for (int i = 0; i < kLossThreads / 32; ++i) a = ff_add(a, FF{part[i], 0.0f});
    atomicAdd(out, (double)a.hi + (double)a.lo);
  }
}

__global__ void __launch_bounds__(kLossThreads) mse_grad_kernel(
    const float2* __restrict__ y, const float* __restrict__ tg, long long count,
    const float* __restrict__ upstream, float scale, float2* __restrict__ g) {
  const float c = scale * __ldg(upstream);
  for (long long i = (long long)blockIdx.x * kLossThreads + threadIdx.x; i < count;
       i += (long long)gridDim.x * kLossThreads) {
    const float2 v = __ldg(y + i);
    const float d = fmaf(v.x, v.x, fmaf(v.y, v.y, -__ldg(tg + i))) * c;
    g[i] = make_float2(d * v.x, d * v.y);
  }
}

__global__ void __launch_bounds__(kLossThreads) phase_grad_kernel(
    const float2* __restrict__ x, const float2* __restrict__ g, long long count,
    float* __restrict__ out) {
  for (long long i = (long long)blockIdx.x * kLossThreads + threadIdx.x; i < count;
       i += (long long)gridDim.x * kLossThreads) {
    const float2 a = __ldg(x + i), b = __ldg(g + i);
    out[i] = fmaf(a.x, b.y, -a.y * b.x);  // Im(conj(a) * b)
  }
}

int loss_grid(long long count, int per_thread) {
  const long long want = (count + (long long)kLossThreads * per_thread - 1) /
                         ((long long)kLossThreads * per_thread);
  const long long cap = 8LL * (g_sms_metrics > 0 ? g_sms_metrics : 1);
  return (int)(want < 1 ? 1 : want < cap ? want : cap);
}

lp_status loss_args(const void* y, const void* target, long long count, const void* out) {
  using namespace lp;
  if (!y || !target || !out)
    return (lp_status)set_last_error(LP_ERR_INVALID_ARGUMENT, "intensity loss: NULL pointer");
  if (count < 1)
    return (lp_status)set_last_error(LP_ERR_INVALID_ARGUMENT, "intensity loss: count >= 1");
  if ((reinterpret_cast<uintptr_t>(y) & 7u) || (reinterpret_cast<uintptr_t>(target) & 3u) ||
      (reinterpret_cast<uintptr_t>(out) & 3u))
    return (lp_status)set_last_error(LP_ERR_MISALIGNED, "intensity loss: alignment");
  if (!g_sms_metrics) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&g_sms_metrics, cudaDevAttrMultiProcessorCount, dev);
    if (g_sms_metrics <= 0) g_sms_metrics = 1;
  }
  return LP_OK;
}

}  // namespace

extern "C" lp_status lp_intensity_mse(const lp_cfloat* y, const float* target, long long count,
                                      double* loss_sum, void* stream) {
  using namespace lp;
  lp_status s = loss_args(y, target, count, loss_sum);
  if (s != LP_OK) return s;
  if (reinterpret_cast<uintptr_t>(loss_sum) & 7u)
    return (lp_status)set_last_error(LP_ERR_MISALIGNED, "lp_intensity_mse: loss_sum alignment");
  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e = cudaMemsetAsync(loss_sum, 0, sizeof(double), st);
  if (e == cudaSuccess) {
    mse_sum_kernel<<<loss_grid(count, 4), kLossThreads, 0, st>>>(
        reinterpret_cast<const float2*>(y), target, count, loss_sum);
    e = cudaGetLastError();
  }
  return e == cudaSuccess ? LP_OK
                          : (lp_status)set_last_error(LP_ERR_CUDA, cudaGetErrorString(e));
}

extern "C" lp_status lp_intensity_mse_grad(const lp_cfloat* y, const float* target,
                                           long long count, const float* upstream, float scale,
                                           lp_cfloat* grad_y, void* stream) {
  using namespace lp;
  lp_status s = loss_args(y, target, count, grad_y);
  if (s != LP_OK) return s;
  if (!upstream || (reinterpret_cast<uintptr_t>(upstream) & 3u) ||
      (reinterpret_cast<uintptr_t>(grad_y) & 7u))
    return (lp_status)set_last_error(LP_ERR_INVALID_ARGUMENT,
                                     "lp_intensity_mse_grad: upstream / grad_y pointer");
  mse_grad_kernel<<<loss_grid(count, 1), kLossThreads, 0, (cudaStream_t)stream>>>(
      reinterpret_cast<const float2*>(y), target, count, upstream, scale,
      reinterpret_cast<float2*>(grad_y));
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? LP_OK
                          : (lp_status)set_last_error(LP_ERR_CUDA, cudaGetErrorString(e));
}

extern "C" lp_status lp_phase_grad(const lp_cfloat* x, const lp_cfloat* g, long long count,
                                   float* out, void* stream) {
  using namespace lp;
  lp_status s = loss_args(x, out, count, out);
  if (s != LP_OK) return s;
  if (!g || (reinterpret_cast<uintptr_t>(g) & 7u))
    return (lp_status)set_last_error(LP_ERR_INVALID_ARGUMENT, "lp_phase_grad: g pointer");
  phase_grad_kernel<<<loss_grid(count, 1), kLossThreads, 0, (cudaStream_t)stream>>>(
      reinterpret_cast<const float2*>(x), reinterpret_cast<const float2*>(g), count, out);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? LP_OK
                          : (lp_status)set_last_error(LP_ERR_CUDA, cudaGetErrorString(e));
}
