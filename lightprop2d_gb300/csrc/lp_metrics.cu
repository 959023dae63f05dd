// Intensity moments of a field for Beam2D.centroid / D4sigma /
// centroid_intensity (beam2d.py:669-752): two read-only passes over the grid.
//
//   pass 1:  m0 = sum I,  m1 = sum jx*I,  m2 = sum jy*I
//   pass 2:  m3 = sum (jx - xc)^2 I,  m4 = sum (jy - yc)^2 I,
//            xc = m1/m0, yc = m2/m0 read from pass 1's result on the device
//
// with I = |field|^2 and jx = ix - n/2, jy = iy - n/2 (n even; grid-index offsets
// from the centre; the caller scales by dL).  The second moments are taken
// about the centroid, as the reference does, so an off-centre beam loses no
// precision to cancellation.  Each thread accumulates in FP32 over a strided
// share of the grid (8 loads in flight, tens of points), then warps and CTAs
// reduce in FP64 and one atomicAdd per CTA lands in the 5-double result.
#include <cuda_runtime.h>

#include <cstdint>

#include "lightprop2d_gb300.h"
#include "lp_internal.h"

namespace {

// One 1024-thread CTA per SM with 16 loads in flight per thread keeps ~20 MB
// in flight on GB300 (a 2048^2 grid in two round trips); few CTAs keep the
// final FP64 atomics (3 per CTA onto the same 40 bytes) from contending.
constexpr int kThreads = 1024;
constexpr int kUnroll = 16;  // loads in flight per thread

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// v[u] = f[i0 + u*stride] (0 past n2), all kUnroll loads issued before any
// is used.
__device__ __forceinline__ void load_block(float2 (&v)[kUnroll], const float2* __restrict__ f,
                                           int i0, int stride, int n2) {
  if (i0 + (kUnroll - 1) * stride < n2) {
#pragma unroll
    for (int u = 0; u < kUnroll; ++u) v[u] = __ldg(f + i0 + u * stride);
  } else {
#pragma unroll
    for (int u = 0; u < kUnroll; ++u) {
      const int i = i0 + u * stride;
      v[u] = i < n2 ? __ldg(f + i) : make_float2(0.0f, 0.0f);
    }
  }
}

// Adds v[0..K) over the CTA into out[0..K) (one atomicAdd per value per CTA).
template <int K>
__device__ __forceinline__ void cta_add(const float (&v)[K], double* out) {
  __shared__ double part[K][kThreads / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < K; ++k) {
    const double s = warp_sum((double)v[k]);
    if (lane == 0) part[k][w] = s;
  }
  __syncthreads();
  if (threadIdx.x < 32) {
#pragma unroll
    for (int k = 0; k < K; ++k) {
      double s = threadIdx.x < kThreads / 32 ? part[k][threadIdx.x] : 0.0;
      s = warp_sum(s);
      if (threadIdx.x == 0) atomicAdd(out + k, s);
    }
  }
}

// The launch makes the grid stride (gridDim.x * kThreads points) a multiple
// of n, so a thread's points all lie in one column: its jx is a constant
// (sum jx I = jx * sum I) and jy advances by stride / n rows per step.
__global__ void __launch_bounds__(kThreads) moments1_kernel(const float2* __restrict__ f,
                                                            int n, double* out) {
  // let the second pass's CTAs be scheduled as this pass's CTAs retire
  asm volatile("griddepcontrol.launch_dependents;");
  const int h = n >> 1;
  const int n2 = n * n;
  const int stride = (int)gridDim.x * kThreads;
  const int first = (int)blockIdx.x * kThreads + (int)threadIdx.x;
  const float jx = (float)((first % n) - h);
  const float djy = (float)(stride / n);
  float jy = (float)((first / n) - h);
  float s0 = 0.0f, s2 = 0.0f;
  for (int i0 = first; i0 < n2; i0 += kUnroll * stride) {
    float2 v[kUnroll];
    load_block(v, f, i0, stride, n2);
#pragma unroll
    for (int u = 0; u < kUnroll; ++u) {
      const float I = fmaf(v[u].x, v[u].x, v[u].y * v[u].y);
      s0 += I;
      s2 = fmaf(fmaf((float)u, djy, jy), I, s2);
    }
    jy = fmaf((float)kUnroll, djy, jy);
  }
  const float s[3] = {s0, jx * s0, s2};
  cta_add<3>(s, out);
}

__global__ void __launch_bounds__(kThreads) moments2_kernel(const float2* __restrict__ f,
                                                            int n, double* out) {
  const int h = n >> 1;
  const int n2 = n * n;
  const int stride = (int)gridDim.x * kThreads;
  const int first = (int)blockIdx.x * kThreads + (int)threadIdx.x;
  // launched with programmatic dependent launch: wait for pass 1's sums
  asm volatile("griddepcontrol.wait;" ::: "memory");
  const double m0 = out[0];
  const float xc = m0 > 0.0 ? (float)(out[1] / m0) : 0.0f;
  const float yc = m0 > 0.0 ? (float)(out[2] / m0) : 0.0f;
  const float dx = (float)((first % n) - h) - xc;
  const float ddy = (float)(stride / n);
  float dy = (float)((first / n) - h) - yc;
  float s0 = 0.0f, s1 = 0.0f;
  for (int i0 = first; i0 < n2; i0 += kUnroll * stride) {
    float2 v[kUnroll];
    load_block(v, f, i0, stride, n2);
#pragma unroll
    for (int u = 0; u < kUnroll; ++u) {
      const float I = fmaf(v[u].x, v[u].x, v[u].y * v[u].y);
      const float d = fmaf((float)u, ddy, dy);
      s0 += I;
      s1 = fmaf(d * d, I, s1);
    }
    dy = fmaf((float)kUnroll, ddy, dy);
  }
  const float s[2] = {dx * dx * s0, s1};
  cta_add<2>(s, out + 3);
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
  // grid: about one CTA per SM (fewer for small grids), a multiple of
  // mult = n / gcd(n, 1024) so that the stride (grid * 1024 points) is a
  // multiple of n.
  const int n2 = n * n;
  const int want = (n2 + kThreads * kUnroll - 1) / (kThreads * kUnroll);
  int g = n, b = kThreads;
  while (b) {
    const int r = g % b;
    g = b;
    b = r;
  }
  const int mult = n / g;
  int grid = want < g_sms_metrics ? want : g_sms_metrics;
  grid = grid / mult * mult;
  if (grid < mult) grid = mult;
  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e = cudaMemsetAsync(moments, 0, 5 * sizeof(double), st);
  if (e == cudaSuccess) {
    moments1_kernel<<<grid, kThreads, 0, st>>>(reinterpret_cast<const float2*>(field), n,
                                               moments);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(kThreads);
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    e = cudaLaunchKernelEx(&cfg, moments2_kernel, reinterpret_cast<const float2*>(field), n,
                           moments);
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
  __shared__ double part[kLossThreads / 32];
  double a = warp_sum((double)s);
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = a;
  __syncthreads();
  if (threadIdx.x < 32) {
    a = threadIdx.x < kLossThreads / 32 ? part[threadIdx.x] : 0.0;
    a = warp_sum(a);
    if (threadIdx.x == 0) atomicAdd(out, a);
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
