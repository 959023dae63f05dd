// Intensity moments of a field for Beam2D.centroid / D4sigma /
// centroid_intensity (beam2d.py:669-752): two read-only passes over the grid.
//
//   pass 1:  m0 = sum I,  m1 = sum jx*I,  m2 = sum jy*I
//   pass 2:  m3 = sum (jx - xc)^2 I,  m4 = sum (jy - yc)^2 I,
//            xc = m1/m0, yc = m2/m0 read from pass 1's result on the device
//
// with I = |field|^2 and jx = ix - n/2, jy = iy - n/2 (grid-index offsets
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
                                                            int logn, double* out) {
  // let the second pass's CTAs be scheduled as this pass's CTAs retire
  asm volatile("griddepcontrol.launch_dependents;");
  const int n = 1 << logn, h = n >> 1;
  const int n2 = n * n;
  const int stride = (int)gridDim.x * kThreads;
  const int first = (int)blockIdx.x * kThreads + (int)threadIdx.x;
  const float jx = (float)((first & (n - 1)) - h);
  const float djy = (float)(stride >> logn);
  float jy = (float)((first >> logn) - h);
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
                                                            int logn, double* out) {
  const int n = 1 << logn, h = n >> 1;
  const int n2 = n * n;
  const int stride = (int)gridDim.x * kThreads;
  const int first = (int)blockIdx.x * kThreads + (int)threadIdx.x;
  // launched with programmatic dependent launch: wait for pass 1's sums
  asm volatile("griddepcontrol.wait;" ::: "memory");
  const double m0 = out[0];
  const float xc = m0 > 0.0 ? (float)(out[1] / m0) : 0.0f;
  const float yc = m0 > 0.0 ? (float)(out[2] / m0) : 0.0f;
  const float dx = (float)((first & (n - 1)) - h) - xc;
  const float ddy = (float)(stride >> logn);
  float dy = (float)((first >> logn) - h) - yc;
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
  if (!lp_is_supported_n(n))
    return (lp_status)set_last_error(LP_ERR_UNSUPPORTED_SIZE,
                                     "lp_beam_moments: npoints must be a power of two in 16..4096");
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
  int logn = 0;
  while ((1 << logn) < n) ++logn;
  // grid: about one CTA per SM (fewer for small grids), a multiple of
  // mult = n / 1024 when n > 1024 so that the stride (grid * 1024 points) is
  // a multiple of n.
  const int n2 = n * n;
  const int want = (n2 + kThreads * kUnroll - 1) / (kThreads * kUnroll);
  const int mult = n > kThreads ? n / kThreads : 1;
  int grid = want < g_sms_metrics ? want : g_sms_metrics;
  grid = grid / mult * mult;
  if (grid < mult) grid = mult;
  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e = cudaMemsetAsync(moments, 0, 5 * sizeof(double), st);
  if (e == cudaSuccess) {
    moments1_kernel<<<grid, kThreads, 0, st>>>(reinterpret_cast<const float2*>(field), logn,
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
    e = cudaLaunchKernelEx(&cfg, moments2_kernel, reinterpret_cast<const float2*>(field), logn,
                           moments);
  }
  if (e != cudaSuccess)
    return (lp_status)set_last_error(LP_ERR_CUDA, cudaGetErrorString(e));
  return LP_OK;
}
