// Grid management of Beam2D (beam2d.py:375-460): expand (edge-replicated
// padding), coarse (block mean) and crop (linear resampling of a central
// window onto a new grid).  Each is one gather kernel over the output grid;
// the caller recomputes the spectrum with lp_fft2, as the reference does.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>

#include "lightprop2d_gb300.h"
#include "lp_internal.h"

using namespace lp;

namespace {

constexpr int kThreads = 256;

lp_status fail(lp_status s, const char* msg) { return (lp_status)set_last_error((int)s, msg); }

bool aligned8(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 7u) == 0; }

// CTAs for kernels that loop over output rows: per_sm per SM, at most one
// per row (the crop kernel's per-CTA column table is amortised over the CTA's
// rows, so it takes fewer CTAs than the plain copy).
int g_sms_grid = 0;
int rows_grid(int rows, int per_sm) {
  if (!g_sms_grid) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&g_sms_grid, cudaDevAttrMultiProcessorCount, dev);
    if (g_sms_grid <= 0) g_sms_grid = 1;
  }
  const int g = per_sm * g_sms_grid;
  return rows < g ? rows : g;
}

int grid_for(size_t points) {
  const size_t g = (points + kThreads - 1) / kThreads;
  return (int)(g < 65535u * 64u ? g : 65535u * 64u);
}

// out[y][x] = in[clamp(y - d)][clamp(x - d)] (beam2d.py:386-402).  A CTA
// copies whole output rows (rows blockIdx.x, += gridDim.x), four points per
// thread in flight.
__global__ void __launch_bounds__(kThreads) expand_kernel(const float2* __restrict__ in,
                                                          int n_in, float2* __restrict__ out,
                                                          int n_out, int d) {
  for (int y = blockIdx.x; y < n_out; y += gridDim.x) {
    const int sy = min(max(y - d, 0), n_in - 1);
    const float2* src = in + (size_t)sy * n_in;
    float2* dst = out + (size_t)y * n_out;
    for (int x0 = threadIdx.x; x0 < n_out; x0 += 4 * kThreads) {
      float2 v[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int x = x0 + u * kThreads;
        v[u] = x < n_out ? __ldg(src + min(max(x - d, 0), n_in - 1)) : make_float2(0.0f, 0.0f);
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int x = x0 + u * kThreads;
        if (x < n_out) dst[x] = v[u];
      }
    }
  }
}

// Mean over order x order blocks (beam2d.py:455-459).
__global__ void coarse_kernel(const float2* __restrict__ in, int n_in, float2* __restrict__ out,
                              int order) {
  const int n_out = n_in / order;
  const size_t total = (size_t)n_out * n_out;
  const float inv = 1.0f / ((float)order * (float)order);
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total;
       i += (size_t)gridDim.x * blockDim.x) {
    const int y = (int)(i / n_out), x = (int)(i % n_out);
    if (order == 2) {  // the common case: four independent loads
      const float2* r0 = in + (size_t)(2 * y) * n_in + (size_t)x * 2;
      const float2* r1 = r0 + n_in;
      const float2 a = __ldg(r0), b = __ldg(r0 + 1), c = __ldg(r1), d = __ldg(r1 + 1);
      out[i] = make_float2(((a.x + b.x) + (c.x + d.x)) * inv, ((a.y + b.y) + (c.y + d.y)) * inv);
      continue;
    }
    float2 s = make_float2(0.0f, 0.0f);
    for (int a = 0; a < order; ++a) {
      const float2* row = in + (size_t)(y * order + a) * n_in + (size_t)x * order;
      for (int b = 0; b < order; ++b) {
        s.x += row[b].x;
        s.y += row[b].y;
      }
    }
    out[i] = make_float2(s.x * inv, s.y * inv);
  }
}

// Position of output index j on the input window axis, in window points:
// p = (j - n_out/2) * ratio - offset, evaluated in float-float so the
// interpolation weight is exact to FP32 for any grid size.
__device__ __forceinline__ void axis_pos(int j, int half, float r_hi, float r_lo, float o_hi,
                                         float o_lo, int n_keep, int& i0, float& w) {
  const float jj = (float)(j - half);
  float p_hi, p_e;
  two_prod(jj, r_hi, p_hi, p_e);
  float s, e;
  two_sum(p_hi, -o_hi, s, e);
  const float lo = e + fmaf(jj, r_lo, p_e) - o_lo;
  // nearest-point extrapolation outside the window, linear inside
  if (!(s > -1.0f)) {
    i0 = 0;
    w = 0.0f;
    return;
  }
  if (!(s < (float)n_keep)) {
    i0 = n_keep - 1;
    w = 0.0f;
    return;
  }
  const float fl = floorf(s);
  float frac = (s - fl) + lo;
  int i = (int)fl;
  if (frac >= 1.0f) { i += 1; frac -= 1.0f; }
  if (frac < 0.0f) { i -= 1; frac += 1.0f; }
  if (i < 0) { i = 0; frac = 0.0f; }
  if (i >= n_keep - 1) { i = n_keep - 1; frac = 0.0f; }
  i0 = i;
  w = frac;
}

// A CTA owns a kThreads-wide column strip and a run of at most kMaxRun
// output rows: a thread finds its column's window position once, the CTA's
// row positions go to shared memory, and each thread blends four rows per
// iteration (16 gathers in flight), so a point costs four gathers and a
// bilinear blend.
constexpr int kMaxOut = 8192;  // the largest grid the transforms take
constexpr int kMaxRun = 64;
constexpr int kCropRows = 4;

__global__ void __launch_bounds__(kThreads) crop_kernel(const float2* __restrict__ in, int n_in,
                                                        int k0, int n_keep,
                                                        float2* __restrict__ out, int n_out,
                                                        int run, float r_hi, float r_lo,
                                                        float o_hi, float o_lo) {
  __shared__ int s_iy[kMaxRun];
  __shared__ float s_wy[kMaxRun];
  const int half = n_out / 2;
  const int y0 = blockIdx.y * run, y1 = min(n_out, y0 + run);
  if ((int)threadIdx.x < y1 - y0)
    axis_pos(y0 + threadIdx.x, half, r_hi, r_lo, o_hi, o_lo, n_keep, s_iy[threadIdx.x],
             s_wy[threadIdx.x]);
  const int x = blockIdx.x * kThreads + threadIdx.x;
  const int xc = min(x, n_out - 1);
  int ix;
  float wx;
  axis_pos(xc, half, r_hi, r_lo, o_hi, o_lo, n_keep, ix, wx);
  const int ix1 = min(ix + 1, n_keep - 1);
  const float ux = 1.0f - wx;
  const float2* win = in + (size_t)k0 * n_in + k0;
  __syncthreads();
  for (int y = y0; y < y1; y += kCropRows) {
    float2 a[kCropRows], b[kCropRows], c[kCropRows], d[kCropRows];
#pragma unroll
    for (int u = 0; u < kCropRows; ++u) {
      const int k = min(y + u, y1 - 1) - y0;
      const int iy = s_iy[k], iy1 = min(iy + 1, n_keep - 1);
      const float2* r0 = win + (size_t)iy * n_in;
      const float2* r1 = win + (size_t)iy1 * n_in;
      a[u] = __ldg(r0 + ix);
      b[u] = __ldg(r0 + ix1);
      c[u] = __ldg(r1 + ix);
      d[u] = __ldg(r1 + ix1);
    }
#pragma unroll
    for (int u = 0; u < kCropRows; ++u) {
      if (x < n_out && y + u < y1) {
        const float wy = s_wy[y + u - y0], uy = 1.0f - wy;
        out[(size_t)(y + u) * n_out + x] =
            make_float2(uy * (ux * a[u].x + wx * b[u].x) + wy * (ux * c[u].x + wx * d[u].x),
                        uy * (ux * a[u].y + wx * b[u].y) + wy * (ux * c[u].y + wx * d[u].y));
      }
    }
  }
}

lp_status launch_check(const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(LP_ERR_CUDA, cudaGetErrorString(e));
  (void)what;
  return LP_OK;
}

}  // namespace

extern "C" {

lp_status lp_expand(const lp_cfloat* in, int n_in, lp_cfloat* out, int n_out, void* stream) {
  if (!in || !out) return fail(LP_ERR_INVALID_ARGUMENT, "lp_expand: NULL pointer");
  if (!aligned8(in) || !aligned8(out)) return fail(LP_ERR_MISALIGNED, "lp_expand: 8-byte alignment");
  if (n_in < 1 || n_out < n_in || ((n_out - n_in) & 1))
    return fail(LP_ERR_INVALID_ARGUMENT, "lp_expand: need n_out >= n_in with an even difference");
  if ((const void*)in == (const void*)out && n_out != n_in)
    return fail(LP_ERR_INVALID_ARGUMENT, "lp_expand: in and out must be different grids");
  expand_kernel<<<rows_grid(n_out, 8), kThreads, 0, (cudaStream_t)stream>>>(
      reinterpret_cast<const float2*>(in), n_in, reinterpret_cast<float2*>(out), n_out,
      (n_out - n_in) / 2);
  return launch_check("lp_expand");
}

lp_status lp_coarse(const lp_cfloat* in, int n_in, lp_cfloat* out, int order, void* stream) {
  if (!in || !out) return fail(LP_ERR_INVALID_ARGUMENT, "lp_coarse: NULL pointer");
  if (!aligned8(in) || !aligned8(out)) return fail(LP_ERR_MISALIGNED, "lp_coarse: 8-byte alignment");
  if (order < 1 || n_in < order || n_in % order)
    return fail(LP_ERR_INVALID_ARGUMENT, "lp_coarse: order must divide n_in");
  if ((const void*)in == (const void*)out && order != 1)
    return fail(LP_ERR_INVALID_ARGUMENT, "lp_coarse: in and out must be different grids");
  const int n_out = n_in / order;
  coarse_kernel<<<grid_for((size_t)n_out * n_out), kThreads, 0, (cudaStream_t)stream>>>(
      reinterpret_cast<const float2*>(in), n_in, reinterpret_cast<float2*>(out), order);
  return launch_check("lp_coarse");
}

lp_status lp_crop(const lp_cfloat* in, int n_in, int first, int n_keep, double x0, double dL_in,
                  lp_cfloat* out, int n_out, double dL_out, void* stream) {
  if (!in || !out) return fail(LP_ERR_INVALID_ARGUMENT, "lp_crop: NULL pointer");
  if (!aligned8(in) || !aligned8(out)) return fail(LP_ERR_MISALIGNED, "lp_crop: 8-byte alignment");
  if (n_keep < 1 || first < 0 || first + n_keep > n_in || n_out < 1)
    return fail(LP_ERR_INVALID_ARGUMENT, "lp_crop: window outside the input grid");
  if (!(dL_in > 0) || !std::isfinite(dL_out) || dL_out == 0.0 || !std::isfinite(x0))
    return fail(LP_ERR_INVALID_ARGUMENT, "lp_crop: dL_in > 0 and finite, non-zero dL_out");
  if ((const void*)in == (const void*)out)
    return fail(LP_ERR_INVALID_ARGUMENT, "lp_crop: in and out must be different grids");
  if (n_out > kMaxOut) return fail(LP_ERR_UNSUPPORTED_SIZE, "lp_crop: n_out <= 8192");
  const FF r = ff_from_double(dL_out / dL_in);
  const FF o = ff_from_double(x0 / dL_in);
  // strips x row runs: about six CTAs per SM, runs of at most kMaxRun rows
  const int strips = (n_out + kThreads - 1) / kThreads;
  int runs = (rows_grid(1 << 30, 6) + strips - 1) / strips;
  if (runs > n_out) runs = n_out;
  int run = (n_out + runs - 1) / runs;
  if (run > kMaxRun) run = kMaxRun;
  runs = (n_out + run - 1) / run;
  crop_kernel<<<dim3(strips, runs), kThreads, 0, (cudaStream_t)stream>>>(
      reinterpret_cast<const float2*>(in), n_in, first, n_keep, reinterpret_cast<float2*>(out),
      n_out, run, r.hi, r.lo, o.hi, o.lo);
  return launch_check("lp_crop");
}

}  // extern "C"
