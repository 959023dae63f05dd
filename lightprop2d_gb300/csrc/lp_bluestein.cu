// Transforms and pointwise passes for grid sizes that the power-of-two pass
// kernels do not cover: any npoints from 2 to 4096 that is not a power of two
// in 16..8192 (the reference accepts any npoints; its FFT library does the
// rest, beam2d.py:207-229).
//
// Bluestein's algorithm (chirp z-transform).  With w[j] = exp(-i*pi*j^2/n),
//     X[k] = sum_j x[j] exp(-2*pi*i*j*k/n) = w[k] * sum_j (x[j] w[j]) conj(w[k-j]),
// a linear convolution of x*w with conj(w), evaluated as a circular
// convolution of length M (a power of two >= 2n-1).  In 2-D both axes
// separate, so the 2-D convolution kernel's spectrum is Bv[k1]*Bv[k2] with
// Bv = FFT_M(b), b = conj(w) wrapped onto M points.  One n x n transform is
//   pad:    y[j1,j2] = x[j1,j2] w[j1] w[j2] on an M x M grid (zero elsewhere)
//   the power-of-two fused passes on y with the separable complex k-domain
//           multiplier Bv (x) Bv / M^2 (forward rows, forward columns x
//           multiplier, inverse columns, inverse rows: a circular convolution)
//   crop:   X[k1,k2] = y[k1,k2] w[k1] w[k2] * scale
// The inverse transform uses conj(w) and FFT_M(conj(b)).  The chirp and both
// kernel spectra are computed once per (device, n) on the host in double
// precision (chirp phases reduced exactly: j^2 mod 2n) and rounded once.
#include <cuda_runtime.h>

#include <cmath>
#include <complex>
#include <map>
#include <mutex>
#include <utility>
#include <vector>

#include "lightprop2d_gb300.h"
#include "lp_fft_core.cuh"

namespace lp {
namespace {

constexpr int kMaxM = 8192;

struct BlueTables {
  float2* chirp = nullptr;  // w[0..n)
  float2* kfwd = nullptr;   // Bv[0..M), Bv[0..M): an LP_MASK_SEP_C64 table
  float2* kinv = nullptr;   // the same for the inverse transform
  int m = 0;
};

std::mutex g_blue_mu;
std::map<std::pair<int, int>, BlueTables> g_blue;  // (device, n)

// In-place radix-2 FFT of length m (power of two), sign -1 (forward).
void host_fft(std::vector<std::complex<double>>& a) {
  const int m = (int)a.size();
  for (int i = 1, j = 0; i < m; ++i) {
    int bit = m >> 1;
    for (; j & bit; bit >>= 1) j ^= bit;
    j ^= bit;
    if (i < j) std::swap(a[i], a[j]);
  }
  for (int len = 2; len <= m; len <<= 1) {
    for (int i = 0; i < m; i += len)
      for (int k = 0; k < len / 2; ++k) {
        const double ang = -2.0 * kPi * k / len;
        const std::complex<double> w(std::cos(ang), std::sin(ang));
        const std::complex<double> u = a[i + k], v = a[i + k + len / 2] * w;
        a[i + k] = u + v;
        a[i + k + len / 2] = u - v;
      }
  }
}

cudaError_t build_tables(int n, BlueTables* t) {
  const int m = bluestein_m(n);
  std::vector<std::complex<double>> w(n);
  for (int j = 0; j < n; ++j) {
    const long long r = ((long long)j * j) % (2LL * n);  // exact: w has period 2n in j^2
    const double ang = -kPi * (double)r / (double)n;
    w[j] = std::complex<double>(std::cos(ang), std::sin(ang));
  }
  std::vector<std::complex<double>> bf(m, 0.0), bi(m, 0.0);
  for (int j = 0; j < n; ++j) {
    bf[j] = std::conj(w[j]);
    bi[j] = w[j];
    if (j > 0) {
      bf[m - j] = std::conj(w[j]);
      bi[m - j] = w[j];
    }
  }
  host_fft(bf);
  host_fft(bi);
  std::vector<float2> h((size_t)n + 4 * (size_t)m);
  for (int j = 0; j < n; ++j) h[j] = make_float2((float)w[j].real(), (float)w[j].imag());
  for (int k = 0; k < m; ++k) {
    const float2 f = make_float2((float)bf[k].real(), (float)bf[k].imag());
    const float2 g = make_float2((float)bi[k].real(), (float)bi[k].imag());
    h[n + k] = h[n + m + k] = f;
    h[n + 2 * m + k] = h[n + 3 * m + k] = g;
  }
  float2* d = nullptr;
  cudaError_t e = cudaMalloc(&d, h.size() * sizeof(float2));
  if (e != cudaSuccess) return e;
  e = cudaMemcpy(d, h.data(), h.size() * sizeof(float2), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    cudaFree(d);
    return e;
  }
  t->chirp = d;
  t->kfwd = d + n;
  t->kinv = d + n + 2 * m;
  t->m = m;
  return cudaSuccess;
}

__global__ void blue_pad_kernel(const float2* __restrict__ in, int n, float2* __restrict__ ws,
                                int logm, const float2* __restrict__ chirp, int conj) {
  const int m = 1 << logm;
  const int total = m * m;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
    const int r = i >> logm, c = i & (m - 1);
    float2 v = make_float2(0.0f, 0.0f);
    if (r < n && c < n) {
      float2 w = cmul(__ldg(chirp + r), __ldg(chirp + c));
      if (conj) w = cconj(w);
      v = cmul(in[(size_t)r * n + c], w);
    }
    ws[i] = v;
  }
}

__global__ void blue_crop_kernel(const float2* __restrict__ ws, int logm, float2* __restrict__ out,
                                 int n, const float2* __restrict__ chirp, int conj, float scale) {
  const int total = n * n;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
    const int r = i / n, c = i - r * n;
    float2 w = cmul(__ldg(chirp + r), __ldg(chirp + c));
    if (conj) w = cconj(w);
    out[i] = cscale(cmul(ws[((size_t)r << logm) + c], w), scale);
  }
}

// x-domain multiplier (lens phase and/or mask, conjugated for the adjoint)
// at every point, out of place.  The grid centre is the reference's:
// X = arange(-n//2, n//2) * dL, so jx = x - (n+1)/2 for any n.
__global__ void generic_xmul_kernel(const float2* __restrict__ in, float2* __restrict__ out, int n,
                                    RowOps ops) {
  const int total = n * n, h = (n + 1) / 2;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
    const int y = i / n, x = i - y * n;
    float2 m = make_float2(1.0f, 0.0f);
    if (ops.lens) {
      const int jx = x - h, jy = y - h;
      m = cis_cycles(lens_cycles(ops.kap_hi, ops.kap_lo, jx * jx + jy * jy), 1.0f);
    }
    if (ops.xmask) m = cmul(m, mask_value_xy(ops.xmask, ops.xmask_type, y, x, n));
    if (ops.conj) m = cconj(m);
    out[i] = cmul(in[i], m);
  }
}

// Spectral multipliers at every point of an unshifted spectrum (fftfreq
// order: index k holds k for k < (n+1)/2, k - n above): H(z) (with the d/dz
// factor, evanescent rule and adjoint conjugation of ColOps), the k-domain
// mask, the optional spectrum write (before the scale) and the scale.
__global__ void generic_spectral_kernel(const float2* __restrict__ in, float2* __restrict__ out,
                                        int n, ColOps ops) {
  const int total = n * n, h = (n + 1) / 2;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
    const int ky = i / n, kx = i - ky * n;
    float2 v = in[i];
    if (ops.apply_h || ops.kmask) {
      float2 m = make_float2(1.0f, 0.0f);
      if (ops.apply_h) {
        const int sx = kx < h ? kx : kx - n, sy = ky < h ? ky : ky - n;
        const float qx = (float)(sx * sx), qy = (float)(sy * sy);
        float a_hi = 0.0f, a_lo = 0.0f;
        if (!ops.phase_fp32) column_constant(ops.kp, qx, a_hi, a_lo);
        m = transfer_value_cc<0>(qx, a_hi, a_lo, qy, ops);
      }
      if (ops.kmask) {
        float2 km = mask_value_xy(ops.kmask, ops.kmask_type, ky, kx, n);
        if (ops.conj) km = cconj(km);
        m = cmul(m, km);
      }
      v = cmul(v, m);
    }
    if (ops.spectrum_out) ops.spectrum_out[i] = v;
    out[i] = ops.scale != 1.0f ? cscale(v, ops.scale) : v;
  }
}

int ew_blocks(long long total) {
  const long long b = (total + 255) / 256;
  return (int)(b > 152 * 16 ? 152 * 16 : (b ? b : 1));
}

}  // namespace

bool bluestein_n(int n) { return n >= 2 && 2 * n - 1 <= kMaxM && !size_ops(n); }

int bluestein_m(int n) {
  int m = 16;
  while (m < 2 * n - 1) m <<= 1;
  return m;
}

cudaError_t bluestein_dft2(const float2* in, float2* out, int n, int inverse, float scale,
                           float2* ws, cudaStream_t st) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  BlueTables t;
  {
    std::lock_guard<std::mutex> lk(g_blue_mu);
    auto it = g_blue.find({dev, n});
    if (it == g_blue.end()) {
      // first transform of this size on this device: host set-up (copies)
      // that a stream capture must not contain
      cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
      e = cudaStreamIsCapturing(st, &cs);
      if (e != cudaSuccess) return e;
      if (cs != cudaStreamCaptureStatusNone) return cudaErrorStreamCaptureUnsupported;
      e = build_tables(n, &t);
      if (e != cudaSuccess) return e;
      g_blue[{dev, n}] = t;
    } else {
      t = it->second;
    }
  }
  const int m = t.m;
  int logm = 0;
  while ((1 << logm) < m) ++logm;
  const SizeOps* so = size_ops(m);
  blue_pad_kernel<<<ew_blocks((long long)m * m), 256, 0, st>>>(in, n, ws, logm, t.chirp, inverse);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  ColOps c = col_ops_none();
  c.kmask = inverse ? t.kinv : t.kfwd;
  c.kmask_type = LP_MASK_SEP_C64;
  c.scale = 1.0f / ((float)m * (float)m);
  e = so->row(0, ws, ws, row_ops_none(), st);
  if (e == cudaSuccess) e = so->col(COL_FUSED, ws, ws, c, st);
  if (e == cudaSuccess) e = so->row(1, ws, ws, row_ops_none(), st);
  if (e != cudaSuccess) return e;
  blue_crop_kernel<<<ew_blocks((long long)n * n), 256, 0, st>>>(ws, logm, out, n, t.chirp, inverse,
                                                                 scale);
  return cudaGetLastError();
}

cudaError_t generic_xmul(const float2* in, float2* out, int n, const RowOps& ops,
                         cudaStream_t st) {
  generic_xmul_kernel<<<ew_blocks((long long)n * n), 256, 0, st>>>(in, out, n, ops);
  return cudaGetLastError();
}

cudaError_t generic_spectral(const float2* in, float2* out, int n, const ColOps& ops,
                             cudaStream_t st) {
  generic_spectral_kernel<<<ew_blocks((long long)n * n), 256, 0, st>>>(in, out, n, ops);
  return cudaGetLastError();
}

void bluestein_release() {
  std::lock_guard<std::mutex> lk(g_blue_mu);
  int prev = 0;
  cudaGetDevice(&prev);
  for (auto& kv : g_blue) {
    cudaSetDevice(kv.first.first);
    cudaFree(kv.second.chirp);
  }
  g_blue.clear();
  cudaSetDevice(prev);
}

}  // namespace lp
