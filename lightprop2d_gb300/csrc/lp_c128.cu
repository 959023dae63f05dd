// complex128 path: the reference's default precision (complex_bits=128,
// beam2d.py:88, :112-113), with results that agree with its numpy complex128
// path to ~1e-14, not just to complex64's ~1e-7.
//
// GB300 runs FP64 at a small fraction of its FP32 rate, so the transforms
// carry each complex128 value through the line passes as float-float pairs
// (value = hi + lo per component, 48 significant bits) and run on the FP32
// pipes.  Error-free transformations build the arithmetic: Knuth's two-sum,
// the FMA two-product and Dekker's fast two-sum.  What must match the
// reference bit for bit stays FP64: the transfer function's Kz and its
// phase trunc(Kz z) - Kz z (a one-ulp difference in Kz z moves the phase by
// ~1e-11 at z = 1 cm), the lens phase and the masks.  Conversions between
// double and float-float use integer bit operations, not FP64 instructions.
// Magnitudes below ~2^-100 lose their low half and below 2^-126 flush to
// zero (FP32's exponent range).
//
// A 2-D transform is a line pass over rows and a line pass over columns.  A
// line pass holds whole lines in shared memory (N <= 8192: at most 128 KB)
// and transforms them with a Stockham sequence of radix-4 stages (one
// radix-2 stage first when log2 N is odd): each thread keeps 8 points in
// registers between the read and write halves of a stage, so the line is
// transformed in place (8 rather than 16 points a thread: 64 registers, four
// 256-thread CTAs per SM; 0.44 against 0.52 ms per 2048^2 propagate, and 4
// points a thread measured 0.49).  A column pass takes two adjacent columns
// per CTA, so a warp's loads cover whole 32-byte sectors, and reads the grid
// in place; at 8192 (two lines would need 2048 threads) the grid is
// transposed in place around a row pass instead.  Stage twiddles come from a
// per-size table W_N^k (k < N) computed on the host in double and split into
// float-float.  Intermediate grids between the passes hold float-float
// values (16 bytes a point, like a complex128); the first pass reads the
// caller's complex128 and the last writes complex128.
//
// A propagate is
//   rows:     [x-domain multipliers] forward FFT
//   columns:  forward FFT, H(z) = exp(2*pi*i*(trunc(Kz z) - Kz z)) with Kz in
//             float64 exactly as beam2d.py:305-308 and :485-489 compute it
//             (once per |ky|: H(kx, ky) = H(kx, -ky)), k-domain mask, 1/N^2,
//             inverse FFT
//   rows:     inverse FFT, |field|^2 epilogue (float64)
// and a propagate of a stored spectrum (Beam2D.propagate) is
//   rows:     H(z) and k-domain mask as each spectrum row loads (once per
//             |kx|), [multiplied spectrum written back], inverse FFT
//   columns:  inverse FFT, 1/N^2
// Sizes that are not powers of two use Bluestein's algorithm (as the
// complex64 path does, lp_bluestein.cu) on a per-stream work grid.
#include <cuda_runtime.h>

#include <cmath>
#include <complex>
#include <cstdarg>
#include <cstdio>
#include <map>
#include <mutex>
#include <string>
#include <utility>
#include <vector>

#include "lightprop2d_gb300.h"
#include "lp_c128_lines.cuh"
#include "lp_device.cuh"
#include "lp_internal.h"

namespace lp {
namespace {
// In-place transpose of an n x n complex128 grid: a CTA swaps tile (bi, bj)
// with tile (bj, bi) (bi <= bj) through shared memory.
constexpr int kTT = 32;
__global__ void __launch_bounds__(256) ztranspose_kernel(z2* a, int n, int tiles) {
  __shared__ z2 s0[kTT][kTT + 1], s1[kTT][kTT + 1];
  // blockIdx.x enumerates pairs bi <= bj
  int p = blockIdx.x, bi = 0;
  while (p >= tiles - bi) {
    p -= tiles - bi;
    ++bi;
  }
  const int bj = bi + p;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8
  for (int r = ty; r < kTT; r += 8) {
    const int y0 = bi * kTT + r, x0 = bj * kTT + tx;
    if (y0 < n && x0 < n) s0[r][tx] = a[(size_t)y0 * n + x0];
    const int y1 = bj * kTT + r, x1 = bi * kTT + tx;
    if (y1 < n && x1 < n) s1[r][tx] = a[(size_t)y1 * n + x1];
  }
  __syncthreads();
  for (int r = ty; r < kTT; r += 8) {
    const int y0 = bi * kTT + r, x0 = bj * kTT + tx;  // receives tile (bj, bi) transposed
    if (y0 < n && x0 < n) a[(size_t)y0 * n + x0] = s1[tx][r];
    const int y1 = bj * kTT + r, x1 = bi * kTT + tx;
    if (y1 < n && x1 < n) a[(size_t)y1 * n + x1] = s0[tx][r];
  }
}

// Pointwise kernels: field <- spectrum * k multipliers (+ spectrum write),
// x multipliers, |field|^2, and the Bluestein pad / separable multiply / crop.
__global__ void zspectral_kernel(const z2* __restrict__ in, z2* out, int n, ZOps o) {
  const long long total = (long long)n * n;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const int ky = (int)(i / n), kx = (int)(i - (long long)ky * n);
    z2 v = in[i];
    if (o.apply_h || o.kmask) v = zf_to_z2(zf_mul(z2_to_zf(v), zkmul_ff(o, ky, kx, n)));
    if (o.spectrum_out) o.spectrum_out[i] = v;
    out[i] = zscale(v, o.scale);
  }
}

__global__ void zxmul_kernel(const z2* __restrict__ in, z2* out, int n, ZOps o) {
  const long long total = (long long)n * n;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const int y = (int)(i / n), x = (int)(i - (long long)y * n);
    out[i] = zf_to_z2(zf_mul(z2_to_zf(in[i]), zxmul_ff(o, y, x, n)));
  }
}

__global__ void ziprofile_kernel(const z2* __restrict__ f, double* __restrict__ out,
                                 long long total) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const z2 v = f[i];
    out[i] = fma(v.x, v.x, v.y * v.y);
  }
}

__global__ void zpad_kernel(const z2* __restrict__ in, int n, z2* ws, int m,
                            const z2* __restrict__ chirp, int conj) {
  const long long total = (long long)m * m;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(i / m), c = (int)(i - (long long)r * m);
    z2 v = make_double2(0.0, 0.0);
    if (r < n && c < n) {
      z2 w = zmul(__ldg(chirp + r), __ldg(chirp + c));
      if (conj) w = zconj(w);
      v = zmul(in[(size_t)r * n + c], w);
    }
    ws[i] = v;
  }
}

__global__ void zsepmul_kernel(z2* ws, int m, const z2* __restrict__ k, double scale) {
  const long long total = (long long)m * m;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(i / m), c = (int)(i - (long long)r * m);
    ws[i] = zscale(zmul(ws[i], zmul(__ldg(k + r), __ldg(k + c))), scale);
  }
}

__global__ void zcrop_kernel(const z2* __restrict__ ws, int m, z2* out, int n,
                             const z2* __restrict__ chirp, int conj, double scale) {
  const long long total = (long long)n * n;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(i / n), c = (int)(i - (long long)r * n);
    z2 w = zmul(__ldg(chirp + r), __ldg(chirp + c));
    if (conj) w = zconj(w);
    out[i] = zscale(zmul(ws[(size_t)r * m + c], w), scale);
  }
}

int zblocks(long long total) {
  const long long b = (total + 255) / 256;
  return (int)(b > 152 * 16 ? 152 * 16 : (b ? b : 1));
}

// ------------------------------------------------------------------ state --
lp_status zfail(lp_status s, const char* fmt, ...) {
  char msg[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(msg, sizeof(msg), fmt, ap);
  va_end(ap);
  return (lp_status)set_last_error((int)s, msg);
}

std::mutex g_zmu;
std::map<std::pair<int, int>, zf*> g_ztw;  // (device, log2 N) -> W_N^k (float-float)
bool g_zsmem_set[64][kMaxLog + 1] = {};
struct ZBlue {
  z2* chirp;
  z2* kf;
  z2* ki;
  int m;
};
std::map<std::pair<int, int>, ZBlue> g_zblue;          // (device, n)
std::map<std::pair<int, uintptr_t>, std::pair<z2*, size_t>> g_zws;  // (device, stream)

bool is_pow2(int n) { return n >= 16 && n <= 8192 && (n & (n - 1)) == 0; }

lp_status capture_guard(cudaStream_t st, const char* what) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(st, &cs) != cudaSuccess)
    return zfail(LP_ERR_CUDA, "cudaStreamIsCapturing failed");
  if (cs != cudaStreamCaptureStatusNone)
    return zfail(LP_ERR_NOT_INITIALIZED,
                 "%s: first complex128 call of this size builds tables; make it before "
                 "stream capture", what);
  return LP_OK;
}

// Per-device, per-size set-up (twiddle table, shared-memory attributes).
lp_status ztables(int n, cudaStream_t st, const zf** tw) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64)
    return zfail(LP_ERR_CUDA, "cudaGetDevice failed");
  int lg = 0;
  while ((1 << lg) < n) ++lg;
  std::lock_guard<std::mutex> lk(g_zmu);
  auto it = g_ztw.find({dev, lg});
  if (it != g_ztw.end()) {
    *tw = it->second;
    return LP_OK;
  }
  lp_status s = capture_guard(st, "complex128 transform");
  if (s != LP_OK) return s;
  std::vector<zf> h(n);
  for (int k = 0; k < n; ++k) {
    const double a = -2.0 * kPi * (double)k / (double)n;
    const double c = std::cos(a), sn = std::sin(a);
    const float ch = (float)c, sh = (float)sn;
    h[k] = make_float4(ch, (float)(c - (double)ch), sh, (float)(sn - (double)sh));
  }
  zf* d = nullptr;
  cudaError_t e = cudaMalloc(&d, sizeof(zf) * n);
  if (e == cudaSuccess) e = cudaMemcpy(d, h.data(), sizeof(zf) * n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && !g_zsmem_set[dev][lg]) e = zline_smem(n);
  if (e != cudaSuccess) {
    if (d) cudaFree(d);
    cudaGetLastError();
    return zfail(e == cudaErrorMemoryAllocation ? LP_ERR_OUT_OF_MEMORY : LP_ERR_CUDA,
                 "complex128 set-up for npoints=%d: %s", n, cudaGetErrorString(e));
  }
  g_zsmem_set[dev][lg] = true;
  g_ztw[{dev, lg}] = d;
  *tw = d;
  return LP_OK;
}

}  // namespace

cudaError_t zline_any(int n, int mode, bool in_d, bool out_d, bool cols, const void* in,
                      void* out, const ZOps& o, const float4* tw, cudaStream_t st) {
  if (n <= 128) return zline_g16_128(n, mode, in_d, out_d, cols, in, out, o, tw, st);
  if (n <= 512) return zline_g256_512(n, mode, in_d, out_d, cols, in, out, o, tw, st);
  if (n <= 2048) return zline_g1024_2048(n, mode, in_d, out_d, cols, in, out, o, tw, st);
  if (n == 4096) return zline_g4096(n, mode, in_d, out_d, cols, in, out, o, tw, st);
  return zline_g8192(n, mode, in_d, out_d, cols, in, out, o, tw, st);
}

cudaError_t zline_smem(int n) {
  if (n <= 128) return zsmem_g16_128(n);
  if (n <= 512) return zsmem_g256_512(n);
  if (n <= 2048) return zsmem_g1024_2048(n);
  if (n == 4096) return zsmem_g4096(n);
  return zsmem_g8192(n);
}

namespace {

cudaError_t ztranspose(z2* a, int n, cudaStream_t st) {
  const int tiles = (n + kTT - 1) / kTT;
  ztranspose_kernel<<<tiles * (tiles + 1) / 2, 256, 0, st>>>(a, n, tiles);
  return cudaGetLastError();
}

ZOps zops_none() {
  ZOps o{};
  o.scale = 1.0;
  return o;
}

// Columns as lines: n <= 4096 reads them in place (two adjacent columns per
// CTA); 8192 transposes and runs row passes.
bool zcols(int n) { return n <= 4096; }

// Power-of-two n: out = [post] F^-1 [k] F [pre] in, as selected by the ops.
//   rows (pre x ops, forward), columns (forward, k ops, scale, inverse),
//   rows (inverse, post x ops, iprofile); 8192 transposes around a row pass
//   in place of the column pass.
lp_status zpropagate_pow2(const z2* in, z2* out, int n, const ZOps& x_pre, const ZOps& k,
                          const ZOps& x_post, cudaStream_t st) {
  const zf* tw;
  lp_status s = ztables(n, st, &tw);
  if (s != LP_OK) return s;
  const bool cols = zcols(n);
  cudaError_t e = zline_any(n, Z_FWD, true, false, false, in, out, x_pre, tw, st);
  if (e == cudaSuccess && !cols) e = ztranspose(out, n, st);
  if (e == cudaSuccess) e = zline_any(n, Z_FUSED, false, false, cols, out, out, k, tw, st);
  if (e == cudaSuccess && !cols) e = ztranspose(out, n, st);
  if (e == cudaSuccess) e = zline_any(n, Z_INV, false, true, false, out, out, x_post, tw, st);
  if (e != cudaSuccess) return zfail(LP_ERR_CUDA, "complex128 passes: %s", cudaGetErrorString(e));
  return LP_OK;
}

// Power-of-two n: forward (inverse) 2-D transform times scale.
lp_status zfft2_pow2(const z2* in, z2* out, int n, int inverse, double scale, cudaStream_t st) {
  const zf* tw;
  lp_status s = ztables(n, st, &tw);
  if (s != LP_OK) return s;
  ZOps o = zops_none();
  o.scale = scale;
  const int mode = inverse ? Z_INV : Z_FWD;
  ZOps first = zops_none();
  const bool cols = zcols(n);
  cudaError_t e = zline_any(n, mode, true, false, false, in, out, first, tw, st);
  if (e == cudaSuccess && !cols) e = ztranspose(out, n, st);
  if (e == cudaSuccess) e = zline_any(n, mode, false, true, cols, out, out, o, tw, st);
  if (e == cudaSuccess && !cols) e = ztranspose(out, n, st);
  if (e != cudaSuccess) return zfail(LP_ERR_CUDA, "complex128 transform: %s", cudaGetErrorString(e));
  return LP_OK;
}

// ------------------------------------------------------------- Bluestein --
void zhost_fft(std::vector<std::complex<double>>& a) {
  const int m = (int)a.size();
  for (int i = 1, j = 0; i < m; ++i) {
    int bit = m >> 1;
    for (; j & bit; bit >>= 1) j ^= bit;
    j ^= bit;
    if (i < j) std::swap(a[i], a[j]);
  }
  for (int len = 2; len <= m; len <<= 1)
    for (int i = 0; i < m; i += len)
      for (int q = 0; q < len / 2; ++q) {
        const double ang = -2.0 * kPi * q / len;
        const std::complex<double> w(std::cos(ang), std::sin(ang));
        const std::complex<double> u = a[i + q], v = a[i + q + len / 2] * w;
        a[i + q] = u + v;
        a[i + q + len / 2] = u - v;
      }
}

lp_status zblue_tables(int n, cudaStream_t st, ZBlue* out) {
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lk(g_zmu);
  auto it = g_zblue.find({dev, n});
  if (it != g_zblue.end()) {
    *out = it->second;
    return LP_OK;
  }
  lp_status s = capture_guard(st, "complex128 transform");
  if (s != LP_OK) return s;
  const int m = bluestein_m(n);
  std::vector<std::complex<double>> w(n), bf(m, 0.0), bi(m, 0.0);
  for (int j = 0; j < n; ++j) {
    const long long r = ((long long)j * j) % (2LL * n);
    const double ang = -kPi * (double)r / (double)n;
    w[j] = std::complex<double>(std::cos(ang), std::sin(ang));
    bf[j] = std::conj(w[j]);
    bi[j] = w[j];
    if (j > 0) {
      bf[m - j] = std::conj(w[j]);
      bi[m - j] = w[j];
    }
  }
  zhost_fft(bf);
  zhost_fft(bi);
  std::vector<z2> h((size_t)n + 2 * (size_t)m);
  for (int j = 0; j < n; ++j) h[j] = make_double2(w[j].real(), w[j].imag());
  for (int q = 0; q < m; ++q) {
    h[n + q] = make_double2(bf[q].real(), bf[q].imag());
    h[n + m + q] = make_double2(bi[q].real(), bi[q].imag());
  }
  z2* d = nullptr;
  cudaError_t e = cudaMalloc(&d, sizeof(z2) * h.size());
  if (e == cudaSuccess) e = cudaMemcpy(d, h.data(), sizeof(z2) * h.size(), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    if (d) cudaFree(d);
    cudaGetLastError();
    return zfail(LP_ERR_CUDA, "complex128 Bluestein tables: %s", cudaGetErrorString(e));
  }
  ZBlue b{d, d + n, d + n + m, m};
  g_zblue[{dev, n}] = b;
  *out = b;
  return LP_OK;
}

lp_status zworkspace(int n, cudaStream_t st, z2** ws) {
  int dev = 0;
  cudaGetDevice(&dev);
  const int m = bluestein_m(n);
  const size_t need = sizeof(z2) * (size_t)m * m;
  std::lock_guard<std::mutex> lk(g_zmu);
  auto& slot = g_zws[{dev, (uintptr_t)st}];
  if (slot.second < need) {
    lp_status s = capture_guard(st, "complex128 work grid");
    if (s != LP_OK) return s;
    if (slot.first) cudaFree(slot.first);
    slot = {nullptr, 0};
    z2* p = nullptr;
    if (cudaMalloc(&p, need) != cudaSuccess) {
      cudaGetLastError();
      return zfail(LP_ERR_OUT_OF_MEMORY, "complex128 work grid of %zu bytes", need);
    }
    slot = {p, need};
  }
  *ws = slot.first;
  return LP_OK;
}

// Any n: forward (inverse) 2-D DFT times scale.
lp_status zdft2(const z2* in, z2* out, int n, int inverse, double scale, cudaStream_t st) {
  if (is_pow2(n)) return zfft2_pow2(in, out, n, inverse, scale, st);
  ZBlue b;
  lp_status s = zblue_tables(n, st, &b);
  if (s != LP_OK) return s;
  z2* ws;
  s = zworkspace(n, st, &ws);
  if (s != LP_OK) return s;
  const int m = b.m;
  zpad_kernel<<<zblocks((long long)m * m), 256, 0, st>>>(in, n, ws, m, b.chirp, inverse);
  s = zfft2_pow2(ws, ws, m, 0, 1.0, st);
  if (s != LP_OK) return s;
  zsepmul_kernel<<<zblocks((long long)m * m), 256, 0, st>>>(ws, m, inverse ? b.ki : b.kf,
                                                           1.0 / ((double)m * m));
  s = zfft2_pow2(ws, ws, m, 1, 1.0, st);
  if (s != LP_OK) return s;
  zcrop_kernel<<<zblocks((long long)n * n), 256, 0, st>>>(ws, m, out, n, b.chirp, inverse, scale);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return zfail(LP_ERR_CUDA, "complex128 transform: %s", cudaGetErrorString(e));
  return LP_OK;
}

// ----------------------------------------------------------------- checks --
lp_status zcheck(int n, const void* p, const char* name, bool required) {
  if (!lp_is_supported_n(n))
    return zfail(LP_ERR_UNSUPPORTED_SIZE,
                 "npoints=%d is not supported (2..4096, or a power of two up to 8192)", n);
  if (!p) return required ? zfail(LP_ERR_INVALID_ARGUMENT, "%s is NULL", name) : LP_OK;
  if (reinterpret_cast<uintptr_t>(p) & 15u)
    return zfail(LP_ERR_MISALIGNED, "%s is not 16-byte aligned", name);
  return LP_OK;
}

lp_status zcheck_mask(const void* m, int type, const char* name) {
  if (type < LP_MASK_NONE || type > LP_MASK_SEP_C128)
    return zfail(LP_ERR_INVALID_ARGUMENT, "%s: unknown mask type %d", name, type);
  if (type != LP_MASK_NONE && !m)
    return zfail(LP_ERR_INVALID_ARGUMENT, "%s: NULL with mask type %d", name, type);
  return LP_OK;
}

void zset_k(ZOps& o, int n, double area, double wl, double z, uint32_t flags) {
  o.apply_h = z != 0.0;
  o.k0 = 1.0 / wl;
  o.z = z;
  o.val = 1.0 / (n * (area / n));
  o.evan_mask = (flags & LP_FLAG_EVANESCENT_MASK) ? 1 : 0;
}

void zset_lens(ZOps& o, int n, double area, double wl, double f) {
  o.lens = 1;
  o.dL = area / n;
  o.lens_c = (1.0 / wl) / (2.0 * f);
}

constexpr uint32_t kZFlags = LP_FLAG_EVANESCENT_MASK | LP_FLAG_SPECTRUM_READONLY;

}  // namespace
}  // namespace lp

using namespace lp;

extern "C" {

lp_status lp_fft2_c128(const lp_cdouble* in, lp_cdouble* out, int n, int inverse, void* stream) {
  lp_status s = zcheck(n, in, "in", true);
  if (s == LP_OK) s = zcheck(n, out, "out", true);
  if (s != LP_OK) return s;
  return zdft2(reinterpret_cast<const z2*>(in), reinterpret_cast<z2*>(out), n, inverse ? 1 : 0,
               inverse ? 1.0 / ((double)n * n) : 1.0, (cudaStream_t)stream);
}

lp_status lp_propagate_c128(lp_cdouble* spectrum, lp_cdouble* field, int n, double area_size,
                            double wl, double z, const void* kmask, int kmask_type,
                            uint32_t flags, void* stream) {
  lp_status s = zcheck(n, spectrum, "spectrum", true);
  if (s == LP_OK) s = zcheck(n, field, "field", true);
  if (s == LP_OK) s = zcheck_mask(kmask, kmask_type, "kmask");
  if (s != LP_OK) return s;
  if (!(std::isfinite(area_size) && area_size > 0 && std::isfinite(wl) && wl > 0 &&
        std::isfinite(z)))
    return zfail(LP_ERR_INVALID_ARGUMENT, "area_size, wl must be finite and > 0, z finite");
  if (flags & ~kZFlags)
    return zfail(LP_ERR_INVALID_ARGUMENT,
                 "complex128 propagate takes LP_FLAG_EVANESCENT_MASK and "
                 "LP_FLAG_SPECTRUM_READONLY only");
  if ((const void*)spectrum == (const void*)field)
    return zfail(LP_ERR_INVALID_ARGUMENT, "spectrum and field must be different grids");
  cudaStream_t st = (cudaStream_t)stream;
  ZOps k = zops_none();
  zset_k(k, n, area_size, wl, z, flags);
  k.kmask = kmask_type ? kmask : nullptr;
  k.kmask_type = kmask_type;
  if (!(flags & LP_FLAG_SPECTRUM_READONLY)) k.spectrum_out = reinterpret_cast<z2*>(spectrum);
  if (is_pow2(n)) {
    // rows: k multipliers on load (+ spectrum write), inverse row FFT;
    // columns: inverse FFT, 1/N^2 (8192: T, rows, T)
    const zf* tw;
    s = ztables(n, st, &tw);
    if (s != LP_OK) return s;
    ZOps inv = zops_none();
    inv.scale = 1.0 / ((double)n * n);
    const bool cols = zcols(n);
    z2* fz = reinterpret_cast<z2*>(field);
    cudaError_t e = zline_any(n, Z_KINV, true, false, false, spectrum, field, k, tw, st);
    if (e == cudaSuccess && !cols) e = ztranspose(fz, n, st);
    if (e == cudaSuccess) e = zline_any(n, Z_INV, false, true, cols, field, field, inv, tw, st);
    if (e == cudaSuccess && !cols) e = ztranspose(fz, n, st);
    if (e != cudaSuccess)
      return zfail(LP_ERR_CUDA, "complex128 propagate: %s", cudaGetErrorString(e));
    return LP_OK;
  }
  zspectral_kernel<<<zblocks((long long)n * n), 256, 0, st>>>(
      reinterpret_cast<const z2*>(spectrum), reinterpret_cast<z2*>(field), n, k);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return zfail(LP_ERR_CUDA, "spectral multipliers: %s", cudaGetErrorString(e));
  return zdft2(reinterpret_cast<z2*>(field), reinterpret_cast<z2*>(field), n, 1,
               1.0 / ((double)n * n), st);
}

lp_status lp_propagate_field_c128(const lp_cdouble* field_in, lp_cdouble* field_out,
                                  lp_cdouble* spectrum_out, double* iprofile_out, int n,
                                  double area_size, double wl, double z, double lens_f,
                                  const void* xmask, int xmask_type, const void* kmask,
                                  int kmask_type, uint32_t flags, void* stream) {
  lp_status s = zcheck(n, field_in, "field_in", true);
  if (s == LP_OK) s = zcheck(n, field_out, "field_out", true);
  if (s == LP_OK) s = zcheck(n, spectrum_out, "spectrum_out", false);
  if (s == LP_OK) s = zcheck_mask(xmask, xmask_type, "xmask");
  if (s == LP_OK) s = zcheck_mask(kmask, kmask_type, "kmask");
  if (s != LP_OK) return s;
  if (iprofile_out && (reinterpret_cast<uintptr_t>(iprofile_out) & 7u))
    return zfail(LP_ERR_MISALIGNED, "iprofile_out is not 8-byte aligned");
  if (!(std::isfinite(area_size) && area_size > 0 && std::isfinite(wl) && wl > 0 &&
        std::isfinite(z) && std::isfinite(lens_f)))
    return zfail(LP_ERR_INVALID_ARGUMENT, "area_size, wl > 0; z and lens_f finite");
  if (flags & ~LP_FLAG_EVANESCENT_MASK)
    return zfail(LP_ERR_INVALID_ARGUMENT,
                 "complex128 fused propagate takes LP_FLAG_EVANESCENT_MASK only");
  if (spectrum_out && (const void*)spectrum_out == (const void*)field_out)
    return zfail(LP_ERR_INVALID_ARGUMENT, "spectrum_out and field_out must be different grids");
  cudaStream_t st = (cudaStream_t)stream;
  ZOps x = zops_none();
  if (lens_f != 0.0) zset_lens(x, n, area_size, wl, lens_f);
  x.xmask = xmask_type ? xmask : nullptr;
  x.xmask_type = xmask_type;
  ZOps k = zops_none();
  zset_k(k, n, area_size, wl, z, flags);
  k.kmask = kmask_type ? kmask : nullptr;
  k.kmask_type = kmask_type;
  k.spectrum_out = reinterpret_cast<z2*>(spectrum_out);
  k.scale = 1.0 / ((double)n * n);
  ZOps post = zops_none();
  post.iprofile = iprofile_out;
  const z2* in = reinterpret_cast<const z2*>(field_in);
  z2* out = reinterpret_cast<z2*>(field_out);
  if (is_pow2(n)) return zpropagate_pow2(in, out, n, x, k, post, st);
  // other sizes: pointwise passes around Bluestein transforms
  const long long n2 = (long long)n * n;
  if (x.lens || x.xmask) {
    zxmul_kernel<<<zblocks(n2), 256, 0, st>>>(in, out, n, x);
    in = out;
  }
  s = zdft2(in, out, n, 0, 1.0, st);
  if (s != LP_OK) return s;
  zspectral_kernel<<<zblocks(n2), 256, 0, st>>>(out, out, n, k);
  s = zdft2(out, out, n, 1, 1.0, st);
  if (s != LP_OK) return s;
  if (iprofile_out) ziprofile_kernel<<<zblocks(n2), 256, 0, st>>>(out, iprofile_out, n2);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return zfail(LP_ERR_CUDA, "complex128 propagate: %s", cudaGetErrorString(e));
  return LP_OK;
}

static lp_status zxdomain(lp_cdouble* field, lp_cdouble* spectrum_out, int n, const ZOps& x,
                          void* stream) {
  cudaStream_t st = (cudaStream_t)stream;
  z2* f = reinterpret_cast<z2*>(field);
  zxmul_kernel<<<zblocks((long long)n * n), 256, 0, st>>>(f, f, n, x);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return zfail(LP_ERR_CUDA, "x-domain multiply: %s", cudaGetErrorString(e));
  if (!spectrum_out) return LP_OK;
  return zdft2(f, reinterpret_cast<z2*>(spectrum_out), n, 0, 1.0, st);
}

lp_status lp_lens_c128(lp_cdouble* field, lp_cdouble* spectrum_out, int n, double area_size,
                       double wl, double f, void* stream) {
  lp_status s = zcheck(n, field, "field", true);
  if (s == LP_OK) s = zcheck(n, spectrum_out, "spectrum_out", false);
  if (s != LP_OK) return s;
  if (!(std::isfinite(area_size) && area_size > 0 && std::isfinite(wl) && wl > 0))
    return zfail(LP_ERR_INVALID_ARGUMENT, "area_size and wl must be finite and > 0");
  if (!std::isfinite(f) || f == 0.0)
    return zfail(LP_ERR_INVALID_ARGUMENT, "focal length must be finite and non-zero");
  ZOps x = zops_none();
  zset_lens(x, n, area_size, wl, f);
  return zxdomain(field, spectrum_out, n, x, stream);
}

lp_status lp_coordinate_filter_c128(lp_cdouble* field, lp_cdouble* spectrum_out, int n,
                                    const void* mask, int mask_type, void* stream) {
  lp_status s = zcheck(n, field, "field", true);
  if (s == LP_OK) s = zcheck(n, spectrum_out, "spectrum_out", false);
  if (s == LP_OK) s = zcheck_mask(mask, mask_type, "mask");
  if (s != LP_OK) return s;
  if (mask_type == LP_MASK_NONE) return zfail(LP_ERR_INVALID_ARGUMENT, "mask is required");
  ZOps x = zops_none();
  x.xmask = mask;
  x.xmask_type = mask_type;
  return zxdomain(field, spectrum_out, n, x, stream);
}

lp_status lp_spectral_filter_c128(lp_cdouble* spectrum, lp_cdouble* field_out, int n,
                                  const void* mask, int mask_type, void* stream) {
  if (mask_type == LP_MASK_NONE) return zfail(LP_ERR_INVALID_ARGUMENT, "mask is required");
  return lp_propagate_c128(spectrum, field_out, n, 1.0, 1.0, 0.0, mask, mask_type, 0u, stream);
}

lp_status lp_apply_transfer_c128(lp_cdouble* spectrum, int n, double area_size, double wl,
                                 double z, uint32_t flags, void* stream) {
  lp_status s = zcheck(n, spectrum, "spectrum", true);
  if (s != LP_OK) return s;
  if (!(std::isfinite(area_size) && area_size > 0 && std::isfinite(wl) && wl > 0 &&
        std::isfinite(z)))
    return zfail(LP_ERR_INVALID_ARGUMENT, "area_size, wl must be finite and > 0, z finite");
  if (flags & ~LP_FLAG_EVANESCENT_MASK)
    return zfail(LP_ERR_INVALID_ARGUMENT, "complex128 transfer takes LP_FLAG_EVANESCENT_MASK only");
  if (z == 0.0) return LP_OK;
  ZOps k = zops_none();
  zset_k(k, n, area_size, wl, z, flags);
  z2* sp = reinterpret_cast<z2*>(spectrum);
  zspectral_kernel<<<zblocks((long long)n * n), 256, 0, (cudaStream_t)stream>>>(sp, sp, n, k);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return zfail(LP_ERR_CUDA, "transfer: %s", cudaGetErrorString(e));
  return LP_OK;
}

lp_status lp_iprofile_c128(const lp_cdouble* field, double* out, int n, void* stream) {
  lp_status s = zcheck(n, field, "field", true);
  if (s != LP_OK) return s;
  if (!out || (reinterpret_cast<uintptr_t>(out) & 7u))
    return zfail(LP_ERR_INVALID_ARGUMENT, "out must be an 8-byte aligned device pointer");
  const long long n2 = (long long)n * n;
  ziprofile_kernel<<<zblocks(n2), 256, 0, (cudaStream_t)stream>>>(
      reinterpret_cast<const z2*>(field), out, n2);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return zfail(LP_ERR_CUDA, "iprofile: %s", cudaGetErrorString(e));
  return LP_OK;
}

}  // extern "C"
