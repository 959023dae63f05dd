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
// A 2-D transform is a line pass over rows, an in-place square transpose, a
// line pass over the (former) columns and a transpose back.  A line pass
// holds whole lines in shared memory (N <= 8192: at most 128 KB) and
// transforms them with a Stockham sequence of radix-4 stages (one radix-2
// stage first when log2 N is odd): each thread keeps 16 points in registers
// between the read and write halves of a stage, so the line is transformed
// in place.  Stage twiddles come from a per-size table W_N^k (k < N) computed
// on the host in double and split into float-float.  Intermediate grids
// between the passes hold float-float values (16 bytes a point, like a
// complex128); the first pass reads the caller's complex128 and the last
// writes complex128.
//
// A propagate is
//   rows:     [x-domain multipliers] forward FFT
//   transpose
//   lines:    forward FFT, H(z) = exp(2*pi*i*(trunc(Kz z) - Kz z)) with Kz in
//             float64 exactly as beam2d.py:305-308 and :485-489 compute it
//             (once per |ky|: H(kx, ky) = H(kx, -ky)), k-domain mask, 1/N^2,
//             inverse FFT
//   transpose
//   rows:     inverse FFT, |field|^2 epilogue (float64)
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
#include "lp_device.cuh"
#include "lp_internal.h"

namespace lp {
namespace {

using z2 = double2;

__device__ __forceinline__ z2 zmul(z2 a, z2 b) {
  return make_double2(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ z2 zconj(z2 a) { return make_double2(a.x, -a.y); }
__device__ __forceinline__ z2 zscale(z2 a, double s) { return make_double2(a.x * s, a.y * s); }

constexpr int kMaxLog = 13;  // 8192

template <int N>
struct ZGeo {
  static constexpr int TL = N >= 16 ? N / 16 : 1;        // threads per line
  static constexpr int L = TL >= 256 ? 1 : 256 / TL;     // lines per CTA
  static constexpr int NT = TL * L;
  static constexpr int HT = N / 2 + 1;                   // H table entries per line
  static constexpr size_t SMEM = 16 * (size_t)L * N;
  static constexpr size_t SMEM_FUSED = 16 * (size_t)L * (N + HT);
  static constexpr int LOG = N == 16 ? 4 : N == 32 ? 5 : N == 64 ? 6 : N == 128 ? 7
                           : N == 256 ? 8 : N == 512 ? 9 : N == 1024 ? 10 : N == 2048 ? 11
                           : N == 4096 ? 12 : 13;
};

// Multipliers of a line pass.  Row passes (x domain, line = y): lens phase
// and mask, before the forward transform (pre) or after the inverse (post),
// and the |field|^2 epilogue.  The fused pass (k domain, line = kx after the
// transpose): H(z), mask, spectrum write, scale.
struct ZOps {
  // x domain
  int lens;          // multiply by exp(i*(X^2+Y^2)*k0/(2f))
  double lens_c;     // k0 / (2 f)
  double dL;
  const void* xmask;
  int xmask_type;
  int post;          // apply the x-domain multiplier after the transform
  double* iprofile;  // optional |out|^2
  // k domain
  int apply_h;
  double k0, z, val;  // val = 1 / (n dL): fftfreq spacing
  int evan_mask;
  const void* kmask;
  int kmask_type;
  z2* spectrum_out;   // natural layout [ky * n + kx]
  double scale;
  float scale_h, scale_l;  // scale as float-float (set by the launcher)
};

// Mask element (y, x) of an n x n mask (or 2n table) as complex128.
__device__ __forceinline__ z2 zmask(const void* mask, int type, int y, int x, int n) {
  const size_t i = (size_t)y * n + x;
  switch (type) {
    case LP_MASK_F32: return make_double2(__ldg(reinterpret_cast<const float*>(mask) + i), 0.0);
    case LP_MASK_C64: {
      const float2 v = __ldg(reinterpret_cast<const float2*>(mask) + i);
      return make_double2(v.x, v.y);
    }
    case LP_MASK_U8:
      return make_double2((double)__ldg(reinterpret_cast<const uint8_t*>(mask) + i), 0.0);
    case LP_MASK_PHASE_F32: {
      double s, c;
      sincos((double)__ldg(reinterpret_cast<const float*>(mask) + i), &s, &c);
      return make_double2(c, s);
    }
    case LP_MASK_F64: return make_double2(__ldg(reinterpret_cast<const double*>(mask) + i), 0.0);
    case LP_MASK_C128: return __ldg(reinterpret_cast<const double2*>(mask) + i);
    case LP_MASK_SEP_F32: {
      const float* t = reinterpret_cast<const float*>(mask);
      return make_double2((double)__ldg(t + x) * (double)__ldg(t + n + y), 0.0);
    }
    case LP_MASK_SPAN_I32: {
      const int* t = reinterpret_cast<const int*>(mask);
      return make_double2((y >= __ldg(t + x) && y < __ldg(t + n + x)) ? 1.0 : 0.0, 0.0);
    }
    case LP_MASK_SEP_C64: {
      const float2* t = reinterpret_cast<const float2*>(mask);
      const float2 a = __ldg(t + x), b = __ldg(t + n + y);
      return zmul(make_double2(a.x, a.y), make_double2(b.x, b.y));
    }
    case LP_MASK_SEP_C128: {
      const double2* t = reinterpret_cast<const double2*>(mask);
      return zmul(__ldg(t + x), __ldg(t + n + y));
    }
    default: return make_double2(1.0, 0.0);
  }
}

// x-domain multiplier at (y, x): the reference's lens phase
// (X^2+Y^2)*k0/(2f) with X = (x - (n+1)/2) dL (beam2d.py:299-300, :508-510)
// times the mask.
__device__ __forceinline__ z2 zxmul(const ZOps& o, int y, int x, int n) {
  z2 m = make_double2(1.0, 0.0);
  if (o.lens) {
    const double X = (double)(x - (n + 1) / 2) * o.dL, Y = (double)(y - (n + 1) / 2) * o.dL;
    double s, c;
    sincos((X * X + Y * Y) * o.lens_c, &s, &c);
    m = make_double2(c, s);
  }
  if (o.xmask) m = zmul(m, zmask(o.xmask, o.xmask_type, y, x, n));
  return m;
}

// H at (ky, kx) as beam2d.py computes it: Kx = fftfreq(n, dL),
// Kz = nan_to_num(sqrt(k0**2 - Kx**2 - Ky**2)), phase = 2*pi*(trunc(Kz z) - Kz z).
__device__ __forceinline__ z2 zkmul(const ZOps& o, int ky, int kx, int n) {
  z2 m = make_double2(1.0, 0.0);
  if (o.apply_h) {
    const int h = (n + 1) / 2;
    const double fx = (double)(kx < h ? kx : kx - n) * o.val;
    const double fy = (double)(ky < h ? ky : ky - n) * o.val;
    const double v = (o.k0 * o.k0 - fx * fx) - fy * fy;
    if (v >= 0.0) {
      const double dk = sqrt(v) * o.z;
      double s, c;
      sincos(2.0 * kPi * (trunc(dk) - dk), &s, &c);
      m = make_double2(c, s);
    } else if (o.evan_mask) {
      m = make_double2(0.0, 0.0);
    }
  }
  if (o.kmask) m = zmul(m, zmask(o.kmask, o.kmask_type, ky, kx, n));
  return m;
}

// ------------------------------------------------------ float-float values --
// zf = (re.hi, re.lo, im.hi, im.lo), 16 bytes like a double2.
using zf = float4;

__device__ __forceinline__ void fast_two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  e = __fsub_rn(b, __fsub_rn(s, a));
}
// (ah + al) + (bh + bl)
__device__ __forceinline__ void ff_add2(float ah, float al, float bh, float bl, float& h,
                                        float& l) {
  float s, e;
  two_sum(ah, bh, s, e);
  fast_two_sum(s, __fadd_rn(e, __fadd_rn(al, bl)), h, l);
}
// (ah + al) * (bh + bl)
__device__ __forceinline__ void ff_mul2(float ah, float al, float bh, float bl, float& h,
                                        float& l) {
  const float p = __fmul_rn(ah, bh);
  fast_two_sum(p, fmaf(ah, bl, fmaf(al, bh, fmaf(ah, bh, -p))), h, l);
}

__device__ __forceinline__ zf zf_add(zf a, zf b) {
  zf r;
  ff_add2(a.x, a.y, b.x, b.y, r.x, r.y);
  ff_add2(a.z, a.w, b.z, b.w, r.z, r.w);
  return r;
}
__device__ __forceinline__ zf zf_sub(zf a, zf b) {
  return zf_add(a, make_float4(-b.x, -b.y, -b.z, -b.w));
}
__device__ __forceinline__ zf zf_conj(zf a) { return make_float4(a.x, a.y, -a.z, -a.w); }
// a * w: each real part is a difference (sum) of two products formed exactly
// by two-products, then one pair sum.
__device__ __forceinline__ zf zf_mul(zf a, zf w) {
  zf r;
  float s, t;
  const float p1 = __fmul_rn(a.x, w.x), p2 = __fmul_rn(a.z, w.z);
  const float e1 = fmaf(a.x, w.y, fmaf(a.y, w.x, fmaf(a.x, w.x, -p1)));
  const float e2 = fmaf(a.z, w.w, fmaf(a.w, w.z, fmaf(a.z, w.z, -p2)));
  two_sum(p1, -p2, s, t);
  fast_two_sum(s, __fadd_rn(t, __fsub_rn(e1, e2)), r.x, r.y);
  const float p3 = __fmul_rn(a.x, w.z), p4 = __fmul_rn(a.z, w.x);
  const float e3 = fmaf(a.x, w.w, fmaf(a.y, w.z, fmaf(a.x, w.z, -p3)));
  const float e4 = fmaf(a.z, w.y, fmaf(a.w, w.x, fmaf(a.z, w.x, -p4)));
  two_sum(p3, p4, s, t);
  fast_two_sum(s, __fadd_rn(t, __fadd_rn(e3, e4)), r.z, r.w);
  return r;
}
__device__ __forceinline__ zf zf_scale(zf a, float sh, float sl) {
  zf r;
  ff_mul2(a.x, a.y, sh, sl, r.x, r.y);
  ff_mul2(a.z, a.w, sh, sl, r.z, r.w);
  return r;
}

// double -> float-float by integer operations: hi takes the top 24
// significant bits, lo the next 24 (both truncated), so the pair holds the
// double to 2^-47 relative.  Below 2^-126 the value flushes to +-0; infinities
// and NaNs carry over in hi.
__device__ __forceinline__ void d2ff(double d, float& h, float& l) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(d);
  const unsigned int w1 = (unsigned int)(b >> 32), w0 = (unsigned int)b;
  const unsigned int sgn = w1 & 0x80000000u;
  const int e = (int)((w1 >> 20) & 0x7FFu) - 1023;
  l = __uint_as_float(sgn);
  if (e < -126) {
    h = l;
    return;
  }
  if (e > 127) {
    const bool nan = e == 1024 && ((w1 & 0xFFFFFu) | w0) != 0;
    h = __uint_as_float(nan ? 0x7FC00000u : (sgn | 0x7F800000u));
    return;
  }
  h = __uint_as_float(sgn | ((unsigned int)(e + 127) << 23) | ((w1 & 0xFFFFFu) << 3) |
                      (w0 >> 29));
  const unsigned int r = w0 & 0x1FFFFFFFu;  // the remaining 29 bits, weight 2^(e-52)
  if (r == 0) return;
  const int p = 31 - __clz((int)r);        // leading bit of r: 0..28
  const int el = e - 52 + p;               // exponent of lo
  if (el < -126) return;
  const unsigned int mr = (p >= 23 ? (r >> (p - 23)) : (r << (23 - p))) & 0x7FFFFFu;
  l = __uint_as_float(sgn | ((unsigned int)(el + 127) << 23) | mr);
}
// float -> double exactly by integer operations (FP32 subnormals give +-0).
__device__ __forceinline__ double f2d(float f) {
  const unsigned int u = __float_as_uint(f);
  const unsigned int ef = (u >> 23) & 0xFFu;
  unsigned long long r = (unsigned long long)(u & 0x80000000u) << 32;
  if (ef == 0xFFu)
    r |= 0x7FF0000000000000ull | ((unsigned long long)(u & 0x7FFFFFu) << 29);
  else if (ef != 0)
    r |= ((unsigned long long)(ef + 896u) << 52) | ((unsigned long long)(u & 0x7FFFFFu) << 29);
  return __longlong_as_double((long long)r);
}
__device__ __forceinline__ zf z2_to_zf(z2 v) {
  zf r;
  d2ff(v.x, r.x, r.y);
  d2ff(v.y, r.z, r.w);
  return r;
}
__device__ __forceinline__ z2 zf_to_z2(zf v) {
  return make_double2(f2d(v.x) + f2d(v.y), f2d(v.z) + f2d(v.w));
}

// Taylor coefficients 1/n! (n! is exact in double up to 18!) as float-float.
constexpr double zfact(int n) { return n <= 1 ? 1.0 : n * zfact(n - 1); }
constexpr float zinv_h(int n) { return (float)(1.0 / zfact(n)); }
constexpr float zinv_l(int n) { return (float)(1.0 / zfact(n) - (double)(float)(1.0 / zfact(n))); }
constexpr double kHalfPiD = 1.57079632679489661923132169163975144;
constexpr float kHalfPiH = (float)kHalfPiD;
constexpr float kHalfPiL = (float)(kHalfPiD - (double)(float)kHalfPiD);

// acc <- c + s * acc, c = (-1)^k / n! (float-float)
__device__ __forceinline__ void zhorner(float sh, float sl, int sign, float ch, float cl,
                                        float& ah, float& al) {
  float ph, pl;
  ff_mul2(sh, sl, ah, al, ph, pl);
  ff_add2(sign * ch, sign * cl, ph, pl, ah, al);
}

// cos(2 pi f) + i sin(2 pi f) for a double f with |f| < 2^21, as float-float.
// Quarter turns: 4f = q + rho (q an integer, |rho| <= 1/2, both exact), so
// theta = rho pi/2 has |theta| <= pi/4; sin(theta)/theta and cos(theta) are
// their Taylor series in s = theta^2 (terms from s^5 on, below 3e-8 of the
// result, in FP32; the first five in float-float; truncation below 1e-17),
// and the quadrant q mod 4 rotates the result.
__device__ __forceinline__ zf zcis_2pi(double f) {
  float fh, fl;
  d2ff(f, fh, fl);
  const float q = rintf(4.0f * fh);
  float rh, rl, th, tl, sh, sl;
  two_sum(__fsub_rn(4.0f * fh, q), 4.0f * fl, rh, rl);
  ff_mul2(rh, rl, kHalfPiH, kHalfPiL, th, tl);
  ff_mul2(th, tl, th, tl, sh, sl);
  // FP32 tails: sin: -1/11! + s/13! - s^2/15! + s^3/17!; cos: -1/10! + ... - s^4/18!
  float ts = fmaf(fmaf(fmaf(zinv_h(17), sh, -zinv_h(15)), sh, zinv_h(13)), sh, -zinv_h(11));
  float tc = fmaf(fmaf(fmaf(fmaf(-zinv_h(18), sh, zinv_h(16)), sh, -zinv_h(14)), sh,
                       zinv_h(12)), sh, -zinv_h(10));
  float sah = ts, sal = 0.0f, cah = tc, cal = 0.0f;
  zhorner(sh, sl, 1, zinv_h(9), zinv_l(9), sah, sal);
  zhorner(sh, sl, -1, zinv_h(7), zinv_l(7), sah, sal);
  zhorner(sh, sl, 1, zinv_h(5), zinv_l(5), sah, sal);
  zhorner(sh, sl, -1, zinv_h(3), zinv_l(3), sah, sal);
  zhorner(sh, sl, 1, 1.0f, 0.0f, sah, sal);
  zhorner(sh, sl, 1, zinv_h(8), zinv_l(8), cah, cal);
  zhorner(sh, sl, -1, zinv_h(6), zinv_l(6), cah, cal);
  zhorner(sh, sl, 1, zinv_h(4), zinv_l(4), cah, cal);
  zhorner(sh, sl, -1, zinv_h(2), zinv_l(2), cah, cal);
  zhorner(sh, sl, 1, 1.0f, 0.0f, cah, cal);
  float snh, snl;
  ff_mul2(th, tl, sah, sal, snh, snl);
  switch ((int)q & 3) {
    case 0: return make_float4(cah, cal, snh, snl);
    case 1: return make_float4(-snh, -snl, cah, cal);
    case 2: return make_float4(-cah, -cal, -snh, -snl);
    default: return make_float4(snh, snl, -cah, -cal);
  }
}

// H at kx (a = k0^2 - fx^2 of this line) and |ky| = j, as the reference
// computes it in float64, with cos/sin of the reduced phase in float-float.
__device__ __forceinline__ zf zh_value(const ZOps& o, double a, int j) {
  const double fy = (double)j * o.val;
  const double v = a - fy * fy;
  if (v >= 0.0) {
    const double dk = sqrt(v) * o.z;
    return zcis_2pi(trunc(dk) - dk);
  }
  return o.evan_mask ? make_float4(0.0f, 0.0f, 0.0f, 0.0f) : make_float4(1.0f, 0.0f, 0.0f, 0.0f);
}

// In-place Stockham transform of one line (buf, N points) by TL threads
// (t = 0..TL-1), 16 points per thread per stage.  S = -1 forward, +1 inverse
// (unscaled).  tw[k] = W_N^k.  Barriers are CTA-wide (every line of the CTA
// runs the same stages).
template <int N, int R, int S>
__device__ __forceinline__ void zstage(zf* buf, int t, int ns, const zf* __restrict__ tw) {
  constexpr int TL = ZGeo<N>::TL, NB = N / R, QB = NB / TL;  // butterflies per thread
  zf v[QB * R];
#pragma unroll
  for (int q = 0; q < QB; ++q)
#pragma unroll
    for (int r = 0; r < R; ++r) v[q * R + r] = buf[t + q * TL + r * NB];
  __syncthreads();
#pragma unroll
  for (int q = 0; q < QB; ++q) {
    const int b = t + q * TL, k = b & (ns - 1);
    zf a[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
      a[r] = v[q * R + r];
      if (r > 0 && ns > 1) {
        zf w = __ldg(tw + (size_t)r * k * (N / (ns * R)));
        if (S > 0) w = zf_conj(w);
        a[r] = zf_mul(a[r], w);
      }
    }
    const int o = (b - k) * R + k;
    if constexpr (R == 2) {
      buf[o] = zf_add(a[0], a[1]);
      buf[o + ns] = zf_sub(a[0], a[1]);
    } else {
      const zf t0 = zf_add(a[0], a[2]), t1 = zf_sub(a[0], a[2]);
      const zf t2 = zf_add(a[1], a[3]);
      zf t3 = zf_sub(a[1], a[3]);
      t3 = S < 0 ? make_float4(t3.z, t3.w, -t3.x, -t3.y)
                 : make_float4(-t3.z, -t3.w, t3.x, t3.y);  // * (S*i)
      buf[o] = zf_add(t0, t2);
      buf[o + ns] = zf_add(t1, t3);
      buf[o + 2 * ns] = zf_sub(t0, t2);
      buf[o + 3 * ns] = zf_sub(t1, t3);
    }
  }
  __syncthreads();
}

template <int N, int S>
__device__ __forceinline__ void zfft(zf* buf, int t, const zf* __restrict__ tw) {
  constexpr int LOG = ZGeo<N>::LOG;
  int ns = 1;
  if constexpr (LOG & 1) {
    zstage<N, 2, S>(buf, t, ns, tw);
    ns = 2;
  }
#pragma unroll 1
  for (int s = 0; s < LOG / 2; ++s) {
    zstage<N, 4, S>(buf, t, ns, tw);
    ns *= 4;
  }
}

enum ZMode { Z_FWD = 0, Z_INV = 1, Z_FUSED = 2 };

// One line pass over N lines.  Z_FWD: [pre x multiplier] forward; Z_INV:
// inverse, scale, [post x multiplier], [iprofile]; Z_FUSED (lines are
// columns after a transpose; line index = kx): forward, k multipliers,
// [spectrum write], scale, inverse.  IN_D / OUT_D: the pass reads / writes
// complex128 (else float-float intermediates).
template <int N, int MODE, bool IN_D, bool OUT_D>
__global__ void __launch_bounds__(ZGeo<N>::NT, ZGeo<N>::NT <= 256 ? (MODE == Z_FUSED ? 2 : 3) : 1)
    zline_kernel(const void* __restrict__ in,
                                                           void* out, ZOps o,
                                                           const zf* __restrict__ tw) {
  using G = ZGeo<N>;
  extern __shared__ float4 zs[];
  const int g = threadIdx.x / G::TL, t = threadIdx.x % G::TL;
  const int line = blockIdx.x * G::L + g;
  zf* buf = zs + (size_t)g * N;
  const size_t base = (size_t)line * N;
  const bool live = line < N;  // N < L: a CTA has more line slots than lines
#pragma unroll
  for (int i = 0; i < 16 && i * G::TL < N; ++i) {
    const int x = t + G::TL * i;
    zf v = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (live) {
      if constexpr (IN_D) {
        v = z2_to_zf(reinterpret_cast<const z2*>(in)[base + x]);
      } else {
        v = reinterpret_cast<const zf*>(in)[base + x];
      }
    }
    if (MODE == Z_FWD && live && (o.lens || o.xmask) && !o.post)
      v = zf_mul(v, z2_to_zf(zxmul(o, line, x, N)));
    buf[x] = v;
  }
  __syncthreads();
  if constexpr (MODE == Z_INV) {
    zfft<N, 1>(buf, t, tw);
  } else {
    zfft<N, -1>(buf, t, tw);
  }
  if constexpr (MODE == Z_FUSED) {
    // H of this line at |ky| = 0..N/2 once each (H(kx, ky) = H(kx, -ky))
    zf* hb = zs + (size_t)G::L * N + (size_t)g * G::HT;
    if (o.apply_h) {
      const int h = (N + 1) / 2;
      const double fx = (double)(line < h ? line : line - N) * o.val;
      const double a = o.k0 * o.k0 - fx * fx;
      for (int j = t; j < G::HT; j += G::TL) hb[j] = zh_value(o, a, j);
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < 16 && i * G::TL < N; ++i) {
      const int ky = t + G::TL * i;
      zf v = buf[ky];
      if (o.apply_h) v = zf_mul(v, hb[ky <= N / 2 ? ky : N - ky]);
      if (o.kmask && live) v = zf_mul(v, z2_to_zf(zmask(o.kmask, o.kmask_type, ky, line, N)));
      if (o.spectrum_out && live) o.spectrum_out[(size_t)ky * N + line] = zf_to_z2(v);
      buf[ky] = zf_scale(v, o.scale_h, o.scale_l);
    }
    __syncthreads();
    zfft<N, 1>(buf, t, tw);
  }
  if (!live) return;
#pragma unroll
  for (int i = 0; i < 16 && i * G::TL < N; ++i) {
    const int x = t + G::TL * i;
    zf v = buf[x];
    if (MODE == Z_INV) {
      v = zf_scale(v, o.scale_h, o.scale_l);
      if ((o.lens || o.xmask) && o.post) v = zf_mul(v, z2_to_zf(zxmul(o, line, x, N)));
      if (o.iprofile) {
        float ah, al, bh, bl, ph, pl;
        ff_mul2(v.x, v.y, v.x, v.y, ah, al);
        ff_mul2(v.z, v.w, v.z, v.w, bh, bl);
        ff_add2(ah, al, bh, bl, ph, pl);
        o.iprofile[base + x] = f2d(ph) + f2d(pl);
      }
    }
    if constexpr (OUT_D) {
      reinterpret_cast<z2*>(out)[base + x] = zf_to_z2(v);
    } else {
      reinterpret_cast<zf*>(out)[base + x] = v;
    }
  }
}

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
    if (o.apply_h || o.kmask) v = zmul(v, zkmul(o, ky, kx, n));
    if (o.spectrum_out) o.spectrum_out[i] = v;
    out[i] = zscale(v, o.scale);
  }
}

__global__ void zxmul_kernel(const z2* __restrict__ in, z2* out, int n, ZOps o) {
  const long long total = (long long)n * n;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const int y = (int)(i / n), x = (int)(i - (long long)y * n);
    out[i] = zmul(in[i], zxmul(o, y, x, n));
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

// The line-pass variants a size uses: (mode, reads complex128, writes complex128).
#define LP_ZLINE_VARIANTS(X) \
  X(Z_FWD, true, false) X(Z_FWD, false, true) X(Z_INV, true, false) X(Z_INV, false, true) \
  X(Z_FUSED, false, false)

template <int N>
cudaError_t set_smem() {
  cudaError_t e = cudaSuccess;
#define LP_ZSET(M, I, O)                                                                  \
  if (e == cudaSuccess)                                                                   \
    e = cudaFuncSetAttribute(zline_kernel<N, M, I, O>,                                    \
                             cudaFuncAttributeMaxDynamicSharedMemorySize,                 \
                             (int)(M == Z_FUSED ? ZGeo<N>::SMEM_FUSED : ZGeo<N>::SMEM));
  LP_ZLINE_VARIANTS(LP_ZSET)
#undef LP_ZSET
  return e;
}

cudaError_t set_smem_for(int n) {
  switch (n) {
    case 16: return set_smem<16>();
    case 32: return set_smem<32>();
    case 64: return set_smem<64>();
    case 128: return set_smem<128>();
    case 256: return set_smem<256>();
    case 512: return set_smem<512>();
    case 1024: return set_smem<1024>();
    case 2048: return set_smem<2048>();
    case 4096: return set_smem<4096>();
    default: return set_smem<8192>();
  }
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
  if (e == cudaSuccess && !g_zsmem_set[dev][lg]) e = set_smem_for(n);
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

template <int N>
cudaError_t zline(int mode, bool in_d, bool out_d, const void* in, void* out, ZOps o,
                  const zf* tw, cudaStream_t st) {
  using G = ZGeo<N>;
  const int grid = (N + G::L - 1) / G::L;
  const float sh = (float)o.scale;
  o.scale_h = sh;
  o.scale_l = (float)(o.scale - (double)sh);
  bool done = false;
#define LP_ZLAUNCH(M, I, O)                                                                 \
  if (!done && mode == M && in_d == I && out_d == O) {                                      \
    zline_kernel<N, M, I, O>                                                                \
        <<<grid, G::NT, M == Z_FUSED ? G::SMEM_FUSED : G::SMEM, st>>>(in, out, o, tw);      \
    done = true;                                                                            \
  }
  LP_ZLINE_VARIANTS(LP_ZLAUNCH)
#undef LP_ZLAUNCH
  return done ? cudaGetLastError() : cudaErrorInvalidValue;
}

cudaError_t zline_any(int n, int mode, bool in_d, bool out_d, const void* in, void* out,
                      const ZOps& o, const zf* tw, cudaStream_t st) {
  switch (n) {
    case 16: return zline<16>(mode, in_d, out_d, in, out, o, tw, st);
    case 32: return zline<32>(mode, in_d, out_d, in, out, o, tw, st);
    case 64: return zline<64>(mode, in_d, out_d, in, out, o, tw, st);
    case 128: return zline<128>(mode, in_d, out_d, in, out, o, tw, st);
    case 256: return zline<256>(mode, in_d, out_d, in, out, o, tw, st);
    case 512: return zline<512>(mode, in_d, out_d, in, out, o, tw, st);
    case 1024: return zline<1024>(mode, in_d, out_d, in, out, o, tw, st);
    case 2048: return zline<2048>(mode, in_d, out_d, in, out, o, tw, st);
    case 4096: return zline<4096>(mode, in_d, out_d, in, out, o, tw, st);
    default: return zline<8192>(mode, in_d, out_d, in, out, o, tw, st);
  }
}

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

// Power-of-two n: out = [post] F^-1 [k] F [pre] in, as selected by the ops.
//   rows (pre x ops, forward), T, lines (forward, k ops, scale, inverse), T,
//   rows (inverse, post x ops, iprofile).
lp_status zpropagate_pow2(const z2* in, z2* out, int n, const ZOps& x_pre, const ZOps& k,
                          const ZOps& x_post, cudaStream_t st) {
  const zf* tw;
  lp_status s = ztables(n, st, &tw);
  if (s != LP_OK) return s;
  cudaError_t e = zline_any(n, Z_FWD, true, false, in, out, x_pre, tw, st);
  if (e == cudaSuccess) e = ztranspose(out, n, st);
  if (e == cudaSuccess) e = zline_any(n, Z_FUSED, false, false, out, out, k, tw, st);
  if (e == cudaSuccess) e = ztranspose(out, n, st);
  if (e == cudaSuccess) e = zline_any(n, Z_INV, false, true, out, out, x_post, tw, st);
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
  cudaError_t e = zline_any(n, mode, true, false, in, out, first, tw, st);
  if (e == cudaSuccess) e = ztranspose(out, n, st);
  if (e == cudaSuccess) e = zline_any(n, mode, false, true, out, out, o, tw, st);
  if (e == cudaSuccess) e = ztranspose(out, n, st);
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
