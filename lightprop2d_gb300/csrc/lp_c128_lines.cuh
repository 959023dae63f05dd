// complex128 line passes (float-float arithmetic), shared by lp_c128.cu and
// the per-size translation units lp_c128_lines_*.cu, which instantiate the
// pass kernels of a few sizes each so that the build compiles them in
// parallel.  See lp_c128.cu for the design.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "lightprop2d_gb300.h"
#include "lp_device.cuh"
#include "lp_internal.h"

namespace lp {

using z2 = double2;

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

// Line pass over the N lines of an N x N grid (n a power of two 16..8192):
// mode Z_FWD / Z_INV / Z_FUSED / Z_KINV; in_d / out_d: the pass reads /
// writes complex128 (else float-float intermediates); cols: the lines are
// the grid's columns (n <= 4096), else its rows.  Defined per size group in
// lp_c128_lines_*.cu.
cudaError_t zline_any(int n, int mode, bool in_d, bool out_d, bool cols, const void* in,
                      void* out, const ZOps& o, const float4* tw, cudaStream_t st);
// Sets the line kernels' shared-memory limits for size n.
cudaError_t zline_smem(int n);
cudaError_t zline_g16_128(int n, int mode, bool in_d, bool out_d, bool cols, const void* in,
                          void* out, const ZOps& o, const float4* tw, cudaStream_t st);
cudaError_t zline_g256_512(int n, int mode, bool in_d, bool out_d, bool cols, const void* in,
                          void* out, const ZOps& o, const float4* tw, cudaStream_t st);
cudaError_t zline_g1024_2048(int n, int mode, bool in_d, bool out_d, bool cols, const void* in,
                          void* out, const ZOps& o, const float4* tw, cudaStream_t st);
cudaError_t zline_g4096(int n, int mode, bool in_d, bool out_d, bool cols, const void* in,
                          void* out, const ZOps& o, const float4* tw, cudaStream_t st);
cudaError_t zline_g8192(int n, int mode, bool in_d, bool out_d, bool cols, const void* in,
                          void* out, const ZOps& o, const float4* tw, cudaStream_t st);
cudaError_t zsmem_g16_128(int n);
cudaError_t zsmem_g256_512(int n);
cudaError_t zsmem_g1024_2048(int n);
cudaError_t zsmem_g4096(int n);
cudaError_t zsmem_g8192(int n);

namespace {



__device__ __forceinline__ z2 zmul(z2 a, z2 b) {
  return make_double2(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ z2 zconj(z2 a) { return make_double2(a.x, -a.y); }
__device__ __forceinline__ z2 zscale(z2 a, double s) { return make_double2(a.x * s, a.y * s); }

constexpr int kMaxLog = 13;  // 8192

// Line geometry; LMIN: least lines per CTA (2 for column passes, so that a
// warp's loads cover whole 32-byte sectors of two adjacent columns).
template <int N, int LMIN = 1>
struct ZGeo {
  static constexpr int PT = 8;                            // points per thread
  static constexpr int TL = N >= PT ? N / PT : 1;         // threads per line
  static constexpr int L0 = TL >= 256 ? 1 : 256 / TL;
  static constexpr int L = L0 < LMIN ? LMIN : L0;         // lines per CTA
  static constexpr int NT = TL * L;
  static constexpr int HT = N / 2 + 1;                   // H table entries per line
  static constexpr size_t SMEM = 16 * (size_t)L * N;
  static constexpr size_t SMEM_FUSED = 16 * (size_t)L * (N + HT);
  // first row pass: the lens's x factors over |x - N/2| and one y factor a line
  static constexpr size_t SMEM_FWD = 16 * ((size_t)L * N + HT + L);
  static constexpr int LOG = N == 16 ? 4 : N == 32 ? 5 : N == 64 ? 6 : N == 128 ? 7
                           : N == 256 ? 8 : N == 512 ? 9 : N == 1024 ? 10 : N == 2048 ? 11
                           : N == 4096 ? 12 : 13;
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

// cos(2 pi f) + i sin(2 pi f) for a double f with |f| < 2^50, as float-float.
// Quarter turns in FP64: 4f = q + rho (q an integer, |rho| <= 1/2, both
// exact), so theta = rho pi/2 has |theta| <= pi/4 and rho converts to
// float-float within 2^-48; sin(theta)/theta and cos(theta) are their Taylor
// series in s = theta^2 (terms from s^5 on, below 3e-8 of the result, in
// FP32; the first five in float-float; truncation below 1e-17), and the
// quadrant q mod 4 rotates the result.
__device__ __forceinline__ zf zcis_2pi(double f) {
  const double f4 = 4.0 * f, qd = rint(f4);
  float rh, rl, th, tl, sh, sl;
  d2ff(f4 - qd, rh, rl);
  const long long q = (long long)qd;
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

// 1/(2 pi) as a double-double (the pair sums to it within 6e-34).
constexpr double kInv2PiH = 0.15915494309189535;
constexpr double kInv2PiL = -9.839338337591243e-18;

// x-domain multiplier at (y, x) as float-float: the reference's lens phase
// (X^2+Y^2)*k0/(2f) with X = (x - (n+1)/2) dL (beam2d.py:299-300, :508-510)
// evaluated in FP64, turned into turns by the double-double 1/(2 pi) (error
// ~1e-16 turn for any phase below ~1e15 rad) and taken by zcis_2pi; times
// the mask.
__device__ __forceinline__ zf zxmul_ff(const ZOps& o, int y, int x, int n) {
  zf m = make_float4(1.0f, 0.0f, 0.0f, 0.0f);
  if (o.lens) {
    const double X = (double)(x - (n + 1) / 2) * o.dL, Y = (double)(y - (n + 1) / 2) * o.dL;
    const double ph = (X * X + Y * Y) * o.lens_c;
    const double p = ph * kInv2PiH;
    const double e = fma(ph, kInv2PiH, -p) + ph * kInv2PiL;
    m = zcis_2pi((p - rint(p)) + e);
  }
  if (o.xmask) m = zf_mul(m, z2_to_zf(zmask(o.xmask, o.xmask_type, y, x, n)));
  return m;
}

// cos + i sin of lens_c * u^2 (u = j dL: one coordinate of the reference's
// lens phase, beam2d.py:508-510), the phase in FP64 turned into turns by the
// double-double 1/(2 pi).  exp(i c (X^2 + Y^2)) is the product of the x and
// y factors (which rounds differently from one float64 phase by ~1e-16 of
// the phase).
__device__ __forceinline__ zf zlens_axis(const ZOps& o, int j) {
  const double u = (double)j * o.dL;
  const double ph = (u * u) * o.lens_c;
  const double p = ph * kInv2PiH;
  const double e = fma(ph, kInv2PiH, -p) + ph * kInv2PiL;
  return zcis_2pi((p - rint(p)) + e);
}

// k-domain multiplier at (ky, kx) as float-float: H as zh_value computes it
// (the reference's float64 Kz and phase), times the mask.
__device__ __forceinline__ zf zkmul_ff(const ZOps& o, int ky, int kx, int n) {
  zf m = make_float4(1.0f, 0.0f, 0.0f, 0.0f);
  if (o.apply_h) {
    const int h = (n + 1) / 2;
    const double fx = (double)(kx < h ? kx : kx - n) * o.val;
    const double fy = (double)(ky < h ? ky : ky - n) * o.val;
    const double v = (o.k0 * o.k0 - fx * fx) - fy * fy;
    if (v >= 0.0) {
      const double dk = sqrt(v) * o.z;
      m = zcis_2pi(trunc(dk) - dk);
    } else if (o.evan_mask) {
      m = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
  }
  if (o.kmask) m = zf_mul(m, z2_to_zf(zmask(o.kmask, o.kmask_type, ky, kx, n)));
  return m;
}

// H at ky (fy2 = fy^2 of this row) and |kx| = j, in the reference's order
// (k0^2 - Kx^2) - Ky^2.
__device__ __forceinline__ zf zh_value_kx(const ZOps& o, double fy2, int j) {
  const double fx = (double)j * o.val;
  const double v = (o.k0 * o.k0 - fx * fx) - fy2;
  if (v >= 0.0) {
    const double dk = sqrt(v) * o.z;
    return zcis_2pi(trunc(dk) - dk);
  }
  return o.evan_mask ? make_float4(0.0f, 0.0f, 0.0f, 0.0f) : make_float4(1.0f, 0.0f, 0.0f, 0.0f);
}

// In-place Stockham transform of one line (buf, N points) by TL threads
// (t = 0..TL-1), PT points per thread per stage; element i of the line at
// buf[i * LS].  S = -1 forward, +1 inverse
// (unscaled).  tw[k] = W_N^k.  Barriers are CTA-wide (every line of the CTA
// runs the same stages).
template <int N, int R, int S, int LS>
__device__ __forceinline__ void zstage(zf* buf, int t, int ns, const zf* __restrict__ tw) {
  constexpr int TL = ZGeo<N>::TL, NB = N / R, QB = NB / TL;  // butterflies per thread
  zf v[QB * R];
#pragma unroll
  for (int q = 0; q < QB; ++q)
#pragma unroll
    for (int r = 0; r < R; ++r) v[q * R + r] = buf[(t + q * TL + r * NB) * LS];
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
      buf[o * LS] = zf_add(a[0], a[1]);
      buf[(o + ns) * LS] = zf_sub(a[0], a[1]);
    } else {
      const zf t0 = zf_add(a[0], a[2]), t1 = zf_sub(a[0], a[2]);
      const zf t2 = zf_add(a[1], a[3]);
      zf t3 = zf_sub(a[1], a[3]);
      t3 = S < 0 ? make_float4(t3.z, t3.w, -t3.x, -t3.y)
                 : make_float4(-t3.z, -t3.w, t3.x, t3.y);  // * (S*i)
      buf[o * LS] = zf_add(t0, t2);
      buf[(o + ns) * LS] = zf_add(t1, t3);
      buf[(o + 2 * ns) * LS] = zf_sub(t0, t2);
      buf[(o + 3 * ns) * LS] = zf_sub(t1, t3);
    }
  }
  __syncthreads();
}

template <int N, int S, int LS>
__device__ __forceinline__ void zfft(zf* buf, int t, const zf* __restrict__ tw) {
  constexpr int LOG = ZGeo<N>::LOG;
  int ns = 1;
  if constexpr (LOG & 1) {
    zstage<N, 2, S, LS>(buf, t, ns, tw);
    ns = 2;
  }
#pragma unroll 1
  for (int s = 0; s < LOG / 2; ++s) {
    zstage<N, 4, S, LS>(buf, t, ns, tw);
    ns *= 4;
  }
}

enum ZMode { Z_FWD = 0, Z_INV = 1, Z_FUSED = 2, Z_KINV = 3 };

// One line pass over N lines.  Z_FWD: [pre x multiplier] forward; Z_INV:
// inverse, scale, [post x multiplier], [iprofile]; Z_FUSED (lines are
// columns after a transpose; line index = kx): forward, k multipliers,
// [spectrum write], scale, inverse; Z_KINV (lines are spectrum rows, line
// index = ky): k multipliers, [spectrum write], inverse.  IN_D / OUT_D: the pass reads / writes
// complex128 (else float-float intermediates).
// Lines per CTA of a pass: column passes take at least two adjacent columns.
// 1: the k-first row pass (Z_KINV) takes rows ky and N - ky in one CTA and
// evaluates their common H (Ky**2 is the same) once.
#ifndef LP_ZKINV_PAIRS
#define LP_ZKINV_PAIRS 1
#endif
template <int N, int MODE, bool COLS>
constexpr bool zpairs() {
  // N <= 2048: two rows in at most 512 threads (measured at 2048^2: 0.256 vs
  // 0.290 ms per spectrum-state propagate; 4096 would need 1024-thread CTAs)
  return LP_ZKINV_PAIRS && MODE == Z_KINV && !COLS && ZGeo<N>::TL <= 256;
}
// Geometry of a pass: at least two lines per CTA for column passes and for
// the paired k-first row pass.
template <int N, int MODE, bool COLS>
using ZGM = ZGeo<N, (COLS || zpairs<N, MODE, COLS>()) ? 2 : 1>;

template <int N, int MODE, bool COLS>
constexpr int zmin_blocks() {
  constexpr int nt = ZGM<N, MODE, COLS>::NT;
  // 64 registers (four CTAs a SM) for the plain passes; the passes with H
  // or lens tables take 85 (three)
  constexpr bool tables = MODE >= Z_FUSED || (MODE == Z_FWD && !COLS);
  return nt <= 256 ? (tables ? 3 : 4) : (nt <= 512 ? 2 : 1);
}

// One line pass over N lines.  Rows (COLS false): line = row, element x at
// [line * N + x].  Columns (COLS true): line = column, element x at
// [x * N + line]; neighbouring threads take neighbouring columns of a row
// and the shared-memory lines interleave (element i of line g at i * L + g),
// so loads, stores and the stage exchanges stay coalesced and conflict-free.
// Modes: Z_FWD: [pre x multiplier] forward; Z_INV: inverse, scale, [post x
// multiplier], [iprofile]; Z_FUSED (line index = kx): forward, k
// multipliers, [spectrum write], scale, inverse; Z_KINV (rows of a spectrum,
// line index = ky): k multipliers, [spectrum write], inverse.  IN_D / OUT_D:
// the pass reads / writes complex128 (else float-float intermediates).
template <int N, int MODE, bool IN_D, bool OUT_D, bool COLS>
__global__ void __launch_bounds__(ZGM<N, MODE, COLS>::NT, zmin_blocks<N, MODE, COLS>())
    zline_kernel(const void* __restrict__ in, void* out, ZOps o, const zf* __restrict__ tw) {
  using G = ZGM<N, MODE, COLS>;
  constexpr bool PAIRS = zpairs<N, MODE, COLS>();
  constexpr int LS = COLS ? G::L : 1;  // element stride of a line in shared memory
  extern __shared__ float4 zs[];
  const int g = COLS ? (int)(threadIdx.x % G::L) : (int)(threadIdx.x / G::TL);
  const int t = COLS ? (int)(threadIdx.x / G::L) : (int)(threadIdx.x % G::TL);
  // PAIRS: lines g = 2p, 2p + 1 of the CTA are rows b and N - b of pair
  // base b = blockIdx.x * L/2 + p (b = 0 .. N/2; rows 0 and N/2 are their
  // own mirrors, so the second line of those pairs is idle)
  const int pb = (int)blockIdx.x * (G::L / 2) + g / 2;
  const int line = PAIRS ? ((g & 1) ? N - pb : pb) : (int)blockIdx.x * G::L + g;
  zf* buf = COLS ? zs + g : zs + (size_t)g * N;
  // grid offset of element x of this line
  auto at = [&](int x) -> size_t {
    return COLS ? (size_t)x * N + line : (size_t)line * N + x;
  };
  // N < L: a CTA has more line slots than lines
  const bool live = PAIRS ? ((g & 1) ? (pb >= 1 && pb < N / 2) : pb <= N / 2) : line < N;
  if constexpr (MODE == Z_KINV) {
    // H of this row (ky = line) at |kx| = 0..N/2 once each (H(kx, ky) =
    // H(-kx, ky)), filled while the row's loads are in flight; with PAIRS one
    // table serves rows ky and N - ky and both rows' threads fill it
    zf v[G::PT];
#pragma unroll
    for (int i = 0; i < G::PT && i * G::TL < N; ++i)
      v[i] = live ? z2_to_zf(reinterpret_cast<const z2*>(in)[at(t + G::TL * i)])
                  : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    zf* hb = zs + (size_t)G::L * N + (size_t)(PAIRS ? g / 2 : g) * G::HT;
    if (o.apply_h) {
      const int h = (N + 1) / 2;
      const int ky = PAIRS ? pb : line;  // Ky**2 of row N - b equals that of row b
      const double fy = (double)(ky < h ? ky : ky - N) * o.val;
      const double fy2 = fy * fy;
      if constexpr (PAIRS) {
        for (int j = t + (g & 1) * G::TL; j < G::HT; j += 2 * G::TL) hb[j] = zh_value_kx(o, fy2, j);
      } else {
        for (int j = t; j < G::HT; j += G::TL) hb[j] = zh_value_kx(o, fy2, j);
      }
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < G::PT && i * G::TL < N; ++i) {
      const int kx = t + G::TL * i;
      zf w = v[i];
      if (o.apply_h) w = zf_mul(w, hb[kx <= N / 2 ? kx : N - kx]);
      if (o.kmask && live) w = zf_mul(w, z2_to_zf(zmask(o.kmask, o.kmask_type, line, kx, N)));
      if (o.spectrum_out && live) o.spectrum_out[at(kx)] = zf_to_z2(w);
      buf[kx * LS] = w;
    }
  } else if constexpr (MODE == Z_FWD && !COLS && IN_D) {
    // first row pass: loads in flight while the lens's x factors over
    // |x - N/2| (shared by the CTA's lines) and each line's y factor fill
    zf v[G::PT];
#pragma unroll
    for (int i = 0; i < G::PT && i * G::TL < N; ++i)
      v[i] = live ? z2_to_zf(reinterpret_cast<const z2*>(in)[at(t + G::TL * i)])
                  : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    const bool lens = o.lens && !o.post;
    zf* lt = zs + (size_t)G::L * N;  // [0, HT): x factors; [HT + g]: line g's y factor
    if (lens) {
      for (int j = threadIdx.x; j < G::HT; j += G::NT) lt[j] = zlens_axis(o, j);
      if (t == 0) lt[G::HT + g] = zlens_axis(o, abs(line - N / 2));
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < G::PT && i * G::TL < N; ++i) {
      const int x = t + G::TL * i;
      zf w = v[i];
      if (lens && live) w = zf_mul(zf_mul(w, lt[abs(x - N / 2)]), lt[G::HT + g]);
      if (o.xmask && live && !o.post)
        w = zf_mul(w, z2_to_zf(zmask(o.xmask, o.xmask_type, line, x, N)));
      buf[x * LS] = w;
    }
  } else if constexpr (MODE == Z_FUSED) {
    // loads in flight while the H of this line (kx = line) at |ky| =
    // 0..N/2 fills once each (H(kx, ky) = H(kx, -ky)); the table is read
    // after the forward transform's barriers
    zf v[G::PT];
#pragma unroll
    for (int i = 0; i < G::PT && i * G::TL < N; ++i)
      v[i] = live ? reinterpret_cast<const zf*>(in)[at(t + G::TL * i)]
                  : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (o.apply_h) {
      zf* hb = zs + (size_t)G::L * N + (size_t)g * G::HT;
      const int h = (N + 1) / 2;
      const double fx = (double)(line < h ? line : line - N) * o.val;
      const double a = o.k0 * o.k0 - fx * fx;
      for (int j = t; j < G::HT; j += G::TL) hb[j] = zh_value(o, a, j);
    }
#pragma unroll
    for (int i = 0; i < G::PT && i * G::TL < N; ++i) buf[(t + G::TL * i) * LS] = v[i];
  } else {
#pragma unroll
    for (int i = 0; i < G::PT && i * G::TL < N; ++i) {
      const int x = t + G::TL * i;
      zf v = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
      if (live) {
        if constexpr (IN_D) {
          v = z2_to_zf(reinterpret_cast<const z2*>(in)[at(x)]);
        } else {
          v = reinterpret_cast<const zf*>(in)[at(x)];
        }
      }
      if (MODE == Z_FWD && live && (o.lens || o.xmask) && !o.post)
        v = zf_mul(v, COLS ? zxmul_ff(o, x, line, N) : zxmul_ff(o, line, x, N));
      buf[x * LS] = v;
    }
  }
  __syncthreads();
  if constexpr (MODE == Z_INV || MODE == Z_KINV) {
    zfft<N, 1, LS>(buf, t, tw);
  } else {
    zfft<N, -1, LS>(buf, t, tw);
  }
  if constexpr (MODE == Z_FUSED) {
    const zf* hb = zs + (size_t)G::L * N + (size_t)g * G::HT;
#pragma unroll
    for (int i = 0; i < G::PT && i * G::TL < N; ++i) {
      const int ky = t + G::TL * i;
      zf v = buf[ky * LS];
      if (o.apply_h) v = zf_mul(v, hb[ky <= N / 2 ? ky : N - ky]);
      if (o.kmask && live) v = zf_mul(v, z2_to_zf(zmask(o.kmask, o.kmask_type, ky, line, N)));
      if (o.spectrum_out && live) o.spectrum_out[(size_t)ky * N + line] = zf_to_z2(v);
      buf[ky * LS] = zf_scale(v, o.scale_h, o.scale_l);
    }
    __syncthreads();
    zfft<N, 1, LS>(buf, t, tw);
  }
  if (!live) return;
#pragma unroll
  for (int i = 0; i < G::PT && i * G::TL < N; ++i) {
    const int x = t + G::TL * i;
    zf v = buf[x * LS];
    if (MODE == Z_INV) {
      v = zf_scale(v, o.scale_h, o.scale_l);
      if ((o.lens || o.xmask) && o.post)
        v = zf_mul(v, COLS ? zxmul_ff(o, x, line, N) : zxmul_ff(o, line, x, N));
      if (o.iprofile) {
        float ah, al, bh, bl, ph, pl;
        ff_mul2(v.x, v.y, v.x, v.y, ah, al);
        ff_mul2(v.z, v.w, v.z, v.w, bh, bl);
        ff_add2(ah, al, bh, bl, ph, pl);
        o.iprofile[at(x)] = f2d(ph) + f2d(pl);
      }
    }
    if constexpr (OUT_D) {
      reinterpret_cast<z2*>(out)[at(x)] = zf_to_z2(v);
    } else {
      reinterpret_cast<zf*>(out)[at(x)] = v;
    }
  }
}

// The line-pass variants a size uses: (mode, reads complex128, writes
// complex128, column pass).  Column passes exist for N <= 4096 (two 8192
// lines would need 2048 threads per CTA); 8192 transposes instead.
#define LP_ZLINE_ROWS(X)                                                              \
  X(Z_FWD, true, false, false) X(Z_FWD, false, true, false) X(Z_INV, true, false, false) \
  X(Z_INV, false, true, false) X(Z_FUSED, false, false, false) X(Z_KINV, true, false, false)
#define LP_ZLINE_COLS(X) \
  X(Z_FWD, false, true, true) X(Z_INV, false, true, true) X(Z_FUSED, false, false, true)

// Dynamic shared memory of a pass: lines, plus the H table (fused, k-first
// passes) or the lens tables (first row pass).
template <int N, int M, bool I, bool C>
constexpr size_t zsmem_bytes() {
  using G = ZGM<N, M, C>;
  if constexpr (zpairs<N, M, C>()) return 16 * ((size_t)G::L * N + (size_t)(G::L / 2) * G::HT);
  return M >= Z_FUSED ? G::SMEM_FUSED : (M == Z_FWD && !C && I) ? G::SMEM_FWD : G::SMEM;
}

// CTAs of a pass: N / L lines, or N/2 + 1 row pairs for the paired pass.
template <int N, int M, bool C>
constexpr int zgrid() {
  using G = ZGM<N, M, C>;
  if constexpr (zpairs<N, M, C>()) return (N / 2 + 1 + G::L / 2 - 1) / (G::L / 2);
  return (N + G::L - 1) / G::L;
}

template <int N>
cudaError_t set_smem() {
  cudaError_t e = cudaSuccess;
#define LP_ZSET(M, I, O, C)                                                               \
  if (e == cudaSuccess)                                                                   \
    e = cudaFuncSetAttribute(zline_kernel<N, M, I, O, C>,                                 \
                             cudaFuncAttributeMaxDynamicSharedMemorySize,                 \
                             (int)zsmem_bytes<N, M, I, C>());
  LP_ZLINE_ROWS(LP_ZSET)
  if constexpr (N <= 4096) {
    LP_ZLINE_COLS(LP_ZSET)
  }
#undef LP_ZSET
  return e;
}

template <int N>
cudaError_t zline(int mode, bool in_d, bool out_d, bool cols, const void* in, void* out, ZOps o,
                  const zf* tw, cudaStream_t st) {
  const float sh = (float)o.scale;
  o.scale_h = sh;
  o.scale_l = (float)(o.scale - (double)sh);
  bool done = false;
#define LP_ZLAUNCH(M, I, O, C)                                                              \
  if (!done && mode == M && in_d == I && out_d == O && cols == C) {                         \
    using G = ZGM<N, M, C>;                                                                 \
    zline_kernel<N, M, I, O, C><<<zgrid<N, M, C>(), G::NT, zsmem_bytes<N, M, I, C>(),      \
                                  st>>>(in, out, o, tw);                                    \
    done = true;                                                                            \
  }
  LP_ZLINE_ROWS(LP_ZLAUNCH)
  if constexpr (N <= 4096) {
    LP_ZLINE_COLS(LP_ZLAUNCH)
  }
#undef LP_ZLAUNCH
  return done ? cudaGetLastError() : cudaErrorInvalidValue;
}

}  // namespace
}  // namespace lp
