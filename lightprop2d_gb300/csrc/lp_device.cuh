// Device building blocks for the angular-spectrum propagation kernels:
// compile-time twiddle constants, register-resident DFTs of size 2..64,
// float-float ("double-FP32") arithmetic and the per-point phase functions.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

namespace lp {

// ---------------------------------------------------------------------------
// Compile-time loops.
// ---------------------------------------------------------------------------
template <int I, int N, class F>
__device__ __forceinline__ void static_for_impl(F&& f) {
  if constexpr (I < N) {
    f(std::integral_constant<int, I>{});
    static_for_impl<I + 1, N>(f);
  }
}
template <int N, class F>
__device__ __forceinline__ void static_for(F&& f) {
  static_for_impl<0, N>(f);
}

// ---------------------------------------------------------------------------
// Compile-time cos/sin of 2*pi*k/R (Taylor series on an angle reduced to
// [0, pi/4], evaluated in double at compile time and rounded to float once).
// ---------------------------------------------------------------------------
constexpr double kPi = 3.14159265358979323846264338327950288;

constexpr double ct_sin(double x) {
  double x2 = x * x, term = x, sum = x;
  for (int k = 1; k < 16; ++k) {
    term *= -x2 / double((2 * k) * (2 * k + 1));
    sum += term;
  }
  return sum;
}
constexpr double ct_cos(double x) {
  double x2 = x * x, term = 1.0, sum = 1.0;
  for (int k = 1; k < 16; ++k) {
    term *= -x2 / double((2 * k - 1) * (2 * k));
    sum += term;
  }
  return sum;
}
// cos(2*pi*k/R) (which = 0) or sin(2*pi*k/R) (which = 1).
constexpr double ct_trig(int k, int R, int which) {
  k = ((k % R) + R) % R;
  const int quad = (4 * k) / R;   // quadrant
  const int rem = 4 * k - quad * R;  // angle within quadrant = (pi/2)*rem/R
  double c = 1.0, s = 0.0;
  if (rem != 0) {
    if (2 * rem <= R) {
      const double a = (kPi / 2) * double(rem) / double(R);
      c = ct_cos(a);
      s = ct_sin(a);
    } else {
      const double a = (kPi / 2) * double(R - rem) / double(R);
      c = ct_sin(a);
      s = ct_cos(a);
    }
  }
  double cc = c, ss = s;
  if (quad == 1) { cc = -s; ss = c; }
  if (quad == 2) { cc = -c; ss = -s; }
  if (quad == 3) { cc = s; ss = -c; }
  return which == 0 ? cc : ss;
}

// ---------------------------------------------------------------------------
// Complex helpers on float2 (x = re, y = im).
// ---------------------------------------------------------------------------
__device__ __forceinline__ float2 cadd(float2 a, float2 b) {
  return make_float2(a.x + b.x, a.y + b.y);
}
__device__ __forceinline__ float2 csub(float2 a, float2 b) {
  return make_float2(a.x - b.x, a.y - b.y);
}
__device__ __forceinline__ float2 cmul(float2 a, float2 w) {
  return make_float2(fmaf(a.x, w.x, -a.y * w.y), fmaf(a.x, w.y, a.y * w.x));
}
__device__ __forceinline__ float2 cconj(float2 a) { return make_float2(a.x, -a.y); }
__device__ __forceinline__ float2 cscale(float2 a, float s) {
  return make_float2(a.x * s, a.y * s);
}

// Multiply by the compile-time twiddle W_R^K, W_R = exp(S * 2*pi*i / R),
// S = -1 (forward) or +1 (inverse).  Trivial angles cost no multiply.
template <int R, int K, int S>
__device__ __forceinline__ float2 twc(float2 a) {
  constexpr int k = ((K % R) + R) % R;
  if constexpr (k == 0) {
    return a;
  } else if constexpr (2 * k == R) {
    return make_float2(-a.x, -a.y);
  } else if constexpr (4 * k == R) {  // W = S*i
    if constexpr (S < 0) return make_float2(a.y, -a.x);
    else return make_float2(-a.y, a.x);
  } else if constexpr (4 * k == 3 * R) {  // W = -S*i
    if constexpr (S < 0) return make_float2(-a.y, a.x);
    else return make_float2(a.y, -a.x);
  } else if constexpr ((8 * k) % R == 0) {  // odd multiples of pi/4
    constexpr float h = 0.70710678118654752440f;
    constexpr double c = ct_trig(k, R, 0);
    constexpr double s = S * ct_trig(k, R, 1);
    // (x + iy)(c + is) with |c| = |s| = h
    if constexpr (c > 0 && s > 0) return make_float2(h * (a.x - a.y), h * (a.x + a.y));
    else if constexpr (c > 0 && s < 0) return make_float2(h * (a.x + a.y), h * (a.y - a.x));
    else if constexpr (c < 0 && s > 0) return make_float2(-h * (a.x + a.y), h * (a.x - a.y));
    else return make_float2(h * (a.y - a.x), -h * (a.x + a.y));
  } else {
    constexpr float c = (float)ct_trig(k, R, 0);
    constexpr float s = (float)(S * ct_trig(k, R, 1));
    return make_float2(fmaf(a.x, c, -a.y * s), fmaf(a.x, s, a.y * c));
  }
}

// ---------------------------------------------------------------------------
// In-register DFT of size R (power of two <= 64), natural order in and out:
//   X[k] = sum_n x[n] * exp(S * 2*pi*i * n*k / R).
// Sizes above 8 use one Cooley-Tukey split R = A*B (decimation in time,
// n = B*n1 + n2, k = k1 + A*k2) with compile-time internal twiddles.
// ---------------------------------------------------------------------------
template <int R, int S>
struct Dft;

template <int S>
struct Dft<1, S> {
  __device__ __forceinline__ static void run(float2 (&)[1]) {}
};

template <int S>
struct Dft<2, S> {
  __device__ __forceinline__ static void run(float2 (&v)[2]) {
    const float2 a = v[0], b = v[1];
    v[0] = cadd(a, b);
    v[1] = csub(a, b);
  }
};

template <int S>
struct Dft<4, S> {
  __device__ __forceinline__ static void run(float2 (&v)[4]) {
    const float2 t0 = cadd(v[0], v[2]), t1 = csub(v[0], v[2]);
    const float2 t2 = cadd(v[1], v[3]);
    const float2 t3 = twc<4, 1, S>(csub(v[1], v[3]));
    v[0] = cadd(t0, t2);
    v[2] = csub(t0, t2);
    v[1] = cadd(t1, t3);
    v[3] = csub(t1, t3);
  }
};

template <int S>
struct Dft<8, S> {
  __device__ __forceinline__ static void run(float2 (&v)[8]) {
    // radix-2 first layer, then two radix-4 DFTs (even / odd outputs).
    float2 e[4], o[4];
    static_for<4>([&](auto n) {
      constexpr int i = decltype(n)::value;
      e[i] = cadd(v[i], v[i + 4]);
      o[i] = twc<8, i, S>(csub(v[i], v[i + 4]));
    });
    Dft<4, S>::run(e);
    Dft<4, S>::run(o);
    static_for<4>([&](auto n) {
      constexpr int i = decltype(n)::value;
      v[2 * i] = e[i];
      v[2 * i + 1] = o[i];
    });
  }
};

template <int R>
struct DftSplit {
  // R = A * B with A the first (stride-B) factor.
  static constexpr int A = (R == 16) ? 4 : (R == 32) ? 4 : (R == 64) ? 8 : 2;
  static constexpr int B = R / A;
};

template <int R, int S>
struct Dft {
  static_assert(R == 16 || R == 32 || R == 64, "unsupported register DFT size");
  __device__ __forceinline__ static void run(float2 (&v)[R]) {
    constexpr int A = DftSplit<R>::A, B = DftSplit<R>::B;
    float2 y[R];
    static_for<B>([&](auto n2c) {
      constexpr int n2 = decltype(n2c)::value;
      float2 a[A];
      static_for<A>([&](auto n1) { a[decltype(n1)::value] = v[B * decltype(n1)::value + n2]; });
      Dft<A, S>::run(a);
      static_for<A>([&](auto k1c) {
        constexpr int k1 = decltype(k1c)::value;
        y[k1 * B + n2] = twc<R, n2 * k1, S>(a[k1]);
      });
    });
    static_for<A>([&](auto k1c) {
      constexpr int k1 = decltype(k1c)::value;
      float2 b[B];
      static_for<B>([&](auto n2) { b[decltype(n2)::value] = y[k1 * B + decltype(n2)::value]; });
      Dft<B, S>::run(b);
      static_for<B>([&](auto k2) { v[k1 + A * decltype(k2)::value] = b[decltype(k2)::value]; });
    });
  }
};

// ---------------------------------------------------------------------------
// Float-float arithmetic (value = hi + lo, |lo| <= ulp(hi)/2).  Used to
// reduce the transfer-function phase kz*z (up to ~1e6 cycles) mod 1 with an
// absolute error of ~1e-8 cycles without FP64 instructions.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void two_prod(float a, float b, float& p, float& e) {
  p = a * b;
  e = fmaf(a, b, -p);
}
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// Split a double into a float-float pair (host and device).
struct FF {
  float hi, lo;
};

// Sum of two pairs, accurate to ~2^-44 relative.
__device__ __forceinline__ FF ff_add(FF a, FF b) {
  float s, e;
  two_sum(a.hi, b.hi, s, e);
  e = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
  FF r;
  r.hi = __fadd_rn(s, e);
  r.lo = __fsub_rn(e, __fsub_rn(r.hi, s));
  return r;
}
// a*b + c with the product exact (two_prod), then a pair sum.
__device__ __forceinline__ FF ff_fma(float a, float b, FF c) {
  FF p;
  two_prod(a, b, p.hi, p.lo);
  return ff_add(p, c);
}
__host__ __device__ inline FF ff_from_double(double d) {
  FF r;
  r.hi = (float)d;
  r.lo = (float)(d - (double)r.hi);
  return r;
}

// ---------------------------------------------------------------------------
// Transfer function of free-space propagation at one spectral point.
//
// Reference (beam2d.py:485-489): phase = 2*pi*(trunc(Kz*z) - Kz*z),
// H = cos(phase) + i*sin(phase) = exp(-2*pi*i * Kz*z), with
// Kz = sqrt(k0^2 - kx^2 - ky^2) (0 where negative, beam2d.py:307-308).
//
// With kx = sx/(N dL), ky = sy/(N dL), k0 = 1/wl:
//   Kz*z = R * sqrt(v),  v = 1 - beta*(sx^2 + sy^2),
//   R = z/wl (cycles), beta = (wl/(N dL))^2.
// The caller passes a = 1 - beta*sx^2 (float-float, per column) and
// q = sy^2 (exact in float for |sy| <= 4096).  Returns the phase in cycles
// reduced to about [-0.5, 0.5], or sets *evanescent when v <= 0.
// ---------------------------------------------------------------------------
struct KParams {
  float beta_hi, beta_lo;  // (wl / (N dL))^2
  float R_hi, R_lo;        // z / wl
  float two_pi_k0;         // 2*pi*k0 in FP32 (for the d/dz multiplier, cycles->rad)
};

__device__ __forceinline__ void column_constant(const KParams& kp, float qx, float& a_hi,
                                                float& a_lo) {
  float t_hi, t_lo;
  two_prod(kp.beta_hi, qx, t_hi, t_lo);
  t_lo = fmaf(kp.beta_lo, qx, t_lo);
  float e;
  two_sum(1.0f, -t_hi, a_hi, e);
  a_lo = e - t_lo;
}

// Returns phase (cycles, ~[-0.5,0.5]); sqrt_v receives sqrt(v) (0 if evanescent).
__device__ __forceinline__ float kz_phase_ff(const KParams& kp, float a_hi, float a_lo,
                                             float qy, bool& evanescent, float& sqrt_v) {
  float u_hi, u_lo;
  two_prod(kp.beta_hi, qy, u_hi, u_lo);
  u_lo = fmaf(kp.beta_lo, qy, u_lo);
  float v0, e, v_hi, v_lo;
  two_sum(a_hi, -u_hi, v0, e);
  // Renormalise: near the evanescent cut-off v0 is tiny after cancellation
  // and the low part can exceed ulp(v0); the one-step Newton square root
  // below needs |v_lo| <= ulp(v_hi) or its quadratic error reaches 1e-4
  // cycles there.
  two_sum(v0, e + (a_lo - u_lo), v_hi, v_lo);
  evanescent = !(v_hi > 0.0f);
  const float vv = evanescent ? 1.0f : v_hi;
  const float y = rsqrtf(vv);
  const float s0 = vv * y;
  const float r = fmaf(-s0, s0, vv) + (evanescent ? 0.0f : v_lo);
  const float c = r * (0.5f * y);
  float p_hi, p_e;
  two_prod(kp.R_hi, s0, p_hi, p_e);
  const float p_lo = p_e + fmaf(kp.R_hi, c, kp.R_lo * s0);
  sqrt_v = evanescent ? 0.0f : s0 + c;
  return (p_hi - rintf(p_hi)) + p_lo;
}

// Plain-FP32 phase (comparison variant only: loses the phase at large k0*z).
__device__ __forceinline__ float kz_phase_f32(const KParams& kp, float qx, float qy,
                                              bool& evanescent, float& sqrt_v) {
  const float beta = kp.beta_hi;
  const float v = 1.0f - beta * (qx + qy);
  evanescent = !(v > 0.0f);
  const float s = evanescent ? 0.0f : sqrtf(v);
  sqrt_v = s;
  const float p = (kp.R_hi + kp.R_lo) * s;
  return p - rintf(p);
}

// exp(sign * 2*pi*i * f) for a phase f in cycles already reduced to about
// [-0.5, 0.5].  Default: the special-function-unit sine/cosine (__sincosf) of
// the angle 2*pi*f, absolute error <= 2^-21.4 (3.6e-7) on [-pi, pi] -- a
// field error of a few 1e-7 relative L2, inside the 1e-5 bar, at two SFU
// operations per point.  LP_ACCURATE_SINCOS selects sincospif instead.
__device__ __forceinline__ float2 cis_cycles(float f, float sign) {
  float s, c;
#ifdef LP_ACCURATE_SINCOS
  sincospif(2.0f * f, &s, &c);
#else
  __sincosf(6.28318530717958647692f * f, &s, &c);
#endif
  return make_float2(c, sign * s);
}

// exp(i*phi) for an FP32 phase mask value in radians.  phi is first reduced
// to [-pi, pi] by Cody-Waite reduction (k = rint(phi / 2pi), r = phi - k*2pi
// with 2pi split into two floats, hi = fl(2pi) and lo = fl(2pi - hi); the
// FMA keeps r to ~1 ulp for |phi| < 2^22), then the special-function unit's
// sine/cosine (absolute error ~4e-7 on [-pi, pi]), a few instructions where
// the accurate sincosf takes tens.  LP_ACCURATE_SINCOS selects sincosf.
__device__ __forceinline__ float2 cis_radians(float phi) {
  float s, c;
#ifdef LP_ACCURATE_SINCOS
  sincosf(phi, &s, &c);
#else
  constexpr float kInv2Pi = 0.15915493667125702f;
  constexpr float k2PiHi = 6.2831854820251465f;
  constexpr float k2PiLo = -1.7484555314695172e-07f;
  const float k = rintf(phi * kInv2Pi);
  const float r = fmaf(-k, k2PiLo, fmaf(-k, k2PiHi, phi));
  __sincosf(r, &s, &c);
#endif
  return make_float2(c, s);
}

// Lens phase in cycles at integer offsets (jx, jy) from the grid centre:
// (X^2+Y^2)*k0/(2f) radians = kappa*(jx^2+jy^2) cycles, kappa = dL^2 k0/(4 pi f).
// m = jx^2 + jy^2 is an exact integer (up to 2^25 at N = 8192); above 2^24 it
// does not fit a float, so it is split into m_hi = fl(m) and the exact
// remainder m_lo.
__device__ __forceinline__ float lens_cycles(float kap_hi, float kap_lo, int m) {
  const float m_hi = (float)m;
  const float m_lo = (float)(m - (int)m_hi);
  float c_hi, c_e;
  two_prod(kap_hi, m_hi, c_hi, c_e);
  const float c_lo = fmaf(kap_lo, m_hi, c_e) + kap_hi * m_lo;
  return (c_hi - rintf(c_hi)) + c_lo;
}

// Mask element fetch (x- or k-domain multiplier).
__device__ __forceinline__ float2 mask_value(const void* mask, int type, size_t idx) {
  switch (type) {
    case 1: return make_float2(__ldg(reinterpret_cast<const float*>(mask) + idx), 0.0f);
    case 2: return __ldg(reinterpret_cast<const float2*>(mask) + idx);
    case 3: return make_float2((float)__ldg(reinterpret_cast<const uint8_t*>(mask) + idx), 0.0f);
    case 4: {
      const float ph = __ldg(reinterpret_cast<const float*>(mask) + idx);
      float s, c;
      sincosf(ph, &s, &c);
      return make_float2(c, s);
    }
    case 5: return make_float2((float)__ldg(reinterpret_cast<const double*>(mask) + idx), 0.0f);
    case 6: {
      const double2 d = __ldg(reinterpret_cast<const double2*>(mask) + idx);
      return make_float2((float)d.x, (float)d.y);
    }
    default: return make_float2(1.0f, 0.0f);
  }
}

// Multiplier at row y, column x of an N x N mask of any type, including the
// compact generator tables (7: separable fx[x]*fy[y], 8: per-column row span,
// 9: complex separable fx[x]*fy[y]).
__device__ __forceinline__ float2 mask_value_xy(const void* mask, int type, int y, int x, int n) {
  if (type == 9) {
    const float2* t = reinterpret_cast<const float2*>(mask);
    return cmul(__ldg(t + x), __ldg(t + n + y));
  }
  if (type == 7) {
    const float* t = reinterpret_cast<const float*>(mask);
    return make_float2(__ldg(t + x) * __ldg(t + n + y), 0.0f);
  }
  if (type == 8) {
    const int* t = reinterpret_cast<const int*>(mask);
    return make_float2((y >= __ldg(t + x) && y < __ldg(t + n + x)) ? 1.0f : 0.0f, 0.0f);
  }
  return mask_value(mask, type, (size_t)y * n + x);
}

}  // namespace lp
