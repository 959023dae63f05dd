// 2-D FFT building blocks for any grid size N (templated; usable from any
// translation unit): the per-line transform, the x-domain and spectral
// multipliers, and "tiles" -- L rows or C columns of one N x N grid processed
// by one CTA -- which the per-size pass kernels and the batched persistent
// kernel are made of.
//
// A 1-D transform of length N runs on T = N/16 threads that each keep 16
// points in registers.  Thread t holds the elements {t + T*j : j < 16} of its
// line both before and after the transform (natural order), so a forward
// transform, a pointwise spectral multiply and an inverse transform chain
// with no reordering.
//
// The transform is a mixed-radix Stockham sequence (radix 16, then 16, then
// 16/8/4/2 as N needs).  Stage s with radix R and Ns = product of the
// earlier radices computes, for each butterfly b < N/R,
//     a[r] = x[b + r*N/R] * W_(Ns*R)^(r*(b mod Ns))      (r < R)
//     y[(b/Ns)*Ns*R + (b mod Ns) + r*Ns] = DFT_R(a)[r],
// thread t doing butterflies b = t + q*T (q < 16/R).  Between stages the
// line goes through one padded shared-memory buffer (element i at
// i + i/16, which keeps the stride-16 writes of the first stage free of bank
// conflicts).  Every stage is one small register butterfly, so the kernels
// stay small enough for the SM instruction cache; per-point multipliers are
// evaluated in rolled loops for the same reason.
#pragma once

#include <cmath>

#include "lightprop2d_gb300.h"
#include "lp_device.cuh"
#include "lp_internal.h"

namespace lp {

template <int N>
struct Plan;  // radices of the stages (0 = no stage)
template <> struct Plan<16> { static constexpr int R[4] = {16, 0, 0, 0}; };
template <> struct Plan<32> { static constexpr int R[4] = {16, 2, 0, 0}; };
template <> struct Plan<64> { static constexpr int R[4] = {16, 4, 0, 0}; };
template <> struct Plan<128> { static constexpr int R[4] = {16, 8, 0, 0}; };
template <> struct Plan<256> { static constexpr int R[4] = {16, 16, 0, 0}; };
template <> struct Plan<512> { static constexpr int R[4] = {16, 16, 2, 0}; };
template <> struct Plan<1024> { static constexpr int R[4] = {16, 16, 4, 0}; };
template <> struct Plan<2048> { static constexpr int R[4] = {16, 16, 8, 0}; };
template <> struct Plan<4096> { static constexpr int R[4] = {16, 16, 16, 0}; };
template <> struct Plan<8192> { static constexpr int R[4] = {16, 16, 16, 2}; };

constexpr int cmin(int a, int b) { return a < b ? a : b; }
constexpr int cmax(int a, int b) { return a > b ? a : b; }

template <int N>
struct FftGeo {
  using P = Plan<N>;
  static constexpr int T = N / 16;  // threads per line
  static constexpr int NST = P::R[3] ? 4 : P::R[2] ? 3 : P::R[1] ? 2 : 1;
  static constexpr int BUF = N + N / 16;  // padded line buffer (float2)
  // Twiddles of stage s (s >= 1): W_(NS*R)^(r*k) for r = 1..R-1, k < NS, at
  // TW_OFF_s + (r-1)*NS + k (the r = 0 row, all ones, is not stored).
  static constexpr int NS1 = 16, NS2 = 16 * P::R[1], NS3 = NS2 * cmax(P::R[2], 1);
  static constexpr int TW_OFF1 = 0;
  static constexpr int TW_OFF2 = TW_OFF1 + cmax(P::R[1] - 1, 0) * NS1;
  static constexpr int TW_OFF3 = TW_OFF2 + cmax(P::R[2] - 1, 0) * NS2;
  static constexpr int TW_SIZE = TW_OFF3 + cmax(P::R[3] - 1, 0) * NS3 + 1;
};

// Host: the stage twiddles of size N (forward sign), computed in double and
// rounded once; layout as in FftGeo.
template <int N>
inline void fill_twiddles(float2* tw) {
  using G = FftGeo<N>;
  auto fill = [&](int off, int R, int NS) {
    for (int r = 1; r < R; ++r)
      for (int k = 0; k < NS; ++k) {
        const double ang = -2.0 * kPi * (double)(r * k) / (double)(NS * R);
        tw[off + (r - 1) * NS + k] = make_float2((float)std::cos(ang), (float)std::sin(ang));
      }
  };
  if (G::NST >= 2) fill(G::TW_OFF1, Plan<N>::R[1], G::NS1);
  if (G::NST >= 3) fill(G::TW_OFF2, Plan<N>::R[2], G::NS2);
  if (G::NST >= 4) fill(G::TW_OFF3, Plan<N>::R[3], G::NS3);
  tw[G::TW_SIZE - 1] = make_float2(1.0f, 0.0f);
}

__device__ __forceinline__ int pad16(int i) { return i + (i >> 4); }

// Programmatic dependent launch: wait for the previous kernel's results, and
// let the next kernel's CTAs be scheduled as this grid's CTAs retire.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_release() { asm volatile("griddepcontrol.launch_dependents;"); }

// Shared-memory slot of line element i: interleaved (IL: lines fastest, for
// column CTAs whose lanes run across lines) or one buffer per line (rows).
template <int N, bool IL, int LINES>
__device__ __forceinline__ int sidx(int i, int line) {
  if constexpr (IL) return pad16(i) * LINES + line;
  else return line * FftGeo<N>::BUF + pad16(i);
}

// Barrier over the threads that share an exchange buffer.  SY = 0: the warp
// (lines of <= 32 threads); SY = 1: the whole CTA; SY = 2: the calling
// thread's group of 256 threads (named barrier 1 + threadIdx.x / 256), for
// kernels whose CTA holds several independent tile groups; SY >= 32 (a
// multiple of 32): the calling thread's group of SY threads (named barrier
// 1 + threadIdx.x / SY; at most 15 groups per CTA).
template <int SY>
constexpr int group_threads() {
  return SY == 2 ? 256 : SY;
}

template <int SY>
__device__ __forceinline__ void group_sync() {
  if constexpr (SY == 0) {
    __syncwarp();
  } else if constexpr (SY == 1) {
    __syncthreads();
  } else {
    constexpr int GT = group_threads<SY>();
    static_assert(GT % 32 == 0, "group barriers cover whole warps");
    asm volatile("bar.sync %0, %1;" ::"r"(1 + (int)(threadIdx.x / GT)), "n"(GT) : "memory");
  }
}

// Thread index within the exchange group.
template <int SY>
__device__ __forceinline__ int group_tid() {
  if constexpr (SY >= 2) return (int)(threadIdx.x % (unsigned)group_threads<SY>());
  else return (int)threadIdx.x;
}

// Global loads / stores; CG = cache at L2 only (data produced by other CTAs
// of the same launch must not be served from a stale L1 line).
template <bool CG>
__device__ __forceinline__ float2 gld(const float2* p) {
  if constexpr (CG) return __ldcg(p); else return *p;
}
template <bool CG>
__device__ __forceinline__ void gst(float2* p, float2 v) {
  if constexpr (CG) __stcg(p, v); else *p = v;
}

// Stage 0 (radix 16, Ns = 1): element t + T*r of the input is v[r]; output r
// goes to element t*16 + r of the buffer.  The buffer must be free.
template <int N, int S, bool IL, int LINES>
__device__ __forceinline__ void fft_first(float2 (&v)[16], float2* buf, int t, int line) {
  Dft<16, S>::run(v);
  if constexpr (FftGeo<N>::NST > 1) {
    static_for<16>([&](auto rc) {
      constexpr int r = decltype(rc)::value;
      buf[sidx<N, IL, LINES>(t * 16 + r, line)] = v[r];
    });
  }
}

// Stage s > 0: inputs from shared memory, twiddled, DFT, outputs to shared
// memory (middle stage) or to registers in natural order (last stage).
template <int N, int S, int s, bool IL, int LINES, int SY>
__device__ __forceinline__ void fft_stage(float2 (&v)[16], float2* buf, const float2* tw, int t,
                                          int line) {
  using G = FftGeo<N>;
  constexpr int R = Plan<N>::R[s], T = G::T, nb = 16 / R;
  constexpr int NS = (s == 1) ? G::NS1 : (s == 2) ? G::NS2 : G::NS3;
  constexpr int OFF = (s == 1) ? G::TW_OFF1 : (s == 2) ? G::TW_OFF2 : G::TW_OFF3;
  constexpr bool LAST = (s == G::NST - 1);
  group_sync<SY>();
  static_for<nb>([&](auto qc) {
    constexpr int q = decltype(qc)::value;
    const int b = t + q * T;
    static_for<R>([&](auto rc) {
      constexpr int r = decltype(rc)::value;
      v[q + nb * r] = buf[sidx<N, IL, LINES>(b + r * (N / R), line)];
    });
  });
  if constexpr (!LAST) group_sync<SY>();
  static_for<nb>([&](auto qc) {
    constexpr int q = decltype(qc)::value;
    const int b = t + q * T;
    const int k = b & (NS - 1);
    float2 a[R];
    static_for<R>([&](auto rc) { a[decltype(rc)::value] = v[q + nb * decltype(rc)::value]; });
    static_for<R - 1>([&](auto rc) {
      constexpr int r = decltype(rc)::value + 1;
      float2 w = tw[OFF + (r - 1) * NS + k];
      if constexpr (S > 0) w.y = -w.y;
      a[r] = cmul(a[r], w);
    });
    Dft<R, S>::run(a);
    if constexpr (LAST) {
      static_for<R>([&](auto rc) { v[q + nb * decltype(rc)::value] = a[decltype(rc)::value]; });
    } else {
      const int o = (b / NS) * NS * R + k;
      static_for<R>([&](auto rc) {
        constexpr int r = decltype(rc)::value;
        buf[sidx<N, IL, LINES>(o + r * NS, line)] = a[r];
      });
    }
  });
}

// Stages after the first (natural-order result in registers).  tw: the
// stage twiddles of size N (shared memory).
template <int N, int S, bool IL, int LINES, int SY>
__device__ __forceinline__ void fft_rest(float2 (&v)[16], float2* buf, const float2* tw, int t,
                                         int line) {
  if constexpr (FftGeo<N>::NST >= 2) fft_stage<N, S, 1, IL, LINES, SY>(v, buf, tw, t, line);
  if constexpr (FftGeo<N>::NST >= 3) fft_stage<N, S, 2, IL, LINES, SY>(v, buf, tw, t, line);
  if constexpr (FftGeo<N>::NST >= 4) fft_stage<N, S, 3, IL, LINES, SY>(v, buf, tw, t, line);
}

// Column modes of the size kernels only: COL_FUSED / COL_INV with H and the
// scale as the only spectral multipliers (the launcher picks them when ops
// allow).
constexpr int COL_FUSED_LEAN = 3;
constexpr int COL_INV_LEAN = 4;

struct NoHook {
  __device__ __forceinline__ void operator()() const {}
};

__device__ __forceinline__ void conj16(float2 (&v)[16]) {
  static_for<16>([&](auto jc) { v[decltype(jc)::value] = cconj(v[decltype(jc)::value]); });
}

// ------------------------------------------------------------------ rows --
// Multiply the thread's 16 points of row y (columns t + T*j) by an x-domain
// mask.  The 16 loads are issued before any is used (independent requests
// in flight); real masks ignore `conj`.
template <int N, int MT = -1>
__device__ __forceinline__ void apply_mask_row(float2 (&v)[16], const void* mask, int type,
                                               int conj, int y, int t, float2* slots,
                                               int nthreads, int tid) {
  constexpr int T = FftGeo<N>::T;
  const size_t row = (size_t)y * N + t;
  switch (MT >= 0 ? MT : type) {  // MT >= 0: the mask type is known when compiling
    case 1: {  // float32
      const float* p = reinterpret_cast<const float*>(mask) + row;
      float m[16];
      static_for<16>([&](auto jc) { m[jc.value] = __ldg(p + T * jc.value); });
      static_for<16>([&](auto jc) { v[jc.value] = cscale(v[jc.value], m[jc.value]); });
      break;
    }
    case 3: {  // uint8 / bool
      const uint8_t* p = reinterpret_cast<const uint8_t*>(mask) + row;
      uint8_t m[16];
      static_for<16>([&](auto jc) { m[jc.value] = __ldg(p + T * jc.value); });
      static_for<16>([&](auto jc) { v[jc.value] = cscale(v[jc.value], (float)m[jc.value]); });
      break;
    }
    case 2: {  // complex64
      const float2* p = reinterpret_cast<const float2*>(mask) + row;
      float2 m[16];
      static_for<16>([&](auto jc) { m[jc.value] = __ldg(p + T * jc.value); });
      static_for<16>([&](auto jc) {
        v[jc.value] = cmul(v[jc.value], conj ? cconj(m[jc.value]) : m[jc.value]);
      });
      break;
    }
    case 4: {  // float32 phase: exp(i*phi)
      const float* p = reinterpret_cast<const float*>(mask) + row;
      static_for<16>([&](auto jc) { slots[jc.value * nthreads + tid].x = __ldg(p + T * jc.value); });
#pragma unroll 1
      for (int j0 = 0; j0 < 16; j0 += 4) {  // four independent evaluations in flight
        float ph[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) ph[u] = slots[(j0 + u) * nthreads + tid].x;
#pragma unroll
        for (int u = 0; u < 4; ++u) slots[(j0 + u) * nthreads + tid] = cis_radians(ph[u]);
      }
      static_for<16>([&](auto jc) {
        const float2 m = slots[jc.value * nthreads + tid];
        v[jc.value] = cmul(v[jc.value], conj ? cconj(m) : m);
      });
      break;
    }
    case 7: {  // separable table: fx[x] * fy[y]
      const float* fx = reinterpret_cast<const float*>(mask);
      const float fy = __ldg(fx + N + y);
      float m[16];
      static_for<16>([&](auto jc) { m[jc.value] = __ldg(fx + t + T * jc.value); });
      static_for<16>([&](auto jc) { v[jc.value] = cscale(v[jc.value], m[jc.value] * fy); });
      break;
    }
    case 8: {  // per-column row span: lo[x] <= y < hi[x]
      const int* lo = reinterpret_cast<const int*>(mask);
      int a[16], b[16];
      static_for<16>([&](auto jc) {
        a[jc.value] = __ldg(lo + t + T * jc.value);
        b[jc.value] = __ldg(lo + N + t + T * jc.value);
      });
      static_for<16>([&](auto jc) {
        if (!(y >= a[jc.value] && y < b[jc.value])) v[jc.value] = make_float2(0.0f, 0.0f);
      });
      break;
    }
    case 9: {  // complex separable table: fx[x] * fy[y]
      const float2* fx = reinterpret_cast<const float2*>(mask);
      float2 fy = __ldg(fx + N + y);
      if (conj) fy = cconj(fy);
      float2 m[16];
      static_for<16>([&](auto jc) { m[jc.value] = __ldg(fx + t + T * jc.value); });
      static_for<16>([&](auto jc) {
        v[jc.value] = cmul(cmul(v[jc.value], conj ? cconj(m[jc.value]) : m[jc.value]), fy);
      });
      break;
    }
    default: {  // float64, complex128: rolled
#pragma unroll 1
      for (int j = 0; j < 16; ++j) {
        float2 m = mask_value_xy(mask, type, y, t + T * j, N);
        if (conj) m = cconj(m);
        // v[j] with a run-time j would spill the array: rotate instead
        static_for<16>([&](auto jc) {
          if (jc.value == j) v[jc.value] = cmul(v[jc.value], m);
        });
      }
      break;
    }
  }
}

// Row-tile features compiled into a kernel (a bit clear: that part of RowOps
// is known to be unused, so its code is left out of the kernel).
constexpr int ROW_LENS = 1, ROW_XMASK = 2, ROW_XSTORE = 4, ROW_SCALE = 8, ROW_IPROF = 16,
              ROW_MOMENTS = 32;
constexpr int ROW_ALL = 63, ROW_LEAN = 0;
// Row-kernel variants of the per-size passes: every multiplier; the
// transform alone; an FP32 phase mask (mask type 4) before or after the
// transform and nothing else (phase-mask design and split-step screens).
static_assert(LP_MASK_PHASE_F32 == 4, "apply_mask_row's case 4 is the FP32 phase mask");
enum RowVariant { ROWV_ALL = 0, ROWV_LEAN = 1, ROWV_PHASE = 2 };
template <int V>
constexpr int row_feat() {
  return V == ROWV_LEAN ? ROW_LEAN : V == ROWV_PHASE ? (ROW_XMASK | ROW_XSTORE) : ROW_ALL;
}
template <int V>
constexpr int row_mask_type() {
  return V == ROWV_PHASE ? (int)LP_MASK_PHASE_F32 : -1;
}
#ifndef LP_ROW_PHASE
#define LP_ROW_PHASE 1
#endif
__host__ __device__ inline int row_variant(const RowOps& o) {
  const bool plain = !o.lens && o.scale == 1.0f && !o.iprofile && !o.moments;
  if (plain && !o.xmask) return ROWV_LEAN;
  if (LP_ROW_PHASE && plain && o.xmask_type == LP_MASK_PHASE_F32) return ROWV_PHASE;
  return ROWV_ALL;
}

// Multiply the thread's 16 points of row y by the x-domain multipliers: the
// lens phase, evaluated in a rolled loop into the thread's own buffer slots
// (one copy of the phase code), then the mask.  The slots must be free.
template <int N, int SY = 1, int FEAT = ROW_ALL, int MT = -1>
__device__ __forceinline__ void apply_xops(float2 (&v)[16], float2* slots, int nthreads, int y,
                                           int t, const RowOps& ops) {
  constexpr int T = FftGeo<N>::T;
  const int tid = group_tid<SY>();
  if ((FEAT & ROW_LENS) && ops.lens) {
    const int jy = y - N / 2;
#pragma unroll 1
    for (int j = 0; j < 16; ++j) {
      const int jx = t + T * j - N / 2;
      float2 m = cis_cycles(lens_cycles(ops.kap_hi, ops.kap_lo, jx * jx + jy * jy), 1.0f);
      if (ops.conj) m = cconj(m);
      slots[j * nthreads + tid] = m;
    }
    static_for<16>([&](auto jc) {
      constexpr int j = decltype(jc)::value;
      v[j] = cmul(v[j], slots[j * nthreads + tid]);
    });
  }
  if ((FEAT & ROW_XMASK) && ops.xmask)
    apply_mask_row<N, MT>(v, ops.xmask, ops.xmask_type, ops.conj, y, t, slots, nthreads, tid);
}

template <int N, bool CG = false>
__device__ __forceinline__ void load_row(float2 (&v)[16], const float2* in, int y, int t) {
  constexpr int T = FftGeo<N>::T;
  const float2* src = in + (size_t)y * N + t;
  static_for<16>([&](auto jc) { v[decltype(jc)::value] = gld<CG>(src + T * decltype(jc)::value); });
}

// Intensity moments of the thread's 16 points of row y (columns t + T*j),
// reduced over the exchange group (FP32 per thread and across a warp's
// lanes, FP64 across warps) and added to out[0..5) with one atomic per value per group:
// sum I, sum jx I, sum jy I, sum jx^2 I, sum jy^2 I (offsets from the centre).
template <int N, int SY>
__device__ __forceinline__ void tile_moments(const float2 (&v)[16], int y, int t, double* out) {
  constexpr int T = FftGeo<N>::T;
  float s0 = 0.0f, s1 = 0.0f, s3 = 0.0f;
  static_for<16>([&](auto jc) {
    constexpr int j = decltype(jc)::value;
    const float I = fmaf(v[j].x, v[j].x, v[j].y * v[j].y);
    const float jx = (float)(t + T * j - N / 2);
    s0 += I;
    s1 = fmaf(jx, I, s1);
    s3 = fmaf(jx * jx, I, s3);
  });
  // Warp sums in FP32 (the offsets are integers with squares below 2^24, so
  // each product is exact to FP32 rounding), the group's warps in
  // float-float, and one FP64 conversion per value for the atomic: FP64 runs
  // at a small fraction of the FP32 rate on this part.
  const float jy = (float)(y - N / 2);
  float m[5] = {s0, s1, jy * s0, s3, jy * jy * s0};
  __shared__ float red[2][5][32];  // [group][value][warp of the group]
  const int tid = group_tid<SY>(), lane = tid & 31, w = tid >> 5;
  const int grp = SY == 2 ? (int)(threadIdx.x >> 8) : 0;
#pragma unroll
  for (int k = 0; k < 5; ++k) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m[k] += __shfl_down_sync(0xffffffffu, m[k], o);
    if (lane == 0) red[grp][k][w] = m[k];
  }
  group_sync<SY>();
  if (tid < 5) {
    FF a = {0.0f, 0.0f};
    const int nw = (SY == 2 ? 256 : (int)blockDim.x) >> 5;
    for (int i = 0; i < nw; ++i) a = ff_add(a, FF{red[grp][tid][i], 0.0f});
    atomicAdd(out + tid, (double)a.hi + (double)a.lo);
  }
  group_sync<SY>();
}

// Row tile: rows tile*L .. tile*L+L-1 by the first L*T threads of the
// exchange group (SY: the CTA, or a 256-thread group), thread (line
// g = tid / T, t = tid % T).  FEAT: the parts of RowOps the kernel supports
// (ROW_* bits; ROW_LEAN = the transform alone; the caller guarantees that
// ops uses nothing outside FEAT).  v holds the thread's loaded points of row
// tile*L + g; `after_first` runs after the first stage (the per-size kernels
// prefetch the next tile there).  The exchange buffer (L * BUF floats2) must
// be free on entry.
template <int N, int S, int L, int NT, bool CG, int SY = 1, class Hook, int FEAT = ROW_ALL,
          int MT = -1>
__device__ __forceinline__ void row_tile(float2 (&v)[16], float2* out, int tile, const RowOps& ops,
                                         float2* buf, const float2* tw, Hook after_first) {
  constexpr int T = FftGeo<N>::T;
  constexpr int LS = T > 32 ? SY : 0;  // a line spans several warps
  const int tid = group_tid<SY>();
  const int g = tid / T, t = tid % T;
  const int y = tile * L + g;
  const bool xops = ((FEAT & ROW_LENS) && ops.lens) || ((FEAT & ROW_XMASK) && ops.xmask);
  const bool at_store = (FEAT & ROW_XSTORE) && ops.x_at_store;
  if (xops && !at_store) {
    apply_xops<N, SY, FEAT, MT>(v, buf, NT, y, t, ops);
    group_sync<SY>();
  }
  fft_first<N, S, false, L>(v, buf, t, g);
  after_first();
  fft_rest<N, S, false, L, LS>(v, buf, tw, t, g);
  if ((FEAT & ROW_SCALE) && ops.scale != 1.0f) {
    static_for<16>([&](auto jc) { v[decltype(jc)::value] = cscale(v[decltype(jc)::value], ops.scale); });
  }
  if (xops && at_store) {
    group_sync<SY>();
    apply_xops<N, SY, FEAT, MT>(v, buf, NT, y, t, ops);
  }
  float2* dst = out + (size_t)y * N + t;
  static_for<16>([&](auto jc) { gst<CG>(dst + T * decltype(jc)::value, v[decltype(jc)::value]); });
  if ((FEAT & ROW_IPROF) && ops.iprofile) {
    float* ip = ops.iprofile + (size_t)y * N + t;
    static_for<16>([&](auto jc) {
      constexpr int j = decltype(jc)::value;
      ip[T * j] = fmaf(v[j].x, v[j].x, v[j].y * v[j].y);
    });
  }
  if constexpr (NT >= 32 && (FEAT & ROW_MOMENTS) != 0) {  // whole warps (batch: 256 threads)
    if (ops.moments) tile_moments<N, SY>(v, y, t, ops.moments);
  }
}

// --------------------------------------------------------------- columns --
// Spectral multiplier without the mask at (qx = sx^2, qy = sy^2): H(z)
// [* d/dz factor].  (a_hi, a_lo) = 1 - beta*qx, the column constant of the
// float-float phase (unused by the plain-FP32 variant).
template <int N, bool LEAN = false>
__device__ __forceinline__ float2 transfer_value_cc(float qx, float a_hi, float a_lo, float qy,
                                                    const ColOps& ops) {
  bool evan;
  float sv, f;
  if (!LEAN && ops.phase_fp32) {
    f = kz_phase_f32(ops.kp, qx, qy, evan, sv);
  } else {
    f = kz_phase_ff(ops.kp, a_hi, a_lo, qy, evan, sv);
  }
  // H = exp(-2*pi*i*f); the adjoint uses conj(H).
  float2 m = cis_cycles(f, ops.conj ? 1.0f : -1.0f);
  if (evan) m = ops.evan_mask ? make_float2(0.0f, 0.0f) : make_float2(1.0f, 0.0f);
  if (!LEAN && ops.dz) {
    // d/dz exp(-2*pi*i*kz*z) = -2*pi*i*kz * H with kz = k0*sqrt(v).
    const float gz = ops.kp.two_pi_k0 * sv * (ops.conj ? 1.0f : -1.0f);
    m = make_float2(-gz * m.y, gz * m.x);
  }
  return m;
}

// The same at (|sy|, sx).
template <int N>
__device__ __forceinline__ float2 transfer_value(int sy_abs, int sx, const ColOps& ops) {
  const float qx = (float)(sx * sx), qy = (float)(sy_abs * sy_abs);
  float a_hi = 0.0f, a_lo = 0.0f;
  if (!ops.phase_fp32) column_constant(ops.kp, qx, a_hi, a_lo);
  return transfer_value_cc<N>(qx, a_hi, a_lo, qy, ops);
}

// Spectral multiply of the thread's 16 points of column kx (rows t + T*j).
// The transfer function of the tile's C columns is first tabulated in shared
// memory over |ky| = 0..N/2 (C*(N/2+1) evaluations shared by all threads),
// then each point reads its entry.  Table entry (a, cc) sits at a*C + cc and
// thread tid fills column tid % C, so each thread computes its column's
// float-float constant once.  The buffer must be free on entry; it is in use
// on exit (callers sync before the next transform).  LEAN: H with the scale
// folded into the table, and no k mask, spectrum write, d/dz or plain-FP32
// phase (the caller checks ops for these).
template <int N, int C, int SY = 1, bool LEAN = false>
__device__ __forceinline__ void apply_spectral(float2 (&v)[16], float2* tab, int x0, int c, int t,
                                               const ColOps& ops) {
  constexpr int T = FftGeo<N>::T, NT = C * T, HE = N / 2 + 1;
  const int kx = x0 + c;
  if constexpr (LEAN) {
    const int tid = group_tid<SY>();
    const int cc = tid % C, x = x0 + cc;
    const int sx = x < N / 2 ? x : x - N;
    const float qx = (float)(sx * sx);
    float a_hi, a_lo;
    column_constant(ops.kp, qx, a_hi, a_lo);
#pragma unroll 1
    for (int a = tid / C; a < HE; a += NT / C)
      tab[a * C + cc] = cscale(transfer_value_cc<N, true>(qx, a_hi, a_lo, (float)(a * a), ops),
                               ops.scale);
    group_sync<SY>();
    static_for<16>([&](auto jc) {
      constexpr int j = decltype(jc)::value;
      const int ky = t + T * j;
      const int a = ky <= N / 2 ? ky : N - ky;
      v[j] = cmul(v[j], tab[a * C + c]);
    });
    return;
  }
  if (ops.apply_h) {
    const int tid = group_tid<SY>();
    const int cc = tid % C, x = x0 + cc;
    const int sx = x < N / 2 ? x : x - N;
    const float qx = (float)(sx * sx);
    float a_hi = 0.0f, a_lo = 0.0f;
    if (!ops.phase_fp32) column_constant(ops.kp, qx, a_hi, a_lo);
#pragma unroll 1
    for (int a = tid / C; a < HE; a += NT / C)
      tab[a * C + cc] = transfer_value_cc<N>(qx, a_hi, a_lo, (float)(a * a), ops);
    group_sync<SY>();
  }
  static_for<16>([&](auto jc) {
    constexpr int j = decltype(jc)::value;
    const int ky = t + T * j;
    float2 m = make_float2(1.0f, 0.0f);
    if (ops.apply_h) {
      const int a = ky <= N / 2 ? ky : N - ky;
      m = tab[a * C + c];
    }
    if (ops.kmask) {
      float2 km = mask_value_xy(ops.kmask, ops.kmask_type, ky, kx, N);
      if (ops.conj) km = cconj(km);
      m = cmul(m, km);
    }
    if (ops.apply_h || ops.kmask) v[j] = cmul(v[j], m);
    if (ops.spectrum_out) ops.spectrum_out[(size_t)ky * N + kx] = v[j];
    if (ops.scale != 1.0f) v[j] = cscale(v[j], ops.scale);
  });
}

template <int N, bool CG = false>
__device__ __forceinline__ void load_col(float2 (&v)[16], const float2* in, int x, int t) {
  constexpr int T = FftGeo<N>::T;
  const float2* src = in + (size_t)t * N + x;
  static_for<16>([&](auto jc) {
    v[decltype(jc)::value] = gld<CG>(src + (size_t)T * N * decltype(jc)::value);
  });
}

// Column tile: columns tile*C .. tile*C+C-1 by the first C*T threads of the
// exchange group (SY), thread (c = tid % C, t = tid / C).  MODE: COL_FWD forward
// transform; COL_INV spectral multiply then inverse transform; COL_FUSED
// forward, spectral multiply, inverse (one copy of the transform code:
// inverse(x) = conj(forward(conj(x)))); COL_FUSED_LEAN / COL_INV_LEAN the
// same with H and the scale only (apply_spectral's LEAN form).  v holds the thread's loaded points;
// `after_first` runs after the first stage of the first transform and
// `before_store` after the last stage has read the buffer into registers.
// The buffer (C * BUF float2) must be free on entry; callers sync the group
// before reusing it.
template <int N, int MODE, int C, bool CG, int SY = 1, class Hook, class Hook2 = NoHook>
__device__ __forceinline__ void col_tile(float2 (&v)[16], float2* out, int tile, const ColOps& ops,
                                         float2* buf, const float2* tw, Hook after_first,
                                         Hook2 before_store = NoHook{}) {
  constexpr int T = FftGeo<N>::T;
  const int tid = group_tid<SY>();
  const int c = tid % C, t = tid / C;
  const int x0 = tile * C, x = x0 + c;
  if constexpr (MODE == COL_FWD) {
    fft_first<N, -1, true, C>(v, buf, t, c);
    after_first();
    fft_rest<N, -1, true, C, SY>(v, buf, tw, t, c);
  } else if constexpr (MODE == COL_INV || MODE == COL_INV_LEAN) {
    apply_spectral<N, C, SY, MODE == COL_INV_LEAN>(v, buf, x0, c, t, ops);
    group_sync<SY>();
    fft_first<N, 1, true, C>(v, buf, t, c);
    after_first();
    fft_rest<N, 1, true, C, SY>(v, buf, tw, t, c);
  } else {
#pragma unroll 1
    for (int pass = 0; pass < 2; ++pass) {
      fft_first<N, -1, true, C>(v, buf, t, c);
      if (pass == 0) after_first();
      fft_rest<N, -1, true, C, SY>(v, buf, tw, t, c);
      if (pass == 0) {
        group_sync<SY>();
        apply_spectral<N, C, SY, MODE == COL_FUSED_LEAN>(v, buf, x0, c, t, ops);
        group_sync<SY>();
        conj16(v);
      }
    }
    conj16(v);
  }
  before_store();
  float2* dst = out + (size_t)t * N + x;
  static_for<16>([&](auto jc) {
    gst<CG>(dst + (size_t)T * N * decltype(jc)::value, v[decltype(jc)::value]);
  });
}

}  // namespace lp
