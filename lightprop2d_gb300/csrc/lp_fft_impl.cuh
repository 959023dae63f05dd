// 2-D FFT passes for one grid size N (the including file defines LP_N).
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
// stay small enough for the SM instruction cache; per-point multipliers
// (transfer function, lens phase) are computed in rolled loops into
// per-thread shared-memory slots for the same reason.
#pragma once

#include "lp_device.cuh"
#include "lp_internal.h"

#ifndef LP_N
#error "define LP_N before including lp_fft_impl.cuh"
#endif

namespace lp {
namespace {

template <int N>
struct Plan;  // radices of the stages (0 = no stage)
template <> struct Plan<16> { static constexpr int R[3] = {16, 0, 0}; };
template <> struct Plan<32> { static constexpr int R[3] = {16, 2, 0}; };
template <> struct Plan<64> { static constexpr int R[3] = {16, 4, 0}; };
template <> struct Plan<128> { static constexpr int R[3] = {16, 8, 0}; };
template <> struct Plan<256> { static constexpr int R[3] = {16, 16, 0}; };
template <> struct Plan<512> { static constexpr int R[3] = {16, 16, 2}; };
template <> struct Plan<1024> { static constexpr int R[3] = {16, 16, 4}; };
template <> struct Plan<2048> { static constexpr int R[3] = {16, 16, 8}; };
template <> struct Plan<4096> { static constexpr int R[3] = {16, 16, 16}; };

constexpr int cmin(int a, int b) { return a < b ? a : b; }
constexpr int cmax(int a, int b) { return a > b ? a : b; }

template <int N>
struct Geo {
  static constexpr int P = 16;                    // points per thread
  static constexpr int T = N / P;                 // threads per line
  static constexpr int NST = Plan<N>::R[2] ? 3 : Plan<N>::R[1] ? 2 : 1;
  static constexpr int BUF = N + N / 16;          // padded line buffer (float2)
  static constexpr int LINES = cmin(N, cmax(1, 256 / T));  // lines per CTA
  static constexpr int THREADS = LINES * T;
  static constexpr size_t SMEM = sizeof(float2) * LINES * BUF;
  // Twiddle table offsets: stage 1 at 0 (R1*16 entries), stage 2 after it.
  static constexpr int NS1 = 16, NS2 = 16 * Plan<N>::R[1];
  static constexpr int TW_OFF1 = 0, TW_OFF2 = Plan<N>::R[1] * NS1;
  static constexpr int TW_SIZE = TW_OFF2 + Plan<N>::R[2] * NS2 + 1;
};

#ifndef LP_MIN_BLOCKS
#define LP_MIN_BLOCKS 2
#endif

// Stage twiddles, layout per stage [r][k] = W_(Ns*R)^(r*k), forward sign.
__device__ float2 g_tw[Geo<LP_N>::TW_SIZE];

__device__ __forceinline__ int pad16(int i) { return i + (i >> 4); }

// Shared-memory slot of line element i: interleaved (IL: lines fastest, for
// column CTAs whose lanes run across lines) or one buffer per line (rows).
template <int N, bool IL>
__device__ __forceinline__ int sidx(int i, int line) {
  if constexpr (IL) return pad16(i) * Geo<N>::LINES + line;
  else return line * Geo<N>::BUF + pad16(i);
}

template <bool CTA>
__device__ __forceinline__ void line_sync() {
  if constexpr (CTA) __syncthreads(); else __syncwarp();
}

// Stage s > 0: inputs from shared memory, twiddled, DFT, outputs to shared
// memory (middle stage) or to registers in natural order (last stage).
template <int N, int S, int s, bool IL, bool CTA>
__device__ __forceinline__ void fft_stage(float2 (&v)[16], float2* buf, int t, int line) {
  constexpr int R = Plan<N>::R[s], T = Geo<N>::T, nb = 16 / R;
  constexpr int NS = (s == 1) ? Geo<N>::NS1 : Geo<N>::NS2;
  constexpr int OFF = (s == 1) ? Geo<N>::TW_OFF1 : Geo<N>::TW_OFF2;
  constexpr bool LAST = (s == Geo<N>::NST - 1);
  line_sync<CTA>();
  static_for<nb>([&](auto qc) {
    constexpr int q = decltype(qc)::value;
    const int b = t + q * T;
    static_for<R>([&](auto rc) {
      constexpr int r = decltype(rc)::value;
      v[q + nb * r] = buf[sidx<N, IL>(b + r * (N / R), line)];
    });
  });
  if constexpr (!LAST) line_sync<CTA>();
  static_for<nb>([&](auto qc) {
    constexpr int q = decltype(qc)::value;
    const int b = t + q * T;
    const int k = b & (NS - 1);
    float2 a[R];
    static_for<R>([&](auto rc) { a[decltype(rc)::value] = v[q + nb * decltype(rc)::value]; });
    static_for<R - 1>([&](auto rc) {
      constexpr int r = decltype(rc)::value + 1;
      float2 w = g_tw[OFF + r * NS + k];
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
        buf[sidx<N, IL>(o + r * NS, line)] = a[r];
      });
    }
  });
}

// One 1-D transform of the thread's 16 register points (natural order in and
// out).  The first stage reads the registers; the buffer must be free
// (callers sync before reuse).
template <int N, int S, bool IL, bool CTA>
__device__ __forceinline__ void fft_line(float2 (&v)[16], float2* buf, int t, int line) {
  Dft<16, S>::run(v);
  if constexpr (Geo<N>::NST > 1) {
    // stage 0 (radix 16, Ns = 1): element t + T*r of the input is v[r];
    // output r goes to element t*16 + r.
    static_for<16>([&](auto rc) {
      constexpr int r = decltype(rc)::value;
      buf[sidx<N, IL>(t * 16 + r, line)] = v[r];
    });
    fft_stage<N, S, 1, IL, CTA>(v, buf, t, line);
    if constexpr (Geo<N>::NST == 3) fft_stage<N, S, 2, IL, CTA>(v, buf, t, line);
  }
}

// ------------------------------------------------------------------ rows --
// x-domain multiplier (lens phase and/or mask) for row y at column x.
template <int N>
__device__ __forceinline__ float2 xop_value(int y, int x, const RowOps& ops) {
  float2 m = make_float2(1.0f, 0.0f);
  if (ops.lens) {
    const float jx = (float)(x - N / 2), jy = (float)(y - N / 2);
    m = cis_cycles(lens_cycles(ops.kap_hi, ops.kap_lo, fmaf(jx, jx, jy * jy)), 1.0f);
  }
  if (ops.xmask) m = cmul(m, mask_value(ops.xmask, ops.xmask_type, (size_t)y * N + x));
  if (ops.conj) m = cconj(m);
  return m;
}

// Multiply the thread's 16 points of row y by the x-domain multiplier.  The
// multiplier is evaluated in a rolled loop into the thread's own buffer slots
// (one copy of the phase code), then applied.  The slots must be free.
template <int N>
__device__ __forceinline__ void apply_xops(float2 (&v)[16], float2* slots, int nthreads, int tid,
                                           int y, int t, const RowOps& ops) {
  constexpr int T = Geo<N>::T;
#pragma unroll 1
  for (int j = 0; j < 16; ++j) slots[j * nthreads + tid] = xop_value<N>(y, t + T * j, ops);
  static_for<16>([&](auto jc) {
    constexpr int j = decltype(jc)::value;
    v[j] = cmul(v[j], slots[j * nthreads + tid]);
  });
}

template <int N, int S>
__global__ void __launch_bounds__(Geo<N>::THREADS, LP_MIN_BLOCKS)
    row_kernel(const float2* in, float2* out, RowOps ops) {
  constexpr int T = Geo<N>::T, L = Geo<N>::LINES;
  constexpr bool CTA = T > 32;
  extern __shared__ float2 smem[];
  const int g = threadIdx.x / T, t = threadIdx.x % T;
  const int y = blockIdx.x * L + g;
  const size_t row0 = (size_t)y * N;

  float2 v[16];
  static_for<16>([&](auto jc) {
    constexpr int j = decltype(jc)::value;
    v[j] = in[row0 + t + T * j];
  });
  const bool xops = ops.lens || ops.xmask;
  if (xops && !ops.x_at_store) {
    apply_xops<N>(v, smem, Geo<N>::THREADS, threadIdx.x, y, t, ops);
    __syncthreads();
  }
  fft_line<N, S, false, CTA>(v, smem, t, g);
  if (ops.scale != 1.0f) {
    static_for<16>([&](auto jc) { v[decltype(jc)::value] = cscale(v[decltype(jc)::value], ops.scale); });
  }
  if (xops && ops.x_at_store) {
    __syncthreads();
    apply_xops<N>(v, smem, Geo<N>::THREADS, threadIdx.x, y, t, ops);
  }
  static_for<16>([&](auto jc) {
    constexpr int j = decltype(jc)::value;
    out[row0 + t + T * j] = v[j];
  });
  if (ops.iprofile) {
    static_for<16>([&](auto jc) {
      constexpr int j = decltype(jc)::value;
      ops.iprofile[row0 + t + T * j] = fmaf(v[j].x, v[j].x, v[j].y * v[j].y);
    });
  }
}

// --------------------------------------------------------------- columns --
// Multiplier at spectral point (ky, kx): kmask * H(z) [* d/dz factor].
template <int N>
__device__ __forceinline__ float2 spectral_value(int ky, int kx, float a_hi, float a_lo,
                                                 float qx, const ColOps& ops) {
  float2 m = make_float2(1.0f, 0.0f);
  if (ops.apply_h) {
    const int sy = ky < N / 2 ? ky : ky - N;
    const float qy = (float)(sy * sy);
    bool evan;
    float sv;
    const float f = ops.phase_fp32 ? kz_phase_f32(ops.kp, qx, qy, evan, sv)
                                   : kz_phase_ff(ops.kp, a_hi, a_lo, qy, evan, sv);
    // H = exp(-2*pi*i*f); the adjoint uses conj(H).
    m = cis_cycles(f, ops.conj ? 1.0f : -1.0f);
    if (evan) m = ops.evan_mask ? make_float2(0.0f, 0.0f) : make_float2(1.0f, 0.0f);
    if (ops.dz) {
      // d/dz exp(-2*pi*i*kz*z) = -2*pi*i*kz * H with kz = k0*sqrt(v).
      const float g = ops.kp.two_pi_k0 * sv * (ops.conj ? 1.0f : -1.0f);
      m = make_float2(-g * m.y, g * m.x);
    }
  }
  if (ops.kmask) {
    float2 km = mask_value(ops.kmask, ops.kmask_type, (size_t)ky * N + kx);
    if (ops.conj) km = cconj(km);
    m = cmul(m, km);
  }
  return m;
}

// Spectral multiply of the thread's 16 points of column kx (rows t + T*j),
// multiplier evaluated in a rolled loop into the thread's slots (which must
// be free), then optional spectrum write and scale.
template <int N>
__device__ __forceinline__ void apply_spectral(float2 (&v)[16], float2* slots, int nthreads,
                                               int tid, int kx, int t, const ColOps& ops) {
  constexpr int T = Geo<N>::T;
  const int sx = kx < N / 2 ? kx : kx - N;
  const float qx = (float)(sx * sx);
  float a_hi = 1.0f, a_lo = 0.0f;
  if (ops.apply_h && !ops.phase_fp32) column_constant(ops.kp, qx, a_hi, a_lo);
  if (ops.apply_h || ops.kmask) {
#pragma unroll 1
    for (int j = 0; j < 16; ++j)
      slots[j * nthreads + tid] = spectral_value<N>(t + T * j, kx, a_hi, a_lo, qx, ops);
    static_for<16>([&](auto jc) {
      constexpr int j = decltype(jc)::value;
      v[j] = cmul(v[j], slots[j * nthreads + tid]);
    });
  }
  if (ops.spectrum_out) {
    static_for<16>([&](auto jc) {
      constexpr int j = decltype(jc)::value;
      ops.spectrum_out[(size_t)(t + T * j) * N + kx] = v[j];
    });
  }
  if (ops.scale != 1.0f) {
    static_for<16>([&](auto jc) { v[decltype(jc)::value] = cscale(v[decltype(jc)::value], ops.scale); });
  }
}

template <int N, int MODE>
__global__ void __launch_bounds__(Geo<N>::THREADS, LP_MIN_BLOCKS)
    col_kernel(const float2* in, float2* out, ColOps ops) {
  constexpr int T = Geo<N>::T, C = Geo<N>::LINES, NT = Geo<N>::THREADS;
  extern __shared__ float2 smem[];
  const int c = threadIdx.x % C, t = threadIdx.x / C;
  const int x = blockIdx.x * C + c;

  float2 v[16];
  static_for<16>([&](auto jc) {
    constexpr int j = decltype(jc)::value;
    v[j] = in[(size_t)(t + T * j) * N + x];
  });

  if constexpr (MODE == COL_FWD) {
    fft_line<N, -1, true, true>(v, smem, t, c);
  } else if constexpr (MODE == COL_INV) {
    apply_spectral<N>(v, smem, NT, threadIdx.x, x, t, ops);
    __syncthreads();
    fft_line<N, 1, true, true>(v, smem, t, c);
  } else {
    // Forward transform, spectral multiply, inverse transform through one
    // copy of the transform code: inverse(x) = conj(forward(conj(x))).
#pragma unroll 1
    for (int pass = 0; pass < 2; ++pass) {
      if (pass == 1) {
        static_for<16>([&](auto jc) { v[decltype(jc)::value] = cconj(v[decltype(jc)::value]); });
      }
      fft_line<N, -1, true, true>(v, smem, t, c);
      __syncthreads();
      if (pass == 0) {
        apply_spectral<N>(v, smem, NT, threadIdx.x, x, t, ops);
        __syncthreads();
      }
    }
    static_for<16>([&](auto jc) { v[decltype(jc)::value] = cconj(v[decltype(jc)::value]); });
  }

  static_for<16>([&](auto jc) {
    constexpr int j = decltype(jc)::value;
    out[(size_t)(t + T * j) * N + x] = v[j];
  });
}

// ------------------------------------------------------------- launchers --
cudaError_t init_size() {
  constexpr int N = LP_N;
  static float2 host_tw[Geo<N>::TW_SIZE];
  auto fill = [&](int off, int R, int NS) {
    for (int r = 0; r < R; ++r)
      for (int k = 0; k < NS; ++k) {
        const double ang = -2.0 * kPi * (double)(r * k) / (double)(NS * R);
        host_tw[off + r * NS + k] = make_float2((float)cos(ang), (float)sin(ang));
      }
  };
  if (Geo<N>::NST >= 2) fill(Geo<N>::TW_OFF1, Plan<N>::R[1], Geo<N>::NS1);
  if (Geo<N>::NST >= 3) fill(Geo<N>::TW_OFF2, Plan<N>::R[2], Geo<N>::NS2);
  cudaError_t e = cudaMemcpyToSymbol(g_tw, host_tw, sizeof(host_tw));
  const int smem = (int)Geo<N>::SMEM;
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(row_kernel<N, -1>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(row_kernel<N, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(col_kernel<N, COL_FWD>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(col_kernel<N, COL_INV>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(col_kernel<N, COL_FUSED>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  return e;
}

cudaError_t launch_row(int inverse, const float2* in, float2* out, const RowOps& ops,
                       cudaStream_t st) {
  constexpr int N = LP_N;
  const dim3 grid(N / Geo<N>::LINES), block(Geo<N>::THREADS);
  if (inverse)
    row_kernel<N, 1><<<grid, block, Geo<N>::SMEM, st>>>(in, out, ops);
  else
    row_kernel<N, -1><<<grid, block, Geo<N>::SMEM, st>>>(in, out, ops);
  return cudaGetLastError();
}

cudaError_t launch_col(int mode, const float2* in, float2* out, const ColOps& ops,
                       cudaStream_t st) {
  constexpr int N = LP_N;
  const dim3 grid(N / Geo<N>::LINES), block(Geo<N>::THREADS);
  switch (mode) {
    case COL_FWD:
      col_kernel<N, COL_FWD><<<grid, block, Geo<N>::SMEM, st>>>(in, out, ops);
      break;
    case COL_INV:
      col_kernel<N, COL_INV><<<grid, block, Geo<N>::SMEM, st>>>(in, out, ops);
      break;
    default:
      col_kernel<N, COL_FUSED><<<grid, block, Geo<N>::SMEM, st>>>(in, out, ops);
      break;
  }
  return cudaGetLastError();
}

}  // namespace
}  // namespace lp

#define LP_CAT2(a, b) a##b
#define LP_CAT(a, b) LP_CAT2(a, b)
namespace lp {
extern const SizeOps LP_CAT(size_ops_, LP_N);
const SizeOps LP_CAT(size_ops_, LP_N) = {LP_N, &init_size, &launch_row, &launch_col};
}  // namespace lp
