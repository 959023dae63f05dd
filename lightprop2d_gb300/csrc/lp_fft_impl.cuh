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
// stay small enough for the SM instruction cache.
//
// Kernels are persistent: a CTA loops over units (a few rows, or a few
// columns) and loads the next unit's points into a second register set while
// it transforms the current one, so global-memory latency overlaps the
// arithmetic.  The per-point transfer function is tabulated per column over
// |ky| (it depends on ky only through ky^2), halving its evaluations.
#pragma once

#include "lp_device.cuh"
#include "lp_internal.h"

#ifndef LP_N
#error "define LP_N before including lp_fft_impl.cuh"
#endif
// Columns per CTA of the column kernels for 1024 <= N <= 2048.
#ifndef LP_COL_C
#define LP_COL_C 4
#endif
// 1: load the next unit into a second register set while transforming the
// current one; 0: load it at the top of the next iteration.
#ifndef LP_PREFETCH
#define LP_PREFETCH 1
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
  // rows per CTA: 256 threads for large N, one warp's worth for small N
  static constexpr int ROWS = N >= 1024 ? cmax(1, 256 / T) : cmin(N, cmax(1, 32 / T));
  // columns per CTA: at least 4 so every row segment is a full 32-byte sector
  static constexpr int COLS = N >= 4096 ? 2 : N >= 1024 ? LP_COL_C : cmin(N, cmax(4, 32 / T));
  static constexpr int ROW_THREADS = ROWS * T;
  static constexpr int COL_THREADS = COLS * T;
  static constexpr int ROW_UNITS = N / ROWS;
  static constexpr int COL_UNITS = N / COLS;
  // Twiddle table offsets: stage 1 at 0 (R1*16 entries), stage 2 after it.
  static constexpr int NS1 = 16, NS2 = 16 * Plan<N>::R[1];
  static constexpr int TW_OFF1 = 0, TW_OFF2 = Plan<N>::R[1] * NS1;
  static constexpr int TW_SIZE = TW_OFF2 + Plan<N>::R[2] * NS2 + 1;
  // Shared memory: exchange buffer of the CTA's lines, then the twiddles.
  static constexpr size_t ROW_SMEM = sizeof(float2) * (ROWS * BUF + TW_SIZE);
  static constexpr size_t COL_SMEM = sizeof(float2) * (COLS * BUF + TW_SIZE);
};

// Stage twiddles, layout per stage [r][k] = W_(Ns*R)^(r*k), forward sign.
__device__ float2 g_tw[Geo<LP_N>::TW_SIZE];

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
  else return line * Geo<N>::BUF + pad16(i);
}

template <bool CTA>
__device__ __forceinline__ void line_sync() {
  if constexpr (CTA) __syncthreads(); else __syncwarp();
}

// Stage 0 (radix 16, Ns = 1): element t + T*r of the input is v[r]; output r
// goes to element t*16 + r of the buffer.  The buffer must be free.
template <int N, int S, bool IL, int LINES>
__device__ __forceinline__ void fft_first(float2 (&v)[16], float2* buf, int t, int line) {
  Dft<16, S>::run(v);
  if constexpr (Geo<N>::NST > 1) {
    static_for<16>([&](auto rc) {
      constexpr int r = decltype(rc)::value;
      buf[sidx<N, IL, LINES>(t * 16 + r, line)] = v[r];
    });
  }
}

// Stage s > 0: inputs from shared memory, twiddled, DFT, outputs to shared
// memory (middle stage) or to registers in natural order (last stage).
template <int N, int S, int s, bool IL, int LINES, bool CTA>
__device__ __forceinline__ void fft_stage(float2 (&v)[16], float2* buf, const float2* tw, int t,
                                          int line) {
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
      v[q + nb * r] = buf[sidx<N, IL, LINES>(b + r * (N / R), line)];
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
      float2 w = tw[OFF + r * NS + k];
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

// Stages after the first (natural-order result in registers).  The stage
// twiddles sit after the CTA's exchange buffer (copied there by load_twiddles).
template <int N, int S, bool IL, int LINES, bool CTA>
__device__ __forceinline__ void fft_rest(float2 (&v)[16], float2* buf, int t, int line) {
  const float2* tw = buf + LINES * Geo<N>::BUF;
  if constexpr (Geo<N>::NST >= 2) fft_stage<N, S, 1, IL, LINES, CTA>(v, buf, tw, t, line);
  if constexpr (Geo<N>::NST == 3) fft_stage<N, S, 2, IL, LINES, CTA>(v, buf, tw, t, line);
}

// Copies the stage twiddles into shared memory after the exchange buffer.  It
// reads only this file's table, so it runs before the wait on the previous
// kernel; the first barrier of the unit loop orders it before any use.
template <int N, int LINES, int NT>
__device__ __forceinline__ void load_twiddles(float2* smem) {
  float2* tw = smem + LINES * Geo<N>::BUF;
  for (int i = threadIdx.x; i < Geo<N>::TW_SIZE; i += NT) tw[i] = g_tw[i];
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

// Multiply the thread's 16 points of row y by the x-domain multiplier,
// evaluated in a rolled loop into the thread's own buffer slots (one copy of
// the phase code), then applied.  The slots must be free.
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

template <int N>
__device__ __forceinline__ void load_row(float2 (&v)[16], const float2* in, int y, int t) {
  constexpr int T = Geo<N>::T;
  const float2* src = in + (size_t)y * N + t;
  static_for<16>([&](auto jc) { v[decltype(jc)::value] = src[T * decltype(jc)::value]; });
}

template <int N, int S>
__global__ void __launch_bounds__(Geo<N>::ROW_THREADS)
    row_kernel(const float2* in, float2* out, RowOps ops) {
  constexpr int T = Geo<N>::T, L = Geo<N>::ROWS, NU = Geo<N>::ROW_UNITS;
  constexpr int NT = Geo<N>::ROW_THREADS;
  constexpr bool CTA = T > 32;
  extern __shared__ float2 smem[];
  const int g = threadIdx.x / T, t = threadIdx.x % T;
  const bool xops = ops.lens || ops.xmask;
  load_twiddles<N, L, NT>(smem);
  pdl_wait();
  pdl_release();
  int unit = blockIdx.x;
  float2 v[16];
#if LP_PREFETCH
  float2 p[16];
  if (unit < NU) load_row<N>(v, in, unit * L + g, t);
#endif
#pragma unroll 1
  while (unit < NU) {
    const int y = unit * L + g, next = unit + gridDim.x;
#if !LP_PREFETCH
    load_row<N>(v, in, y, t);
#endif
    __syncthreads();  // buffer free: previous unit's last-stage reads are done
    if (xops && !ops.x_at_store) {
      apply_xops<N>(v, smem, NT, threadIdx.x, y, t, ops);
      __syncthreads();
    }
    fft_first<N, S, false, L>(v, smem, t, g);
#if LP_PREFETCH
    if (next < NU) load_row<N>(p, in, next * L + g, t);
#endif
    fft_rest<N, S, false, L, CTA>(v, smem, t, g);
    if (ops.scale != 1.0f) {
      static_for<16>([&](auto jc) { v[decltype(jc)::value] = cscale(v[decltype(jc)::value], ops.scale); });
    }
    if (xops && ops.x_at_store) {
      __syncthreads();
      apply_xops<N>(v, smem, NT, threadIdx.x, y, t, ops);
    }
    float2* dst = out + (size_t)y * N + t;
    static_for<16>([&](auto jc) { dst[T * decltype(jc)::value] = v[decltype(jc)::value]; });
    if (ops.iprofile) {
      float* ip = ops.iprofile + (size_t)y * N + t;
      static_for<16>([&](auto jc) {
        constexpr int j = decltype(jc)::value;
        ip[T * j] = fmaf(v[j].x, v[j].x, v[j].y * v[j].y);
      });
    }
#if LP_PREFETCH
    static_for<16>([&](auto jc) { v[decltype(jc)::value] = p[decltype(jc)::value]; });
#endif
    unit = next;
  }
}

// --------------------------------------------------------------- columns --
// Spectral multiplier without the mask at (|sy|, sx): H(z) [* d/dz factor].
template <int N>
__device__ __forceinline__ float2 transfer_value(int sy_abs, int sx, const ColOps& ops) {
  const float qx = (float)(sx * sx), qy = (float)(sy_abs * sy_abs);
  bool evan;
  float sv, f;
  if (ops.phase_fp32) {
    f = kz_phase_f32(ops.kp, qx, qy, evan, sv);
  } else {
    float a_hi, a_lo;
    column_constant(ops.kp, qx, a_hi, a_lo);
    f = kz_phase_ff(ops.kp, a_hi, a_lo, qy, evan, sv);
  }
  // H = exp(-2*pi*i*f); the adjoint uses conj(H).
  float2 m = cis_cycles(f, ops.conj ? 1.0f : -1.0f);
  if (evan) m = ops.evan_mask ? make_float2(0.0f, 0.0f) : make_float2(1.0f, 0.0f);
  if (ops.dz) {
    // d/dz exp(-2*pi*i*kz*z) = -2*pi*i*kz * H with kz = k0*sqrt(v).
    const float gz = ops.kp.two_pi_k0 * sv * (ops.conj ? 1.0f : -1.0f);
    m = make_float2(-gz * m.y, gz * m.x);
  }
  return m;
}

// Spectral multiply of the thread's 16 points of column kx (rows t + T*j).
// The transfer function of the CTA's C columns is first tabulated in shared
// memory over |ky| = 0..N/2 (C*(N/2+1) evaluations shared by all threads),
// then each point reads its entry.  The buffer must be free on entry; it is
// in use on exit (callers sync before the next transform).
template <int N, int C>
__device__ __forceinline__ void apply_spectral(float2 (&v)[16], float2* tab, int x0, int c, int t,
                                               const ColOps& ops) {
  constexpr int T = Geo<N>::T, NT = C * T, E = (N / 2 + 1) * C;
  const int kx = x0 + c;
  if (ops.apply_h) {
#pragma unroll 1
    for (int i = threadIdx.x; i < E; i += NT) {
      const int cc = i % C, a = i / C;
      const int x = x0 + cc;
      tab[i] = transfer_value<N>(a, x < N / 2 ? x : x - N, ops);
    }
    __syncthreads();
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
      float2 km = mask_value(ops.kmask, ops.kmask_type, (size_t)ky * N + kx);
      if (ops.conj) km = cconj(km);
      m = cmul(m, km);
    }
    if (ops.apply_h || ops.kmask) v[j] = cmul(v[j], m);
    if (ops.spectrum_out) ops.spectrum_out[(size_t)ky * N + kx] = v[j];
    if (ops.scale != 1.0f) v[j] = cscale(v[j], ops.scale);
  });
}

template <int N>
__device__ __forceinline__ void load_col(float2 (&v)[16], const float2* in, int x, int t) {
  constexpr int T = Geo<N>::T;
  const float2* src = in + (size_t)t * N + x;
  static_for<16>([&](auto jc) { v[decltype(jc)::value] = src[(size_t)T * N * decltype(jc)::value]; });
}

template <int N, int MODE>
__global__ void __launch_bounds__(Geo<N>::COL_THREADS)
    col_kernel(const float2* in, float2* out, ColOps ops) {
  constexpr int T = Geo<N>::T, C = Geo<N>::COLS, NU = Geo<N>::COL_UNITS;
  extern __shared__ float2 smem[];
  const int c = threadIdx.x % C, t = threadIdx.x / C;
  load_twiddles<N, C, C * T>(smem);
  pdl_wait();
  pdl_release();
  int unit = blockIdx.x;
  float2 v[16];
#if LP_PREFETCH
  float2 p[16];
  if (unit < NU) load_col<N>(v, in, unit * C + c, t);
#define LP_PREFETCH_COL(cond) \
  if (cond) load_col<N>(p, in, next * C + c, t)
#else
#define LP_PREFETCH_COL(cond)
#endif
#pragma unroll 1
  while (unit < NU) {
    const int x0 = unit * C, x = x0 + c, next = unit + gridDim.x;
#if !LP_PREFETCH
    load_col<N>(v, in, x, t);
#endif
    __syncthreads();  // buffer free: previous unit's last-stage reads are done
    if constexpr (MODE == COL_FWD) {
      fft_first<N, -1, true, C>(v, smem, t, c);
      LP_PREFETCH_COL(next < NU);
      fft_rest<N, -1, true, C, true>(v, smem, t, c);
    } else if constexpr (MODE == COL_INV) {
      apply_spectral<N, C>(v, smem, x0, c, t, ops);
      __syncthreads();
      fft_first<N, 1, true, C>(v, smem, t, c);
      LP_PREFETCH_COL(next < NU);
      fft_rest<N, 1, true, C, true>(v, smem, t, c);
    } else {
      // Forward transform, spectral multiply, inverse transform through one
      // copy of the transform code: inverse(x) = conj(forward(conj(x))).
#pragma unroll 1
      for (int pass = 0; pass < 2; ++pass) {
        fft_first<N, -1, true, C>(v, smem, t, c);
        LP_PREFETCH_COL(pass == 0 && next < NU);
        fft_rest<N, -1, true, C, true>(v, smem, t, c);
        __syncthreads();
        if (pass == 0) {
          apply_spectral<N, C>(v, smem, x0, c, t, ops);
          __syncthreads();
          static_for<16>([&](auto jc) { v[decltype(jc)::value] = cconj(v[decltype(jc)::value]); });
        }
      }
      static_for<16>([&](auto jc) { v[decltype(jc)::value] = cconj(v[decltype(jc)::value]); });
    }
    float2* dst = out + (size_t)t * N + x;
    static_for<16>([&](auto jc) { dst[(size_t)T * N * decltype(jc)::value] = v[decltype(jc)::value]; });
#if LP_PREFETCH
    static_for<16>([&](auto jc) { v[decltype(jc)::value] = p[decltype(jc)::value]; });
#endif
    unit = next;
  }
#undef LP_PREFETCH_COL
}

// ------------------------------------------------------------- launchers --
int g_sms = 0;                 // SM count of the device set up last
int g_occ_row = 1, g_occ_col = 1;  // max resident CTAs per SM
int g_ctas_row = 0, g_ctas_col = 0;  // tuned CTAs per SM (0 = built-in choice)

// Built-in choice: as many resident CTAs per SM as fit (measured on GB300:
// latency hiding from more resident warps outweighs a fuller last wave).
// The autotuner may pick fewer.
int ctas_in_effect(int occ, int tuned) { return tuned > 0 ? (tuned < occ ? tuned : occ) : occ; }

int grid_for(int units, int occ, int tuned) {
  const int g = g_sms * ctas_in_effect(occ, tuned);
  return g < units ? g : units;
}

template <class K, class... Args>
cudaError_t launch_pdl(K kernel, int grid, int block, size_t smem, cudaStream_t st,
                       Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(block);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, args...);
}

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
  const int rs = (int)Geo<N>::ROW_SMEM, cs = (int)Geo<N>::COL_SMEM;
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(row_kernel<N, -1>, cudaFuncAttributeMaxDynamicSharedMemorySize, rs);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(row_kernel<N, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, rs);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(col_kernel<N, COL_FWD>, cudaFuncAttributeMaxDynamicSharedMemorySize, cs);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(col_kernel<N, COL_INV>, cudaFuncAttributeMaxDynamicSharedMemorySize, cs);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(col_kernel<N, COL_FUSED>, cudaFuncAttributeMaxDynamicSharedMemorySize, cs);
  int dev = 0;
  if (e == cudaSuccess) e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&g_sms, cudaDevAttrMultiProcessorCount, dev);
  int occ = 0;
  if (e == cudaSuccess)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, row_kernel<N, 1>,
                                                      Geo<N>::ROW_THREADS, rs);
  g_occ_row = occ > 0 ? occ : 1;
  if (e == cudaSuccess)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, col_kernel<N, COL_FUSED>,
                                                      Geo<N>::COL_THREADS, cs);
  g_occ_col = occ > 0 ? occ : 1;
  return e;
}

cudaError_t launch_row(int inverse, const float2* in, float2* out, const RowOps& ops,
                       cudaStream_t st) {
  constexpr int N = LP_N;
  const int grid = grid_for(Geo<N>::ROW_UNITS, g_occ_row, g_ctas_row);
  if (inverse)
    return launch_pdl(row_kernel<N, 1>, grid, Geo<N>::ROW_THREADS, Geo<N>::ROW_SMEM, st, in, out,
                      ops);
  return launch_pdl(row_kernel<N, -1>, grid, Geo<N>::ROW_THREADS, Geo<N>::ROW_SMEM, st, in, out,
                    ops);
}

cudaError_t launch_col(int mode, const float2* in, float2* out, const ColOps& ops,
                       cudaStream_t st) {
  constexpr int N = LP_N;
  const int grid = grid_for(Geo<N>::COL_UNITS, g_occ_col, g_ctas_col);
  const int bs = Geo<N>::COL_THREADS;
  const size_t sm = Geo<N>::COL_SMEM;
  switch (mode) {
    case COL_FWD: return launch_pdl(col_kernel<N, COL_FWD>, grid, bs, sm, st, in, out, ops);
    case COL_INV: return launch_pdl(col_kernel<N, COL_INV>, grid, bs, sm, st, in, out, ops);
    default: return launch_pdl(col_kernel<N, COL_FUSED>, grid, bs, sm, st, in, out, ops);
  }
}

int set_ctas_per_sm(int kind, int value) {
  int& slot = kind == 0 ? g_ctas_row : g_ctas_col;
  const int occ = kind == 0 ? g_occ_row : g_occ_col;
  slot = value < 0 ? 0 : value;
  return ctas_in_effect(occ, slot);
}

}  // namespace
}  // namespace lp

#define LP_CAT2(a, b) a##b
#define LP_CAT(a, b) LP_CAT2(a, b)
namespace lp {
extern const SizeOps LP_CAT(size_ops_, LP_N);
const SizeOps LP_CAT(size_ops_, LP_N) = {LP_N, &init_size, &launch_row, &launch_col,
                                         &set_ctas_per_sm};
}  // namespace lp
