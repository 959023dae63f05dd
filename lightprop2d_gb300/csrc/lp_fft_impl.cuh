// 2-D FFT passes for one grid size N (the including file defines LP_N).
//
// Each 1-D transform of length N = R1*R2 runs as two Stockham stages on
// T = N/max(R1,R2) threads that each keep P = max(R1,R2) points in registers:
//
//   thread t holds elements {t + T*j : j < P} of its line, both before and
//   after the transform (natural order), so a forward transform, a pointwise
//   spectral multiply and an inverse transform chain in registers with no
//   reordering between them.
//
//   stage 1 (radix R1, no twiddles):   in[b + r*N/R1]      -> buf[b*R1 + r]
//   stage 2 (radix R2, twiddles W_N^(r*(b mod R1))):
//                                      buf[b + r*R1]       -> out[b + r*R1]
//
// The only data exchange is one padded shared-memory buffer per line
// (index i stored at i + i/R1, which keeps the stride-R1 stage-1 writes free
// of bank conflicts).  Rows are read and written with consecutive threads on
// consecutive addresses; columns are processed C at a time with the column
// index fastest across lanes so every row segment is C*8 contiguous bytes.
#pragma once

#include "lp_device.cuh"
#include "lp_internal.h"

#ifndef LP_N
#error "define LP_N before including lp_fft_impl.cuh"
#endif

namespace lp {
namespace {

template <int N>
struct Plan;
template <> struct Plan<16> { static constexpr int R1 = 4, R2 = 4; };
template <> struct Plan<32> { static constexpr int R1 = 8, R2 = 4; };
template <> struct Plan<64> { static constexpr int R1 = 8, R2 = 8; };
template <> struct Plan<128> { static constexpr int R1 = 16, R2 = 8; };
template <> struct Plan<256> { static constexpr int R1 = 16, R2 = 16; };
template <> struct Plan<512> { static constexpr int R1 = 32, R2 = 16; };
template <> struct Plan<1024> { static constexpr int R1 = 32, R2 = 32; };
template <> struct Plan<2048> { static constexpr int R1 = 64, R2 = 32; };
template <> struct Plan<4096> { static constexpr int R1 = 64, R2 = 64; };

constexpr int cmin(int a, int b) { return a < b ? a : b; }
constexpr int cmax(int a, int b) { return a > b ? a : b; }

template <int N>
struct Geo {
  static constexpr int R1 = Plan<N>::R1, R2 = Plan<N>::R2;
  static constexpr int P = cmax(R1, R2);
  static constexpr int T = N / P;                       // threads per line
  static constexpr int BUF = N + N / R1;                // padded line buffer (float2)
  static constexpr int ROWS = cmin(N, cmax(1, 128 / T));  // rows per CTA
  static constexpr int COLS = cmin(N, cmax(1, 128 / T));  // columns per CTA
  static constexpr int ROW_THREADS = ROWS * T;
  static constexpr int COL_THREADS = COLS * T;
  static constexpr size_t ROW_SMEM = sizeof(float2) * ROWS * BUF;
  static constexpr size_t COL_SMEM = sizeof(float2) * COLS * BUF;
};

// Stage-2 twiddles of size N, layout [r][k] = W_N^(r*k) = exp(-2*pi*i*r*k/N),
// r < R2, k < R1 (N entries).  Filled once per device by init().
__device__ float2 g_tw[LP_N];

// One 1-D transform of the thread's P register points (see file comment).
// C lines share one interleaved buffer: line c uses buf[(padded index)*C + c].
template <int N, int S, int C, bool CTA_SYNC>
__device__ __forceinline__ void fft_line(float2 (&v)[Geo<N>::P], float2* buf, int t, int c) {
  constexpr int R1 = Geo<N>::R1, R2 = Geo<N>::R2, P = Geo<N>::P, T = Geo<N>::T;
  constexpr int nb1 = P / R1, nb2 = P / R2;
  static_for<nb1>([&](auto qc) {
    constexpr int q = decltype(qc)::value;
    float2 a[R1];
    static_for<R1>([&](auto rc) { a[decltype(rc)::value] = v[q + nb1 * decltype(rc)::value]; });
    Dft<R1, S>::run(a);
    const int b = t + q * T;
    static_for<R1>([&](auto rc) {
      constexpr int r = decltype(rc)::value;
      buf[(b * (R1 + 1) + r) * C + c] = a[r];
    });
  });
  if constexpr (CTA_SYNC) __syncthreads(); else __syncwarp();
  static_for<nb2>([&](auto qc) {
    constexpr int q = decltype(qc)::value;
    const int b2 = t + q * T;
    const int k = b2 & (R1 - 1);
    const int base = b2 + (b2 / R1);  // padded index of b2
    float2 a[R2];
    static_for<R2>([&](auto rc) {
      constexpr int r = decltype(rc)::value;
      // index i = b2 + r*R1 -> padded i + i/R1 = base + r*(R1+1)
      a[r] = buf[(base + r * (R1 + 1)) * C + c];
    });
    static_for<R2 - 1>([&](auto rc) {
      constexpr int r = decltype(rc)::value + 1;
      float2 w = g_tw[r * R1 + k];
      if constexpr (S > 0) w.y = -w.y;
      a[r] = cmul(a[r], w);
    });
    Dft<R2, S>::run(a);
    static_for<R2>([&](auto rc) { v[q + nb2 * decltype(rc)::value] = a[decltype(rc)::value]; });
  });
}

// ------------------------------------------------------------------ rows --
template <int N, int S>
__global__ void __launch_bounds__(Geo<N>::ROW_THREADS)
    row_kernel(const float2* in, float2* out, RowOps ops) {
  constexpr int P = Geo<N>::P, T = Geo<N>::T, ROWS = Geo<N>::ROWS;
  extern __shared__ float2 smem[];
  const int g = threadIdx.x / T, t = threadIdx.x % T;
  const int y = blockIdx.x * ROWS + g;
  float2* buf = smem + g * Geo<N>::BUF;
  const size_t row0 = (size_t)y * N;

  float2 v[P];
  static_for<P>([&](auto jc) {
    constexpr int j = decltype(jc)::value;
    v[j] = in[row0 + t + T * j];
  });

  if (ops.lens || ops.xmask) {
    const float jy = (float)(y - N / 2);
    static_for<P>([&](auto jc) {
      constexpr int j = decltype(jc)::value;
      const int x = t + T * j;
      float2 m = make_float2(1.0f, 0.0f);
      if (ops.lens) {
        const float jx = (float)(x - N / 2);
        const float f = lens_cycles(ops.kap_hi, ops.kap_lo, fmaf(jx, jx, jy * jy));
        m = cis_cycles(f, 1.0f);
      }
      if (ops.xmask) m = cmul(m, mask_value(ops.xmask, ops.xmask_type, row0 + x));
      if (ops.conj) m = cconj(m);
      v[j] = cmul(v[j], m);
    });
  }

  fft_line<N, S, 1, (T > 32)>(v, buf, t, 0);

  if (ops.scale != 1.0f) {
    static_for<P>([&](auto jc) { v[decltype(jc)::value] = cscale(v[decltype(jc)::value], ops.scale); });
  }
  if (ops.ymask) {
    static_for<P>([&](auto jc) {
      constexpr int j = decltype(jc)::value;
      float2 m = mask_value(ops.ymask, ops.ymask_type, row0 + t + T * j);
      if (ops.conj) m = cconj(m);
      v[j] = cmul(v[j], m);
    });
  }
  static_for<P>([&](auto jc) {
    constexpr int j = decltype(jc)::value;
    out[row0 + t + T * j] = v[j];
  });
  if (ops.iprofile) {
    static_for<P>([&](auto jc) {
      constexpr int j = decltype(jc)::value;
      ops.iprofile[row0 + t + T * j] = fmaf(v[j].x, v[j].x, v[j].y * v[j].y);
    });
  }
}

// --------------------------------------------------------------- columns --
template <int N>
__device__ __forceinline__ void spectral_point(float2& val, int ky, int kx, float a_hi,
                                               float a_lo, float qx, const ColOps& ops) {
  const size_t idx = (size_t)ky * N + kx;
  if (ops.kmask) {
    float2 m = mask_value(ops.kmask, ops.kmask_type, idx);
    if (ops.conj) m = cconj(m);
    val = cmul(val, m);
  }
  if (ops.apply_h) {
    const int sy = ky < N / 2 ? ky : ky - N;
    const float qy = (float)(sy * sy);
    bool evan;
    float sv;
    const float f = ops.phase_fp32 ? kz_phase_f32(ops.kp, qx, qy, evan, sv)
                                   : kz_phase_ff(ops.kp, a_hi, a_lo, qy, evan, sv);
    // H = exp(-2*pi*i*f); the adjoint uses conj(H).
    float2 h = cis_cycles(f, ops.conj ? 1.0f : -1.0f);
    if (evan) h = ops.evan_mask ? make_float2(0.0f, 0.0f) : make_float2(1.0f, 0.0f);
    if (ops.dz) {
      // d/dz exp(-2*pi*i*kz*z) = -2*pi*i*kz * H with kz = k0*sqrt(v).
      const float g = ops.kp.two_pi_k0 * sv * (ops.conj ? 1.0f : -1.0f);
      h = make_float2(-g * h.y, g * h.x);
    }
    val = cmul(val, h);
  }
  if (ops.spectrum_out) ops.spectrum_out[idx] = val;
  if (ops.scale != 1.0f) val = cscale(val, ops.scale);
}

template <int N, int MODE>
__global__ void __launch_bounds__(Geo<N>::COL_THREADS)
    col_kernel(const float2* in, float2* out, ColOps ops) {
  constexpr int P = Geo<N>::P, T = Geo<N>::T, C = Geo<N>::COLS;
  extern __shared__ float2 smem[];
  const int c = threadIdx.x % C, t = threadIdx.x / C;
  const int x = blockIdx.x * C + c;

  float2 v[P];
  static_for<P>([&](auto jc) {
    constexpr int j = decltype(jc)::value;
    v[j] = in[(size_t)(t + T * j) * N + x];
  });

  if constexpr (MODE == COL_FWD) {
    fft_line<N, -1, C, true>(v, smem, t, c);
  } else {
    if constexpr (MODE == COL_FUSED) {
      fft_line<N, -1, C, true>(v, smem, t, c);
      __syncthreads();  // the inverse transform reuses the exchange buffer
    }
    const int sx = x < N / 2 ? x : x - N;
    const float qx = (float)(sx * sx);
    float a_hi = 1.0f, a_lo = 0.0f;
    if (ops.apply_h && !ops.phase_fp32) column_constant(ops.kp, qx, a_hi, a_lo);
    static_for<P>([&](auto jc) {
      constexpr int j = decltype(jc)::value;
      spectral_point<N>(v[j], t + T * j, x, a_hi, a_lo, qx, ops);
    });
    fft_line<N, 1, C, true>(v, smem, t, c);
  }

  static_for<P>([&](auto jc) {
    constexpr int j = decltype(jc)::value;
    out[(size_t)(t + T * j) * N + x] = v[j];
  });
}

// ------------------------------------------------------------- launchers --
cudaError_t init_size() {
  constexpr int N = LP_N, R1 = Geo<N>::R1, R2 = Geo<N>::R2;
  static float2 host_tw[N];
  for (int r = 0; r < R2; ++r)
    for (int k = 0; k < R1; ++k) {
      const double ang = -2.0 * kPi * (double)((r * k) % N) / (double)N;
      host_tw[r * R1 + k] = make_float2((float)cos(ang), (float)sin(ang));
    }
  cudaError_t e = cudaMemcpyToSymbol(g_tw, host_tw, sizeof(host_tw));
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(row_kernel<N, -1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)Geo<N>::ROW_SMEM);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(row_kernel<N, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)Geo<N>::ROW_SMEM);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(col_kernel<N, COL_FWD>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)Geo<N>::COL_SMEM);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(col_kernel<N, COL_INV>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)Geo<N>::COL_SMEM);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(col_kernel<N, COL_FUSED>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)Geo<N>::COL_SMEM);
  return e;
}

cudaError_t launch_row(int inverse, const float2* in, float2* out, const RowOps& ops,
                       cudaStream_t st) {
  constexpr int N = LP_N;
  const dim3 grid(N / Geo<N>::ROWS), block(Geo<N>::ROW_THREADS);
  if (inverse)
    row_kernel<N, 1><<<grid, block, Geo<N>::ROW_SMEM, st>>>(in, out, ops);
  else
    row_kernel<N, -1><<<grid, block, Geo<N>::ROW_SMEM, st>>>(in, out, ops);
  return cudaGetLastError();
}

cudaError_t launch_col(int mode, const float2* in, float2* out, const ColOps& ops,
                       cudaStream_t st) {
  constexpr int N = LP_N;
  const dim3 grid(N / Geo<N>::COLS), block(Geo<N>::COL_THREADS);
  switch (mode) {
    case COL_FWD:
      col_kernel<N, COL_FWD><<<grid, block, Geo<N>::COL_SMEM, st>>>(in, out, ops);
      break;
    case COL_INV:
      col_kernel<N, COL_INV><<<grid, block, Geo<N>::COL_SMEM, st>>>(in, out, ops);
      break;
    default:
      col_kernel<N, COL_FUSED><<<grid, block, Geo<N>::COL_SMEM, st>>>(in, out, ops);
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
