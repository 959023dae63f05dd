// Pass kernels and launchers for one grid size N (the including file defines
// LP_N); the transform code itself is in lp_fft_core.cuh.
//
// Kernels are persistent: a CTA loops over tiles (a few rows, or a few
// columns) and loads the next tile's points into a second register set while
// it transforms the current one, so global-memory latency overlaps the
// arithmetic.  Stage twiddles are copied into shared memory once per CTA.
// Launches use programmatic dependent launch so the next pass's CTAs are
// scheduled as this pass retires.
//
// Each pass exists in a general form (every multiplier a run-time option)
// and in forms compiled for what most calls use: the row transform alone, a
// row pass with only an FP32 phase mask, and column passes whose only
// spectral multiplier is H.  The launchers pick by the call's ops; the
// specialised kernels leave the unused code out, which removes the general
// column kernel's instruction-cache stalls.
#pragma once

#include "lp_async.cuh"
#include "lp_fft_core.cuh"

#ifndef LP_N
#error "define LP_N before including lp_fft_impl.cuh"
#endif
// Columns per CTA of the column kernels for N = 1024, 2048 and 4096 (2048:
// eight columns, 1024 threads, measured 41.0 vs 42.2 us against four, 41.7
// us for two four-column CTAs per SM and 43.6 us for seven-column tiles,
// which even out the SMs' work but not a tile's latency; 4096: four
// columns, 1024 threads without prefetch, 155.8 vs 192.9 us against two
// columns with prefetch and 222 us for two two-column CTAs per SM).
#ifndef LP_COL_C1024
#define LP_COL_C1024 4
#endif
#ifndef LP_COL_C2048
#define LP_COL_C2048 8
#endif
#ifndef LP_COL_C4096
#define LP_COL_C4096 4
#endif
// 8192: a line is 512 threads and 68 KB of exchange buffer, so column tiles
// hold two columns (1024 threads, 204 KB with the twiddles).
#ifndef LP_COL_C8192
#define LP_COL_C8192 2
#endif
// Per-size choices below were measured on GB300 (fused propagate, inputs
// larger than L2); each can be overridden with -D for tuning experiments.
// 1: load the next tile into a second register set while transforming the
// current one; 0: load it at the top of the next iteration.
#ifndef LP_ROW_PREFETCH
#define LP_ROW_PREFETCH (LP_N < 8192 && LP_N != 1024)
#endif
// Rows loaded ahead by the transform-only row kernel (0, 1 or 2; measured:
// two rows ahead at 2048^2 57.2 vs 56.6 us per propagate, one row ahead at
// 1024^2 18.1 vs 17.9 us).
#ifndef LP_ROW_PREFETCH_LEAN
#define LP_ROW_PREFETCH_LEAN LP_ROW_PREFETCH
#endif
#ifndef LP_COL_PREFETCH
#define LP_COL_PREFETCH 0
#endif
// Minimum resident CTAs per SM requested from the register allocator
// (2 with 512-thread column CTAs caps them at 64 registers).
//
// Row passes at 1024-2048 run one- or two-row CTAs of 128 threads, several
// per SM: a CTA's barriers then hold only its own rows, so one CTA's loads,
// exchanges and barrier waits overlap another's arithmetic.  Measured on
// GB300 (back-to-back fused propagates, inputs larger than L2): 2048^2 with
// three 170-register CTAs per SM and next-row prefetch 63.2 us, against
// 65.8 us for one 256-thread CTA (two rows, 225 registers) per SM, 63.6 us
// with two CTAs per SM, 64.1 us with four, 64.9-66.0 us without prefetch at
// three to five; 1024^2 with four 128-register CTAs per SM without prefetch
// 20.5 us, against 22.2 us for one 256-thread CTA (four rows) per SM and
// 21.3-22.5 us for 64-thread one-row CTAs or 128-thread CTAs with prefetch.
#ifndef LP_ROW_MINB
#define LP_ROW_MINB (LP_N == 2048 ? 3 : LP_N == 1024 ? 4 : 1)
#endif
// Threads per row-kernel CTA for N >= 1024 (whole rows per CTA).
#ifndef LP_ROW_THREADS
#define LP_ROW_THREADS (LP_N == 2048 || LP_N == 1024 ? 128 : 256)
#endif
#ifndef LP_COL_MINB
#define LP_COL_MINB (LP_N >= 2048 ? 1 : 2)
#endif
// TMA-staged row kernels (1) or register-prefetch kernels (0); used for
// N >= 1024 only.  TMA wins at 4096 (rows of 32 KB); at 1024-2048 the
// register kernels, which use every SM, are faster.
#ifndef LP_ROW_TMA
#define LP_ROW_TMA (LP_N == 4096)
#endif
// The TMA row kernel's tiles are 4096 points of whole rows: N in 1024..4096.
#define LP_ROW_TMA_SIZE (LP_N >= 1024 && LP_N <= 4096)
// TMA-staged column kernel (eight-column tiles, 16-byte aligned grids).
#ifndef LP_COL_TMA
#define LP_COL_TMA 0
#endif
// 1: fused column passes whose only spectral multipliers are H and the scale
// run a kernel built for that case (no k-mask, spectrum-write or d/dz code;
// the scale folded into the H table).
#ifndef LP_COL_LEAN
#define LP_COL_LEAN 1
#endif
// 1: row passes with no multiplier, scale or epilogue run a kernel built for
// the transform alone.
#ifndef LP_ROW_LEAN
#define LP_ROW_LEAN 1
#endif
// Preferred shared-memory carveout (percent) of every pass kernel of this
// size; -1 leaves the driver's default.
#ifndef LP_CARVEOUT
#define LP_CARVEOUT -1
#endif
// TMA row kernels: equal contiguous tile runs per group on as many SMs as
// that needs (1), or tiles strided over every SM (0).
#ifndef LP_TMA_BALANCED
#define LP_TMA_BALANCED 1
#endif

namespace lp {
namespace {

template <int N>
struct Geo : FftGeo<N> {
  using F = FftGeo<N>;
  // rows per CTA: LP_ROW_THREADS threads for large N, one warp's worth for small N
  static constexpr int ROWS = N >= 1024 ? cmax(1, LP_ROW_THREADS / F::T) : cmin(N, cmax(1, 32 / F::T));
  // columns per CTA: at least 4 so every row segment is a full 32-byte sector
  static constexpr int COLS = N >= 8192   ? LP_COL_C8192
                              : N >= 4096 ? LP_COL_C4096
                              : N >= 2048 ? LP_COL_C2048
                              : N >= 1024 ? LP_COL_C1024
                                          : cmin(N, cmax(4, 32 / F::T));
  static constexpr int ROW_THREADS = ROWS * F::T;
  static constexpr int COL_THREADS = COLS * F::T;
  static constexpr int ROW_UNITS = N / ROWS;
  static constexpr int COL_UNITS = N / COLS;
  // Shared memory: exchange buffer of the CTA's lines, then the twiddles.
  static constexpr size_t ROW_SMEM = sizeof(float2) * (ROWS * F::BUF + F::TW_SIZE);
  static constexpr size_t COL_SMEM = sizeof(float2) * (COLS * F::BUF + F::TW_SIZE);
};

// Stage twiddles of this size (filled once per device by init_size).
__device__ float2 g_tw[FftGeo<LP_N>::TW_SIZE];

// Copies the stage twiddles into shared memory at `dst`.  It reads only this
// file's table, so it runs before the wait on the previous kernel; the first
// barrier of the tile loop orders it before any use.
template <int NT>
__device__ __forceinline__ void load_twiddles(float2* dst) {
  for (int i = threadIdx.x; i < FftGeo<LP_N>::TW_SIZE; i += NT) dst[i] = g_tw[i];
}

template <int N, int S, int V = ROWV_ALL>
__global__ void __launch_bounds__(Geo<N>::ROW_THREADS, LP_ROW_MINB)
    row_kernel(const float2* in, float2* out, RowOps ops) {
  constexpr int T = Geo<N>::T, L = Geo<N>::ROWS, NU = Geo<N>::ROW_UNITS;
  constexpr int NT = Geo<N>::ROW_THREADS;
  extern __shared__ float2 smem[];
  float2* tw = smem + L * Geo<N>::BUF;
  const int g = threadIdx.x / T, t = threadIdx.x % T;
  load_twiddles<NT>(tw);
  pdl_wait();
  pdl_release();
  // rows loaded ahead of the one being transformed (0: none)
  constexpr int PF = (V == ROWV_LEAN) ? LP_ROW_PREFETCH_LEAN : LP_ROW_PREFETCH;
  int tile = blockIdx.x;
  const int step = gridDim.x;
  float2 v[16], p[PF >= 1 ? 16 : 1], q[PF >= 2 ? 16 : 1];
  if constexpr (PF >= 1) {
    if (tile < NU) load_row<N>(v, in, tile * L + g, t);
  }
  if constexpr (PF >= 2) {
    if (tile + step < NU) load_row<N>(p, in, (tile + step) * L + g, t);
  }
#pragma unroll 1
  while (tile < NU) {
    if constexpr (PF == 0) load_row<N>(v, in, tile * L + g, t);
    __syncthreads();  // buffer free: previous tile's last-stage reads are done
    if constexpr (PF == 0) {
      row_tile<N, S, L, NT, false, 1, NoHook, row_feat<V>(), row_mask_type<V>()>(
          v, out, tile, ops, smem, tw, NoHook{});
    } else {
      const int ahead = tile + PF * step;
      auto pf = [&] {
        if (ahead < NU) {
          if constexpr (PF == 1) load_row<N>(p, in, ahead * L + g, t);
          else load_row<N>(q, in, ahead * L + g, t);
        }
      };
      row_tile<N, S, L, NT, false, 1, decltype(pf), row_feat<V>(), row_mask_type<V>()>(
          v, out, tile, ops, smem, tw, pf);
      static_for<16>([&](auto jc) { v[decltype(jc)::value] = p[decltype(jc)::value]; });
      if constexpr (PF >= 2)
        static_for<16>([&](auto jc) { p[decltype(jc)::value] = q[decltype(jc)::value]; });
    }
    tile += step;
  }
}

template <int N, int MODE>
__global__ void __launch_bounds__(Geo<N>::COL_THREADS, LP_COL_MINB)
    col_kernel(const float2* in, float2* out, ColOps ops) {
  constexpr int T = Geo<N>::T, C = Geo<N>::COLS, NU = Geo<N>::COL_UNITS;
  extern __shared__ float2 smem[];
  float2* tw = smem + C * Geo<N>::BUF;
  const int c = threadIdx.x % C, t = threadIdx.x / C;
  load_twiddles<C * T>(tw);
  pdl_wait();
  pdl_release();
  int tile = blockIdx.x;
  float2 v[16];
#if LP_COL_PREFETCH
  float2 p[16];
  if (tile < NU) load_col<N>(v, in, tile * C + c, t);
#endif
#pragma unroll 1
  while (tile < NU) {
    const int next = tile + gridDim.x;
#if !LP_COL_PREFETCH
    load_col<N>(v, in, tile * C + c, t);
#endif
    __syncthreads();  // buffer free: previous tile's last-stage reads are done
#if LP_COL_PREFETCH
    col_tile<N, MODE, C, false>(v, out, tile, ops, smem, tw, [&] {
      if (next < NU) load_col<N>(p, in, next * C + c, t);
    });
    static_for<16>([&](auto jc) { v[decltype(jc)::value] = p[decltype(jc)::value]; });
#else
    col_tile<N, MODE, C, false>(v, out, tile, ops, smem, tw, NoHook{});
#endif
    tile = next;
  }
}

// ------------------------------------------------------ TMA-staged rows --
// Set when a bounded wait of this size's kernels gave up (read and cleared by
// take_async_error on the host).
__device__ int g_async_err;

#if LP_COL_TMA
// --------------------------------------------------- TMA-staged columns --
// Column pass with tiles moved by the tensor-copy (TMA) engine instead of
// per-thread loads: an eight-column tile (C x N complex64, 64-byte row
// segments) arrives as 2-D boxes of C x 256 elements in two halves.  The
// first half of the next tile lands in its own buffer while the current
// tile is transformed; the second half lands in the exchange buffer as soon
// as the current tile's last stage has read it, while the threads store
// their results.  Threads read their 16 points from the landed rows (whole
// 256-byte warp rows, no bank conflicts); stores stay per-thread.
template <int N>
struct ColTma {
  static constexpr int C = Geo<N>::COLS, H = N / 2, BOX = 256;
  static constexpr uint32_t HALF_BYTES = (uint32_t)C * H * sizeof(float2);
  static constexpr size_t XB = (size_t)C * FftGeo<N>::BUF;  // exchange (float2)
  static constexpr size_t OFF_LAND = XB;
  static constexpr size_t OFF_TW = OFF_LAND + (size_t)C * H;
  static constexpr size_t OFF_BAR =
      ((OFF_TW + FftGeo<N>::TW_SIZE) * sizeof(float2) + 15) / 16 * 16;
  static constexpr size_t SMEM = OFF_BAR + 2 * sizeof(uint64_t);
  static_assert((OFF_LAND * sizeof(float2)) % 128 == 0, "TMA destinations are 128-byte aligned");
};

template <int N, int MODE>
__global__ void __launch_bounds__(Geo<N>::COL_THREADS, 1)
    col_kernel_tma(const __grid_constant__ CUtensorMap tin, float2* out, ColOps ops) {
  using CT = ColTma<N>;
  constexpr int T = Geo<N>::T, C = CT::C, H = CT::H, BOX = CT::BOX, NU = Geo<N>::COL_UNITS;
  extern __shared__ __align__(128) float2 smem_ct[];
  float2* xbuf = smem_ct;
  float2* land = smem_ct + CT::OFF_LAND;
  float2* tw = smem_ct + CT::OFF_TW;
  uint64_t* bars = reinterpret_cast<uint64_t*>(reinterpret_cast<char*>(smem_ct) + CT::OFF_BAR);
  const int c = threadIdx.x % C, t = threadIdx.x / C;
  load_twiddles<C * T>(tw);
  if (threadIdx.x == 0) {
    mbar_init(bars, 1);
    mbar_init(bars + 1, 1);
    mbar_init_fence();
  }
  __syncthreads();
  const int first = blockIdx.x, step = gridDim.x;
  const int count = first < NU ? (NU - 1 - first) / step + 1 : 0;
  // rows half*H .. half*H+H-1 of tile `tile` into dst ([row][C], dense)
  auto load_half = [&](float2* dst, uint64_t* bar, int tile, int half) {
    mbar_expect_tx(bar, CT::HALF_BYTES);
#pragma unroll 1
    for (int b = 0; b < H / BOX; ++b)
      tma_load_2d(dst + (size_t)b * BOX * C, &tin, tile * C, half * H + b * BOX, bar);
  };
  pdl_wait();
  pdl_release();
  if (threadIdx.x == 0 && count > 0) {
    load_half(land, bars, first, 0);
    load_half(xbuf, bars + 1, first, 1);
  }
  bool ok = true;
#pragma unroll 1
  for (int j = 0; j < count; ++j) {
    const int tile = first + j * step;
    const bool more = j + 1 < count;
    ok = mbar_wait(bars, j & 1, &g_async_err) && ok;
    ok = mbar_wait(bars + 1, j & 1, &g_async_err) && ok;
    float2 v[16];
    static_for<8>([&](auto jc) {
      constexpr int jj = decltype(jc)::value;
      v[jj] = land[(t + T * jj) * C + c];
      v[jj + 8] = xbuf[(t + T * jj) * C + c];
    });
    __syncthreads();  // both landing areas read
    if (threadIdx.x == 0 && more) {
      fence_proxy_async();
      load_half(land, bars, tile + step, 0);
    }
    col_tile<N, MODE, C, false>(v, out, tile, ops, xbuf, tw, NoHook{}, [&] {
      __syncthreads();  // exchange buffer read by the last stage
      if (threadIdx.x == 0 && more) {
        fence_proxy_async();
        load_half(xbuf, bars + 1, tile + step, 1);
      }
    });
  }
  if (!ok && threadIdx.x == 0 && count > 0) {
    // A wait gave up: let both areas' last copies land (bounded) before exit.
    mbar_wait(bars, (count - 1) & 1, &g_async_err);
    mbar_wait(bars + 1, (count - 1) & 1, &g_async_err);
  }
}
#endif

#if LP_ROW_TMA_SIZE
// Row pass for N >= 1024 on 16-byte aligned grids.  One CTA per SM holds two
// independent groups of 256 threads.  A tile is 4096 points (4096/N whole
// rows, contiguous in memory); each group owns a contiguous run of `tpg`
// tiles and SL landing slots that the TMA engine fills with one bulk copy per
// tile.  A group reads a landed tile into registers, hands the slot straight
// back to the copy engine for its tile SL ahead, and transforms in its own
// exchange buffer, so up to 2*SL tiles per SM are in flight while the SM
// computes, and no registers are spent on prefetching.  The grid is sized so
// every group gets the same number of tiles (a memory-bound pass is balanced
// by its copies in flight, not by using every SM).
template <int N>
struct RowTma {
  static constexpr int TILE = 4096;
  static constexpr int L = TILE / N;
  static constexpr int G = 2;
  static constexpr int SL = N >= 4096 ? 1 : 2;
  static constexpr int NU = N / L;
  static constexpr size_t XBUF = (size_t)L * FftGeo<N>::BUF;         // float2 per group
  static constexpr size_t OFF_LAND = G * XBUF;                        // float2
  static constexpr size_t OFF_TW = OFF_LAND + (size_t)G * SL * TILE;  // float2
  static constexpr size_t BAR_BYTES =
      ((OFF_TW + FftGeo<N>::TW_SIZE) * sizeof(float2) + 15) / 16 * 16;
  static constexpr size_t SMEM = BAR_BYTES + G * SL * sizeof(uint64_t);
};

template <int N, int S, int V = ROWV_ALL>
__global__ void __launch_bounds__(512, 1)
    row_kernel_tma(const float2* in, float2* out, RowOps ops, int tpg) {
  using RT = RowTma<N>;
  constexpr int T = FftGeo<N>::T, L = RT::L, SL = RT::SL, TILE = RT::TILE;
  constexpr uint32_t BYTES = TILE * sizeof(float2);
  extern __shared__ __align__(16) float2 smem[];
  const int grp = threadIdx.x >> 8, lt = threadIdx.x & 255;
  float2* xbuf = smem + grp * RT::XBUF;
  float2* land = smem + RT::OFF_LAND + (size_t)grp * SL * TILE;
  float2* tw = smem + RT::OFF_TW;
  uint64_t* bars = reinterpret_cast<uint64_t*>(reinterpret_cast<char*>(smem) + RT::BAR_BYTES);
  load_twiddles<512>(tw);
  if (threadIdx.x == 0) {
    for (int k = 0; k < RT::G * SL; ++k) mbar_init(bars + k, 1);
    mbar_init_fence();
  }
  __syncthreads();
  bars += grp * SL;
#if LP_TMA_BALANCED
  // tiles first .. first+count-1 (count <= 0 for idle groups of the last CTA)
  const int first = (blockIdx.x * RT::G + grp) * tpg, step = 1;
  const int count = min(tpg, RT::NU - first);
#else
  // tiles first, first+step, ... over the whole grid
  const int first = blockIdx.x * RT::G + grp, step = gridDim.x * RT::G;
  const int count = first < RT::NU ? (RT::NU - 1 - first) / step + 1 : 0;
#endif
  pdl_wait();
  pdl_release();
  if (lt == 0) {
    for (int k = 0; k < SL && k < count; ++k)
      bulk_load(land + k * TILE, in + (size_t)(first + k * step) * TILE, BYTES, bars + k);
  }
  const int g = lt / T, t = lt % T;
  bool ok = true;
#pragma unroll 1
  for (int j = 0; j < count; ++j) {
    const int k = j % SL;
    ok = mbar_wait(bars + k, (j / SL) & 1, &g_async_err) && ok;
    float2 v[16];
    const float2* src = land + k * TILE + g * N + t;
    static_for<16>([&](auto jc) { v[decltype(jc)::value] = src[T * decltype(jc)::value]; });
    group_sync<2>();  // slot k read by the whole group; exchange buffer free
    if (lt == 0 && j + SL < count) {
      fence_proxy_async();
      bulk_load(land + k * TILE, in + (size_t)(first + (j + SL) * step) * TILE, BYTES, bars + k);
    }
    row_tile<N, S, L, 256, false, 2, NoHook, row_feat<V>(), row_mask_type<V>()>(
        v, out, first + j * step, ops, xbuf, tw, NoHook{});
  }
  if (!ok && lt == 0) {
    // A wait gave up: let each slot's last copy land (bounded) before exit.
    for (int k = 0; k < SL && k < count; ++k) {
      const int jl = k + ((count - 1 - k) / SL) * SL;
      mbar_wait(bars + k, (jl / SL) & 1, &g_async_err);
    }
  }
}

#endif

// ------------------------------------------------------------- launchers --
int g_sms = 0;                       // SM count of the device set up last
int g_occ_row = 1, g_occ_col = 1;    // max resident CTAs per SM
int g_ctas_row = 0, g_ctas_col = 0;  // tuned CTAs per SM (0 = built-in choice)
const float2* g_tw_dev[64] = {};    // device address of g_tw, per device

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
  static float2 host_tw[FftGeo<N>::TW_SIZE];
  fill_twiddles<N>(host_tw);
  cudaError_t e = cudaMemcpyToSymbol(g_tw, host_tw, sizeof(host_tw));
  void* p = nullptr;
  int dev = 0;
  if (e == cudaSuccess) e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaGetSymbolAddress(&p, g_tw);
  if (e == cudaSuccess && dev >= 0 && dev < 64) g_tw_dev[dev] = reinterpret_cast<const float2*>(p);
  const int rs = (int)Geo<N>::ROW_SMEM, cs = (int)Geo<N>::COL_SMEM;
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(row_kernel<N, -1>, cudaFuncAttributeMaxDynamicSharedMemorySize, rs);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(row_kernel<N, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, rs);
#if LP_ROW_TMA_SIZE
  {
    const int ts = (int)RowTma<N>::SMEM;
    for (const void* k : {(const void*)row_kernel_tma<N, -1>, (const void*)row_kernel_tma<N, 1>,
                          (const void*)row_kernel_tma<N, -1, ROWV_LEAN>,
                          (const void*)row_kernel_tma<N, 1, ROWV_LEAN>,
                          (const void*)row_kernel_tma<N, -1, ROWV_PHASE>,
                          (const void*)row_kernel_tma<N, 1, ROWV_PHASE>})
      if (e == cudaSuccess) e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, ts);
  }
#endif
#if LP_COL_TMA
  {
    const int ts = (int)ColTma<N>::SMEM;
    for (const void* k : {(const void*)col_kernel_tma<N, COL_FWD>,
                          (const void*)col_kernel_tma<N, COL_INV>,
                          (const void*)col_kernel_tma<N, COL_FUSED>})
      if (e == cudaSuccess) e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, ts);
  }
#endif
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(col_kernel<N, COL_FWD>, cudaFuncAttributeMaxDynamicSharedMemorySize, cs);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(col_kernel<N, COL_INV>, cudaFuncAttributeMaxDynamicSharedMemorySize, cs);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(col_kernel<N, COL_FUSED>, cudaFuncAttributeMaxDynamicSharedMemorySize, cs);
#if LP_COL_LEAN
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(col_kernel<N, COL_FUSED_LEAN>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, cs);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(col_kernel<N, COL_INV_LEAN>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, cs);
#endif
#if LP_ROW_LEAN
  for (const void* k : {(const void*)row_kernel<N, -1, ROWV_LEAN>,
                        (const void*)row_kernel<N, 1, ROWV_LEAN>,
                        (const void*)row_kernel<N, -1, ROWV_PHASE>,
                        (const void*)row_kernel<N, 1, ROWV_PHASE>})
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, rs);
#endif
#if LP_CARVEOUT >= 0
  for (const void* k : {(const void*)row_kernel<N, -1>, (const void*)row_kernel<N, 1>,
                        (const void*)col_kernel<N, COL_FWD>, (const void*)col_kernel<N, COL_INV>,
                        (const void*)col_kernel<N, COL_FUSED>})
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, LP_CARVEOUT);
#if LP_COL_TMA
  for (const void* k : {(const void*)col_kernel_tma<N, COL_FWD>,
                        (const void*)col_kernel_tma<N, COL_INV>,
                        (const void*)col_kernel_tma<N, COL_FUSED>})
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, LP_CARVEOUT);
#endif
#endif
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
#if LP_ROW_TMA_SIZE && LP_ROW_TMA
  {
    if ((reinterpret_cast<uintptr_t>(in) & 15u) == 0) {
      using RT = RowTma<N>;
      const int tpg = (RT::NU + RT::G * g_sms - 1) / (RT::G * g_sms);
      const int grid = LP_TMA_BALANCED ? (RT::NU + RT::G * tpg - 1) / (RT::G * tpg)
                                       : cmin(g_sms, (RT::NU + RT::G - 1) / RT::G);
      const int v = LP_ROW_LEAN ? row_variant(ops) : ROWV_ALL;
      auto k = inverse ? (v == ROWV_LEAN    ? row_kernel_tma<N, 1, ROWV_LEAN>
                          : v == ROWV_PHASE ? row_kernel_tma<N, 1, ROWV_PHASE>
                                            : row_kernel_tma<N, 1>)
                       : (v == ROWV_LEAN    ? row_kernel_tma<N, -1, ROWV_LEAN>
                          : v == ROWV_PHASE ? row_kernel_tma<N, -1, ROWV_PHASE>
                                            : row_kernel_tma<N, -1>);
      return launch_pdl(k, grid, 512, RT::SMEM, st, in, out, ops, tpg);
    }
  }
#endif
  const int grid = grid_for(Geo<N>::ROW_UNITS, g_occ_row, g_ctas_row);
#if LP_ROW_LEAN
  {
    const int v = row_variant(ops);
    if (v != ROWV_ALL) {
      auto k = inverse ? (v == ROWV_LEAN ? row_kernel<N, 1, ROWV_LEAN> : row_kernel<N, 1, ROWV_PHASE>)
                       : (v == ROWV_LEAN ? row_kernel<N, -1, ROWV_LEAN>
                                         : row_kernel<N, -1, ROWV_PHASE>);
      return launch_pdl(k, grid, Geo<N>::ROW_THREADS, Geo<N>::ROW_SMEM, st, in, out, ops);
    }
  }
#endif
  if (inverse)
    return launch_pdl(row_kernel<N, 1>, grid, Geo<N>::ROW_THREADS, Geo<N>::ROW_SMEM, st, in, out,
                      ops);
  return launch_pdl(row_kernel<N, -1>, grid, Geo<N>::ROW_THREADS, Geo<N>::ROW_SMEM, st, in, out,
                    ops);
}

cudaError_t launch_col(int mode, const float2* in, float2* out, const ColOps& ops,
                       cudaStream_t st) {
  constexpr int N = LP_N;
  const int bs = Geo<N>::COL_THREADS;
#if LP_COL_TMA
  {
    CUtensorMap tm;
    if ((reinterpret_cast<uintptr_t>(in) & 15u) == 0 &&
        grid_tensor_map(&tm, in, N, ColTma<N>::C, ColTma<N>::BOX)) {
      const int grid = cmin(g_sms, Geo<N>::COL_UNITS);
      const size_t ts = ColTma<N>::SMEM;
      switch (mode) {
        case COL_FWD: return launch_pdl(col_kernel_tma<N, COL_FWD>, grid, bs, ts, st, tm, out, ops);
        case COL_INV: return launch_pdl(col_kernel_tma<N, COL_INV>, grid, bs, ts, st, tm, out, ops);
        default: return launch_pdl(col_kernel_tma<N, COL_FUSED>, grid, bs, ts, st, tm, out, ops);
      }
    }
  }
#endif
  const int grid = grid_for(Geo<N>::COL_UNITS, g_occ_col, g_ctas_col);
  const size_t sm = Geo<N>::COL_SMEM;
#if LP_COL_LEAN
  if (ops.apply_h && !ops.kmask && !ops.spectrum_out && !ops.dz && !ops.phase_fp32) {
    if (mode == COL_FUSED)
      return launch_pdl(col_kernel<N, COL_FUSED_LEAN>, grid, bs, sm, st, in, out, ops);
    if (mode == COL_INV)
      return launch_pdl(col_kernel<N, COL_INV_LEAN>, grid, bs, sm, st, in, out, ops);
  }
#endif
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

int take_async_error() {
  int v = 0;
  if (cudaMemcpyFromSymbol(&v, g_async_err, sizeof(int)) != cudaSuccess) return -1;
  if (v) {
    const int zero = 0;
    if (cudaMemcpyToSymbol(g_async_err, &zero, sizeof(int)) != cudaSuccess) return -1;
  }
  return v ? 1 : 0;
}

const float2* twiddles_dev() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
  return g_tw_dev[dev];
}

}  // namespace
}  // namespace lp

#define LP_CAT2(a, b) a##b
#define LP_CAT(a, b) LP_CAT2(a, b)
namespace lp {
extern const SizeOps LP_CAT(size_ops_, LP_N);
const SizeOps LP_CAT(size_ops_, LP_N) = {LP_N, &init_size, &launch_row, &launch_col,
                                         &set_ctas_per_sm, &twiddles_dev,
                                         &take_async_error};
}  // namespace lp
