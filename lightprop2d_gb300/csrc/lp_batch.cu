// Batched propagation of many beams of uneven grid sizes in ONE persistent
// launch (lp_batch_* in include/lightprop2d_gb300.h).
//
// Each beam needs three passes over its own grid, in place:
//   pass 0  rows:    x-domain lens multiply, forward row FFT
//   pass 1  columns: forward column FFT, H(z) in registers, inverse column FFT
//   pass 2  rows:    inverse row FFT, |field|^2 epilogue
// Every pass is split into tiles (4096 points each: 256 threads x 16) and
// tiles are grouped into work items.  The host orders the items (largest
// beams first; beams in groups of ~2^23 points; pass p+1 of a group is queued
// behind pass p of the next group, so a pass rarely waits and a group's
// passes run while its data is still in L2) and the resident CTAs pull them
// from a device counter.  An item of pass p > 0 waits until its beam's
// completion counter shows every tile of the earlier passes done.  Items are
// taken in queue order and only wait on earlier items, which running CTAs
// already hold, so the waits always end; each wait is still bounded and gives
// up with an error flag (LP_ERR_TIMEOUT on the host) instead of hanging.
// The last CTA to leave resets the queue and counters for the next run, so a
// run is a single launch that can be captured in a CUDA graph.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <mutex>
#include <new>
#include <vector>

#include "lightprop2d_gb300.h"
#include "lp_fft_core.cuh"

using namespace lp;

// 1: column items of beams whose column ops are H and the scale only run the
// column tile built for that case (no k-mask, spectrum-write or d/dz code).
#ifndef LP_BATCH_COL_LEAN
#define LP_BATCH_COL_LEAN 1
#endif
// 1: row items run tiles with only the multipliers a batch can carry (a lens
// in the forward pass, the iprofile and moment epilogues in the inverse).
#ifndef LP_BATCH_ROW_FEAT
#define LP_BATCH_ROW_FEAT 1
#endif

namespace {

constexpr int kBT = 256;          // threads per CTA
constexpr int kTilePts = kBT * 16;  // points per tile
constexpr int kBufF2 = kTilePts + kTilePts / 16;   // exchange buffer (float2)
constexpr int kTwMax = FftGeo<4096>::TW_SIZE;      // largest twiddle table
constexpr size_t kSmem = sizeof(float2) * (kBufF2 + kTwMax);
constexpr int kMinLog = 6, kMaxLog = 12;           // n = 64 .. 4096

template <int N>
struct BGeo {
  static constexpr int T = N / 16;
  static constexpr int L = cmin(N, kBT / T);  // rows per tile (L*T = 256)
  static constexpr int C = cmin(N, kBT / T);  // columns per tile
};

int row_tiles(int n) { return n * (n / 16) / kBT; }  // = N / L for N >= 64
int col_tiles(int n) { return row_tiles(n); }

struct BeamRec {
  float2* field;
  int n;
  int need1, need2;  // completed tiles needed before pass 1 / pass 2
  int col_lean;      // column ops are H and the scale only (COL_FUSED_LEAN)
  RowOps fwd;
  ColOps col;
  RowOps inv;
};

struct Item {
  int beam, pass, tile0, ntiles;
  int need;  // completed tiles of `beam` required before this item starts
};

// state[0] queue head, state[1] CTAs finished, state[2] error flag
struct BatchPlan {
  int count = 0, n_items = 0, grid = 0, ctas = 0, device = 0;
  long long spin_limit = 0;
  BeamRec* d_beams = nullptr;
  Item* d_items = nullptr;
  int* d_done = nullptr;
  int* d_state = nullptr;
  const float2** d_tw = nullptr;  // per log2(n): that size's twiddle table
};

template <int N>
__device__ __forceinline__ void run_tiles(const Item& item, const BeamRec* bp, float2* buf,
                                          const float2* tw) {
  using G = BGeo<N>;
  float2* field = bp->field;
#pragma unroll 1
  for (int k = 0; k < item.ntiles; ++k) {
    const int tile = item.tile0 + k;
    if (k > 0) __syncthreads();  // exchange buffer reused by the next tile
    float2 v[16];
    if (item.pass == 1) {
      const ColOps ops = bp->col;
      load_col<N, true>(v, field, tile * G::C + threadIdx.x % G::C, threadIdx.x / G::C);
      if (LP_BATCH_COL_LEAN && bp->col_lean)
        col_tile<N, COL_FUSED_LEAN, G::C, true>(v, field, tile, ops, buf, tw, NoHook{});
      else
        col_tile<N, COL_FUSED, G::C, true>(v, field, tile, ops, buf, tw, NoHook{});
    } else {
      const int g = threadIdx.x / G::T, t = threadIdx.x % G::T;
      load_row<N, true>(v, field, tile * G::L + g, t);
      // plan_batch gives the forward pass at most a lens and the inverse pass
      // at most the iprofile and moment epilogues (LP_BATCH_ROW_FEAT 0:
      // kernels with every row multiplier compiled in)
      if (item.pass == 0) {
        const RowOps ops = bp->fwd;
        row_tile<N, -1, G::L, kBT, true, 1, NoHook, LP_BATCH_ROW_FEAT ? ROW_LENS : ROW_ALL>(
            v, field, tile, ops, buf, tw, NoHook{});
      } else {
        const RowOps ops = bp->inv;
        row_tile<N, 1, G::L, kBT, true, 1, NoHook,
                 LP_BATCH_ROW_FEAT ? (ROW_IPROF | ROW_MOMENTS) : ROW_ALL>(v, field, tile, ops, buf,
                                                                         tw, NoHook{});
      }
    }
  }
}

__device__ __forceinline__ int tw_count(int n) {
  switch (n) {
    case 64: return FftGeo<64>::TW_SIZE;
    case 128: return FftGeo<128>::TW_SIZE;
    case 256: return FftGeo<256>::TW_SIZE;
    case 512: return FftGeo<512>::TW_SIZE;
    case 1024: return FftGeo<1024>::TW_SIZE;
    case 2048: return FftGeo<2048>::TW_SIZE;
    default: return FftGeo<4096>::TW_SIZE;
  }
}

__global__ void __launch_bounds__(kBT) batch_kernel(const BeamRec* __restrict__ beams,
                                                    const Item* __restrict__ items, int n_items,
                                                    int* done, int* state, int nbeams,
                                                    const float2* const* tw_tables,
                                                    long long spin_limit) {
  extern __shared__ float2 smem[];
  float2* buf = smem;
  float2* tw = smem + kBufF2;
  __shared__ int s_item, s_stop;
  int cur_n = 0;
#pragma unroll 1
  for (;;) {
    if (threadIdx.x == 0) {
      const int it = atomicAdd(&state[0], 1);
      volatile int* err = state + 2;
      int stop = it >= n_items || *err;
      if (!stop) {
        const Item item = items[it];
        if (item.need > 0) {
          volatile int* cnt = done + item.beam;
          long long k = 0;
          while (*cnt < item.need) {
            if (*err) { stop = 1; break; }
            if (++k > spin_limit) {
              atomicExch(&state[2], 1);  // give up: the host sees LP_ERR_TIMEOUT
              stop = 1;
              break;
            }
            __nanosleep(200);
          }
          __threadfence();
        }
      }
      s_item = it;
      s_stop = stop;
    }
    __syncthreads();
    if (s_stop) break;
    const Item item = items[s_item];
    const BeamRec* bp = beams + item.beam;
    const int n = bp->n;
    // The column pass's first item clears the beam's moment sums; every
    // row-pass-2 item runs after all column items (dependency counter).
    if (item.pass == 1 && item.tile0 == 0 && threadIdx.x < 5 && bp->inv.moments)
      bp->inv.moments[threadIdx.x] = 0.0;
    if (n != cur_n) {  // stage twiddles of this size into shared memory
      const float2* src = tw_tables[31 - __clz(n)];
      const int cnt = tw_count(n);
      for (int i = threadIdx.x; i < cnt; i += kBT) tw[i] = src[i];
      cur_n = n;
      __syncthreads();
    }
    switch (n) {
      case 64: run_tiles<64>(item, bp, buf, tw); break;
      case 128: run_tiles<128>(item, bp, buf, tw); break;
      case 256: run_tiles<256>(item, bp, buf, tw); break;
      case 512: run_tiles<512>(item, bp, buf, tw); break;
      case 1024: run_tiles<1024>(item, bp, buf, tw); break;
      case 2048: run_tiles<2048>(item, bp, buf, tw); break;
      default: run_tiles<4096>(item, bp, buf, tw); break;
    }
    __syncthreads();  // every thread's stores of this item are issued
    if (threadIdx.x == 0) {
      __threadfence();
      atomicAdd(done + item.beam, item.ntiles);
    }
  }
  // The last CTA out resets the queue for the next run (the error flag stays
  // for lp_batch_status).
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    s_stop = atomicAdd(&state[1], 1) == (int)gridDim.x - 1;
  }
  __syncthreads();
  if (s_stop) {
    for (int i = threadIdx.x; i < nbeams; i += kBT) done[i] = 0;
    if (threadIdx.x == 0) {
      state[0] = 0;
      state[1] = 0;
    }
    __threadfence();
  }
}

int g_batch_occ = 1;

lp_status fail(lp_status s, const char* msg) { return (lp_status)set_last_error((int)s, msg); }

lp_status cuda_fail(cudaError_t e, const char* where) {
  char msg[256];
  snprintf(msg, sizeof(msg), "%s: %s", where, cudaGetErrorString(e));
  return fail(LP_ERR_CUDA, msg);
}

void free_plan(BatchPlan* p) {
  if (!p) return;
  for (void* q : {(void*)p->d_beams, (void*)p->d_items, (void*)p->d_done, (void*)p->d_state,
                  (void*)p->d_tw})
    if (q) cudaFree(q);
  delete p;
}

}  // namespace

cudaError_t lp::batch_init() {
  cudaError_t e = cudaFuncSetAttribute(batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)kSmem);
  int occ = 0;
  if (e == cudaSuccess)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, batch_kernel, kBT, kSmem);
  g_batch_occ = occ > 0 ? occ : 1;
  return e;
}

struct lp_batch {
  BatchPlan plan;
};

namespace {

// Host part of a batch: argument checks, per-beam records (largest beams
// first) and the work queue.  No CUDA call, so it also plans shards on hosts
// without a GPU (lp_batch_plan).
lp_status plan_batch(const lp_beam_desc* beams, int count, const lp_batch_options* options,
                     std::vector<BeamRec>& recs, std::vector<Item>& items,
                     lp_batch_options& opt) {
  if (!beams || count <= 0) return fail(LP_ERR_INVALID_ARGUMENT, "lp_batch_create: no beams");
  opt = lp_batch_options{};
  if (options) opt = *options;
  const int tpi = opt.tiles_per_item > 0 ? opt.tiles_per_item : 8;
  const int glog = opt.group_points_log2 > 0 ? opt.group_points_log2 : 23;
  for (int i = 0; i < count; ++i) {
    const lp_beam_desc& b = beams[i];
    if (b.n < 64 || b.n > 4096 || (b.n & (b.n - 1)) != 0) {
      char msg[128];
      snprintf(msg, sizeof(msg), "beam %d: n=%d unsupported in a batch (64..4096, power of two)",
               i, b.n);
      return fail(LP_ERR_UNSUPPORTED_SIZE, msg);
    }
    if (!b.field) return fail(LP_ERR_INVALID_ARGUMENT, "beam field is NULL");
    if (reinterpret_cast<uintptr_t>(b.field) & 7u)
      return fail(LP_ERR_MISALIGNED, "beam field must be 8-byte aligned");
    if (b.iprofile && (reinterpret_cast<uintptr_t>(b.iprofile) & 3u))
      return fail(LP_ERR_MISALIGNED, "beam iprofile must be 4-byte aligned");
    if (b.moments && (reinterpret_cast<uintptr_t>(b.moments) & 7u))
      return fail(LP_ERR_MISALIGNED, "beam moments must be 8-byte aligned");
    if (!(b.area_size > 0 && b.wl > 0) || !std::isfinite(b.z) || !std::isfinite(b.lens_f))
      return fail(LP_ERR_INVALID_ARGUMENT, "beam geometry must be finite, area and wl > 0");
    if (b.flags & ~(uint32_t)(LP_FLAG_PHASE_FP32 | LP_FLAG_EVANESCENT_MASK))
      return fail(LP_ERR_INVALID_ARGUMENT,
                  "beam flags: only LP_FLAG_PHASE_FP32 and LP_FLAG_EVANESCENT_MASK apply");
  }
  // Host records: beams sorted by size (largest first).
  std::vector<int> order(count);
  for (int i = 0; i < count; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(),
                   [&](int a, int b) { return beams[a].n > beams[b].n; });
  recs.assign(count, BeamRec{});
  for (int k = 0; k < count; ++k) {
    const lp_beam_desc& b = beams[order[k]];
    BeamRec& r = recs[k];
    r.field = reinterpret_cast<float2*>(b.field);
    r.n = b.n;
    r.need1 = row_tiles(b.n);
    r.need2 = row_tiles(b.n) + col_tiles(b.n);
    r.fwd = row_ops_none();
    if (b.lens_f != 0.0) set_lens(r.fwd, b.n, b.area_size, b.wl, b.lens_f);
    r.col = make_colops(b.n, b.area_size, b.wl, b.z, b.z != 0.0,
                        b.flags & (LP_FLAG_PHASE_FP32 | LP_FLAG_EVANESCENT_MASK));
    r.col.scale = 1.0f / ((float)b.n * (float)b.n);
    r.col_lean = r.col.apply_h && !r.col.phase_fp32 && !r.col.dz && !r.col.kmask &&
                 !r.col.spectrum_out;
    r.inv = row_ops_none();
    r.inv.iprofile = b.iprofile;
    r.inv.moments = b.moments;
  }

  // Work queue: groups of ~2^glog points; pass p of group g is queued after
  // pass p-1 of group g+1 (a software pipeline over groups).
  std::vector<std::pair<int, int>> groups;  // [first, last) beam index
  {
    long long acc = 0;
    int first = 0;
    for (int k = 0; k < count; ++k) {
      acc += (long long)recs[k].n * recs[k].n;
      if (acc >= (1LL << glog) || k == count - 1) {
        groups.push_back({first, k + 1});
        first = k + 1;
        acc = 0;
      }
    }
  }
  items.clear();
  auto emit = [&](int g, int pass) {
    for (int k = groups[g].first; k < groups[g].second; ++k) {
      const int tiles = pass == 1 ? col_tiles(recs[k].n) : row_tiles(recs[k].n);
      const int need = pass == 0 ? 0 : pass == 1 ? recs[k].need1 : recs[k].need2;
      for (int t0 = 0; t0 < tiles; t0 += tpi)
        items.push_back({k, pass, t0, std::min(tpi, tiles - t0), need});
    }
  };
  const int ng = (int)groups.size();
  for (int step = 0; step < ng + 2; ++step)
    for (int pass = 0; pass < 3; ++pass) {
      const int g = step - pass;
      if (g >= 0 && g < ng) emit(g, pass);
    }
  if (opt.debug_unsatisfiable) items.back().need += 1 << 30;

  return LP_OK;
}

}  // namespace

extern "C" {

lp_status lp_batch_create(const lp_beam_desc* beams, int count, const lp_batch_options* options,
                          lp_batch** out) {
  if (!out) return fail(LP_ERR_INVALID_ARGUMENT, "lp_batch_create: out is NULL");
  *out = nullptr;
  std::vector<BeamRec> recs;
  std::vector<Item> items;
  lp_batch_options opt;
  lp_status s = plan_batch(beams, count, options, recs, items, opt);
  if (s != LP_OK) return s;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  s = lp_init(dev);
  if (s != LP_OK) return s;

  BatchPlan* p = new (std::nothrow) BatchPlan();
  if (!p) return fail(LP_ERR_OUT_OF_MEMORY, "lp_batch_create: host allocation failed");
  p->count = count;
  p->n_items = (int)items.size();
  p->device = dev;
  p->spin_limit = opt.spin_limit > 0 ? opt.spin_limit : (1LL << 22);
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  p->ctas = opt.ctas_per_sm > 0 ? std::min(opt.ctas_per_sm, g_batch_occ) : g_batch_occ;
  p->grid = std::max(1, std::min(sms * p->ctas, p->n_items));
  const float2* tws[kMaxLog + 1] = {};
  for (int lg = kMinLog; lg <= kMaxLog; ++lg) {
    tws[lg] = size_ops(1 << lg)->twiddles();
    if (!tws[lg]) {
      free_plan(p);
      return fail(LP_ERR_INTERNAL, "lp_batch_create: twiddle table missing on this device");
    }
  }
  e = cudaMalloc(&p->d_beams, sizeof(BeamRec) * count);
  if (e == cudaSuccess) e = cudaMalloc(&p->d_items, sizeof(Item) * items.size());
  if (e == cudaSuccess) e = cudaMalloc(&p->d_done, sizeof(int) * count);
  if (e == cudaSuccess) e = cudaMalloc(&p->d_state, sizeof(int) * 4);
  if (e == cudaSuccess) e = cudaMalloc(&p->d_tw, sizeof(tws));
  if (e != cudaSuccess) {
    free_plan(p);
    cudaGetLastError();
    return fail(LP_ERR_OUT_OF_MEMORY, "lp_batch_create: device allocation failed");
  }
  e = cudaMemcpy(p->d_beams, recs.data(), sizeof(BeamRec) * count, cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(p->d_items, items.data(), sizeof(Item) * items.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(p->d_done, 0, sizeof(int) * count);
  if (e == cudaSuccess) e = cudaMemset(p->d_state, 0, sizeof(int) * 4);
  if (e == cudaSuccess) e = cudaMemcpy(p->d_tw, tws, sizeof(tws), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    free_plan(p);
    return cuda_fail(e, "lp_batch_create: upload");
  }
  lp_batch* b = new (std::nothrow) lp_batch();
  if (!b) {
    free_plan(p);
    return fail(LP_ERR_OUT_OF_MEMORY, "lp_batch_create: host allocation failed");
  }
  b->plan = *p;
  delete p;
  *out = b;
  return LP_OK;
}

lp_status lp_batch_plan(const lp_beam_desc* beams, int count, const lp_batch_options* options,
                        int* n_items, long long* n_tiles, long long* n_points) {
  std::vector<BeamRec> recs;
  std::vector<Item> items;
  lp_batch_options opt;
  lp_status s = plan_batch(beams, count, options, recs, items, opt);
  if (s != LP_OK) return s;
  long long tiles = 0, points = 0;
  for (const Item& it : items) tiles += it.ntiles;
  for (const BeamRec& r : recs) points += (long long)r.n * r.n;
  if (n_items) *n_items = (int)items.size();
  if (n_tiles) *n_tiles = tiles;
  if (n_points) *n_points = points;
  return LP_OK;
}

lp_status lp_batch_run(lp_batch* batch, void* stream) {
  if (!batch) return fail(LP_ERR_INVALID_ARGUMENT, "lp_batch_run: batch is NULL");
  const BatchPlan& p = batch->plan;
  batch_kernel<<<p.grid, kBT, kSmem, (cudaStream_t)stream>>>(
      p.d_beams, p.d_items, p.n_items, p.d_done, p.d_state, p.count, p.d_tw, p.spin_limit);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? LP_OK : cuda_fail(e, "lp_batch_run");
}

lp_status lp_batch_status(lp_batch* batch, void* stream) {
  if (!batch) return fail(LP_ERR_INVALID_ARGUMENT, "lp_batch_status: batch is NULL");
  const BatchPlan& p = batch->plan;
  cudaError_t e = cudaStreamSynchronize((cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(e, "lp_batch_status: synchronize");
  int err = 0;
  e = cudaMemcpy(&err, p.d_state + 2, sizeof(int), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(e, "lp_batch_status: read flag");
  if (!err) return LP_OK;
  // A run that gave up leaves its counters part-way: clear them for the next run.
  e = cudaMemset(p.d_state, 0, sizeof(int) * 4);
  if (e == cudaSuccess) e = cudaMemset(p.d_done, 0, sizeof(int) * p.count);
  if (e != cudaSuccess) return cuda_fail(e, "lp_batch_status: reset");
  return fail(LP_ERR_TIMEOUT, "lp_batch_run: a bounded device-side wait gave up");
}

lp_status lp_batch_info(const lp_batch* batch, int* n_items, int* grid, int* ctas_per_sm) {
  if (!batch) return fail(LP_ERR_INVALID_ARGUMENT, "lp_batch_info: batch is NULL");
  if (n_items) *n_items = batch->plan.n_items;
  if (grid) *grid = batch->plan.grid;
  if (ctas_per_sm) *ctas_per_sm = batch->plan.ctas;
  return LP_OK;
}

lp_status lp_batch_destroy(lp_batch* batch) {
  if (!batch) return LP_OK;
  BatchPlan* p = new (std::nothrow) BatchPlan(batch->plan);
  delete batch;
  free_plan(p);
  return LP_OK;
}

}  // extern "C"
