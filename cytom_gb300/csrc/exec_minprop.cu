// exec_minprop.cu — BFS, CC and SSSP executors (min-propagation vertex programs).
//
// Replaces ContinuousAlgorithmExecutor::executeAlgorithm with AlgorithmExecutor
// (pull over tiles) and ApplyExecutor (apply over changed vertices)
// (src/include/core/continuous-algorithm-executor.h:72-218,
//  src/include/core/algorithm-executor.h:214-505, src/include/core/apply-executor.h:40-115)
// for the vertex programs examples/bfs.cc, examples/cc.cc and examples/sssp.cc.
//
// One round = gather + apply + control, exactly the reference's Jacobi round:
//   gather: every edge of a tile row that holds an active source (TileManager::isActive,
//     tile-manager.h:403-427) whose own source is active (isEdgeActive) relaxes
//     next[tgt] from current[src] with atomicMin; a lowered value marks `changed`.
//   apply: every changed vertex copies next into current and becomes active for the
//     next round; its tile row is flagged active; the counts of activated vertices and
//     of edges in newly active rows (the reference's processed-edge count,
//     algorithm-executor.h:424-426) accumulate per round.
//   control: ends the run when nothing changed or max_iterations rounds ran, and sets
//     the CUDA-graph while-condition.
// Values are uint32 with UINT32_MAX as "not reached". SSSP sums integer weights
// exactly (the reference's f32 sums are exact for integers below 2^24).
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cstdlib>
#include <cstring>

#include "engine.h"
#include "minprop_dev.cuh"
#include "ptx.cuh"

namespace cytom {

constexpr int GATHER_T = 256;

static int grid_persistent(Ctx* c, int per_sm) { return c->num_sms * per_sm; }

// Clears both parities of the row flags and the loop counters before a run.
__global__ void begin_kernel(const JobDesc* __restrict__ jd, const StoreDesc* __restrict__ sd,
                             unsigned max_iter) {
  LoopState* ls = jd->ls;
  const uint64_t T = sd->T;
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < 2 * T; i += stride)
    jd->rows[i] = 0;
  if (blockIdx.x == 0 && threadIdx.x == 0) minprop_begin_state(ls, max_iter);
}

// Apply over every frontier word (apply_step), then the block's counters (apply_flush);
// the last block to finish runs the round's control step and, inside a captured loop,
// sets the loop's while-condition. Independently of that, block 0 counts the rounds a
// captured loop started and ends the loop with an error status past max_iterations + 1,
// so the loop is bounded whatever the control step does.
__global__ void __launch_bounds__(APPLY_T) apply_minprop_kernel(const JobDesc* __restrict__ jd,
                                                                const StoreDesc* __restrict__ sd, int initial,
                                                                cudaGraphConditionalHandle h, int use_handle) {
  LoopState* ls = jd->ls;
  if (use_handle && blockIdx.x == 0 && threadIdx.x == 0) {
    volatile LoopState* vls = ls;
    const unsigned started = vls->sel_rounds + 1;
    vls->sel_rounds = started;
    if ((uint64_t)started > (uint64_t)vls->max_iter + 2) {
      vls->err = 2;
      vls->cont = 0;
      cudaGraphSetConditional(h, 0u);
    }
  }
  if (!ls->cont) return;
  const unsigned pw = initial ? 0u : ((ls->iter & 1u) ^ 1u);
  const uint64_t nwords = (sd->n + 31) >> 5;
  unsigned cnt = 0;
  unsigned long long teps = 0;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t base = (uint64_t)blockIdx.x * blockDim.x; base < nwords; base += stride)
    apply_step<false>(jd, sd, pw, base, cnt, teps);
  apply_flush(ls, pw, cnt, teps);
  if (threadIdx.x == 0) {
    __threadfence();
    if (atomicAdd(&ls->apply_done, 1u) == gridDim.x - 1) {
      __threadfence();
      atomicExch(&ls->apply_done, 0u);
      const unsigned cont = control_step(jd, sd, initial);
      if (use_handle) cudaGraphSetConditional(h, cont);
    }
  }
}

// Gather for BFS (ALGO 0), CC (1), SSSP (2). A warp owns a 128-edge chunk: lane l
// loads edges [4l, 4l+4) of it with one 128-bit load. The tile of an edge is found
// from the chunk's first tile and tile_ptr (edges are tile-major).
template <int ALGO>
__global__ void __launch_bounds__(GATHER_T) gather_minprop_kernel(const JobDesc* __restrict__ jd,
                                                                  const StoreDesc* __restrict__ sd,
                                                                  int adaptive) {
  LoopState* ls = jd->ls;
  if (!ls->cont || ls->mode != 0) return;
  const unsigned p = ls->iter & 1u;
  const uint64_t T = sd->T;
  const unsigned* __restrict__ rows_cur = jd->rows + p * T;
  round_open<false>(jd, sd, p, adaptive, (uint64_t)blockIdx.x * blockDim.x + threadIdx.x,
                    (uint64_t)gridDim.x * blockDim.x);
  const uint32_t* __restrict__ edges = sd->edges;
  const uint32_t* __restrict__ wts = sd->wts;
  const unsigned long long* __restrict__ tile_ptr = sd->tile_ptr;
  const uint32_t* __restrict__ chunk_tile = sd->chunk_tile;
  const uint32_t* __restrict__ fa = jd->fa;
  const uint32_t* __restrict__ cur = jd->cur;
  const bool async = jd->async != 0;
  uint32_t* next = jd->next;
  uint32_t* ch = jd->ch;
  const uint64_t E = sd->E, nchunks = sd->nchunks;
  const uint32_t lT = sd->lT, lvpt = sd->lvpt;
  const uint32_t ymask = (uint32_t)(T - 1);
  const unsigned lane = threadIdx.x & 31;
  const uint64_t warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  unsigned long long scanned = 0;
  for (uint64_t c = warp; c < nchunks; c += nwarps) {
    const uint32_t t0 = chunk_tile[c];
    const uint32_t t1 = chunk_tile[c + 1];
    if (adaptive) {
      bool any = false;
      for (uint32_t x = t0 >> lT; x <= (t1 >> lT); ++x) any |= rows_cur[x] != 0;
      if (!any) continue;
    }
    const uint64_t e0 = c * kChunk + (uint64_t)lane * 4;
    if (lane == 0) scanned += (E - c * kChunk < (uint64_t)kChunk) ? (E - c * kChunk) : kChunk;
    if (e0 >= E) continue;
    const uint4 ev = *reinterpret_cast<const uint4*>(edges + e0);
    uint4 wv = make_uint4(0, 0, 0, 0);
    if (mp_weighted<ALGO>()) wv = *reinterpret_cast<const uint4*>(wts + e0);
    // locate the tile of e0: last t in [t0, t1] with tile_ptr[t] <= e0
    uint32_t t = t0;
    if (tile_ptr[t + 1] <= e0) {
      uint32_t lo = t0, hi = t1;
      while (lo < hi) {
        uint32_t mid = lo + ((hi - lo + 1) >> 1);
        if (tile_ptr[mid] <= e0) lo = mid;
        else hi = mid - 1;
      }
      t = lo;
    }
    unsigned long long tend = tile_ptr[t + 1];
    const uint32_t evk[4] = {ev.x, ev.y, ev.z, ev.w};
    const uint32_t wvk[4] = {wv.x, wv.y, wv.z, wv.w};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const uint64_t e = e0 + k;
      if (e >= E) break;
      while (tend <= e) {
        ++t;
        tend = tile_ptr[t + 1];
      }
      const uint32_t x = t >> lT, y = t & ymask;
      if (adaptive && rows_cur[x] == 0) continue;
      const uint32_t u = (x << lvpt) | (evk[k] >> 16);
      if (adaptive && !((fa[u >> 5] >> (u & 31)) & 1u)) continue;
      const uint32_t uv = async ? __ldcg(next + u) : cur[u];
      if (uv == kInf) continue;
      const uint32_t cand = mp_cand<ALGO>(uv, wvk[k]);
      if (cand == kInf) continue;
      const uint32_t v = (y << lvpt) | (evk[k] & 0xFFFFu);
      if (cand < __ldcg(next + v)) {
        uint32_t old = atomicMin(next + v, cand);
        if (cand < old) atomicOr(ch + (v >> 5), 1u << (v & 31));
      }
    }
  }
  // edges-scanned counter
  __shared__ unsigned long long s_sc[GATHER_T / 32];
  if (lane == 0) s_sc[threadIdx.x >> 5] = scanned;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long s = 0;
    for (int k = 0; k < GATHER_T / 32; ++k) s += s_sc[k];
    if (s) atomicAdd(&ls->edges_scanned, s);
  }
}

// Streaming gather: the same round as gather_minprop_kernel, with the edge array
// (and weights) streamed through shared memory by bulk copies (cp.async.bulk) in an
// NST-deep mbarrier pipeline, so each SM keeps tens of KB of HBM reads in flight while
// its threads resolve the dependent frontier / value / atomic loads of EPT edges each
// in batches.
//  - Stages are SG_T * EPT-edge slices of the tile-major edge array. A block owns
//    groups of 128 / EPT consecutive stages (group g, g + gridDim.x, ...), so
//    consecutive stages of a block usually lie in one tile row and its frontier words
//    stay in L1.
//  - A stage whose tile rows are all inactive is skipped without being copied.
//  - Single-row stages (the common case at large vertices-per-tile) take the source
//    row from the stage: the frontier test needs no per-edge tile lookup, and only
//    edges with an active source look up their target tile.
// The shape (EPT, NST, blocks per SM) is a variant picked by the autotuner.
template <int ALGO, int EPT, int NST>
__host__ __device__ constexpr size_t gather_stream_smem() {
  return (size_t)NST * SG_T * EPT * 4 * (mp_weighted<ALGO>() ? 2 : 1) + NST * sizeof(uint64_t);
}

template <int ALGO, int EPT, int NST, int MINB>
__global__ void __launch_bounds__(SG_T, MINB) gather_stream_kernel(const JobDesc* __restrict__ jd,
                                                                    const StoreDesc* __restrict__ sd,
                                                                    int adaptive) {
  constexpr uint32_t SE = SG_T * EPT;
  constexpr int SG_GROUP = 128 / EPT;
  extern __shared__ __align__(128) uint8_t smem_raw[];
  uint32_t* ebuf = reinterpret_cast<uint32_t*>(smem_raw);
  uint32_t* wbuf = ebuf + NST * SE;
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem_raw + (size_t)NST * SE * 4 * (mp_weighted<ALGO>() ? 2 : 1));

  LoopState* ls = jd->ls;
  if (!ls->cont || ls->mode != 0) return;
  const unsigned p = ls->iter & 1u;
  round_open<false>(jd, sd, p, adaptive, (uint64_t)blockIdx.x * blockDim.x + threadIdx.x,
                    (uint64_t)gridDim.x * blockDim.x);
  const uint32_t* __restrict__ edges = sd->edges;
  const uint32_t* __restrict__ wts = sd->wts;
  const uint64_t E = sd->E;
  const uint64_t nst = (E + SE - 1) / SE;
  const uint64_t G = gridDim.x;

  // the block's stage sequence: groups blockIdx.x, blockIdx.x + G, ... of SG_GROUP stages
  auto advance = [&](uint64_t s) -> uint64_t {
    uint64_t n1 = s + 1;
    if ((n1 % SG_GROUP) != 0 && n1 < nst) return n1;
    return (s / SG_GROUP + G) * SG_GROUP;
  };
  auto next_active = [&](uint64_t s) -> uint64_t {
    while (s < nst && !stage_active<false, EPT>(jd, sd, s, p, adaptive)) s = advance(s);
    return s < nst ? s : nst;
  };
  auto issue = [&](int slot, uint64_t s) {
    const uint64_t e0 = s * SE;
    const uint64_t rem = E - e0;
    const uint32_t cnt = rem < (uint64_t)SE ? (uint32_t)rem : SE;
    const uint32_t bytes = ((cnt + 3u) & ~3u) * 4u;
    fence_proxy_async_smem();
    mbar_arrive_expect_tx(&bar[slot], bytes * (mp_weighted<ALGO>() ? 2u : 1u));
    bulk_g2s(ebuf + slot * SE, edges + e0, bytes, &bar[slot]);
    if (mp_weighted<ALGO>()) bulk_g2s(wbuf + slot * SE, wts + e0, bytes, &bar[slot]);
  };

  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NST; ++k) mbar_init(&bar[k], 1);
    fence_mbar_init();
  }
  __syncthreads();

  // Thread 0 walks the block's stage sequence (skipping inactive stages) and keeps its
  // queue: stq[k] = the stage in slot (slot + k) % NST, k = 0 the one consumed next. The
  // stage of each slot is published in s_stage when it is issued; every thread reads it
  // there after the block barrier that follows (NST >= 2 barriers later).
  __shared__ unsigned long long s_stage[NST];
  uint64_t stq[NST];
  uint64_t s_next = nst;
  if (threadIdx.x == 0) {
    const uint64_t first = (uint64_t)blockIdx.x * SG_GROUP;
    uint64_t s0 = next_active(first < nst ? first : nst);
#pragma unroll
    for (int k = 0; k < NST; ++k) {
      stq[k] = s0;
      s_stage[k] = s0;
      if (s0 < nst) s0 = next_active(advance(s0));
    }
#pragma unroll
    for (int k = 0; k < NST; ++k)
      if (stq[k] < nst) issue(k, stq[k]);
    s_next = s0;
  }
  __syncthreads();
  uint32_t phases = 0;  // bit k: parity to wait for on slot k
  int slot = 0;
  unsigned long long scanned = 0;
  bool failed = false;

  for (;;) {
    const uint64_t cur = s_stage[slot];
    if (cur >= nst) break;
    // one block barrier per stage: a thread whose bounded wait gave up skips the stage
    // and the barrier after it ends the block
    const bool ok = mbar_wait(&bar[slot], (phases >> slot) & 1u);
    phases ^= 1u << slot;
    if (ok) {
      if (threadIdx.x == 0) {
        const uint64_t rem = E - cur * SE;
        scanned += rem < (uint64_t)SE ? rem : (uint64_t)SE;
      }
      dense_stage<ALGO, false, false, EPT>(jd, sd, ebuf + slot * SE, wbuf + slot * SE, cur, p, adaptive);
    }
    if (__syncthreads_or(!ok)) {  // every thread is done with this slot
      failed = true;
      phases ^= 1u << slot;  // the slot's copy is still owed: the cleanup waits on it
      break;
    }
    if (threadIdx.x == 0) {
      // refill the slot with the next stage of this block
      if (s_next < nst) issue(slot, s_next);
      s_stage[slot] = s_next;
#pragma unroll
      for (int k = 0; k + 1 < NST; ++k) stq[k] = stq[k + 1];
      stq[NST - 1] = s_next;
      if (s_next < nst) s_next = next_active(advance(s_next));
    }
    slot = (slot + 1 == NST) ? 0 : slot + 1;
  }
  if (failed) {
    // give up: record the error, then wait (bounded) for the copies this block still has in flight
    if (threadIdx.x == 0) {
      atomicExch(&ls->err, 1u);
      for (int k = 0; k < NST; ++k) {
        const int sl = (slot + k) % NST;
        if (stq[k] < nst) mbar_wait(&bar[sl], (phases >> sl) & 1u);
      }
    }
    __syncthreads();
    return;
  }
  if (threadIdx.x == 0 && scanned) atomicAdd(&ls->edges_scanned, scanned);
}

// ---- dense round over column-ordered tile stages -----------------------------------
// gather_tiles_kernel: the dense round with the targets of one tile column reduced in
// shared memory, as the reference reduces a tile into its tile-local target buffer before
// writing it back (getLocalNextArray / executeAlgoOnTile / applyTiles,
// src/include/core/algorithm-executor.h:160-200, 214-290, 431-505).
//  - Work: stages of at most TS_P edges that never cross a tile, listed in column-major
//    tile order (column y, then row x, then the tile's pieces). The list is split over the
//    CTAs (one per SM) in contiguous ranges of equal weight (edges + TS_STAGE_COST per
//    stage), so a CTA walks few columns.
//  - Each stage's edges (and weights) arrive by bulk copy (cp.async.bulk) in an NST-deep
//    mbarrier pipeline, as in gather_stream_kernel; a stage of an inactive tile row is
//    skipped without a copy.
//  - While its column holds enough of the CTA's edges, a CTA keeps next values for the
//    column's first S target ids (the ids RMAT graphs hit most: low ids take most edges)
//    in shared memory, neutral kInf, lowered with shared-memory atomics; when the column
//    changes (and at the end) it writes them back in one coalesced pass: a value below
//    next[v] lowers next[v] (red.min) and sets v's changed bit (one red.or per warp and
//    word). That replaces, per relaxed edge, a random pre-check load of next[v] and two
//    global atomics. Targets at or beyond S, and columns with few of the CTA's edges,
//    take that global path directly.
// Values are the same as every other gather's: each target ends the round at the minimum
// over its relaxed edges, exactly.
constexpr int TS_T = 512;                 // threads of a tiles block (8 edges per thread)
constexpr uint32_t TS_BUF = TS_T * 8;     // words per stage buffer (16 KB)
constexpr uint32_t TS_P = TS_BUF - 4;     // edges per stage: a copy starts up to 3 words early
constexpr uint32_t TS_SLICE_MAX = 32768;  // targets held in shared memory (128 KB)
constexpr int TS_NST = 3;
constexpr uint32_t TS_SLICE_MIN = 2;      // slice mode from 2 edges per slice target up
// Partition weight of a stage: its edges plus a fixed cost for its copy, wait and barrier,
// so CTAs whose ranges hold many small tiles get fewer of them.
constexpr uint32_t TS_STAGE_COST = 2048;

template <int ALGO>
__host__ __device__ constexpr size_t tiles_smem_fixed() {
  return (size_t)TS_NST * TS_BUF * 4 * (mp_weighted<ALGO>() ? 2 : 1) + TS_NST * sizeof(uint64_t);
}
static inline uint32_t tiles_slice(uint32_t lvpt) {
  return std::min<uint32_t>(TS_SLICE_MAX, 1u << lvpt);
}

__device__ __forceinline__ uint32_t tiles_lower_bound(const unsigned long long* __restrict__ a, uint32_t n,
                                                      unsigned long long key) {
  uint32_t lo = 0, hi = n;
  while (lo < hi) {
    const uint32_t mid = lo + ((hi - lo) >> 1);
    if (a[mid] < key) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// Writes the shared-memory slice of column y back to next / changed and resets it to
// kInf. Every thread calls it; it ends with a block barrier.
// Slice position of target tl: the low 5 bits are permuted within their group of 32 by
// higher bits, so targets with equal low bits (RMAT ids are skewed in every bit) spread
// over the shared-memory banks. A group of 32 targets stays one group of 32 positions.
__device__ __forceinline__ uint32_t tiles_pos(uint32_t tl) {
  return tl ^ (((tl >> 5) ^ (tl >> 10) ^ (tl >> 15)) & 31u);
}

// A warp covers 32 consecutive targets (one changed word) per step and keeps FL steps'
// loads of next in flight.
constexpr int TS_FL = 8;
__device__ __forceinline__ void tiles_flush(const JobDesc* __restrict__ jd, uint32_t* slice, uint32_t S,
                                            uint32_t yb) {
  uint32_t* next = jd->next;
  uint32_t* ch = jd->ch;
  const unsigned lane = threadIdx.x & 31;
  for (uint32_t base0 = (threadIdx.x & ~31u); base0 < S; base0 += TS_T * TS_FL) {
    uint32_t c[TS_FL], nv[TS_FL];
#pragma unroll
    for (int k = 0; k < TS_FL; ++k) {
      const uint32_t i = tiles_pos(base0 + (uint32_t)k * TS_T + lane);  // target base0 + k*TS_T + lane
      c[k] = (base0 + (uint32_t)k * TS_T < S) ? slice[i] : kInf;
      if (c[k] != kInf) slice[i] = kInf;
    }
#pragma unroll
    for (int k = 0; k < TS_FL; ++k)
      nv[k] = (c[k] != kInf) ? __ldcg(next + yb + base0 + (uint32_t)k * TS_T + lane) : 0u;
#pragma unroll
    for (int k = 0; k < TS_FL; ++k) {
      const uint32_t v = yb + base0 + (uint32_t)k * TS_T + lane;
      const bool imp = c[k] != kInf && c[k] < nv[k];
      if (imp) atomicMin(next + v, c[k]);
      const unsigned m = __ballot_sync(0xFFFFFFFFu, imp);
      if (lane == 0 && m) atomicOr(ch + (v >> 5), m);
    }
  }
  __syncthreads();
}

template <int ALGO>
__global__ void __launch_bounds__(TS_T, 1) gather_tiles_kernel(const JobDesc* __restrict__ jd,
                                                               const StoreDesc* __restrict__ sd, int adaptive) {
  extern __shared__ __align__(128) uint8_t smem_raw[];
  __shared__ uint32_t s_range[2];
  LoopState* ls = jd->ls;
  if (!ls->cont || ls->mode != 0) return;
  const unsigned p = ls->iter & 1u;
  round_open<false>(jd, sd, p, adaptive, (uint64_t)blockIdx.x * blockDim.x + threadIdx.x,
                    (uint64_t)gridDim.x * blockDim.x);
  constexpr bool WT = mp_weighted<ALGO>();
  const uint32_t lvpt = sd->lvpt, lT = sd->lT;
  const uint32_t vpt = 1u << lvpt;
  const uint32_t ymask = (uint32_t)(sd->T - 1);
  const uint32_t S = min(TS_SLICE_MAX, vpt);
  uint32_t* slice = reinterpret_cast<uint32_t*>(smem_raw);
  uint32_t* ebuf = slice + S;
  uint32_t* wbuf = ebuf + TS_NST * TS_BUF;
  uint64_t* bar = reinterpret_cast<uint64_t*>(ebuf + TS_NST * TS_BUF * (WT ? 2 : 1));
  if (sd->xnst == nullptr) {  // no stage list (never launched so): fail loudly
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicExch(&ls->err, 3u);
    return;
  }
  const TileStage* __restrict__ stages = sd->xst;
  const unsigned long long* __restrict__ cum = sd->xcum;
  const unsigned* rows_cur = jd->rows + p * sd->T;
  const uint32_t* __restrict__ edges = sd->edges;
  const uint32_t* __restrict__ wts = sd->wts;
  const uint32_t* fa = jd->fa;
  const bool async = jd->async != 0;
  uint32_t* next = jd->next;
  uint32_t* ch = jd->ch;

  if (threadIdx.x == 0) {
    const uint32_t nst = *sd->xnst;
    const unsigned long long total = cum[nst];
    const unsigned long long lo = total * blockIdx.x / gridDim.x, hi = total * (blockIdx.x + 1) / gridDim.x;
    s_range[0] = tiles_lower_bound(cum, nst, lo);
    s_range[1] = tiles_lower_bound(cum, nst, hi);
#pragma unroll
    for (int k = 0; k < TS_NST; ++k) mbar_init(&bar[k], 1);
    fence_mbar_init();
  }
  for (uint32_t i = threadIdx.x; i < S; i += TS_T) slice[i] = kInf;
  __syncthreads();
  const uint32_t sb = s_range[0], se = s_range[1];
  const unsigned long long cta_lo = cum[sb], cta_hi = cum[se];

  auto next_active = [&](uint32_t s) -> uint32_t {
    if (adaptive)
      while (s < se && ld_plain<false>(rows_cur + (stages[s].tile >> lT)) == 0) ++s;
    return s;
  };
  auto issue = [&](int slot, uint32_t s) {
    const TileStage st = stages[s];
    const unsigned long long a0 = st.e0 & ~3ULL;
    const uint32_t words = ((uint32_t)(st.e0 & 3ULL) + st.count + 3u) & ~3u;
    fence_proxy_async_smem();
    mbar_arrive_expect_tx(&bar[slot], words * 4u * (WT ? 2u : 1u));
    bulk_g2s(ebuf + slot * TS_BUF, edges + a0, words * 4u, &bar[slot]);
    if (WT) bulk_g2s(wbuf + slot * TS_BUF, wts + a0, words * 4u, &bar[slot]);
  };

  uint32_t stq[TS_NST];
  {
    uint32_t s0 = next_active(sb);
#pragma unroll
    for (int k = 0; k < TS_NST; ++k) {
      stq[k] = s0;
      if (s0 < se) s0 = next_active(s0 + 1);
    }
    if (threadIdx.x == 0) {
#pragma unroll
      for (int k = 0; k < TS_NST; ++k)
        if (stq[k] < se) issue(k, stq[k]);
    }
  }
  uint32_t s_next = (stq[TS_NST - 1] < se) ? next_active(stq[TS_NST - 1] + 1) : se;
  uint32_t phases = 0;
  int slot = 0;
  unsigned long long scanned = 0;
  bool failed = false;
  uint32_t cur_col = 0xFFFFFFFFu;
  bool slice_mode = false;

  while (stq[0] < se) {
    const TileStage st = stages[stq[0]];
    const uint32_t y = st.tile & ymask;
    if (y != cur_col) {  // uniform: every thread walks the same stages
      if (slice_mode) tiles_flush(jd, slice, S, cur_col << lvpt);
      cur_col = y;
      slice_mode = false;
      if (sd->traversal == CYTOM_TRAVERSAL_ROW_FIRST) {  // a column's tiles are consecutive
        const unsigned long long c0 = sd->xcolcum[y], c1 = sd->xcolcum[y + 1];
        const unsigned long long seg = min(cta_hi, c1) - max(cta_lo, c0);
        slice_mode = seg >= (unsigned long long)S * TS_SLICE_MIN;
      }
    }
    const bool ok = mbar_wait(&bar[slot], (phases >> slot) & 1u);
    phases ^= 1u << slot;
    if (ok) {
      if (threadIdx.x == 0) scanned += st.count;
      const uint32_t x = st.tile >> lT;
      const uint32_t xb = x << lvpt, yb = y << lvpt;
      const uint32_t off = (uint32_t)(st.e0 & 3ULL), endp = off + st.count;
      const bool full_row = !adaptive || ld_plain<false>(rows_cur + x) == vpt;
      const uint32_t* eb = ebuf + slot * TS_BUF;
      const uint32_t* wb = wbuf + slot * TS_BUF;
      uint32_t qv[8], ww[8], uu[8];
      uint32_t vmask = 0;
#pragma unroll
      for (int k = 0; k < 2; ++k) {
        const uint32_t i0 = threadIdx.x * 4 + (uint32_t)k * (TS_T * 4);
        const uint4 q = *reinterpret_cast<const uint4*>(eb + i0);
        uint4 wq = make_uint4(0, 0, 0, 0);
        if (WT) wq = *reinterpret_cast<const uint4*>(wb + i0);
        qv[4 * k + 0] = q.x;
        qv[4 * k + 1] = q.y;
        qv[4 * k + 2] = q.z;
        qv[4 * k + 3] = q.w;
        ww[4 * k + 0] = wq.x;
        ww[4 * k + 1] = wq.y;
        ww[4 * k + 2] = wq.z;
        ww[4 * k + 3] = wq.w;
#pragma unroll
        for (int j = 0; j < 4; ++j) vmask |= ((i0 + j) >= off && (i0 + j) < endp) ? (1u << (4 * k + j)) : 0u;
      }
#pragma unroll
      for (int idx = 0; idx < 8; ++idx) uu[idx] = xb | (qv[idx] >> 16);
      uint32_t amask = vmask;
      if (!full_row && vmask) {
        uint32_t fw[8];
#pragma unroll
        for (int idx = 0; idx < 8; ++idx) fw[idx] = ((vmask >> idx) & 1u) ? ld_state<false>(fa + (uu[idx] >> 5)) : 0u;
        amask = 0;
#pragma unroll
        for (int idx = 0; idx < 8; ++idx) amask |= ((fw[idx] >> (uu[idx] & 31)) & 1u) << idx;
        amask &= vmask;
      }
      if (amask) {
        uint32_t cand[8];
#pragma unroll
        for (int idx = 0; idx < 8; ++idx) cand[idx] = ((amask >> idx) & 1u) ? ld_src<false>(jd, async, uu[idx]) : kInf;
#pragma unroll
        for (int idx = 0; idx < 8; ++idx)
          if (cand[idx] != kInf) cand[idx] = mp_cand<ALGO>(cand[idx], ww[idx]);
        uint32_t gmask = 0;  // edges taking the global path
#pragma unroll
        for (int idx = 0; idx < 8; ++idx) {
          if (cand[idx] == kInf) continue;
          const uint32_t tl = qv[idx] & 0xFFFFu;
          if (slice_mode && tl < S) {
            uint32_t* sp = slice + tiles_pos(tl);
            if (cand[idx] < *sp) atomicMin(sp, cand[idx]);
          } else {
            gmask |= 1u << idx;
          }
        }
        if (gmask) {
          uint32_t nv[8];
#pragma unroll
          for (int idx = 0; idx < 8; ++idx)
            nv[idx] = ((gmask >> idx) & 1u) ? __ldcg(next + (yb | (qv[idx] & 0xFFFFu))) : 0u;
#pragma unroll
          for (int idx = 0; idx < 8; ++idx) {
            if (((gmask >> idx) & 1u) && cand[idx] < nv[idx]) {
              const uint32_t v = yb | (qv[idx] & 0xFFFFu);
              atomicMin(next + v, cand[idx]);
              atomicOr(ch + (v >> 5), 1u << (v & 31));
            }
          }
        }
      }
    }
    if (__syncthreads_or(!ok)) {
      failed = true;
      phases ^= 1u << slot;  // the slot's copy is still owed: the cleanup waits on it
      break;
    }
    if (threadIdx.x == 0 && s_next < se) issue(slot, s_next);
#pragma unroll
    for (int k = 0; k + 1 < TS_NST; ++k) stq[k] = stq[k + 1];
    stq[TS_NST - 1] = s_next;
    if (s_next < se) s_next = next_active(s_next + 1);
    slot = (slot + 1 == TS_NST) ? 0 : slot + 1;
  }
  if (failed) {
    if (threadIdx.x == 0) {
      atomicExch(&ls->err, 1u);
      for (int k = 0; k < TS_NST; ++k) {
        const int sl = (slot + k) % TS_NST;
        if (stq[k] < se) mbar_wait(&bar[sl], (phases >> sl) & 1u);
      }
    }
    __syncthreads();
    return;
  }
  if (slice_mode) tiles_flush(jd, slice, S, cur_col << lvpt);
  if (threadIdx.x == 0 && scanned) atomicAdd(&ls->edges_scanned, scanned);
}

// Tile at position d of a traversal order (x = source tile, y = target tile, T = 2^lT):
// row-first d = y * T + x, column-first d = x * T + y (src/lib/traversal/row_first.cc,
// column_first.cc), or the Hilbert curve's d -> (x, y) (the published curve-walk
// algorithm that src/lib/traversal/hilbert.cc:35-47 also follows).
__device__ __forceinline__ uint64_t traversal_tile(uint32_t order, uint64_t d, uint32_t lT) {
  const uint64_t tm = (1ULL << lT) - 1ULL;
  uint64_t x, y;
  if (order == CYTOM_TRAVERSAL_COLUMN_FIRST) {
    x = d >> lT;
    y = d & tm;
  } else if (order == CYTOM_TRAVERSAL_HILBERT) {
    x = 0;
    y = 0;
    uint64_t t = d;
    for (uint64_t s = 1; s < (1ULL << lT); s <<= 1) {
      const uint64_t rx = 1 & (t >> 1);
      const uint64_t ry = 1 & (t ^ rx);
      if (ry == 0) {  // rotate the quadrant
        if (rx == 1) {
          x = s - 1 - x;
          y = s - 1 - y;
        }
        const uint64_t tmp = x;
        x = y;
        y = tmp;
      }
      x += s * rx;
      y += s * ry;
      t >>= 2;
    }
  } else {
    y = d >> lT;
    x = d & tm;
  }
  return (x << lT) | y;
}

// Stage list of gather_tiles_kernel, per store version: the tiles in the traversal order
// (rank r names tile traversal_tile(r)), each cut into stages of at most TS_P edges.
__global__ void xs_count_kernel(const unsigned long long* __restrict__ tile_ptr, uint32_t lT, uint64_t ntiles,
                                uint32_t order, uint32_t* __restrict__ cnt, uint32_t* __restrict__ size) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; r < ntiles; r += stride) {
    const uint64_t t = traversal_tile(order, r, lT);
    const uint64_t sz = tile_ptr[t + 1] - tile_ptr[t];
    size[r] = (uint32_t)sz;
    cnt[r] = (uint32_t)((sz + TS_P - 1) / TS_P);
  }
}

__global__ void xs_write_kernel(const unsigned long long* __restrict__ tile_ptr, uint32_t lT, uint64_t ntiles,
                                uint32_t order, const uint32_t* __restrict__ cnt, const uint32_t* __restrict__ off,
                                const uint32_t* __restrict__ size, const uint32_t* __restrict__ ecm,
                                const uint32_t* __restrict__ nst, TileStage* __restrict__ st,
                                unsigned long long* __restrict__ cum, unsigned long long* __restrict__ colcum,
                                unsigned long long E) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  const uint64_t tm = (1ULL << lT) - 1ULL;
  for (uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; r < ntiles; r += stride) {
    const uint64_t t = traversal_tile(order, r, lT);
    const uint32_t n = cnt[r], o = off[r], sz = size[r];
    const unsigned long long wbase = (unsigned long long)ecm[r] + (unsigned long long)o * TS_STAGE_COST;
    if ((r & tm) == 0) colcum[r >> lT] = wbase;  // row-first: the first tile of column r >> lT
    const unsigned long long e0 = tile_ptr[t];
    for (uint32_t k = 0; k < n; ++k) {
      TileStage s;
      s.tile = (uint32_t)t;
      s.count = min(TS_P, sz - k * TS_P);
      s.e0 = e0 + (unsigned long long)k * TS_P;
      st[o + k] = s;
      cum[o + k] = wbase + (unsigned long long)k * (TS_P + TS_STAGE_COST);
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    const unsigned long long total = E + (unsigned long long)(*nst) * TS_STAGE_COST;
    cum[*nst] = total;
    colcum[1ULL << lT] = total;
  }
}

// The column-ordered dense round needs tiles of >= 1024 vertices (a warp-aligned shared
// slice of >= 1024 targets) and 32-bit column offsets.
static bool tiles_geometry(const Ctx* c) { return c->lvpt >= 10; }
static bool tiles_usable(const Ctx* c) { return tiles_geometry(c) && c->E < 0xFFFFFFF0ull; }
constexpr int kTilesVariant = 4;

int build_tile_stages(Ctx* c) {
  if (c->xs_version == c->version) return CYTOM_OK;
  if (!tiles_usable(c)) {
    // a store past 2^32 edges: programs tuned to the tiles kernel go back to the stream
    for (int k = 0; k < 2; ++k)
      if (c->sg_variant[k] == kTilesVariant) {
        c->sg_variant[k] = 0;
        c->tune_epoch++;
      }
    c->xs_version = c->version;
    return CYTOM_OK;
  }
  const uint64_t nt = c->ntiles;
  const uint64_t need = c->E / TS_P + nt + 1;
  if (need > c->xs_cap || !c->xs_tmp) {
    join_runs(c);  // runs in flight may still read the old list
    cudaError_t se = cudaStreamSynchronize(c->stream);
    if (se != cudaSuccess) return cuda_err(c, se, "tile stage list");
    cudaFree(c->xs_stage);
    cudaFree(c->xs_cum);
    c->xs_stage = nullptr;
    c->xs_cum = nullptr;
    c->xs_cap = 0;
    const uint64_t cap = need + need / 2;
    if (cy_malloc(&c->xs_stage, cap * sizeof(TileStage)) != cudaSuccess ||
        cy_malloc(&c->xs_cum, (cap + 1) * 8) != cudaSuccess ||
        (!c->xs_colcum && cy_malloc(&c->xs_colcum, (c->T + 1) * 8) != cudaSuccess) ||
        (!c->xs_tmp && cy_malloc(&c->xs_tmp, (4 * nt + 8) * 4) != cudaSuccess)) {
      cudaGetLastError();
      return set_err(c, CYTOM_ERR_OOM, "tile stage list");
    }
    c->xs_cap = cap;
  }
  uint32_t* cnt = c->xs_tmp;
  uint32_t* off = c->xs_tmp + (nt + 1);
  uint32_t* nst = c->xs_tmp + 2 * (nt + 1);
  uint32_t* tot = nst + 1;
  uint32_t* size = nst + 2;
  uint32_t* ecm = size + nt;
  int slot = prof_begin(c, KC_MERGE);
  xs_count_kernel<<<std::max(1, std::min<int>(grid_persistent(c, 8), (int)((nt + 255) / 256))), 256, 0, c->stream>>>(
      c->tile_ptr, c->lT, nt, (uint32_t)c->cfg.traversal, cnt, size);
  c->launches++;
  int rc = exclusive_scan_u32(c, cnt, off, nt, nst);
  if (!rc) rc = exclusive_scan_u32(c, size, ecm, nt, tot);
  if (rc) return rc;
  xs_write_kernel<<<std::max(1, std::min<int>(grid_persistent(c, 8), (int)((nt + 255) / 256))), 256, 0, c->stream>>>(
      c->tile_ptr, c->lT, nt, (uint32_t)c->cfg.traversal, cnt, off, size, ecm, nst, c->xs_stage, c->xs_cum,
      c->xs_colcum, c->E);
  c->launches++;
  prof_end(c, slot, (double)nt * 28.0 + (double)need * 24.0);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_err(c, e, "tile stage list");
  c->xs_version = c->version;
  return upload_store_desc(c);
}

// Sparse gather (sparse_group over every group of 32 items) and its chunk pass
// (sparse_chunk over the queue the first pass filled).
template <int ALGO>
__global__ void __launch_bounds__(256, 4) gather_sparse_kernel(const JobDesc* __restrict__ jd,
                                                             const StoreDesc* __restrict__ sd, int adaptive) {
  LoopState* ls = jd->ls;
  if (!ls->cont || ls->mode != 1) return;
  const unsigned p = ls->iter & 1u;
  round_open<false>(jd, sd, p, adaptive, (uint64_t)blockIdx.x * blockDim.x + threadIdx.x,
                    (uint64_t)gridDim.x * blockDim.x);
  const unsigned lane = threadIdx.x & 31;
  const uint64_t warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  const uint64_t items = (uint64_t)ls->nact_words[p] << sd->lT;
  unsigned long long scanned = 0;
  uint32_t nread = 0;
  // few groups: up to 8 warps share each group's light edges
  const uint64_t groups = (items + 31) / 32;
  uint32_t nslice = 1;
  while (nslice < 8 && groups * nslice * 2 <= nwarps) nslice *= 2;
  const uint32_t slice = (uint32_t)(warp % nslice);
  for (uint64_t g = (warp / nslice) * 32; g < items; g += (nwarps / nslice) * 32)
    scanned += sparse_group<ALGO, false>(jd, sd, g, items, nread, slice, nslice);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    scanned += __shfl_xor_sync(0xFFFFFFFFu, scanned, o);
    nread += __shfl_xor_sync(0xFFFFFFFFu, nread, o);
  }
  if (lane == 0 && scanned) atomicAdd(&ls->edges_scanned, scanned);
  if (lane == 0 && nread) atomicAdd(&ls->items_read, (unsigned long long)nread);
}

template <int ALGO>
__global__ void __launch_bounds__(256, 4) gather_sparse_chunks(const JobDesc* __restrict__ jd,
                                                             const StoreDesc* __restrict__ sd) {
  LoopState* ls = jd->ls;
  if (!ls->cont || ls->mode != 1) return;
  const unsigned lane = threadIdx.x & 31;
  const uint64_t warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  uint64_t nq = ls->spq_count;
  if (nq > jd->spq_cap) nq = jd->spq_cap;
  const uint64_t items = (uint64_t)ls->nact_words[ls->iter & 1u] << sd->lT;
  unsigned long long scanned = 0;
  for (uint64_t q = warp; q < nq; q += nwarps) scanned += sparse_chunk<ALGO, false>(jd, sd, q, items);
  if (lane == 0 && scanned) atomicAdd(&ls->edges_scanned, scanned);
}

// ---- job state -----------------------------------------------------------

__global__ void init_minprop_kernel(const JobDesc* __restrict__ jd, const StoreDesc* __restrict__ sd,
                                    int algo) {
  const uint64_t n = sd->n;
  const uint64_t nwords = (n + 31) >> 5;
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t v = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += stride) {
    uint32_t val = (algo == CYTOM_ALGO_CC) ? (uint32_t)v : kInf;
    jd->cur[v] = val;
    jd->next[v] = val;
  }
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nwords; i += stride) {
    jd->fa[i] = 0;
    uint32_t m = 0;
    if (algo == CYTOM_ALGO_CC) {
      uint64_t rem = n - (i << 5);
      m = rem >= 32 ? 0xFFFFFFFFu : ((1u << rem) - 1u);
    }
    jd->ch[i] = m;
  }
}

// BFS / SSSP start vertex: next = 0 and changed, so the seeding apply activates it
// (examples/bfs.cc:193-196; for SSSP the start distance the reference never sets,
// examples/sssp.cc:197-202).
__global__ void init_start_kernel(const JobDesc* __restrict__ jd, unsigned long long s) {
  jd->next[s] = 0;
  jd->ch[s >> 5] |= 1u << (s & 31);
}

// edgeChanged(INSERT) for a batch (examples/bfs.cc:115-140, cc.cc:113-131,
// sssp.cc:337-356): a target that the new edge improves gets the better value in
// next and is marked changed; the next run propagates from there. Reads current
// values (equal to next after a converged run).
template <int ALGO>
__global__ void seed_minprop_kernel(const JobDesc* __restrict__ jd, const uint32_t* __restrict__ src,
                                    const uint32_t* __restrict__ tgt, const uint32_t* __restrict__ w,
                                    uint64_t count) {
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  const uint32_t* cur = jd->cur;
  uint32_t* next = jd->next;
  uint32_t* ch = jd->ch;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += stride) {
    uint32_t u = src[i], v = tgt[i];
    uint32_t uv = cur[u];
    if (uv == kInf) continue;
    const uint32_t cand = mp_cand<ALGO>(uv, w ? w[i] : 1u);
    if (cand == kInf) continue;
    if (cand < __ldcg(next + v)) {
      uint32_t old = atomicMin(next + v, cand);
      if (cand < old) atomicOr(ch + (v >> 5), 1u << (v & 31));
    }
  }
}

// edgeChanged(DELETE) (examples/sssp.cc:135-139: the reference re-runs a job when a
// deleted edge was its target's critical neighbour). A deleted edge (u, v, w) matters when
// it is tight: cand(cur[u], w) equals the value v holds (cur, or next when a pending insert
// seeded v through it). Without a tight deleted edge every value is still carried by a
// path of tight edges that all remain stored, and deleting edges cannot lower any value,
// so the values stay the fixed point of the new graph. A run that stopped before
// converging (cont still set) counts as tight. *tight becomes 1 if the job must restart.
template <int ALGO>
__global__ void delete_tight_kernel(const JobDesc* __restrict__ jd, const uint32_t* __restrict__ dsrc,
                                    const uint32_t* __restrict__ dtgt, const uint32_t* __restrict__ dw,
                                    uint64_t count, unsigned* tight) {
  if (blockIdx.x == 0 && threadIdx.x == 0 && *(volatile unsigned*)&jd->ls->cont != 0) *tight = 1u;
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  const uint32_t* cur = jd->cur;
  const uint32_t* next = jd->next;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += stride) {
    const uint32_t uv = cur[dsrc[i]];
    if (uv == kInf) continue;
    const uint32_t cand = mp_cand<ALGO>(uv, dw ? dw[i] : 1u);
    const uint32_t v = dtgt[i];
    if (cand == cur[v] || cand == next[v]) *tight = 1u;
  }
}

// The same seeding from the compaction's sorted keys [x][y][src_local][tgt_local] of the
// edges appended since the last compaction: the jobs are seeded when the merged snapshot is
// installed, after the runs on the previous snapshot have finished; all min-propagation
// jobs of the context in one pass over the keys (each key decoded, its weight read once).
struct SeedJobs {
  const JobDesc* jd[kMaxSeedJobs];
  int algo[kMaxSeedJobs];
  int count;
};

template <int ALGO>
__device__ __forceinline__ void seed_one(const JobDesc* __restrict__ jd, uint32_t u, uint32_t v, uint32_t w) {
  const uint32_t uv = jd->cur[u];
  if (uv == kInf) return;
  const uint32_t cand = mp_cand<ALGO>(uv, w);
  if (cand == kInf) return;
  if (cand < __ldcg(jd->next + v)) {
    uint32_t old = atomicMin(jd->next + v, cand);
    if (cand < old) atomicOr(jd->ch + (v >> 5), 1u << (v & 31));
  }
}

__global__ void seed_keys_multi_kernel(SeedJobs sj, const uint64_t* __restrict__ K, const uint32_t* __restrict__ W,
                                       uint64_t count, uint32_t lvpt, uint32_t lT) {
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  const uint64_t m = (1ULL << lvpt) - 1ULL;
  const uint64_t tmask = (1ULL << lT) - 1ULL;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += stride) {
    const uint64_t key = K[i];
    const uint64_t tile = key >> (2 * lvpt);
    const uint32_t u = (uint32_t)(((tile >> lT) << lvpt) | ((key >> lvpt) & m));
    const uint32_t v = (uint32_t)(((tile & tmask) << lvpt) | (key & m));
    const uint32_t w = W ? W[i] : 1u;
    for (int k = 0; k < sj.count; ++k) {
      switch (sj.algo[k]) {
        case CYTOM_ALGO_BFS: seed_one<0>(sj.jd[k], u, v, w); break;
        case CYTOM_ALGO_CC: seed_one<1>(sj.jd[k], u, v, w); break;
        case CYTOM_ALGO_SSWP: seed_one<3>(sj.jd[k], u, v, w); break;
        default: seed_one<2>(sj.jd[k], u, v, w); break;
      }
    }
  }
}

int minprop_seed_keys_many(Ctx* c, Job* const* jobs, int njobs, const uint64_t* K, const uint32_t* W,
                           uint64_t count) {
  int g = std::max(1, std::min<int>(grid_persistent(c, 8), (int)((count + 255) / 256)));
  for (int base = 0; base < njobs; base += kMaxSeedJobs) {
    SeedJobs sj{};
    sj.count = std::min(kMaxSeedJobs, njobs - base);
    for (int k = 0; k < sj.count; ++k) {
      sj.jd[k] = jobs[base + k]->d;
      sj.algo[k] = jobs[base + k]->algo;
    }
    int slot = prof_begin(c, KC_INSERT);
    seed_keys_multi_kernel<<<g, 256, 0, c->stream>>>(sj, K, W, count, c->lvpt, c->lT);
    c->launches++;
    prof_end(c, slot, (double)count * (12.0 + 8.0 * sj.count));
  }
  return cuda_err(c, cudaGetLastError(), "seed_keys");
}


int minprop_delete_check(Ctx* c, Job* j, const uint32_t* dsrc, const uint32_t* dtgt, const uint32_t* dw,
                         uint64_t count, unsigned* tight) {
  int g = std::max(1, std::min<int>(grid_persistent(c, 8), (int)((count + 255) / 256)));
  switch (j->algo) {
    case CYTOM_ALGO_BFS: delete_tight_kernel<0><<<g, 256, 0, c->stream>>>(j->d, dsrc, dtgt, dw, count, tight); break;
    case CYTOM_ALGO_CC: delete_tight_kernel<1><<<g, 256, 0, c->stream>>>(j->d, dsrc, dtgt, dw, count, tight); break;
    case CYTOM_ALGO_SSWP: delete_tight_kernel<3><<<g, 256, 0, c->stream>>>(j->d, dsrc, dtgt, dw, count, tight); break;
    default: delete_tight_kernel<2><<<g, 256, 0, c->stream>>>(j->d, dsrc, dtgt, dw, count, tight); break;
  }
  c->launches++;
  return cuda_err(c, cudaGetLastError(), "delete_tight");
}

int minprop_alloc(Ctx* c, Job* j) {
  const uint64_t n = c->n;
  const uint64_t nwords = (n + 31) / 32;
  JobDesc& h = j->h;
  cudaError_t e = cy_malloc(&h.cur, n * 4);
  if (e == cudaSuccess) e = cy_malloc(&h.next, n * 4);
  if (e == cudaSuccess) e = cy_malloc(&h.fa, nwords * 4);
  if (e == cudaSuccess) e = cy_malloc(&h.ch, nwords * 4);
  if (e == cudaSuccess) e = cy_malloc(&h.rows, 2 * c->T * 4);
  if (e == cudaSuccess) e = cy_malloc(&h.aw, nwords * 4);
  if (e == cudaSuccess) e = cy_malloc(&h.awm, nwords * 8);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return set_err(c, CYTOM_ERR_OOM, "job state");
  }
  return CYTOM_OK;
}

int minprop_init(Ctx* c, Job* j) {
  int algo = j->algo;
  init_minprop_kernel<<<grid_persistent(c, 8), 256, 0, c->stream>>>(j->d, c->dsd, algo);
  c->launches++;
  if (algo != CYTOM_ALGO_CC) {
    init_start_kernel<<<1, 1, 0, c->stream>>>(j->d, j->params.start_vertex);
    c->launches++;
  }
  return cuda_err(c, cudaGetLastError(), "init_minprop");
}

int minprop_seed(Ctx* c, Job* j, const uint32_t* src, const uint32_t* tgt, const uint32_t* w,
                 uint64_t count) {
  int g = std::max(1, std::min<int>(grid_persistent(c, 8), (int)((count + 255) / 256)));
  int slot = prof_begin(c, KC_INSERT);
  switch (j->algo) {
    case CYTOM_ALGO_BFS: seed_minprop_kernel<0><<<g, 256, 0, c->stream>>>(j->d, src, tgt, w, count); break;
    case CYTOM_ALGO_CC: seed_minprop_kernel<1><<<g, 256, 0, c->stream>>>(j->d, src, tgt, w, count); break;
    case CYTOM_ALGO_SSWP: seed_minprop_kernel<3><<<g, 256, 0, c->stream>>>(j->d, src, tgt, w, count); break;
    default: seed_minprop_kernel<2><<<g, 256, 0, c->stream>>>(j->d, src, tgt, w, count); break;
  }
  c->launches++;
  prof_end(c, slot, (double)count * 16.0);
  return cuda_err(c, cudaGetLastError(), "seed_minprop");
}

// Gather variant: "stream" (bulk-copy pipeline, default) or "simple" (direct
// 128-bit loads, one chunk per warp); CYTOM_GATHER selects it.
static int gather_mode() {
  static int v = -1;
  if (v < 0) {
    const char* s = getenv("CYTOM_GATHER");
    v = (s && strcmp(s, "simple") == 0) ? 0 : 1;
  }
  return v;
}

struct GatherLaunch {
  void* fn;
  dim3 grid, block;
  size_t smem;
};

// Shapes of the streaming gather the autotuner chooses from: edges per thread, pipeline
// depth, resident blocks per SM (shared memory per SM: blocks x depth x stage bytes).
struct SgVariant {
  int ept, nst, minb;
};
static const SgVariant kSgVariants[] = {{16, 3, 2}, {8, 4, 3}, {8, 3, 4}, {4, 6, 4}};
constexpr int kSgVariantCount = 4;

template <int ALGO>
static void* sg_fn(int v) {
  switch (v) {
    case 1: return (void*)gather_stream_kernel<ALGO, 8, 4, 3>;
    case 2: return (void*)gather_stream_kernel<ALGO, 8, 3, 4>;
    case 3: return (void*)gather_stream_kernel<ALGO, 4, 6, 4>;
    default: return (void*)gather_stream_kernel<ALGO, 16, 3, 2>;
  }
}
template <int ALGO>
static size_t sg_smem(int v) {
  switch (v) {
    case 1: return gather_stream_smem<ALGO, 8, 4>();
    case 2: return gather_stream_smem<ALGO, 8, 3>();
    case 3: return gather_stream_smem<ALGO, 4, 6>();
    default: return gather_stream_smem<ALGO, 16, 3>();
  }
}

template <int ALGO>
static GatherLaunch tiles_launch_t(Ctx* c) {
  static int attr_set = 0;
  GatherLaunch g{};
  g.fn = (void*)gather_tiles_kernel<ALGO>;
  g.smem = (size_t)tiles_slice(c->lvpt) * 4 + tiles_smem_fixed<ALGO>();
  const size_t full = (size_t)TS_SLICE_MAX * 4 + tiles_smem_fixed<ALGO>();
  if (!attr_set) {
    cudaFuncSetAttribute(g.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)full);
    attr_set = 1;
  }
  g.grid = dim3(grid_persistent(c, 1));
  g.block = dim3(TS_T);
  return g;
}

static GatherLaunch tiles_launch(Ctx* c, int a) {
  return a == 0 ? tiles_launch_t<0>(c) : a == 1 ? tiles_launch_t<1>(c) : a == 3 ? tiles_launch_t<3>(c)
                                                                         : tiles_launch_t<2>(c);
}

static GatherLaunch stream_launch(Ctx* c, int a, int v) {
  if (v == kTilesVariant) return tiles_launch(c, a);
  static bool attr_set[4][kSgVariantCount] = {};
  GatherLaunch g{};
  g.fn = a == 0 ? sg_fn<0>(v) : a == 1 ? sg_fn<1>(v) : a == 3 ? sg_fn<3>(v) : sg_fn<2>(v);
  g.smem = a >= 2 ? sg_smem<2>(v) : sg_smem<0>(v);
  if (!attr_set[a][v]) {
    cudaFuncSetAttribute(g.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)g.smem);
    attr_set[a][v] = true;
  }
  g.grid = dim3(grid_persistent(c, kSgVariants[v].minb));
  g.block = dim3(SG_T);
  return g;
}

// The variant in use: CYTOM_SG_VARIANT overrides; else the autotuner's choice for the
// program's class (unweighted BFS / CC, weighted SSSP).
static int sg_variant(Ctx* c, int algo) {
  static int env = -2;
  if (env == -2) {
    const char* s = getenv("CYTOM_SG_VARIANT");
    env = s ? atoi(s) : -1;
    if (env > kTilesVariant) env = -1;
  }
  int v = (env >= 0) ? env : c->sg_variant[(algo == CYTOM_ALGO_SSSP || algo == CYTOM_ALGO_SSWP) ? 1 : 0];
  if (v == kTilesVariant && !tiles_usable(c)) v = 0;
  return v;
}

// Whether the runs of program `algo` use the column-ordered tiles kernel (its stage list
// is built only then).
bool tiles_in_use(Ctx* c, int algo) { return gather_mode() != 0 && sg_variant(c, algo) == kTilesVariant; }

static GatherLaunch gather_launch(Ctx* c, int algo) {
  GatherLaunch g{};
  if (gather_mode() == 0) {
    g.fn = algo == CYTOM_ALGO_BFS    ? (void*)gather_minprop_kernel<0>
           : algo == CYTOM_ALGO_CC   ? (void*)gather_minprop_kernel<1>
           : algo == CYTOM_ALGO_SSWP ? (void*)gather_minprop_kernel<3>
                                     : (void*)gather_minprop_kernel<2>;
    g.grid = dim3(grid_persistent(c, 8));
    g.block = dim3(GATHER_T);
    g.smem = 0;
    return g;
  }
  const int a = algo == CYTOM_ALGO_BFS ? 0 : algo == CYTOM_ALGO_CC ? 1 : algo == CYTOM_ALGO_SSWP ? 3 : 2;
  return stream_launch(c, a, sg_variant(c, algo));
}

static int launch_gather(Ctx* c, Job* j, int adaptive) {
  GatherLaunch g = gather_launch(c, j->algo);
  const JobDesc* jd = j->d;
  const StoreDesc* sd = c->dsd;
  void* args[] = {(void*)&jd, (void*)&sd, (void*)&adaptive};
  cudaError_t e = cudaLaunchKernel(g.fn, g.grid, g.block, args, g.smem, c->stream);
  c->launches++;
  return cuda_err(c, e, "gather");
}

// One wave of resident blocks: grid = SMs x blocks of `fn` that fit on an SM at once
// (a larger grid runs in several waves, which costs a sparse round of a few microseconds
// of work one wave per extra set of blocks).
static int resident_grid(Ctx* c, void* fn, int threads) {
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, 0) != cudaSuccess || per_sm < 1) {
    cudaGetLastError();
    per_sm = 1;
  }
  return c->num_sms * per_sm;
}

static void* sparse_fn(int algo) {
  return algo == CYTOM_ALGO_BFS    ? (void*)gather_sparse_kernel<0>
         : algo == CYTOM_ALGO_CC   ? (void*)gather_sparse_kernel<1>
         : algo == CYTOM_ALGO_SSWP ? (void*)gather_sparse_kernel<3>
                                   : (void*)gather_sparse_kernel<2>;
}

static void* chunks_fn(int algo) {
  return algo == CYTOM_ALGO_BFS    ? (void*)gather_sparse_chunks<0>
         : algo == CYTOM_ALGO_CC   ? (void*)gather_sparse_chunks<1>
         : algo == CYTOM_ALGO_SSWP ? (void*)gather_sparse_chunks<3>
                                   : (void*)gather_sparse_chunks<2>;
}

static cudaError_t add_kernel(cudaGraph_t g, cudaGraphNode_t* node, const cudaGraphNode_t* deps,
                              size_t ndeps, void* fn, dim3 grid, dim3 block, void** args,
                              size_t smem = 0) {
  cudaKernelNodeParams kp{};
  kp.func = fn;
  kp.gridDim = grid;
  kp.blockDim = block;
  kp.sharedMemBytes = (unsigned)smem;
  kp.kernelParams = args;
  kp.extra = nullptr;
  return cudaGraphAddKernelNode(node, g, deps, ndeps, &kp);
}

// Graph: begin -> seeding apply + control -> while(cont) { dense gather -> sparse gather ->
// chunk pass -> apply + control }. Dense and sparse are picked on the device per round;
// the kernels not needed exit at once (measured cheaper than conditional IF nodes around
// them: 182-189 vs 166 GTEPS on the RMAT-22 stream).
static int build_minprop_graph(Ctx* c, Job* j) {
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaGraphCreate(&g, 0);
  if (e != cudaSuccess) return cuda_err(c, e, "graph create");
  cudaGraphConditionalHandle h;
  e = cudaGraphConditionalHandleCreate(&h, g, 0, cudaGraphCondAssignDefault);
  const JobDesc* jd = j->d;
  const StoreDesc* sd = c->dsd;
  unsigned max_iter = (unsigned)std::min<uint64_t>(j->params.max_iterations, 0xFFFFFFFFu);
  int adaptive = c->cfg.enable_adaptive_scheduling;
  int zero = 0, one = 1;
  const int g_apply = resident_grid(c, (void*)apply_minprop_kernel, APPLY_T);
  const int g_sparse = resident_grid(c, sparse_fn(j->algo), 256);
  const int g_chunks = resident_grid(c, chunks_fn(j->algo), 256);
  cudaGraphNode_t n_begin, n_apply0, n_while, b_apply, d_gather, s_sparse, c_chunks;
  void* a_begin[] = {(void*)&jd, (void*)&sd, (void*)&max_iter};
  if (e == cudaSuccess)
    e = add_kernel(g, &n_begin, nullptr, 0, (void*)begin_kernel, dim3(std::max(1, c->num_sms)), dim3(256), a_begin);
  void* a_apply0[] = {(void*)&jd, (void*)&sd, (void*)&one, (void*)&h, (void*)&one};
  if (e == cudaSuccess)
    e = add_kernel(g, &n_apply0, &n_begin, 1, (void*)apply_minprop_kernel, dim3(g_apply), dim3(APPLY_T), a_apply0);
  cudaGraphNodeParams cp{};
  cp.type = cudaGraphNodeTypeConditional;
  cp.conditional.handle = h;
  cp.conditional.type = cudaGraphCondTypeWhile;
  cp.conditional.size = 1;
  if (e == cudaSuccess) e = cudaGraphAddNode(&n_while, g, &n_apply0, nullptr, 1, &cp);
  if (e == cudaSuccess) {
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    void* a_g[] = {(void*)&jd, (void*)&sd, (void*)&adaptive};
    GatherLaunch gl = gather_launch(c, j->algo);
    e = add_kernel(body, &d_gather, nullptr, 0, gl.fn, gl.grid, gl.block, a_g, gl.smem);
    if (e == cudaSuccess)
      e = add_kernel(body, &s_sparse, &d_gather, 1, sparse_fn(j->algo), dim3(g_sparse), dim3(256), a_g);
    void* a_q[] = {(void*)&jd, (void*)&sd};
    if (e == cudaSuccess)
      e = add_kernel(body, &c_chunks, &s_sparse, 1, chunks_fn(j->algo), dim3(g_chunks), dim3(256), a_q);
    void* a_a[] = {(void*)&jd, (void*)&sd, (void*)&zero, (void*)&h, (void*)&one};
    if (e == cudaSuccess)
      e = add_kernel(body, &b_apply, &c_chunks, 1, (void*)apply_minprop_kernel, dim3(g_apply), dim3(APPLY_T), a_a);
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(&j->loop_exec, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) {
    cudaGetLastError();
    j->loop_exec = nullptr;
    j->graph_failed = true;
    return CYTOM_ERR_CUDA;
  }
  return CYTOM_OK;
}

static bool use_graphs() {
  static int v = -1;
  if (v < 0) {
    const char* s = getenv("CYTOM_NO_GRAPH");
    v = (s && s[0] == '1') ? 0 : 1;
  }
  return v == 1;
}

// Algorithmic bytes of one gather round, from the loop state before (`a`) and after
// (`b`) it: every scanned edge (+ its weight), one value per active source, a read and a
// reduction per changed target (bounded by the vertices the round activates), and the
// frontier: the whole bitmap for a dense round; for a sparse round the listed words
// (index, word and column mask) and, per (word, tile column) item that a source of the
// word reaches, its two directory entries and tile offset.
static double round_bytes(const Ctx* c, const LoopState& a, const LoopState& b, double wbytes) {
  const unsigned p = a.iter & 1u;
  const double scanned = (double)(b.edges_scanned - a.edges_scanned);
  const double act = (double)a.active[p];
  const double changed = (double)b.active[p ^ 1u];
  double bytes = scanned * (4.0 + wbytes) + act * 4.0 + changed * 8.0;
  if (a.mode == 0) bytes += (double)c->n / 8.0;
  else bytes += (double)a.nact_words[p] * 16.0 + (double)(b.items_read - a.items_read) * 16.0;
  return bytes;
}

int minprop_run(Ctx* c, Job* j) {
  int adaptive = c->cfg.enable_adaptive_scheduling;
  unsigned max_iter = (unsigned)std::min<uint64_t>(j->params.max_iterations, 0xFFFFFFFFu);
  if (!c->profiling && use_graphs() && !j->graph_failed) {
    if (j->loop_exec && j->graph_epoch != c->tune_epoch) {
      cudaGraphExecDestroy(j->loop_exec);
      j->loop_exec = nullptr;
    }
    if (!j->loop_exec) {
      build_minprop_graph(c, j);
      j->graph_epoch = c->tune_epoch;
    }
    if (j->loop_exec) {
      j->last_run_graph = true;
      cudaError_t e = cudaGraphLaunch(j->loop_exec, c->stream);
      c->launches += 2;  // per-round launches are counted from the loop state afterwards
      if (e != cudaSuccess) return cuda_err(c, e, "graph launch");
      return CYTOM_OK;
    }
  }
  // host-driven loop (profiling mode or no graph support)
  j->last_run_graph = false;
  const int g_apply = resident_grid(c, (void*)apply_minprop_kernel, APPLY_T);
  const int g_sparse = resident_grid(c, sparse_fn(j->algo), 256);
  const int g_chunks = resident_grid(c, chunks_fn(j->algo), 256);
  begin_kernel<<<std::max(1, c->num_sms), 256, 0, c->stream>>>(j->d, c->dsd, max_iter);
  apply_minprop_kernel<<<g_apply, APPLY_T, 0, c->stream>>>(j->d, c->dsd, 1, 0, 0);
  c->launches += 2;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_err(c, e, "run prologue");
  const JobDesc* jd = j->d;
  const StoreDesc* sd = c->dsd;
  void* a_g[] = {(void*)&jd, (void*)&sd, (void*)&adaptive};
  // profiling: the gather slot of the previous round and its loop-state snapshot; the
  // round's algorithmic bytes are known once the next snapshot is read
  int prev_slot = -1;
  LoopState prev{};
  const double wbytes = (j->algo == CYTOM_ALGO_SSSP || j->algo == CYTOM_ALGO_SSWP) ? 4.0 : 0.0;
  for (uint64_t round = 0; round < max_iter;) {
    if (c->profiling) {
      // one round at a time, only the gather the device chose, so per-launch times are clean
      LoopState snap;
      e = cudaMemcpyAsync(&snap, j->ls, sizeof(LoopState), cudaMemcpyDeviceToHost, c->stream);
      if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
      if (e != cudaSuccess) return cuda_err(c, e, "run loop");
      if (prev_slot >= 0) c->pending[prev_slot].bytes = round_bytes(c, prev, snap, wbytes);
      prev_slot = -1;
      if (!snap.cont) break;
      prev = snap;
      if (snap.mode == 0) {
        int s1 = prof_begin(c, KC_GATHER);
        int rc = launch_gather(c, j, adaptive);
        if (rc) return rc;
        prof_end(c, s1, 0.0);
        prev_slot = s1;
      } else {
        int s1 = prof_begin(c, KC_OTHER);
        e = cudaLaunchKernel(sparse_fn(j->algo), dim3(g_sparse), dim3(256), a_g, 0, c->stream);
        void* a_q[] = {(void*)&jd, (void*)&sd};
        if (e == cudaSuccess) e = cudaLaunchKernel(chunks_fn(j->algo), dim3(g_chunks), dim3(256), a_q, 0, c->stream);
        c->launches += 2;
        prof_end(c, s1, 0.0);
        prev_slot = s1;
        if (e != cudaSuccess) return cuda_err(c, e, "sparse gather");
      }
      int s2 = prof_begin(c, KC_APPLY);
      apply_minprop_kernel<<<g_apply, APPLY_T, 0, c->stream>>>(j->d, c->dsd, 0, 0, 0);
      prof_end(c, s2, -1.0);
      c->launches += 1;
      ++round;
      continue;
    }
    // launch a few rounds before checking: kernels are no-ops once the run ended
    for (int k = 0; k < 4 && round < max_iter; ++k, ++round) {
      int rc = launch_gather(c, j, adaptive);
      if (rc) return rc;
      e = cudaLaunchKernel(sparse_fn(j->algo), dim3(g_sparse), dim3(256), a_g, 0, c->stream);
      void* a_q[] = {(void*)&jd, (void*)&sd};
      if (e == cudaSuccess) e = cudaLaunchKernel(chunks_fn(j->algo), dim3(g_chunks), dim3(256), a_q, 0, c->stream);
      if (e != cudaSuccess) return cuda_err(c, e, "sparse gather");
      apply_minprop_kernel<<<g_apply, APPLY_T, 0, c->stream>>>(j->d, c->dsd, 0, 0, 0);
      c->launches += 3;
    }
    e = cudaMemcpyAsync(c->h_pinned, &j->ls->cont, 4, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_err(c, e, "run loop");
    if (*(unsigned*)c->h_pinned == 0) break;
  }
  if (prev_slot >= 0) {
    LoopState snap;
    e = cudaMemcpyAsync(&snap, j->ls, sizeof(LoopState), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_err(c, e, "run loop");
    c->pending[prev_slot].bytes = round_bytes(c, prev, snap, wbytes);
  }
  return CYTOM_OK;
}


// ---- autotuner ---------------------------------------------------------------
// Picks the streaming-gather shape (kSgVariants) per program class by timing every
// variant on the context's current graph: a scratch job in a representative dense
// state (current = next = vertex id, every other vertex active, every tile row active
// but not full, so each edge takes the frontier test and about half take the value
// path) runs one round per variant; next and changed are restored before every launch,
// so each variant sees identical input. Best of three launches per variant.
__global__ void tune_state_kernel(JobDesc* jd, const StoreDesc* __restrict__ sd, LoopState* ls, int full) {
  const uint64_t n = sd->n, nwords = (n + 31) >> 5, T = sd->T;
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  const uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  for (uint64_t v = tid; v < n; v += stride) {
    if (full) jd->cur[v] = (uint32_t)v;
    jd->next[v] = (uint32_t)v;
  }
  for (uint64_t i = tid; i < nwords; i += stride) {
    if (full) jd->fa[i] = 0x55555555u;
    jd->ch[i] = 0;
  }
  for (uint64_t x = tid; x < 2 * T; x += stride) jd->rows[x] = x < T ? 1u : 0u;
  if (tid == 0) {
    ls->iter = 0;
    ls->cont = 1;
    ls->mode = 0;
    ls->err = 0;
    ls->teps[0] = ls->teps[1] = 0;
  }
}

// Frontier of the sparse-threshold tuning: word i is non-zero with probability 1/div,
// with one vertex chosen by a hash of i; next = current = vertex id; a fresh loop state.
// The seeding apply (apply_minprop_kernel, initial) then lists the words and flags rows.
__global__ void tune_frontier_kernel(JobDesc* jd, const StoreDesc* __restrict__ sd, LoopState* ls, uint32_t div) {
  const uint64_t n = sd->n, nwords = (n + 31) >> 5, T = sd->T;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  const uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  for (uint64_t v = tid; v < n; v += stride) {
    jd->cur[v] = (uint32_t)v;
    jd->next[v] = (uint32_t)v;
  }
  for (uint64_t i = tid; i < nwords; i += stride) {
    uint32_t h = (uint32_t)i * 0x9E3779B9u + 0x7F4A7C15u;
    h ^= h >> 15;
    h *= 0x2C1B3C6Du;
    h ^= h >> 12;
    jd->ch[i] = (h % div == 0) ? (1u << ((h >> 20) & 31u)) : 0u;
  }
  for (uint64_t x = tid; x < 2 * T; x += stride) jd->rows[x] = 0;
  if (tid == 0) {
    ls->iter = 0;
    ls->max_iter = 1000;
    ls->cont = 1;
    ls->err = 0;
    ls->active[0] = ls->active[1] = 0;
    ls->nact_words[0] = ls->nact_words[1] = 0;
    ls->teps[0] = ls->teps[1] = 0;
    ls->spq_count = 0;
    ls->apply_done = 0;
    ls->sel_rounds = 0;
  }
}

__global__ void tune_mode_kernel(LoopState* ls, unsigned mode) {
  ls->mode = mode;
  ls->cont = 1;
  ls->spq_count = 0;
}

static const uint32_t kDivCandidates[6] = {128, 64, 32, 16, 8, 4};

static bool sparse_div_from_env() {
  static int v = -1;
  if (v < 0) v = getenv("CYTOM_SPARSE_DIV") ? 1 : 0;
  return v == 1;
}

int minprop_autotune(Ctx* c) {
  int brc = build_directory(c);
  if (!brc) brc = build_tile_stages(c);
  if (brc) return brc;
  const uint64_t n = c->n, nwords = (n + 31) / 32;
  JobDesc h{};
  LoopState* ls = nullptr;
  JobDesc* d = nullptr;
  char* buf = nullptr;
  const uint64_t qcap = c->E / 32 + c->E / 256 + 1024;
  const size_t bytes = n * 8 + nwords * 8 + 2 * c->T * 4 + nwords * 12 + sizeof(LoopState) + sizeof(JobDesc) +
                       qcap * sizeof(uint2) + 9 * 256;
  if (cy_malloc_async((void**)&buf, bytes, c->stream) != cudaSuccess) {
    cudaGetLastError();
    return CYTOM_OK;  // no memory to tune with: keep the current shapes
  }
  char* q = buf;
  auto take = [&](size_t b) {
    char* r = q;
    q += (b + 255) & ~(size_t)255;
    return r;
  };
  h.cur = (uint32_t*)take(n * 4);
  h.next = (uint32_t*)take(n * 4);
  h.fa = (uint32_t*)take(nwords * 4);
  h.ch = (uint32_t*)take(nwords * 4);
  h.rows = (uint32_t*)take(2 * c->T * 4);
  h.aw = (uint32_t*)take(nwords * 4);
  h.awm = (unsigned long long*)take(nwords * 8);
  ls = (LoopState*)take(sizeof(LoopState));
  d = (JobDesc*)take(sizeof(JobDesc));
  h.spq = (uint2*)take(qcap * sizeof(uint2));
  h.spq_cap = qcap;
  h.ls = ls;
  cudaMemsetAsync(ls, 0, sizeof(LoopState), c->stream);
  cudaMemcpyAsync(d, &h, sizeof(JobDesc), cudaMemcpyHostToDevice, c->stream);
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  int adaptive = 1;
  const StoreDesc* sd = c->dsd;
  const JobDesc* jd = d;
  void* args[] = {(void*)&jd, (void*)&sd, (void*)&adaptive};
  const int classes = c->wtype == CYTOM_WEIGHT_U32 ? 2 : 1;
  cudaError_t e = cudaSuccess;
  for (int cls = 0; cls < classes && e == cudaSuccess; ++cls) {
    const int algo = cls == 0 ? 1 : 2;
    int best = 0;
    double best_us = 1e300;
    const int nvar = kSgVariantCount + (tiles_usable(c) ? 1 : 0);
    for (int v = 0; v < nvar && e == cudaSuccess; ++v) {
      GatherLaunch g = stream_launch(c, algo, v);
      double vbest = 1e300;
      for (int rep = 0; rep < 3 && e == cudaSuccess; ++rep) {
        tune_state_kernel<<<grid_persistent(c, 4), 256, 0, c->stream>>>(d, sd, ls, rep == 0 && v == 0 ? 1 : 0);
        cudaEventRecord(a, c->stream);
        e = cudaLaunchKernel(g.fn, g.grid, g.block, args, g.smem, c->stream);
        cudaEventRecord(b, c->stream);
        if (e == cudaSuccess) e = cudaEventSynchronize(b);
        float ms = 0.f;
        if (e == cudaSuccess) cudaEventElapsedTime(&ms, a, b);
        vbest = std::min(vbest, (double)ms * 1e3);
        c->launches += 2;
      }
      c->tune_us[cls][v] = vbest;
      if (vbest < best_us) {
        best_us = vbest;
        best = v;
      }
    }
    if (e == cudaSuccess) c->sg_variant[cls] = best;
    // sparse-round threshold of this class: dense (the chosen kernel) against sparse
    // (directory walk + chunk pass) rounds on frontiers of growing density
    c->tune_div[cls] = 0;
    if (e == cudaSuccess && c->hsd.dir_ok && c->cfg.enable_adaptive_scheduling && !sparse_div_from_env()) {
      GatherLaunch gd = stream_launch(c, algo, best);
      const int g_apply = resident_grid(c, (void*)apply_minprop_kernel, APPLY_T);
      const int g_sparse = resident_grid(c, sparse_fn(algo), 256);
      const int g_chunks = resident_grid(c, chunks_fn(algo), 256);
      void* a_q[] = {(void*)&jd, (void*)&sd};
      uint32_t div = 0;
      bool losing = false;
      for (int k = 0; k < 6 && e == cudaSuccess; ++k) {
        double t_mode[2] = {1e300, 1e300};
        for (unsigned mode = 0; mode < 2 && e == cudaSuccess; ++mode) {
          for (int rep = 0; rep < 2 && e == cudaSuccess; ++rep) {
            tune_frontier_kernel<<<grid_persistent(c, 4), 256, 0, c->stream>>>(d, sd, ls, kDivCandidates[k]);
            apply_minprop_kernel<<<g_apply, APPLY_T, 0, c->stream>>>(d, sd, 1, 0, 0);
            tune_mode_kernel<<<1, 1, 0, c->stream>>>(ls, mode);
            cudaEventRecord(a, c->stream);
            if (mode == 0) {
              e = cudaLaunchKernel(gd.fn, gd.grid, gd.block, args, gd.smem, c->stream);
            } else {
              e = cudaLaunchKernel(sparse_fn(algo), dim3(g_sparse), dim3(256), args, 0, c->stream);
              if (e == cudaSuccess) e = cudaLaunchKernel(chunks_fn(algo), dim3(g_chunks), dim3(256), a_q, 0, c->stream);
            }
            cudaEventRecord(b, c->stream);
            if (e == cudaSuccess) e = cudaEventSynchronize(b);
            float ms = 0.f;
            if (e == cudaSuccess) cudaEventElapsedTime(&ms, a, b);
            t_mode[mode] = std::min(t_mode[mode], (double)ms * 1e3);
            c->launches += 5;
          }
        }
        c->tune_dense_us[cls][k] = t_mode[0];
        c->tune_sparse_us[cls][k] = t_mode[1];
        if (!losing && t_mode[1] < t_mode[0]) div = kDivCandidates[k];
        else losing = true;
      }
      if (e == cudaSuccess) c->tune_div[cls] = div ? div : 1024;
    }
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFreeAsync(buf, c->stream);
  if (e != cudaSuccess) return cuda_err(c, e, "autotune");
  c->tune_E = c->E;
  c->tune_epoch++;
  return cuda_err(c, cudaStreamSynchronize(c->stream), "autotune");
}


void sg_shapes(int* ept, int* nst, int* minb, int* count) {
  *count = kSgVariantCount + 1;
  for (int v = 0; v < kSgVariantCount; ++v) {
    ept[v] = kSgVariants[v].ept;
    nst[v] = kSgVariants[v].nst;
    minb[v] = kSgVariants[v].minb;
  }
  // the column-ordered tiles kernel: 8 edges per thread of 512, 3-deep pipeline, 1 block per SM
  ept[kTilesVariant] = 8;
  nst[kTilesVariant] = TS_NST;
  minb[kTilesVariant] = 1;
}

}  // namespace cytom
