// minprop_dev.cuh — device building blocks of one BFS / CC / SSSP round, shared by the
// one-job kernels (exec_minprop.cu) and the batched persistent executor (exec_batch.cu),
// so both compute the same round with the same arithmetic.
//
// The round is the reference's Jacobi round (src/include/core/continuous-algorithm-executor.h:72-218):
//   gather  — AlgorithmExecutor::executeTile / executeAlgorithmSingleEdge[Weighted]
//             (src/include/core/algorithm-executor.h:214-505): every edge whose source is
//             active relaxes next[tgt] from current[src];
//   apply   — ApplyExecutor::run (src/include/core/apply-executor.h:40-115): changed
//             vertices copy next into current and form the next frontier;
//   control — the convergence test and the swap of the active bitmaps
//             (continuous-algorithm-executor.h:193-218).
//
// Load policy: the one-job kernels read state written by earlier launches through the
// read-only path (PERSIST = false). The persistent kernel writes that state in the same
// launch on other SMs, so it reads every mutable word through L2 (PERSIST = true);
// the L1 of an SM is not coherent with stores of other SMs within a launch.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "engine.h"
#include "ptx.cuh"

namespace cytom {

constexpr int APPLY_T = 256;
constexpr int SG_T = 256;     // threads of a dense-stage block
constexpr int SG_E = 4096;    // edges per dense stage
static_assert(SG_E == SG_T * 16, "16 edges per thread per stage");

// Loads of data that a launch may have written (current values, frontier, changed bits,
// row flags): read-only cache path across launches, L2 within a persistent launch.
template <bool PERSIST, class T>
__device__ __forceinline__ T ld_state(const T* p) {
  if constexpr (PERSIST) return __ldcg(p);
  else return __ldg(p);
}
// The same for words that the one-job kernels also read with plain loads.
template <bool PERSIST, class T>
__device__ __forceinline__ T ld_plain(const T* p) {
  if constexpr (PERSIST) return __ldcg(p);
  else return *p;
}

// Programs: ALGO 0 BFS, 1 CC, 2 SSSP, 3 SSWP. SSWP runs on complemented values (v' = ~v),
// which turns its max(v, min(u, w)) into the same min-propagation as the others:
// v' = min(v', max(u', ~w)); unreached (0) is kInf, the start (UINT32_MAX) is 0.
template <int ALGO>
__host__ __device__ constexpr bool mp_weighted() {
  return ALGO >= 2;
}
// The value an edge offers its target from source value c (c != kInf) and weight w.
template <int ALGO>
__device__ __forceinline__ uint32_t mp_cand(uint32_t c, uint32_t w) {
  if (ALGO == 0) return c + 1;
  if (ALGO == 1) return c;
  if (ALGO == 2) {
    const uint32_t sum = c + w;  // c < kInf; a carry out or kInf itself means unreachable
    return (sum < c || sum == kInf) ? kInf : sum;
  }
  return max(c, ~w);
}

// Pre-check of a target's next value before the reduction, through L2. (Any value read
// would do: next only decreases during a round and never exceeds current. Reading the
// one-job kernels' pre-checks through L1 instead measured 2-3 % slower on the RMAT-22
// stream's dense SSSP rounds.)
template <bool PERSIST>
__device__ __forceinline__ uint32_t ld_next(const uint32_t* p) {
  return __ldcg(p);
}

// Source value of a gather. The asynchronous programs (examples/bfs-async.cc,
// cc-async.cc: ASYNC = true) pull from next[src], which other blocks lower during the
// round (algorithm-executor.h:303-312); read through L2, a value is either the one at
// the round's start or a lower one, and both are valid bounds.
template <bool PERSIST>
__device__ __forceinline__ uint32_t ld_src(const JobDesc* __restrict__ jd, bool async, uint64_t u) {
  if (async) return __ldcg(jd->next + u);
  return ld_state<PERSIST>(jd->cur + u);
}

__device__ __forceinline__ unsigned long long row_edges(const StoreDesc* sd, uint64_t x) {
  return sd->tile_ptr[(x + 1) << sd->lT] - sd->tile_ptr[x << sd->lT];
}

// Opening of gather round p: clears the next parity's row flags (threads tid, tid+nthr,
// ...) and, on thread 0, the next parity's counters; adds the round's processed-edge
// count (edges of tile rows with an active source, algorithm-executor.h:424-426).
template <bool PERSIST>
__device__ __forceinline__ void round_open(const JobDesc* __restrict__ jd, const StoreDesc* __restrict__ sd,
                                           unsigned p, int adaptive, uint64_t tid, uint64_t nthr) {
  LoopState* ls = jd->ls;
  const uint64_t T = sd->T;
  unsigned* rows_nxt = jd->rows + (p ^ 1u) * T;
  for (uint64_t i = tid; i < T; i += nthr) rows_nxt[i] = 0;
  if (tid == 0) {
    ls->active[p ^ 1u] = 0;
    ls->nact_words[p ^ 1u] = 0;
    ls->teps[p ^ 1u] = 0;
    atomicAdd(&ls->count_edges, adaptive ? ld_plain<PERSIST>(&ls->teps[p]) : sd->E);
  }
}

// Tile columns in which the active sources of frontier word i (bits w) may have edges:
// the OR of their column masks, read for words with at most four active sources (the
// sparse rounds' words hold about one); all columns for denser words or without masks.
__device__ __forceinline__ unsigned long long word_columns(const StoreDesc* __restrict__ sd, uint64_t i,
                                                           uint32_t w) {
  const unsigned long long* cm = sd->cmask;
  if (!cm || __popc(w) > 4) return ~0ULL;
  unsigned long long m = 0;
  const unsigned long long* row = cm + (i << 5);
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    if (w) {
      m |= row[__ffs(w) - 1];
      w &= w - 1;
    }
  }
  return m;
}

// ---- apply ---------------------------------------------------------------
// One apply step of a block: thread t handles frontier word base + t (base a multiple
// of 32). `initial` apply = the seeding apply before round 0 (writes parity 0).
// rows[parity][x] receives the number of vertices of tile row x that are active in
// the next round (0 = the row is skipped; vpt = every source active, the frontier
// test is skipped). A warp covers 32 consecutive words; when they share one row
// (vpt >= 1024) it adds its row count with a single atomic. The non-zero frontier
// words are listed (warp-ballot compaction) for sparse rounds.
template <bool PERSIST>
__device__ __forceinline__ void apply_step(const JobDesc* __restrict__ jd, const StoreDesc* __restrict__ sd,
                                           unsigned pw, uint64_t base, unsigned& cnt, unsigned long long& teps) {
  LoopState* ls = jd->ls;
  const uint64_t n = sd->n, T = sd->T;
  const uint32_t lvpt = sd->lvpt;
  const uint64_t nwords = (n + 31) >> 5;
  unsigned* rows_w = jd->rows + pw * T;
  uint32_t* __restrict__ ch = jd->ch;
  uint32_t* __restrict__ fa = jd->fa;
  uint32_t* __restrict__ cur = jd->cur;
  const uint32_t* __restrict__ next = jd->next;
  const unsigned lane = threadIdx.x & 31;
  const uint64_t i = base + threadIdx.x;
  uint32_t w = 0;
  if (i < nwords) {
    w = ld_plain<PERSIST>(ch + i);
    fa[i] = w;
    if (w) {
      ch[i] = 0;
      if (!PERSIST && __popc(w) > 2 && ((i + 1) << 5) <= n) {
        // many changed vertices: the whole word's 32 values in one round trip. A vertex
        // without its changed bit holds next == current (every lowering of next sets
        // the bit), so copying it is a no-op. (Not in the persistent kernel, whose
        // register budget would spill the eight vectors.)
        const uint4* src = reinterpret_cast<const uint4*>(next + (i << 5));
        uint4* dst = reinterpret_cast<uint4*>(cur + (i << 5));
        uint4 q[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) q[k] = ld_plain<PERSIST>(src + k);
#pragma unroll
        for (int k = 0; k < 8; ++k) dst[k] = q[k];
      } else {
        uint32_t bits = w;
        while (bits) {
          const int b = __ffs(bits) - 1;
          bits &= bits - 1;
          const uint64_t v = (i << 5) + b;
          cur[v] = ld_plain<PERSIST>(next + v);
        }
      }
    }
  }
  const unsigned pc = __popc(w);
  cnt += pc;
  {
    const unsigned nz = __ballot_sync(0xFFFFFFFFu, w != 0);
    if (nz) {
      unsigned slot0 = 0;
      if (lane == 0) slot0 = atomicAdd(&ls->nact_words[pw], (unsigned)__popc(nz));
      slot0 = __shfl_sync(0xFFFFFFFFu, slot0, 0);
      if (w) {
        const unsigned slot = slot0 + __popc(nz & ((1u << lane) - 1u));
        jd->aw[slot] = (uint32_t)i;
        jd->awm[slot] = word_columns(sd, i, w);
      }
    }
  }
  if (lvpt >= 10) {
    unsigned tot = pc;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) tot += __shfl_xor_sync(0xFFFFFFFFu, tot, o);
    if (lane == 0 && tot) {
      const uint64_t x = ((base + (threadIdx.x & ~31u)) << 5) >> lvpt;
      if (atomicAdd(&rows_w[x], tot) == 0) teps += row_edges(sd, x);
    }
  } else if (w) {
    uint32_t bits = w;
    while (bits) {
      const int b = __ffs(bits) - 1;
      const uint64_t v = (i << 5) + b;
      const uint64_t x = v >> lvpt;
      const uint64_t row_first = x << lvpt;
      const uint64_t row_last = row_first + (1ULL << lvpt);  // exclusive
      uint32_t mrow = bits;
      if (row_last < ((i + 1) << 5)) mrow &= (1u << (uint32_t)(row_last - (i << 5))) - 1u;
      bits &= ~mrow;
      if (atomicAdd(&rows_w[x], (unsigned)__popc(mrow)) == 0) teps += row_edges(sd, x);
    }
  }
}

// Block reduction of the apply counters into the loop state (every thread calls it).
__device__ __forceinline__ void apply_flush(LoopState* ls, unsigned pw, unsigned cnt, unsigned long long teps) {
  __shared__ unsigned s_cnt[APPLY_T / 32];
  __shared__ unsigned long long s_teps[APPLY_T / 32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    cnt += __shfl_xor_sync(0xFFFFFFFFu, cnt, o);
    teps += __shfl_xor_sync(0xFFFFFFFFu, teps, o);
  }
  const unsigned wid = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) {
    s_cnt[wid] = cnt;
    s_teps[wid] = teps;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned c = 0;
    unsigned long long t = 0;
    for (int k = 0; k < APPLY_T / 32; ++k) {
      c += s_cnt[k];
      t += s_teps[k];
    }
    if (c) atomicAdd(&ls->active[pw], c);
    if (t) atomicAdd(&ls->teps[pw], t);
  }
  __syncthreads();
}

// ---- control -------------------------------------------------------------
// Ends a round (or, `initial`, the seeding apply): advances the round counter, ends the
// run when nothing changed or max_iterations rounds ran, and picks the next round's
// gather: sparse (directory, only the listed frontier words) while at most 1/sparse_div
// of the frontier words are non-zero, dense (stream every active row) above.
__device__ __forceinline__ unsigned control_step(const JobDesc* __restrict__ jd, const StoreDesc* __restrict__ sd,
                                                 int initial) {
  volatile LoopState* ls = jd->ls;
  if (ls->cont) {
    unsigned iter = ls->iter;
    unsigned p = 0;
    if (!initial) {
      iter += 1;
      ls->iter = iter;
      p = iter & 1u;
    }
    const unsigned a = ls->active[p];
    ls->active_total = ls->active_total + a;
    ls->cont = (a > 0 && iter < ls->max_iter && ls->err == 0) ? 1u : 0u;
    const uint64_t nwords = (sd->n + 31) >> 5;
    const uint32_t div = jd->sparse_div ? jd->sparse_div : sd->sparse_div;
    ls->mode = (sd->dir_ok && sd->adaptive && (uint64_t)ls->nact_words[p] * div <= nwords) ? 1u : 0u;
    ls->spq_count = 0;
  }
  return ls->cont;
}

// The loop state of a BFS / CC / SSSP / SSWP run before its first round (one thread).
__device__ __forceinline__ void minprop_begin_state(LoopState* ls, unsigned max_iter) {
  ls->iter = 0;
  ls->max_iter = max_iter;
  ls->cont = 1;
  ls->err = 0;
  ls->active[0] = ls->active[1] = 0;
  ls->nact_words[0] = ls->nact_words[1] = 0;
  ls->mode = 0;
  ls->spq_count = 0;
  ls->teps[0] = ls->teps[1] = 0;
  ls->count_edges = 0;
  ls->edges_scanned = 0;
  ls->active_total = 0;
  ls->apply_done = 0;
  ls->sel_rounds = 0;
  ls->items_read = 0;
}

// ---- dense gather: one stage of SG_T * EPT edges ---------------------------
// Processes stage `st` (EPT edges per thread, a multiple of 4) whose edges (and weights) are at eb / wb: shared memory for the
// bulk-copy pipeline, global memory (FROM_GLOBAL, guarded loads) for the persistent
// kernel. Single-row stages (the common case at large vertices-per-tile) take the source
// row from the stage: the frontier test needs no per-edge tile lookup, and only edges
// with an active source look up their target tile. Target updates are fire-and-forget
// red.min / red.or: a candidate below the value read is below current[v] too
// (next <= current), so next[v] ends the round below current[v] and v changed.
template <int ALGO, bool PERSIST, bool FROM_GLOBAL, int EPT = 16>
__device__ __forceinline__ void dense_stage(const JobDesc* __restrict__ jd, const StoreDesc* __restrict__ sd,
                                            const uint32_t* eb, const uint32_t* wb, uint64_t st, unsigned p,
                                            int adaptive) {
  const uint64_t T = sd->T;
  const unsigned* rows_cur = jd->rows + p * T;
  const uint32_t* __restrict__ chunk_tile = sd->chunk_tile;
  const unsigned long long* __restrict__ tile_ptr = sd->tile_ptr;
  const uint32_t* fa = jd->fa;
  const bool async = jd->async != 0;
  uint32_t* next = jd->next;
  uint32_t* ch = jd->ch;
  const uint64_t E = sd->E, nchunks = sd->nchunks;
  const uint32_t lT = sd->lT, lvpt = sd->lvpt;
  const uint32_t ymask = (uint32_t)(T - 1);
  constexpr uint32_t SE = SG_T * EPT;  // edges of a stage
  static_assert(EPT % 4 == 0 && EPT <= 32 && SE % kChunk == 0, "stage shape");
  const uint64_t e0 = st * SE;
  const uint64_t rem = E - e0;
  const uint32_t cnt = rem < (uint64_t)SE ? (uint32_t)rem : SE;
  // tiles of the stage's first edge and of the first edge after it
  uint32_t tf, ta;
  {
    const uint64_t c0 = st * (SE / kChunk);
    uint64_t c1 = c0 + SE / kChunk;
    if (c1 > nchunks) c1 = nchunks;
    tf = chunk_tile[c0];
    ta = chunk_tile[c1];
  }
  const bool single_row = (tf >> lT) == (ta >> lT);
  const bool single_tile = tf == ta;
  const uint32_t vpt = 1u << lvpt;
  // a fully active row needs no frontier test
  const bool full_row = single_row && (!adaptive || ld_plain<PERSIST>(rows_cur + (tf >> lT)) == vpt);

  uint32_t qv[EPT], ww[EPT], uu[EPT];
  uint32_t vmask = 0;
#pragma unroll
  for (int k = 0; k < EPT / 4; ++k) {
    const uint32_t i0 = threadIdx.x * 4 + (uint32_t)k * (SG_T * 4);
    uint4 q, wq = make_uint4(0, 0, 0, 0);
    if (!FROM_GLOBAL || i0 + 4 <= cnt) {
      q = *reinterpret_cast<const uint4*>(eb + i0);
      if (mp_weighted<ALGO>()) wq = *reinterpret_cast<const uint4*>(wb + i0);
    } else {
      q.x = i0 < cnt ? eb[i0] : 0u;
      q.y = i0 + 1 < cnt ? eb[i0 + 1] : 0u;
      q.z = i0 + 2 < cnt ? eb[i0 + 2] : 0u;
      q.w = 0u;
      if (mp_weighted<ALGO>()) {
        wq.x = i0 < cnt ? wb[i0] : 0u;
        wq.y = i0 + 1 < cnt ? wb[i0 + 1] : 0u;
        wq.z = i0 + 2 < cnt ? wb[i0 + 2] : 0u;
      }
    }
    qv[4 * k + 0] = q.x;
    qv[4 * k + 1] = q.y;
    qv[4 * k + 2] = q.z;
    qv[4 * k + 3] = q.w;
    ww[4 * k + 0] = wq.x;
    ww[4 * k + 1] = wq.y;
    ww[4 * k + 2] = wq.z;
    ww[4 * k + 3] = wq.w;
    if (cnt != SE) {
#pragma unroll
      for (int j = 0; j < 4; ++j) vmask |= ((i0 + j) < cnt) ? (1u << (4 * k + j)) : 0u;
    }
  }
  if (cnt == SE) vmask = (EPT == 32) ? 0xFFFFFFFFu : ((1u << EPT) - 1u);  // a full stage
  if (single_row) {
    const uint32_t xb = (tf >> lT) << lvpt;
#pragma unroll
    for (int idx = 0; idx < EPT; ++idx) uu[idx] = xb | (qv[idx] >> 16);
  } else {
    // general path: per-edge tile lookup for the source row
#pragma unroll
    for (int k = 0; k < EPT / 4; ++k) {
      const uint32_t i0 = threadIdx.x * 4 + (uint32_t)k * (SG_T * 4);
      const uint64_t eg = e0 + i0;
      uint32_t t = 0;
      unsigned long long tend = 0;
      if (i0 < cnt) {
        t = chunk_tile[eg >> 7];
        tend = tile_ptr[t + 1];
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int idx = 4 * k + j;
        if ((vmask >> idx) & 1u) {
          while (tend <= eg + j) {
            ++t;
            tend = tile_ptr[t + 1];
          }
          const uint32_t x = t >> lT;
          uu[idx] = (x << lvpt) | (qv[idx] >> 16);
          if (adaptive && ld_plain<PERSIST>(rows_cur + x) == 0) vmask &= ~(1u << idx);
        } else {
          uu[idx] = 0;
        }
      }
    }
  }
  uint32_t amask = vmask;
  if (adaptive && !full_row) {
    uint32_t fw[EPT];
#pragma unroll
    for (int idx = 0; idx < EPT; ++idx) fw[idx] = ((vmask >> idx) & 1u) ? ld_state<PERSIST>(fa + (uu[idx] >> 5)) : 0u;
    amask = 0;
#pragma unroll
    for (int idx = 0; idx < EPT; ++idx) amask |= ((fw[idx] >> (uu[idx] & 31)) & 1u) << idx;
    amask &= vmask;
  }
  if (amask) {
    uint32_t cand[EPT], vv[EPT];
#pragma unroll
    for (int idx = 0; idx < EPT; ++idx) cand[idx] = ((amask >> idx) & 1u) ? ld_src<PERSIST>(jd, async, uu[idx]) : kInf;
    if (single_tile) {
      const uint32_t yb = (tf & ymask) << lvpt;
#pragma unroll
      for (int idx = 0; idx < EPT; ++idx) vv[idx] = yb | (qv[idx] & 0xFFFFu);
    } else {
      // target tiles of the edges with an active source
#pragma unroll
      for (int k = 0; k < EPT / 4; ++k) {
        const uint32_t i0 = threadIdx.x * 4 + (uint32_t)k * (SG_T * 4);
        const uint64_t eg = e0 + i0;
        const uint32_t kmask = (amask >> (4 * k)) & 0xFu;
        uint32_t t = 0;
        unsigned long long tend = 0;
        if (kmask) {
          t = chunk_tile[eg >> 7];
          tend = tile_ptr[t + 1];
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const int idx = 4 * k + j;
          vv[idx] = 0;
          if ((kmask >> j) & 1u) {
            while (tend <= eg + j) {
              ++t;
              tend = tile_ptr[t + 1];
            }
            vv[idx] = ((t & ymask) << lvpt) | (qv[idx] & 0xFFFFu);
          }
        }
      }
    }
#pragma unroll
    for (int idx = 0; idx < EPT; ++idx)
      if (cand[idx] != kInf) cand[idx] = mp_cand<ALGO>(cand[idx], ww[idx]);
    uint32_t nv[EPT];
#pragma unroll
    for (int idx = 0; idx < EPT; ++idx) nv[idx] = (cand[idx] != kInf) ? ld_next<PERSIST>(next + vv[idx]) : 0u;
#pragma unroll
    for (int idx = 0; idx < EPT; ++idx)
      if (cand[idx] != kInf && cand[idx] < nv[idx]) atomicMin(next + vv[idx], cand[idx]);
#pragma unroll
    for (int idx = 0; idx < EPT; ++idx)
      if (cand[idx] != kInf && cand[idx] < nv[idx]) atomicOr(ch + (vv[idx] >> 5), 1u << (vv[idx] & 31));
  }
}

// Whether stage st holds an edge of an active tile row (adaptive scheduling).
template <bool PERSIST, int EPT = 16>
__device__ __forceinline__ bool stage_active(const JobDesc* __restrict__ jd, const StoreDesc* __restrict__ sd,
                                             uint64_t st, unsigned p, int adaptive) {
  if (!adaptive) return true;
  const unsigned* rows_cur = jd->rows + p * sd->T;
  const uint64_t nchunks = sd->nchunks;
  constexpr uint32_t SE = SG_T * EPT;
  const uint64_t c0 = st * (SE / kChunk);
  uint64_t c1 = c0 + SE / kChunk;
  if (c1 > nchunks) c1 = nchunks;
  const uint32_t x0 = sd->chunk_tile[c0] >> sd->lT;
  const uint32_t x1 = sd->chunk_tile[c1] >> sd->lT;
  for (uint32_t x = x0; x <= x1; ++x)
    if (ld_plain<PERSIST>(rows_cur + x)) return true;
  return false;
}

// ---- sparse gather -------------------------------------------------------
// Sparse gather: the round restricted to the edges of the listed non-zero frontier
// words. Work item = (frontier word, tile column y); the source directory gives the
// item's edge range inside tile (x, y), x being the word's tile row. A warp takes 32
// consecutive items (consecutive y of one word) and walks the light items' edges with
// all 32 lanes. Items longer than SP_HEAVY edges, and, when the 32 items of a warp hold
// more than SP_WARP_MAX edges in total, every item longer than SP_LIGHT, are cut into
// SP_CHUNK-edge chunks queued for the chunk pass, so no warp is left with more than
// about SP_WARP_MAX edges of light items or one chunk per queue entry (RMAT hub blocks).
constexpr uint32_t SP_HEAVY = 256;
constexpr uint32_t SP_CHUNK = 256;
constexpr uint32_t SP_LIGHT = 32;
constexpr uint32_t SP_WARP_MAX = 2048;
// Every light item is first narrowed to the edges of its word's active sources
// (sp_narrow). Streaming RMAT-22 by the shortest item narrowed: none 307.6 GTEPS, 64
// edges 313.8, 16 edges 326.7, 4 edges 326-329, every item 335.7; narrowing heavy items
// as well (up to 1,024 / 8,192 / all edges) gained nothing over the chunk pass's own
// skip of inactive chunks.
constexpr uint32_t SP_NARROW = 0;
constexpr int SP_ILP = 8;

struct SpItem {
  uint32_t x, y, bits, lo, hi, b;  // b: the word's 32-source block in its tile row
  unsigned long long base;
};

// Item (word w, tile column y): its frontier bits, directory range and tile base.
template <bool PERSIST>
__device__ __forceinline__ SpItem sp_item_at(const JobDesc* __restrict__ jd, const StoreDesc* __restrict__ sd,
                                             uint32_t w, uint32_t y) {
  const uint32_t lT = sd->lT, lnbw = sd->lvpt - 5, nbw = sd->nbw;
  SpItem r;
  r.y = y;
  r.x = w >> lnbw;
  const uint32_t b = w & (nbw - 1);
  r.b = b;
  r.bits = ld_state<PERSIST>(jd->fa + w);
  const uint64_t dbase = (((uint64_t)r.x << lT) + r.y) * (nbw + 1) + b;
  r.lo = sd->dir[dbase];
  r.hi = sd->dir[dbase + 1];
  r.base = sd->tile_ptr[((uint64_t)r.x << lT) | r.y];
  return r;
}

template <bool PERSIST>
__device__ __forceinline__ SpItem sp_item(const JobDesc* __restrict__ jd, const StoreDesc* __restrict__ sd,
                                          uint64_t it) {
  const uint32_t w = ld_plain<PERSIST>(jd->aw + (it >> sd->lT));
  return sp_item_at<PERSIST>(jd, sd, w, (uint32_t)(it & (sd->T - 1)));
}

// Relaxes SP_ILP edges per lane whose sources are in their item's frontier word; the
// loads of all SP_ILP edges are issued before any of them is used.
template <int ALGO, bool PERSIST>
__device__ __forceinline__ void sp_batch(const JobDesc* __restrict__ jd, const StoreDesc* __restrict__ sd,
                                         const uint32_t (&xs)[SP_ILP], const uint32_t (&ys)[SP_ILP],
                                         const uint32_t (&bits)[SP_ILP], const unsigned long long (&pos)[SP_ILP],
                                         uint32_t valid) {
  const uint32_t lvpt = sd->lvpt;
  const bool async = jd->async != 0;
  uint32_t pk[SP_ILP], wv[SP_ILP], cand[SP_ILP], nv[SP_ILP];
#pragma unroll
  for (int k = 0; k < SP_ILP; ++k) pk[k] = ((valid >> k) & 1u) ? sd->edges[pos[k]] : 0u;
  // the weight is read only for an edge whose source is in the frontier, beside its
  // source value (one dependent step, as before; most listed edges have inactive sources)
#pragma unroll
  for (int k = 0; k < SP_ILP; ++k) {
    const uint32_t sl = pk[k] >> 16;
    const bool act = ((valid >> k) & 1u) && ((bits[k] >> (sl & 31)) & 1u);
    cand[k] = act ? ld_src<PERSIST>(jd, async, (xs[k] << lvpt) | sl) : kInf;
    wv[k] = (mp_weighted<ALGO>() && act) ? sd->wts[pos[k]] : 0u;
  }
#pragma unroll
  for (int k = 0; k < SP_ILP; ++k)
    if (cand[k] != kInf) cand[k] = mp_cand<ALGO>(cand[k], wv[k]);
#pragma unroll
  for (int k = 0; k < SP_ILP; ++k)
    nv[k] = (cand[k] != kInf) ? ld_next<PERSIST>(jd->next + ((ys[k] << lvpt) | (pk[k] & 0xFFFFu))) : 0u;
#pragma unroll
  for (int k = 0; k < SP_ILP; ++k) {
    if (cand[k] != kInf && cand[k] < nv[k]) {
      const uint32_t v = (ys[k] << lvpt) | (pk[k] & 0xFFFFu);
      atomicMin(jd->next + v, cand[k]);
      atomicOr(jd->ch + (v >> 5), 1u << (v & 31));
    }
  }
}

// Narrows item m to the edges whose sources lie between the lowest and the highest
// active source of its word: an item's edges are sorted by (source, target) and packed
// as source << 16 | target, so two lower-bound searches (run side by side) on
// (source << 16) find the span. Sources outside it are inactive; their edges would only
// be read and dropped.
__device__ __forceinline__ void sp_narrow(const StoreDesc* __restrict__ sd, SpItem& m) {
  const uint32_t smin = (m.b << 5) + (uint32_t)(__ffs(m.bits) - 1);
  const uint32_t smax = (m.b << 5) + (31u - (uint32_t)__clz(m.bits));
  const uint32_t klo = smin << 16;
  const bool top = smax == 0xFFFFu;  // the tile's last source: the span runs to the end
  const uint32_t khi = top ? 0u : (smax + 1u) << 16;
  const uint32_t* e = sd->edges + m.base;
  uint32_t a0 = m.lo, a1 = m.hi, c0 = m.lo, c1 = top ? m.lo : m.hi;
  while (a0 < a1 || c0 < c1) {
    const uint32_t ma = (a0 + a1) >> 1, mc = (c0 + c1) >> 1;
    const uint32_t va = a0 < a1 ? e[ma] : 0u;
    const uint32_t vc = c0 < c1 ? e[mc] : 0u;
    if (a0 < a1) {
      if (va < klo) a0 = ma + 1;
      else a1 = ma;
    }
    if (c0 < c1) {
      if (vc < khi) c0 = mc + 1;
      else c1 = mc;
    }
  }
  m.lo = a0;
  m.hi = top ? m.hi : c0;
}

// One group of 32 items [g, g + 32) for the calling warp; returns the light edges walked
// and adds the items whose directory entries it read to `nread` (slice 0 only).
// With nslice > 1 several warps share the group: each reads the group's items, slice 0
// alone queues the heavy ones, and the light edges are dealt out in steps of 32 * SP_ILP
// (slice k takes steps k, k + nslice, ...); if the queue overflowed, slice 0 walks every
// light edge itself (the others' share is then walked twice, which changes nothing).
template <int ALGO, bool PERSIST>
__device__ __forceinline__ uint32_t sparse_group(const JobDesc* __restrict__ jd, const StoreDesc* __restrict__ sd,
                                                 uint64_t g, uint64_t items, uint32_t& nread,
                                                 uint32_t slice = 0, uint32_t nslice = 1) {
  LoopState* ls = jd->ls;
  const unsigned lane = threadIdx.x & 31;
  const uint64_t qcap = jd->spq_cap;
  const uint64_t it = g + lane;
  SpItem m{};
  uint32_t len = 0;
  if (it < items) {
    // an item whose column no active source of its word reaches holds none of their
    // edges: it is left empty without reading the directory
    const uint64_t li = it >> sd->lT;
    const uint32_t y = (uint32_t)(it & (sd->T - 1));
    const uint32_t w = ld_plain<PERSIST>(jd->aw + li);
    const unsigned long long cols = ld_plain<PERSIST>(jd->awm + li);
    if ((cols >> (y >> sd->cshift)) & 1ULL) {
      nread += slice == 0 ? 1u : 0u;
      m = sp_item_at<PERSIST>(jd, sd, w, y);
      len = m.hi > m.lo ? m.hi - m.lo : 0u;
      if (len > SP_NARROW && len <= SP_HEAVY) {
        sp_narrow(sd, m);
        len = m.hi > m.lo ? m.hi - m.lo : 0u;
      }
    }
  }
  uint32_t tot = len;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) tot += __shfl_xor_sync(0xFFFFFFFFu, tot, o);
  const bool heavy = len > SP_HEAVY || (tot > SP_WARP_MAX && len > SP_LIGHT);
  bool queued = heavy && slice != 0;  // slice 0 queues; the others leave those items to it
  bool overflow = false;
  if (heavy && slice == 0) {
    const uint32_t nch = (len + SP_CHUNK - 1) / SP_CHUNK;
    const unsigned slot = atomicAdd(&ls->spq_count, nch);
    if ((uint64_t)slot + nch <= qcap) {
      for (uint32_t k = 0; k < nch; ++k) jd->spq[slot + k] = make_uint2((uint32_t)it, k);
      queued = true;
    } else {
      overflow = true;
    }
  }
  const bool walk_all = nslice > 1 && slice == 0 && __any_sync(0xFFFFFFFFu, overflow);
  // light items: the group's edges are numbered 0..total-1 (warp prefix sum over the
  // items' lengths); lanes take SP_ILP of them per step and find their item by a
  // binary search over the prefix sums held in the lanes
  const uint32_t mine = (len > 0 && !queued) ? len : 0u;
  uint32_t incl = mine;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y2 = __shfl_up_sync(0xFFFFFFFFu, incl, o);
    if (lane >= (unsigned)o) incl += y2;
  }
  const uint32_t total = __shfl_sync(0xFFFFFFFFu, incl, 31);
  const uint32_t step0 = walk_all ? 0u : slice, nstep = walk_all ? 1u : nslice;
  for (uint32_t f0 = step0 * 32 * SP_ILP; f0 < total; f0 += nstep * 32 * SP_ILP) {
    uint32_t xs[SP_ILP], ys[SP_ILP], bits[SP_ILP];
    unsigned long long pos[SP_ILP];
    uint32_t valid = 0;
#pragma unroll
    for (int k = 0; k < SP_ILP; ++k) {
      const uint32_t f = f0 + lane + 32u * k;
      // item j holding flattened edge f: the least j with incl[j] > f
      uint32_t j = 0;
#pragma unroll
      for (int step = 16; step > 0; step >>= 1) {
        const uint32_t probe = __shfl_sync(0xFFFFFFFFu, incl, j + step - 1);
        if (probe <= f) j += step;
      }
      const uint32_t incl_j = __shfl_sync(0xFFFFFFFFu, incl, j);
      const uint32_t mine_j = __shfl_sync(0xFFFFFFFFu, mine, j);
      xs[k] = __shfl_sync(0xFFFFFFFFu, m.x, j);
      ys[k] = __shfl_sync(0xFFFFFFFFu, m.y, j);
      bits[k] = __shfl_sync(0xFFFFFFFFu, m.bits, j);
      const uint32_t lo_j = __shfl_sync(0xFFFFFFFFu, m.lo, j);
      const unsigned long long base_j = __shfl_sync(0xFFFFFFFFu, m.base, j);
      pos[k] = base_j + lo_j + (f - (incl_j - mine_j));
      valid |= (f < total) ? (1u << k) : 0u;
    }
    sp_batch<ALGO, PERSIST>(jd, sd, xs, ys, bits, pos, valid);
  }
  return slice == 0 ? mine : 0u;
}

// Queue entry q (a chunk of a heavy item) for the calling warp; returns the edges walked
// (lane 0). Sources are sorted inside an item, so a chunk whose first and last edges
// span no source of the item's frontier word is skipped after two loads.
template <int ALGO, bool PERSIST>
__device__ __forceinline__ uint32_t sparse_chunk(const JobDesc* __restrict__ jd, const StoreDesc* __restrict__ sd,
                                                 uint64_t q, uint64_t items) {
  const unsigned lane = threadIdx.x & 31;
  const uint2 c = ld_plain<PERSIST>(jd->spq + q);
  if (c.x >= items) return 0;  // never indexes outside this round's items
  SpItem m = sp_item<PERSIST>(jd, sd, c.x);
  {
    // the item as sparse_group cut it into chunks: narrowed by the same rule
    const uint32_t len = m.hi > m.lo ? m.hi - m.lo : 0u;
    if (len > SP_NARROW && len <= SP_HEAVY) sp_narrow(sd, m);
  }
  const uint32_t e0 = m.lo + c.y * SP_CHUNK;
  const uint32_t e1 = min(m.hi, e0 + SP_CHUNK);
  if (e0 >= e1) return 0;
  uint32_t bound = 0;
  if (lane == 0) bound = sd->edges[m.base + e0];
  if (lane == 1) bound = sd->edges[m.base + e1 - 1];
  const uint32_t s_first = (__shfl_sync(0xFFFFFFFFu, bound, 0) >> 16) & 31u;
  const uint32_t s_last = (__shfl_sync(0xFFFFFFFFu, bound, 1) >> 16) & 31u;
  const uint32_t span = (s_last >= 31u ? 0xFFFFFFFFu : ((2u << s_last) - 1u)) & ~((1u << s_first) - 1u);
  if ((m.bits & span) == 0) return 0;
  uint32_t xs[SP_ILP], ys[SP_ILP], bits[SP_ILP];
#pragma unroll
  for (int k = 0; k < SP_ILP; ++k) {
    xs[k] = m.x;
    ys[k] = m.y;
    bits[k] = m.bits;
  }
  for (uint32_t e = e0 + lane; e < e1; e += 32 * SP_ILP) {
    unsigned long long pos[SP_ILP];
    uint32_t valid = 0;
#pragma unroll
    for (int k = 0; k < SP_ILP; ++k) {
      const uint32_t ek = e + 32u * k;
      pos[k] = m.base + ek;
      valid |= (ek < e1) ? (1u << k) : 0u;
    }
    sp_batch<ALGO, PERSIST>(jd, sd, xs, ys, bits, pos, valid);
  }
  return lane == 0 ? e1 - e0 : 0u;
}

}  // namespace cytom
