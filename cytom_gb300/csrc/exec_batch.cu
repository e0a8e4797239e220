// exec_batch.cu — batched persistent executor: many jobs (BFS, CC, SSSP, PageRank,
// PageRank-delta) over one or more graph snapshots run together in ONE kernel launch.
//
// The reference runs every job as its own ContinuousAlgorithmExecutor on its own
// threads (src/include/core/jobs.h:79-83, src/include/main/execute.h:534-771); a job's
// rounds are separated by barriers (continuous-algorithm-executor.h:49-249). Here the
// jobs share the GPU inside one persistent kernel:
//  - every job has a work queue for its current phase: the 4096-edge stages (dense
//    round) or 256-item groups and 256-edge chunks (sparse round) of a gather, the
//    1024-word ranges of an apply, the 4096-vertex ranges of a PageRank contribution
//    pass (every PAGERANK round; PageRank-delta's residual round only, its delta rounds
//    take the contributions the previous pull wrote) and the target bins of its pull;
//  - a block claims a unit of any job with one 64-bit atomic on that job's claim word
//    [phase : 8][units : 24][next unit : 32], so the phase and its size travel with the
//    claim;
//  - the block that completes the last unit of a phase (a per-phase completion
//    counter) runs the job's control step — the same device code as the one-job
//    executors (minprop_dev.cuh, pagerank_dev.cuh) — and publishes the next phase;
//  - no block ever waits on another block: a block that finds no unit polls the claim
//    words again (bounded: after kIdleLimit empty polls in a row -- or the limit a test
//    sets through cytom_set_fault_injection -- it records a timeout and exits, so the
//    launch always ends).
// Values written during the launch are read through L2 (the PERSIST load policy).
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <new>
#include <vector>

#include "engine.h"
#include "minprop_dev.cuh"
#include "pagerank_dev.cuh"

namespace cytom {

int pagerank_batch_prep(Ctx* c, Job* j, PrArgs* out, uint64_t* nb, int* first_mode, uint64_t* begin_edges);

constexpr int BT = 256;  // threads of a batch block (every unit kind is written for 256)
static_assert(BT == APPLY_T && BT == SG_T && BT == PR_BLOCK_T, "one block shape for every unit");

enum BatchPhase : unsigned {
  PH_NONE = 0,
  PH_APPLY0 = 1,     // seeding apply of a BFS / CC / SSSP run
  PH_DENSE = 2,      // dense gather: one 4096-edge stage per unit
  PH_SPARSE = 3,     // sparse gather: 256 items per unit
  PH_CHUNKS = 4,     // sparse chunk pass: 8 queued chunks per unit
  PH_APPLY = 5,      // apply: 1024 frontier words per unit
  PH_PR_CONTRIB = 6, // PageRank contributions: 4096 sources per unit
  PH_PR_PULL = 7,    // PageRank pull: targets of one in-degree bin per unit (pr_bin_unit)
  PH_DONE = 8
};
constexpr uint32_t BU_APPLY_WORDS = 1024;
constexpr uint32_t BU_SPARSE_ITEMS = 256;
constexpr uint32_t BU_CHUNKS = BT / 32;
constexpr uint32_t BU_PR_VERTS = 4096;
// targets per pull unit of each bin: 4 per thread (one thread per target), 4 per group of
// VW lanes, one for the block bin
__host__ __device__ constexpr uint32_t pr_bin_unit(int k) {
  return pr_bin_vw(k) == 1 ? 4 * BT : (pr_bin_vw(k) == 0 ? 1 : 4 * (BT / pr_bin_vw(k)));
}
constexpr uint32_t kMaxUnits = (1u << 24) - 1;
constexpr uint32_t kIdleLimit = 1u << 22;

struct BJob {
  const JobDesc* jd;
  const StoreDesc* sd;
  PrArgs pr;
  PrArgs pr2;                      // paired PAGERANK job (paired = 1): its arguments
  void* cpair;                     // paired jobs: interleaved contributions {job, pr2 job}
  unsigned long long nb[kPrBins];  // PageRank target bins
  LoopState* ls;                   // the job's loop state (statistics read back after the launch)
  int algo;
  int adaptive;
  int paired;
  unsigned begin;                  // batch_begin_kernel: 1 BFS / CC / SSSP reset, 2 PageRank reset, 0 none
  unsigned max_iter;
  unsigned pad_bj;
  double tol;
  unsigned long long begin_edges;  // PageRank: edges a round reads
};

struct __align__(128) BSched {
  unsigned long long claim;  // [phase:8][units:24][next:32]
  unsigned done;             // units of the current phase completed
  int prmode;                // PageRank: mode of the current round
};

struct BCtl {
  unsigned jobs_left;
  unsigned err;
  unsigned long long units;  // units processed (statistics)
  unsigned idle_limit;       // empty polls before a block gives up
};

__host__ __device__ constexpr unsigned long long pack_claim(unsigned phase, unsigned total) {
  return ((unsigned long long)phase << 56) | ((unsigned long long)(total & 0xFFFFFFu) << 32);
}

__device__ __forceinline__ uint32_t ceil_div(uint64_t a, uint64_t b) { return (uint32_t)((a + b - 1) / b); }

// Units of a pull phase: every bin's targets in units of pr_bin_unit(k).
__device__ __forceinline__ uint32_t pr_pull_units(const BJob* J) {
  uint32_t t = 0;
  for (int k = 0; k < kPrBins; ++k) t += ceil_div(J->nb[k], pr_bin_unit(k));
  return t;
}

// Pull units are handed out from the largest in-degree bin down (unit 0 = the last unit
// of the hub bin), so the longest units start first and the short ones fill the phase's
// tail.
__device__ __forceinline__ uint32_t pr_pull_order(const BJob* J, uint32_t unit) { return pr_pull_units(J) - 1u - unit; }


// ---- units -----------------------------------------------------------------

__device__ __forceinline__ unsigned ls_iter(const LoopState* ls) { return *(const volatile unsigned*)&ls->iter; }

__device__ void unit_apply(const BJob* J, bool initial, uint32_t unit) {
  const JobDesc* jd = J->jd;
  const StoreDesc* sd = J->sd;
  const unsigned pw = initial ? 0u : ((ls_iter(jd->ls) & 1u) ^ 1u);
  const uint64_t nwords = (sd->n + 31) >> 5;
  unsigned cnt = 0;
  unsigned long long teps = 0;
  const uint64_t base0 = (uint64_t)unit * BU_APPLY_WORDS;
  for (uint32_t k = 0; k < BU_APPLY_WORDS / BT; ++k) {
    const uint64_t base = base0 + (uint64_t)k * BT;
    if (base < nwords) apply_step<true>(jd, sd, pw, base, cnt, teps);
  }
  apply_flush(jd->ls, pw, cnt, teps);
}

template <int ALGO>
__device__ void unit_dense(const BJob* J, uint32_t st) {
  const JobDesc* jd = J->jd;
  const StoreDesc* sd = J->sd;
  const unsigned p = ls_iter(jd->ls) & 1u;
  if (!stage_active<true>(jd, sd, st, p, J->adaptive)) return;
  const uint64_t e0 = (uint64_t)st * SG_E;
  // two half-stages of 8 edges per thread: the persistent kernel's register budget is
  // set by its largest unit, and a 16-edge stage would cap it at two blocks per SM
#pragma unroll 1
  for (uint32_t h = 0; h < 2; ++h) {
    const uint64_t st8 = 2ull * st + h, h0 = st8 * (SG_E / 2);
    if (h0 >= sd->E) break;
    dense_stage<ALGO, true, true, 8>(jd, sd, sd->edges + h0, mp_weighted<ALGO>() ? sd->wts + h0 : nullptr, st8, p,
                                     J->adaptive);
  }
  if (threadIdx.x == 0) {
    const uint64_t rem = sd->E - e0;
    atomicAdd(&jd->ls->edges_scanned, (unsigned long long)(rem < (uint64_t)SG_E ? rem : (uint64_t)SG_E));
  }
}

template <int ALGO>
__device__ void unit_sparse(const BJob* J, uint32_t unit) {
  const JobDesc* jd = J->jd;
  const StoreDesc* sd = J->sd;
  const unsigned p = ls_iter(jd->ls) & 1u;
  const uint64_t items = (uint64_t)__ldcg(&jd->ls->nact_words[p]) << sd->lT;
  const uint64_t g = (uint64_t)unit * BU_SPARSE_ITEMS + (threadIdx.x >> 5) * 32;
  unsigned long long scanned = 0;
  uint32_t nread = 0;  // items read: the one-job kernels' byte accounting, not kept here
  if (g < items) scanned = sparse_group<ALGO, true>(jd, sd, g, items, nread);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) scanned += __shfl_xor_sync(0xFFFFFFFFu, scanned, o);
  if ((threadIdx.x & 31) == 0 && scanned) atomicAdd(&jd->ls->edges_scanned, scanned);
}

template <int ALGO>
__device__ void unit_chunks(const BJob* J, uint32_t unit) {
  const JobDesc* jd = J->jd;
  const StoreDesc* sd = J->sd;
  const unsigned p = ls_iter(jd->ls) & 1u;
  const uint64_t items = (uint64_t)__ldcg(&jd->ls->nact_words[p]) << sd->lT;
  uint64_t nq = __ldcg(&jd->ls->spq_count);
  if (nq > jd->spq_cap) nq = jd->spq_cap;
  const uint64_t q = (uint64_t)unit * BU_CHUNKS + (threadIdx.x >> 5);
  uint32_t scanned = 0;
  if (q < nq) scanned = sparse_chunk<ALGO, true>(jd, sd, q, items);
  if ((threadIdx.x & 31) == 0 && scanned) atomicAdd(&jd->ls->edges_scanned, (unsigned long long)scanned);
}

template <int MODE>
__device__ void unit_pr_contrib(const BJob* J, uint32_t unit) {
  const PrArgs& a = J->pr;
  const unsigned p = ls_iter(a.ls) & 1u;
  const uint64_t lo = (uint64_t)unit * BU_PR_VERTS;
  const uint64_t hi = std::min<uint64_t>(lo + BU_PR_VERTS, a.n);
  const pr_ff_t<MODE> dangling = pr_contrib_range<MODE, true>(a, p, lo, hi, threadIdx.x, BT);
  pr_dangling_flush<MODE>(a.ls, p, dangling);
}

template <int MODE, int VW>
__device__ __forceinline__ void pull_groups(const PrArgs& a, const pr_val_t<MODE>* cr, uint64_t off, uint64_t cnt,
                                            uint64_t first, unsigned p, pr_ff_t<MODE> dang, PrTally& t) {
  constexpr uint32_t GPB = BT / VW;  // groups per block
  const unsigned gl = threadIdx.x & (VW - 1);
  const uint32_t g = threadIdx.x / VW;
#pragma unroll 1
  for (uint32_t k = 0; k < 4; ++k) {
    const uint64_t i = first + (uint64_t)k * GPB + g;
    uint32_t v = 0, lo = 0, hi = 0;
    if (i < cnt) {
      v = a.bins[off + i];
      lo = a.csc_ptr[v];
      hi = a.csc_ptr[v + 1];
    }
    const pr_ff_t<MODE> sum = pr_sum_group<MODE, true, VW>(a, cr, lo, hi, gl);
    if (gl == 0 && i < cnt) pr_finish<MODE, true>(a, v, sum, p, dang, t);
  }
}

template <int MODE>
__device__ void unit_pr_pull(const BJob* J, uint32_t unit) {
  const PrArgs& a = J->pr;
  LoopState* ls = a.ls;
  const unsigned p = ls_iter(ls) & 1u;
  const pr_ff_t<MODE> dang = pr_dang_arg<MODE, true>(a, ls, p);
  // the bin this unit belongs to
  int k = 0;
  uint64_t off = 0;
  uint32_t u = pr_pull_order(J, unit);
  for (; k < kPrBins - 1; ++k) {
    const uint32_t units_k = ceil_div(J->nb[k], pr_bin_unit(k));
    if (u < units_k) break;
    u -= units_k;
    off += J->nb[k];
  }
  const uint64_t cnt = J->nb[k];
  const uint64_t first = (uint64_t)u * pr_bin_unit(k);
  const pr_val_t<MODE>* cr = pr_cread<MODE>(a, p);
  PrTally t;
  t.init();
  switch (pr_bin_vw(k)) {
    case 1:
#pragma unroll 1
      for (uint32_t r = 0; r < 4; ++r) {
        const uint64_t i = first + (uint64_t)r * BT + threadIdx.x;
        if (i < cnt) {
          const uint32_t v = a.bins[off + i];
          const pr_ff_t<MODE> sum = pr_sum_thread<MODE, true>(a, cr, v);
          pr_finish<MODE, true>(a, v, sum, p, dang, t);
        }
      }
      break;
    case 4: pull_groups<MODE, 4>(a, cr, off, cnt, first, p, dang, t); break;
    case 8: pull_groups<MODE, 8>(a, cr, off, cnt, first, p, dang, t); break;
    case 32: pull_groups<MODE, 32>(a, cr, off, cnt, first, p, dang, t); break;
    default: {
      const uint32_t v = a.bins[off + first];
      const pr_ff_t<MODE> sum = pr_sum_block<MODE, true>(a, cr, v);
      if (threadIdx.x == 0) pr_finish<MODE, true>(a, v, sum, p, dang, t);
    }
  }
  pr_tally_flush<MODE>(ls, p, t);
}

// ---- two PAGERANK jobs of one snapshot in one pass ---------------------------------
// Jobs of one context and form (FP32 compensated, or FP64 plain) share a round's passes:
// the contribution pass writes both jobs' contributions interleaved per source, so the
// pull loads each in-edge's source id once and one pair of contributions for both jobs
// (one L2 sector where two jobs apart take two). Each job keeps its own ranks, loop
// state, parameters and summation order: its sums are those of a pass of its own, bit
// for bit. A job that converges first stops updating; the pair runs until both have.
template <int MODE>
struct PrPairT;
template <>
struct PrPairT<PR_NORM32> {
  using T = float2;
};
template <>
struct PrPairT<PR_NORM64> {
  using T = double2;
};
template <int MODE>
using pr_pair_t = typename PrPairT<MODE>::T;

__device__ __forceinline__ bool pr_on(const LoopState* ls) { return __ldcg(&ls->cont) != 0u; }

// Both jobs' contributions of sources [unit * BU_PR_VERTS, ...), as pr_contrib_range
// computes them (NORM32: FP32 quotient of the rank's high word, the low word entering the
// dangling mass; NORM64: FP64 quotient). A thread loads the degrees and ranks of four
// sources before it uses any (one round trip per four sources); the dangling sums add up
// in source order as in pr_contrib_range.
template <int MODE>
__device__ void unit_pr_contrib_pair(const BJob* J, uint32_t unit) {
  using V = pr_val_t<MODE>;
  constexpr bool k32 = MODE == PR_NORM32;
  const PrArgs& a0 = J->pr;
  const PrArgs& a1 = J->pr2;
  const bool on0 = pr_on(a0.ls), on1 = pr_on(a1.ls);
  const unsigned p0 = ls_iter(a0.ls) & 1u, p1 = ls_iter(a1.ls) & 1u;
  const V* r0 = k32 ? (const V*)((p0 == 0) ? a0.rank : a0.comp) : (const V*)((p0 == 0) ? a0.r64 : a0.r64n);
  const V* r1 = k32 ? (const V*)((p1 == 0) ? a1.rank : a1.comp) : (const V*)((p1 == 0) ? a1.r64 : a1.r64n);
  const float* l0 = (p0 == 0) ? a0.lo0 : a0.lo1;
  const float* l1 = (p1 == 0) ? a1.lo0 : a1.lo1;
  pr_pair_t<MODE>* cw = reinterpret_cast<pr_pair_t<MODE>*>(J->cpair);
  const uint64_t lo = (uint64_t)unit * BU_PR_VERTS;
  const uint64_t hi = std::min<uint64_t>(lo + BU_PR_VERTS, a0.n);
  pr_ff_t<MODE> d0{}, d1{};
  for (uint64_t ub = lo + threadIdx.x; ub < hi; ub += 4 * BT) {
    uint32_t dg[4];
    V h0[4], h1[4];
    float w0[4], w1[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const uint64_t u = ub + (uint64_t)k * BT;
      const bool in = u < hi;
      dg[k] = in ? a0.deg[u] : 1u;  // the snapshot's out-degrees, shared by both jobs
      h0[k] = (in && on0) ? __ldcg(r0 + u) : (V)0;
      h1[k] = (in && on1) ? __ldcg(r1 + u) : (V)0;
      w0[k] = (k32 && in && on0) ? __ldcg(l0 + u) : 0.f;
      w1[k] = (k32 && in && on1) ? __ldcg(l1 + u) : 0.f;
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const uint64_t u = ub + (uint64_t)k * BT;
      if (u < hi) {
        pr_pair_t<MODE> c;
        c.x = (V)0;
        c.y = (V)0;
        if (on0) {
          if (!dg[k]) {
            if constexpr (k32) d0 = ff_add(d0, FF{(float)h0[k], w0[k]});
            else d0 += h0[k];
          }
          c.x = dg[k] ? h0[k] / (V)dg[k] : (V)0;
        }
        if (on1) {
          if (!dg[k]) {
            if constexpr (k32) d1 = ff_add(d1, FF{(float)h1[k], w1[k]});
            else d1 += h1[k];
          }
          c.y = dg[k] ? h1[k] / (V)dg[k] : (V)0;
        }
        cw[u] = c;
      }
    }
  }
  pr_dangling_flush<MODE>(a0.ls, p0, d0);
  pr_dangling_flush<MODE>(a1.ls, p1, d1);
}

// pr_lane_sum over the interleaved pairs: the same edges in the same order for each job.
template <int MODE, int B, class Acc>
__device__ __forceinline__ void pr_lane_sum_pair(const PrArgs& a, const pr_pair_t<MODE>* cp, uint32_t e0, uint32_t hi,
                                                 uint32_t stride, Acc& acc0, Acc& acc1) {
  uint32_t id[B];
#pragma unroll
  for (int k = 0; k < B; ++k) {
    const uint32_t e = e0 + (uint32_t)k * stride;
    id[k] = e < hi ? __ldcs(a.csc_src + e) : 0u;  // streamed: keep L1 for the gathered contributions
  }
  for (uint32_t e = e0; e < hi; e += (uint32_t)B * stride) {
    pr_pair_t<MODE> c[B];
#pragma unroll
    for (int k = 0; k < B; ++k) {
      const uint32_t ek = e + (uint32_t)k * stride;
      if (ek < hi) {
        c[k] = __ldcg(cp + id[k]);
      } else {
        c[k].x = 0;
        c[k].y = 0;
      }
    }
    const uint32_t en = e + (uint32_t)B * stride;
#pragma unroll
    for (int k = 0; k < B; ++k) {
      const uint32_t ek = en + (uint32_t)k * stride;
      id[k] = ek < hi ? __ldcs(a.csc_src + ek) : 0u;
    }
#pragma unroll
    for (int k = 0; k < B; ++k)
      if (e + (uint32_t)k * stride < hi) {
        acc0.add(c[k].x);
        acc1.add(c[k].y);
      }
  }
}

template <int MODE>
using pr_acc_t = typename std::conditional<pr_is64<MODE>(), Acc64, Acc32>::type;

template <int MODE>
__device__ __forceinline__ pr_ff_t<MODE> pr_acc_value(const Acc32& a) {
  return pr_acc32_out<MODE>(a.s, a.e);
}
template <int MODE>
__device__ __forceinline__ double pr_acc_value(const Acc64& a) {
  return a.s;
}

// A group of VW lanes merges its lanes by an xor tree, as pr_sum_group does.
template <int VW>
__device__ __forceinline__ void pr_group_merge(Acc32& acc) {
#pragma unroll
  for (int o = VW / 2; o > 0; o >>= 1) {
    const float s2 = __shfl_xor_sync(0xFFFFFFFFu, acc.s, o, VW);
    const float e2 = __shfl_xor_sync(0xFFFFFFFFu, acc.e, o, VW);
    acc.merge(s2, e2);
  }
}
template <int VW>
__device__ __forceinline__ void pr_group_merge(Acc64& acc) {
#pragma unroll
  for (int o = VW / 2; o > 0; o >>= 1) acc.s += __shfl_xor_sync(0xFFFFFFFFu, acc.s, o, VW);
}

// Whole-block sum (pr_sum_block's reduction) of both jobs; thread 0 holds the sums.
template <int MODE>
__device__ __forceinline__ void pr_block_pair(const PrArgs& a, const pr_pair_t<MODE>* cp, uint32_t v,
                                              pr_ff_t<MODE>& s0, pr_ff_t<MODE>& s1) {
  __shared__ float s_s[2][BT / 32], s_e[2][BT / 32];
  __shared__ double s_d[2][BT / 32];
  const unsigned lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const uint32_t lo = a.csc_ptr[v], hi = a.csc_ptr[v + 1];
  pr_acc_t<MODE> acc0, acc1;
  acc0.init();
  acc1.init();
  pr_lane_sum_pair<MODE, 4>(a, cp, lo + threadIdx.x, hi, BT, acc0, acc1);
  pr_group_merge<32>(acc0);
  pr_group_merge<32>(acc1);
  if constexpr (pr_is64<MODE>()) {
    if (lane == 0) {
      s_d[0][wid] = acc0.s;
      s_d[1][wid] = acc1.s;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      s0 = 0.0;
      s1 = 0.0;
      for (int k = 0; k < BT / 32; ++k) {
        s0 += s_d[0][k];
        s1 += s_d[1][k];
      }
    }
  } else {
    if (lane == 0) {
      s_s[0][wid] = acc0.s;
      s_e[0][wid] = acc0.e;
      s_s[1][wid] = acc1.s;
      s_e[1][wid] = acc1.e;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      Acc32 t0, t1;
      t0.init();
      t1.init();
      for (int k = 0; k < BT / 32; ++k) {
        t0.merge(s_s[0][k], s_e[0][k]);
        t1.merge(s_s[1][k], s_e[1][k]);
      }
      s0 = pr_acc32_out<MODE>(t0.s, t0.e);
      s1 = pr_acc32_out<MODE>(t1.s, t1.e);
    }
  }
  __syncthreads();
}

// Both jobs' updates of target v from their sums and preloaded ranks (pr_finish).
template <int MODE>
struct PairFinish {
  const PrArgs& a0;
  const PrArgs& a1;
  bool on0, on1;
  unsigned p0, p1;
  pr_ff_t<MODE> dang0, dang1;
  PrTally t0, t1;
  __device__ __forceinline__ void old(uint32_t v, PrOld& o0, PrOld& o1) const {
    if (on0) o0 = pr_load_old<MODE, true>(a0, v, p0);
    if (on1) o1 = pr_load_old<MODE, true>(a1, v, p1);
  }
  __device__ __forceinline__ void operator()(uint32_t v, pr_ff_t<MODE> s0, pr_ff_t<MODE> s1, PrOld o0, PrOld o1) {
    if (on0) pr_apply_norm<MODE>(a0, v, s0, p0, dang0, o0, t0);
    if (on1) pr_apply_norm<MODE>(a1, v, s1, p1, dang1, o1, t1);
  }
};

// Targets of in-degree <= 4, one thread each, four per thread: the thread loads the
// four targets' ids and offsets up front, then handles two targets at a time with their
// in-edge ids, then their contributions and ranks, in flight together. Each target's
// edges add up in edge order, as pr_sum_thread adds them.
template <int MODE>
__device__ __forceinline__ void pair_small(const PrArgs& a0, const pr_pair_t<MODE>* cp, uint64_t off, uint64_t cnt,
                                           uint64_t first, PairFinish<MODE>& fin) {
  using Acc = pr_acc_t<MODE>;
  uint32_t v[4], lo[4], hi[4];
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const uint64_t i = first + (uint64_t)r * BT + threadIdx.x;
    v[r] = i < cnt ? a0.bins[off + i] : 0xFFFFFFFFu;
  }
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    lo[r] = v[r] != 0xFFFFFFFFu ? a0.csc_ptr[v[r]] : 0u;
    hi[r] = v[r] != 0xFFFFFFFFu ? a0.csc_ptr[v[r] + 1] : 0u;
  }
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    uint32_t id[2][4];
#pragma unroll
    for (int t = 0; t < 2; ++t)
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const uint32_t e = lo[2 * h + t] + (uint32_t)k;
        id[t][k] = e < hi[2 * h + t] ? a0.csc_src[e] : 0u;
      }
    pr_pair_t<MODE> c[2][4];
    PrOld o0[2] = {}, o1[2] = {};
#pragma unroll
    for (int t = 0; t < 2; ++t) {
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        if (lo[2 * h + t] + (uint32_t)k < hi[2 * h + t]) {
          c[t][k] = __ldcg(cp + id[t][k]);
        } else {
          c[t][k].x = 0;
          c[t][k].y = 0;
        }
      }
      if (v[2 * h + t] != 0xFFFFFFFFu) fin.old(v[2 * h + t], o0[t], o1[t]);
    }
#pragma unroll
    for (int t = 0; t < 2; ++t) {
      if (v[2 * h + t] == 0xFFFFFFFFu) continue;
      Acc acc0, acc1;
      acc0.init();
      acc1.init();
#pragma unroll
      for (int k = 0; k < 4; ++k)
        if (lo[2 * h + t] + (uint32_t)k < hi[2 * h + t]) {
          acc0.add(c[t][k].x);
          acc1.add(c[t][k].y);
        }
      fin(v[2 * h + t], pr_acc_value<MODE>(acc0), pr_acc_value<MODE>(acc1), o0[t], o1[t]);
    }
  }
}

// Targets of one group bin, VW lanes each, four per group (pull_groups): the group loads
// its four targets' ids and offsets up front; the first lane loads each target's ranks
// before the target's sum. Lane order and merge tree as pr_sum_group.
template <int MODE, int VW>
__device__ __forceinline__ void pair_groups(const PrArgs& a0, const pr_pair_t<MODE>* cp, uint64_t off,
                                            uint64_t cnt, uint64_t first, PairFinish<MODE>& fin) {
  constexpr uint32_t GPB = BT / VW;
  const unsigned gl = threadIdx.x & (VW - 1);
  const uint32_t g = threadIdx.x / VW;
  uint32_t v[4], lo[4], hi[4];
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const uint64_t i = first + (uint64_t)r * GPB + g;
    v[r] = i < cnt ? a0.bins[off + i] : 0xFFFFFFFFu;
  }
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    lo[r] = v[r] != 0xFFFFFFFFu ? a0.csc_ptr[v[r]] : 0u;
    hi[r] = v[r] != 0xFFFFFFFFu ? a0.csc_ptr[v[r] + 1] : 0u;
  }
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    PrOld o0 = {}, o1 = {};
    if (gl == 0 && v[r] != 0xFFFFFFFFu) fin.old(v[r], o0, o1);
    pr_acc_t<MODE> acc0, acc1;
    acc0.init();
    acc1.init();
    pr_lane_sum_pair<MODE, 4>(a0, cp, lo[r] + gl, hi[r], VW, acc0, acc1);
    pr_group_merge<VW>(acc0);
    pr_group_merge<VW>(acc1);
    if (gl == 0 && v[r] != 0xFFFFFFFFu)
      fin(v[r], pr_acc_value<MODE>(acc0), pr_acc_value<MODE>(acc1), o0, o1);
  }
}

template <int MODE>
__device__ void unit_pr_pull_pair(const BJob* J, uint32_t unit) {
  const PrArgs& a0 = J->pr;
  const PrArgs& a1 = J->pr2;
  PairFinish<MODE> fin{a0, a1};
  fin.on0 = pr_on(a0.ls);
  fin.on1 = pr_on(a1.ls);
  fin.p0 = ls_iter(a0.ls) & 1u;
  fin.p1 = ls_iter(a1.ls) & 1u;
  fin.dang0 = pr_dang_arg<MODE, true>(a0, a0.ls, fin.p0);
  fin.dang1 = pr_dang_arg<MODE, true>(a1, a1.ls, fin.p1);
  fin.t0.init();
  fin.t1.init();
  int k = 0;
  uint64_t off = 0;
  uint32_t u = pr_pull_order(J, unit);
  for (; k < kPrBins - 1; ++k) {
    const uint32_t units_k = ceil_div(J->nb[k], pr_bin_unit(k));
    if (u < units_k) break;
    u -= units_k;
    off += J->nb[k];
  }
  const uint64_t cnt = J->nb[k];
  const uint64_t first = (uint64_t)u * pr_bin_unit(k);
  const pr_pair_t<MODE>* cp = reinterpret_cast<const pr_pair_t<MODE>*>(J->cpair);
  switch (pr_bin_vw(k)) {
    case 1: pair_small<MODE>(a0, cp, off, cnt, first, fin); break;
    case 4: pair_groups<MODE, 4>(a0, cp, off, cnt, first, fin); break;
    case 8: pair_groups<MODE, 8>(a0, cp, off, cnt, first, fin); break;
    case 32: pair_groups<MODE, 32>(a0, cp, off, cnt, first, fin); break;
    default: {
      const uint32_t v = a0.bins[off + first];
      PrOld o0 = {}, o1 = {};
      if (threadIdx.x == 0) fin.old(v, o0, o1);
      pr_ff_t<MODE> s0{}, s1{};
      pr_block_pair<MODE>(a0, cp, v, s0, s1);
      if (threadIdx.x == 0) fin(v, s0, s1, o0, o1);
    }
  }
  if (fin.on0) pr_tally_flush<MODE>(a0.ls, fin.p0, fin.t0);
  if (fin.on1) pr_tally_flush<MODE>(a1.ls, fin.p1, fin.t1);
}


// ---- phase transitions (whole block, after the last unit of `phase`) --------

__device__ void advance(const BJob* J, BSched* S, BCtl* ctl, unsigned phase) {
  __shared__ unsigned s_next, s_total, s_cont;
  __shared__ int s_mode;
  const JobDesc* jd = J->jd;
  const StoreDesc* sd = J->sd;
  const bool pr = J->algo == CYTOM_ALGO_PR_DELTA || J->algo == CYTOM_ALGO_PAGERANK;
  if (threadIdx.x == 0) {
    s_mode = *(volatile int*)&S->prmode;
    s_next = PH_DONE;
    s_total = 0;
    s_cont = 1;
    if (pr) {
      if (phase == PH_PR_CONTRIB) {
        s_next = PH_PR_PULL;
        s_total = pr_pull_units(J);
      } else {
        s_cont = pr_control_step(J->pr.ls, s_mode);
        if (J->paired) s_cont |= pr_control_step(J->pr2.ls, s_mode);
        if (s_cont) {
          if (s_mode == PR_DELTA_RESIDUAL || s_mode == PR_DELTA_PUSH) {
            // PageRank-delta: the pull wrote the next round's contributions
            s_mode = PR_DELTA_PUSH;
            s_next = PH_PR_PULL;
            s_total = pr_pull_units(J);
          } else {
            s_next = PH_PR_CONTRIB;
            s_total = ceil_div(J->pr.n, BU_PR_VERTS);
          }
        }
      }
    } else if (phase == PH_DENSE || phase == PH_CHUNKS) {
      s_next = PH_APPLY;
    } else if (phase == PH_SPARSE) {
      uint64_t nq = __ldcg(&jd->ls->spq_count);
      if (nq > jd->spq_cap) nq = jd->spq_cap;
      s_next = nq ? PH_CHUNKS : PH_APPLY;
      s_total = nq ? ceil_div(nq, BU_CHUNKS) : 0;
    } else {
      s_cont = control_step(jd, sd, phase == PH_APPLY0 ? 1 : 0);
    }
  }
  __syncthreads();
  if (!pr && (phase == PH_APPLY0 || phase == PH_APPLY) && s_cont) {
    // open the next round (all threads clear the row flags), then pick its gather
    const unsigned p = ls_iter(jd->ls) & 1u;
    round_open<true>(jd, sd, p, J->adaptive, threadIdx.x, BT);
    __syncthreads();
    if (threadIdx.x == 0) {
      const unsigned mode = *(volatile unsigned*)&jd->ls->mode;
      if (mode == 0) {
        s_next = PH_DENSE;
        s_total = ceil_div(sd->E, SG_E);
      } else {
        s_next = PH_SPARSE;
        s_total = ceil_div((uint64_t)__ldcg(&jd->ls->nact_words[p]) << sd->lT, BU_SPARSE_ITEMS);
      }
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    unsigned next = s_next, total = s_total;
    // an empty gather phase goes straight to the apply
    if (!pr && (next == PH_DENSE || next == PH_SPARSE || next == PH_CHUNKS) && total == 0) next = PH_APPLY;
    if (next == PH_APPLY) total = ceil_div((sd->n + 31) >> 5, BU_APPLY_WORDS);
    if (total > kMaxUnits) {
      atomicExch(&ctl->err, 2u);
      next = PH_DONE;
    }
    if (!s_cont || next == PH_DONE) {
      __threadfence();
      atomicExch(&S->claim, pack_claim(PH_DONE, 0));
      atomicSub(&ctl->jobs_left, 1u);
    } else {
      S->done = 0;
      S->prmode = s_mode;
      __threadfence();
      atomicExch(&S->claim, pack_claim(next, total));
    }
  }
  __syncthreads();
}

__device__ void run_unit(const BJob* J, unsigned phase, uint32_t unit, int prmode) {
  const int algo = J->algo;
  switch (phase) {
    case PH_APPLY0:
    case PH_APPLY:
      unit_apply(J, phase == PH_APPLY0, unit);
      break;
    case PH_DENSE:
      if (algo == CYTOM_ALGO_BFS) unit_dense<0>(J, unit);
      else if (algo == CYTOM_ALGO_CC) unit_dense<1>(J, unit);
      else if (algo == CYTOM_ALGO_SSWP) unit_dense<3>(J, unit);
      else unit_dense<2>(J, unit);
      break;
    case PH_SPARSE:
      if (algo == CYTOM_ALGO_BFS) unit_sparse<0>(J, unit);
      else if (algo == CYTOM_ALGO_CC) unit_sparse<1>(J, unit);
      else if (algo == CYTOM_ALGO_SSWP) unit_sparse<3>(J, unit);
      else unit_sparse<2>(J, unit);
      break;
    case PH_CHUNKS:
      if (algo == CYTOM_ALGO_BFS) unit_chunks<0>(J, unit);
      else if (algo == CYTOM_ALGO_CC) unit_chunks<1>(J, unit);
      else if (algo == CYTOM_ALGO_SSWP) unit_chunks<3>(J, unit);
      else unit_chunks<2>(J, unit);
      break;
    case PH_PR_CONTRIB:
      if (J->paired) {
        if (prmode == PR_NORM32) unit_pr_contrib_pair<PR_NORM32>(J, unit);
        else unit_pr_contrib_pair<PR_NORM64>(J, unit);
        break;
      }
      // PageRank-delta: its residual round only (the delta rounds take the previous
      // pull's contributions)
      if (prmode == PR_DELTA_RESIDUAL) unit_pr_contrib<PR_DELTA_RESIDUAL>(J, unit);
      else if (prmode == PR_NORM32) unit_pr_contrib<PR_NORM32>(J, unit);
      else unit_pr_contrib<PR_NORM64>(J, unit);
      break;
    case PH_PR_PULL:
      if (J->paired) {
        if (prmode == PR_NORM32) unit_pr_pull_pair<PR_NORM32>(J, unit);
        else unit_pr_pull_pair<PR_NORM64>(J, unit);
        break;
      }
      if (prmode == PR_DELTA_RESIDUAL) unit_pr_pull<PR_DELTA_RESIDUAL>(J, unit);
      else if (prmode == PR_DELTA_PUSH) unit_pr_pull<PR_DELTA_PUSH>(J, unit);
      else if (prmode == PR_NORM32) unit_pr_pull<PR_NORM32>(J, unit);
      else unit_pr_pull<PR_NORM64>(J, unit);
      break;
    default:
      break;
  }
}

// Five blocks per SM (48 registers, about 1.9 KB spilled per thread): the job rounds are
// latency-bound gathers, and warps in flight matter more than the spills (64 jobs over
// RMAT-14..21 snapshots, incremental job round: 10.9-11.3 ms device time at four blocks
// per SM, 10.4-11.1 at five).
__global__ void __launch_bounds__(BT, 5) batch_kernel(const BJob* __restrict__ jobs, BSched* sched, BCtl* ctl,
                                                        int njobs) {
  __shared__ int s_job, s_state, s_last, s_mode;
  __shared__ unsigned s_unit, s_total, s_phase;
  int cursor = (int)(blockIdx.x % (unsigned)njobs);
  unsigned idle = 0;
  unsigned long long done_units = 0;
  for (;;) {
    if (threadIdx.x < 32) {
      // warp 0 reads 32 claim words at a time (one L2 round trip), in cyclic order from
      // the job this block worked on last, and claims a unit of the first open one
      const unsigned lane = threadIdx.x;
      int found = -1;
      unsigned unit = 0, total = 0, phase = 0;
      for (int base = 0; base < njobs && found < 0; base += 32) {
        const int k = base + (int)lane;
        int jj = cursor + k;
        if (jj >= njobs) jj -= njobs;
        bool open = false;
        if (k < njobs) {
          const unsigned long long cw = *(volatile unsigned long long*)&sched[jj].claim;
          open = (unsigned)cw < ((unsigned)(cw >> 32) & 0xFFFFFFu);
        }
        unsigned m = __ballot_sync(0xFFFFFFFFu, open);
        while (m) {
          const int l = __ffs(m) - 1;
          m &= m - 1;
          int got = 0;
          unsigned long long old = 0;
          if ((int)lane == l) {
            old = atomicAdd(&sched[jj].claim, 1ULL);
            got = (unsigned)old < ((unsigned)(old >> 32) & 0xFFFFFFu) ? 1 : 0;
            if (got) __threadfence();  // the phase's state was published before the claim word
          }
          got = __shfl_sync(0xFFFFFFFFu, got, l);
          if (got) {
            old = __shfl_sync(0xFFFFFFFFu, old, l);
            found = __shfl_sync(0xFFFFFFFFu, jj, l);
            unit = (unsigned)old;
            total = (unsigned)(old >> 32) & 0xFFFFFFu;
            phase = (unsigned)(old >> 56);
            break;
          }
        }
      }
      if (lane == 0) {
        int state = 0;
        if (found >= 0) {
          __threadfence();
          s_mode = *(volatile int*)&sched[found].prmode;
          idle = 0;
        } else if (*(volatile unsigned*)&ctl->jobs_left == 0 || *(volatile unsigned*)&ctl->err != 0) {
          state = 2;
        } else if (++idle > ctl->idle_limit) {
          atomicExch(&ctl->err, 1u);
          state = 2;
        } else {
          state = 1;
          __nanosleep(idle < 16 ? 100u : 800u);  // back off once the block has polled a while
        }
        s_job = found;
        s_unit = unit;
        s_total = total;
        s_phase = phase;
        s_state = state;
      }
    }
    __syncthreads();
    const int state = s_state;
    if (state == 2) break;
    if (state == 1) {
      __syncthreads();
      continue;
    }
    const int jb = s_job;
    const BJob* J = jobs + jb;
    run_unit(J, s_phase, s_unit, s_mode);
    __syncthreads();
    if (threadIdx.x == 0) {
      __threadfence();
      const unsigned d = atomicAdd(&sched[jb].done, 1u);
      s_last = (d + 1 == s_total) ? 1 : 0;
      ++done_units;
    }
    __syncthreads();
    if (s_last) {
      __threadfence();
      advance(J, sched + jb, ctl, s_phase);
    }
    cursor = jb;
  }
  if (threadIdx.x == 0 && done_units) atomicAdd(&ctl->units, done_units);
}

// Every job's loop state reset for its run, one block per job, in one launch: BFS / CC /
// SSSP / SSWP clear both parities of their row flags; PageRank-delta jobs were reset by
// their preparation (their rank sum follows the reset).
__global__ void batch_begin_kernel(const BJob* __restrict__ jobs, int count) {
  const int k = blockIdx.x;
  if (k >= count) return;
  const BJob& J = jobs[k];
  if (J.begin == 1) {
    const JobDesc* jd = J.jd;
    const uint64_t T = J.sd->T;
    uint32_t* rows = jd->rows;
    for (uint64_t i = threadIdx.x; i < 2 * T; i += blockDim.x) rows[i] = 0;
    if (threadIdx.x == 0) minprop_begin_state(jd->ls, J.max_iter);
  } else if (J.begin == 2 && threadIdx.x == 0) {
    pr_begin_state(J.ls, J.max_iter, J.tol, J.begin_edges);
  }
}

// Copies every job's loop state into one array, read back with a single copy.
__global__ void batch_stats_kernel(const BJob* __restrict__ jobs, int count, LoopState* __restrict__ out) {
  const int k = blockIdx.x;
  if (k >= count) return;
  const unsigned* src = reinterpret_cast<const unsigned*>(jobs[k].ls);
  unsigned* dst = reinterpret_cast<unsigned*>(out + k);
  for (unsigned i = threadIdx.x; i < sizeof(LoopState) / 4; i += blockDim.x) dst[i] = __ldcg(src + i);
}

// ---- host ---------------------------------------------------------------------

static bool is_pr(int algo) { return algo == CYTOM_ALGO_PR_DELTA || algo == CYTOM_ALGO_PAGERANK; }

struct BatchBuffers {
  int device = -1;
  BJob* jobs = nullptr;
  BSched* sched = nullptr;
  BCtl* ctl = nullptr;
  LoopState* d_ls = nullptr;  // the jobs' loop states after the launch
  LoopState* h_ls = nullptr;  // pinned copy
  int cap = 0;
  cudaEvent_t a = nullptr, b = nullptr;
};

static int batch_run(Ctx* const* ctxs, const int* job_ids, int count, cytom_run_stats* stats) {
  Ctx* c0 = ctxs[0];
  std::vector<Job*> jobs(count);
  std::vector<Ctx*> uniq;
  for (int k = 0; k < count; ++k) {
    Ctx* c = ctxs[k];
    if (!c) return CYTOM_ERR_INVAL;
    if (c->device != c0->device) return set_err(c0, CYTOM_ERR_INVAL, "batched jobs must share one device");
    if (job_ids[k] < 0 || job_ids[k] >= (int)c->jobs.size() || !c->jobs[job_ids[k]])
      return set_err(c0, CYTOM_ERR_INVAL, "unknown job in batch");
    jobs[k] = c->jobs[job_ids[k]];
    for (int m = 0; m < k; ++m)
      if (ctxs[m] == c && job_ids[m] == job_ids[k]) return set_err(c0, CYTOM_ERR_INVAL, "job listed twice in batch");
    if (std::find(uniq.begin(), uniq.end(), c) == uniq.end()) uniq.push_back(c);
  }
  // per snapshot: merge pending edges, refresh the source directory, then enqueue every
  // snapshot's PageRank CSC update before any is waited for (they run side by side)
  for (Ctx* c : uniq) {
    int rc = compact(c);
    if (!rc) rc = build_directory(c);
    if (rc) {
      if (c != c0) c0->err = c->err;
      return rc;
    }
  }
  for (int k = 0; k < count; ++k) {
    if (!is_pr(jobs[k]->algo)) continue;
    int rc = pagerank_csc_stage(ctxs[k]);
    if (rc) {
      if (ctxs[k] != c0) c0->err = ctxs[k]->err;
      return rc;
    }
  }

  std::vector<BJob> hj(count);
  std::vector<BSched> hs(count);
  for (int k = 0; k < count; ++k) {
    Ctx* c = ctxs[k];
    Job* j = jobs[k];
    int rc = CYTOM_OK;
    if (j->fresh) {
      rc = job_init_state(c, j);
      if (rc) return rc;
      j->fresh = false;
    }
    BJob b{};
    b.jd = j->d;
    b.sd = c->dsd;
    b.ls = j->ls;
    b.algo = j->algo;
    b.adaptive = c->cfg.enable_adaptive_scheduling;
    memset(&hs[k], 0, sizeof(BSched));
    b.max_iter = (unsigned)std::min<uint64_t>(j->params.max_iterations, 0xFFFFFFFFu);
    b.tol = j->params.tolerance;
    if (is_pr(j->algo)) {
      uint64_t nb[kPrBins];
      int mode = 0;
      uint64_t edges = 0;
      rc = pagerank_batch_prep(c, j, &b.pr, nb, &mode, &edges);
      if (rc) return rc;
      b.begin = j->algo == CYTOM_ALGO_PAGERANK ? 2u : 0u;
      b.begin_edges = edges;
      for (int bi = 0; bi < kPrBins; ++bi) b.nb[bi] = nb[bi];
      hs[k].prmode = mode;
      const uint64_t units = (c->n + BU_PR_VERTS - 1) / BU_PR_VERTS;
      if (units > kMaxUnits) return set_err(c, CYTOM_ERR_RANGE, "graph too large for the batched executor");
      hs[k].claim = (j->params.max_iterations > 0) ? pack_claim(PH_PR_CONTRIB, (unsigned)units)
                                                   : pack_claim(PH_DONE, 0);
    } else {
      b.begin = 1;
      const uint64_t units = (((c->n + 31) >> 5) + BU_APPLY_WORDS - 1) / BU_APPLY_WORDS;
      const uint64_t stages = (c->E + SG_E - 1) / SG_E;
      if (units > kMaxUnits || stages > kMaxUnits)
        return set_err(c, CYTOM_ERR_RANGE, "graph too large for the batched executor");
      hs[k].claim = pack_claim(PH_APPLY0, (unsigned)units);
    }
    hj[k] = b;
  }
  // PAGERANK jobs of one context and form run in pairs: one pass per round for both
  // (CYTOM_BATCH_PAIR=0 keeps every job on passes of its own)
  const char* pair_env = getenv("CYTOM_BATCH_PAIR");
  if (!(pair_env && pair_env[0] == '0')) {
    std::vector<char> used(count, 0);
    for (int k1 = 0; k1 < count; ++k1) {
      if (used[k1] || jobs[k1]->algo != CYTOM_ALGO_PAGERANK || (unsigned)(hs[k1].claim >> 56) == PH_DONE) continue;
      for (int k2 = k1 + 1; k2 < count; ++k2) {
        if (used[k2] || ctxs[k2] != ctxs[k1] || jobs[k2]->algo != CYTOM_ALGO_PAGERANK ||
            (unsigned)(hs[k2].claim >> 56) == PH_DONE || jobs[k2]->params.kahan != jobs[k1]->params.kahan ||
            hj[k2].pr.csc_src != hj[k1].pr.csc_src)
          continue;
        Ctx* c = ctxs[k1];
        const size_t need = (size_t)c->n * 16;  // double2 per vertex covers both forms
        if (c->pr_pair_bytes < need) {
          cudaFree(c->pr_pair);
          c->pr_pair = nullptr;
          c->pr_pair_bytes = 0;
          if (cy_malloc(&c->pr_pair, need) != cudaSuccess) {
            cudaGetLastError();
            break;  // no pair buffer: the jobs run on passes of their own
          }
          c->pr_pair_bytes = need;
        }
        hj[k1].paired = 1;
        hj[k1].pr2 = hj[k2].pr;
        hj[k1].cpair = c->pr_pair;
        hs[k2].claim = pack_claim(PH_DONE, 0);
        used[k1] = used[k2] = 1;
        break;
      }
    }
  }
  unsigned left = 0;
  for (int k = 0; k < count; ++k)
    if ((unsigned)(hs[k].claim >> 56) != PH_DONE) ++left;
  // prep work of every snapshot's stream is done before the launch
  for (Ctx* c : uniq) {
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_err(c0, e, "batch prep");
  }
  // device tables, kept by the first context and grown on demand
  BatchBuffers*& bb = reinterpret_cast<BatchBuffers*&>(c0->batch);
  if (!bb) {
    bb = new (std::nothrow) BatchBuffers();
    if (!bb) return set_err(c0, CYTOM_ERR_OOM, "batch buffers");
    cudaEventCreate(&bb->a);
    cudaEventCreate(&bb->b);
  }
  if (bb->cap < count) {
    cudaFree(bb->jobs);
    cudaFree(bb->sched);
    cudaFree(bb->d_ls);
    cudaFreeHost(bb->h_ls);
    bb->jobs = nullptr;
    bb->sched = nullptr;
    bb->d_ls = nullptr;
    bb->h_ls = nullptr;
    bb->cap = 0;
    if (cy_malloc(&bb->jobs, sizeof(BJob) * count) != cudaSuccess ||
        cy_malloc(&bb->sched, sizeof(BSched) * count) != cudaSuccess ||
        cy_malloc(&bb->d_ls, sizeof(LoopState) * count) != cudaSuccess ||
        cy_malloc_host(&bb->h_ls, sizeof(LoopState) * count) != cudaSuccess) {
      cudaGetLastError();
      return set_err(c0, CYTOM_ERR_OOM, "batch tables");
    }
    bb->cap = count;
  }
  if (!bb->ctl && cy_malloc(&bb->ctl, sizeof(BCtl)) != cudaSuccess) {
    cudaGetLastError();
    return set_err(c0, CYTOM_ERR_OOM, "batch control");
  }
  BCtl hctl{};
  // phantom jobs (fault injection) are counted as unfinished but never get work
  const unsigned launch_left = left ? left + c0->inj_phantom_jobs : 0;
  hctl.jobs_left = launch_left;
  hctl.idle_limit = c0->inj_idle_limit ? c0->inj_idle_limit : kIdleLimit;
  cudaStream_t st = c0->stream;
  cudaError_t e = cudaMemcpyAsync(bb->jobs, hj.data(), sizeof(BJob) * count, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(bb->sched, hs.data(), sizeof(BSched) * count, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(bb->ctl, &hctl, sizeof(BCtl), cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return cuda_err(c0, e, "batch upload");
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batch_kernel, BT, 0);
  per_sm = std::max(1, std::min(per_sm, 5));
  const int grid = c0->num_sms * per_sm;
  batch_begin_kernel<<<count, 256, 0, st>>>(bb->jobs, count);
  c0->launches++;
  cudaEventRecord(bb->a, st);
  if (launch_left) {
    batch_kernel<<<grid, BT, 0, st>>>(bb->jobs, bb->sched, bb->ctl, count);
    c0->launches++;
  }
  cudaEventRecord(bb->b, st);
  if (stats) {
    batch_stats_kernel<<<count, 64, 0, st>>>(bb->jobs, count, bb->d_ls);
    c0->launches++;
  }
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(&hctl, bb->ctl, sizeof(BCtl), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess && stats)
    e = cudaMemcpyAsync(bb->h_ls, bb->d_ls, sizeof(LoopState) * count, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_err(c0, e, "batch run");
  float ms = 0.f;
  cudaEventElapsedTime(&ms, bb->a, bb->b);
  c0->batch_units += hctl.units;
  if (hctl.err) {
    // the launch ended with jobs in mid-round: they restart from scratch on their next run
    for (int k = 0; k < count; ++k) jobs[k]->fresh = true;
    if (hctl.err == 1) return set_err(c0, CYTOM_ERR_TIMEOUT, "batched executor: a block found no work for too long");
    return set_err(c0, CYTOM_ERR_RANGE, "batched executor: a phase exceeds the unit limit");
  }
  for (int k = 0; k < count; ++k) {
    Job* j = jobs[k];
    j->last_run_graph = false;
    if (!stats) continue;
    const LoopState& ls = bb->h_ls[k];
    cytom_run_stats& s = stats[k];
    memset(&s, 0, sizeof(s));
    s.iterations = ls.iter;
    s.count_edges = ls.count_edges;
    s.edges_scanned = ls.edges_scanned;
    s.active_vertices = ls.active_total;
    s.converged = ls.cont == 0 ? 1 : 0;
    s.residual = ls.resid_final;
    s.elapsed_ms = ms;
  }
  return CYTOM_OK;
}

void batch_free(Ctx* c) {
  BatchBuffers* bb = reinterpret_cast<BatchBuffers*>(c->batch);
  if (!bb) return;
  if (bb->jobs) cudaFree(bb->jobs);
  if (bb->sched) cudaFree(bb->sched);
  if (bb->ctl) cudaFree(bb->ctl);
  if (bb->d_ls) cudaFree(bb->d_ls);
  if (bb->h_ls) cudaFreeHost(bb->h_ls);
  if (bb->a) cudaEventDestroy(bb->a);
  if (bb->b) cudaEventDestroy(bb->b);
  delete bb;
  c->batch = nullptr;
}

}  // namespace cytom

using namespace cytom;

extern "C" int cytom_run_batch(cytom_ctx* const* ctxs, const int* job_ids, int count, cytom_run_stats* stats) {
  if (!ctxs || !job_ids || count <= 0 || !ctxs[0]) return CYTOM_ERR_INVAL;
  Ctx* const* cs = reinterpret_cast<Ctx* const*>(ctxs);
  for (int k = 0; k < count; ++k)
    if (cs[k]) settle_runs(cs[k]);
  int dev = -1;
  cudaGetDevice(&dev);
  if (dev != cs[0]->device) cudaSetDevice(cs[0]->device);
  int rc = batch_run(cs, job_ids, count, stats);
  if (dev >= 0 && dev != cs[0]->device) cudaSetDevice(dev);
  return rc;
}

extern "C" int cytom_batch_units(const cytom_ctx* ctx, uint64_t* units) {
  const Ctx* c = reinterpret_cast<const Ctx*>(ctx);
  if (!c || !units) return CYTOM_ERR_INVAL;
  *units = c->batch_units;
  return CYTOM_OK;
}
