// pagerank_dev.cuh — device building blocks of one PageRank-family round, shared by the
// one-job kernels (exec_pagerank.cu) and the batched persistent executor (exec_batch.cu).
//
// A round: per-source contributions (and the dangling mass), then a pull over the
// target-sorted CSC — each target's in-edges summed in a fixed order with Neumaier
// compensation, 1 / 4 / 8 / 32 lanes or a whole block per target by in-degree bin —
// then the control step (FP64 residual, convergence). PageRank-delta is
// examples/pagerank-delta.cc (pullGather :127-132, apply :142-174); PAGERANK is the
// normalised PageRank with dangling-mass redistribution.
//
// Fused form (PageRank-delta; pr_fused): a target's new delta fixes its contribution to
// the next round, so the pull writes it as it finishes each target. Contributions are
// kept by round parity: round p reads half p and writes half p^1. Only a run's first
// (residual) round needs a contribution pass. The PAGERANK forms keep the pass: at RMAT
// scale 26 their pull's scattered per-target writes cost more than the pass's streamed ones.
//
// Load policy as in minprop_dev.cuh: PERSIST = the persistent kernel, which reads every
// value written in the same launch (ranks, contributions) through L2.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

#include "engine.h"

namespace cytom {

// Targets are binned by in-degree: bin k holds in-degrees in (pr_bin_hi(k-1), pr_bin_hi(k)];
// its pull uses pr_bin_vw(k) lanes per target (1 = one thread, 0 = one whole block).
constexpr int kPrBins = 5;
__host__ __device__ constexpr uint32_t pr_bin_hi(int k) {
  return k == 0 ? 4u : k == 1 ? 32u : k == 2 ? 256u : k == 3 ? 4096u : 0xFFFFFFFFu;
}
__host__ __device__ constexpr int pr_bin_vw(int k) { return k == 0 ? 1 : k == 1 ? 4 : k == 2 ? 8 : k == 3 ? 32 : 0; }
constexpr int PR_T = 256;
constexpr int PR_BLOCK_T = 256;

// PR_W*: weighted PageRank r = (1-alpha) t + alpha (P r + D t), P[v,u] = w_uv / s_u
// (pull over the CSC with its raw weights; s_u = sum of u's out-weights; t = teleport).
// PR_ADJ*: its adjoint lambda = c + alpha (P^T lambda + a (t . lambda)) (pull over the
// source-major CSR; a_u = 1 when s_u = 0). 32 = FP32 values with compensated sums,
// 64 = FP64 plain.
enum PrMode {
  PR_DELTA_RESIDUAL = 0,
  PR_DELTA_PUSH = 1,
  PR_NORM32 = 2,
  PR_NORM64 = 3,
  PR_W32 = 4,
  PR_W64 = 5,
  PR_ADJ32 = 6,
  PR_ADJ64 = 7
};
template <int MODE>
__host__ __device__ constexpr bool pr_is64() {
  return MODE == PR_NORM64 || MODE == PR_W64 || MODE == PR_ADJ64;
}
template <int MODE>
__host__ __device__ constexpr bool pr_weighted() {
  return MODE >= PR_W32;
}
template <int MODE>
__host__ __device__ constexpr bool pr_fused() {
  return MODE == PR_DELTA_RESIDUAL || MODE == PR_DELTA_PUSH;
}
// Value type of the contributions (and of a lane's partial sums before the merge).
template <int MODE>
using pr_val_t = typename std::conditional<pr_is64<MODE>(), double, float>::type;

// Compensated accumulation (Neumaier): true sum ~= s + e.
struct Acc32 {
  float s, e;
  __device__ __forceinline__ void init() { s = 0.f, e = 0.f; }
  __device__ __forceinline__ void add(float x) {
    const float t = s + x;
    if (fabsf(s) >= fabsf(x)) e += (s - t) + x;
    else e += (x - t) + s;
    s = t;
  }
  __device__ __forceinline__ void merge(float s2, float e2) {
    const float t = s + s2;
    float err;
    if (fabsf(s) >= fabsf(s2)) err = (s - t) + s2;
    else err = (s2 - t) + s;
    s = t;
    e += e2 + err;
  }
  __device__ __forceinline__ float value() const { return s + e; }
};

struct Acc64 {
  double s;
  __device__ __forceinline__ void init() { s = 0.0; }
  __device__ __forceinline__ void add(double x) { s += x; }
  __device__ __forceinline__ void merge(double s2, double) { s += s2; }
  __device__ __forceinline__ double value() const { return s; }
};

// Float-float numbers: an unevaluated pair hi + lo of FP32 values (about 44 significant
// bits), built from error-free transformations -- Knuth's two-sum, Dekker's fast two-sum
// (|a| >= |b|) and the FMA-exact product. GB300 runs FP64 at a small fraction of its FP32
// rate, so the FP32-compensated PageRank keeps its per-target arithmetic (update, change,
// dangling mass) in this form instead of FP64. The _rn intrinsics keep the compiler from
// contracting the transformations' products and sums into FMAs.
struct FF {
  float hi, lo;
};
__device__ __forceinline__ FF ff_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  return {s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}
__device__ __forceinline__ FF ff_fast_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ FF ff_add(FF a, FF b) {
  const FF s = ff_two_sum(a.hi, b.hi);
  const FF t = ff_two_sum(a.lo, b.lo);
  const FF u = ff_fast_two_sum(s.hi, __fadd_rn(s.lo, t.hi));
  return ff_fast_two_sum(u.hi, __fadd_rn(u.lo, t.lo));
}
__device__ __forceinline__ FF ff_mul(FF a, FF b) {
  const float p = __fmul_rn(a.hi, b.hi);
  const float e = __fmaf_rn(a.hi, b.hi, -p);
  return ff_fast_two_sum(p, __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, e)));
}
__device__ __forceinline__ FF ff_abs(FF a) { return a.hi < 0.f ? FF{-a.hi, -a.lo} : a; }
__host__ __device__ inline FF ff_from_double(double x) {
  const float hi = (float)x;
  return {hi, (float)(x - (double)hi)};
}

struct PrArgs {
  const uint32_t* csc_src;
  const uint32_t* csc_ptr;
  const uint32_t* bins;     // targets grouped by in-degree bin (pr_bin_hi), bin after bin
  uint64_t bin_off, bin_count;
  const uint32_t* deg;      // out-degree used for contributions
  float* rank;
  float* comp;
  float* delta;
  float* contrib;           // FP32 contributions (PageRank-delta: 2 x n, by parity)
  double* r64;
  double* r64n;
  double* contrib64;        // FP64 contributions
  float* lo0;               // FP32 PAGERANK / WPAGERANK: low words of the ranks (rank + lo0,
  float* lo1;               //   comp + lo1): each rank is carried as an unevaluated float pair
  const float* csc_w;       // weighted modes: raw weight of each in-edge (CSC) / out-edge (CSR)
  const double* wsum;       // weighted modes: out-weight sum s_u of each vertex
  const double* tele;       // weighted modes: teleport vector (NULL = uniform 1/n)
  const double* cvec;       // adjoint: the loss weights c
  float* pt;                // adjoint FP32: (P^T lambda)_u of the last round
  double* pt64;             // adjoint FP64
  LoopState* ls;
  uint64_t n;
  double alpha, delta_param, base;
  FF alpha_ff, base_ff, inv_n_ff;  // alpha, base and 1/n as float-float (pr_args_ff)
};

// Fills the float-float copies of alpha, base and 1/n (host, after those are set).
inline void pr_args_ff(PrArgs& a) {
  a.alpha_ff = ff_from_double(a.alpha);
  a.base_ff = ff_from_double(a.base);
  a.inv_n_ff = ff_from_double(a.n ? 1.0 / (double)a.n : 0.0);
}

// A round's sums and the dangling term: float-float in the FP32-compensated form, FP64
// in the others.
template <int MODE>
using pr_ff_t = typename std::conditional<MODE == PR_NORM32, FF, double>::type;

template <bool PERSIST, class T>
__device__ __forceinline__ T pr_ld(const T* p) {
  if constexpr (PERSIST) return __ldcg(p);
  else return *p;
}

// The contributions round p reads (fused form: half p; the others: the one vector).
template <int MODE>
__device__ __forceinline__ const pr_val_t<MODE>* pr_cread(const PrArgs& a, unsigned p) {
  const uint64_t off = pr_fused<MODE>() ? (uint64_t)p * a.n : 0;
  if constexpr (pr_is64<MODE>()) return a.contrib64 + off;
  else return a.contrib + off;
}

// Contribution of in-edge e with source s: cr[s], times the edge's raw weight in the
// weighted modes (an FP32 product in the FP32 modes).
template <int MODE, bool PERSIST>
__device__ __forceinline__ pr_val_t<MODE> pr_cval(const PrArgs& a, const pr_val_t<MODE>* cr, uint32_t e, uint32_t s) {
  const pr_val_t<MODE> c = pr_ld<PERSIST>(cr + s);
  if constexpr (pr_weighted<MODE>()) return c * (pr_val_t<MODE>)a.csc_w[e];
  else return c;
}

// Contributions of the sources handled by this thread (u = lo + tid, lo + tid + nthr, ...
// below hi): PageRank-delta's residual round (every source contributes rank / outdeg;
// its later rounds take the previous pull's contributions) and every round of the
// other forms.
// Returns the thread's share of the dangling mass (PAGERANK).
template <int MODE, bool PERSIST>
__device__ __forceinline__ pr_ff_t<MODE> pr_contrib_range(const PrArgs& a, unsigned p, uint64_t lo, uint64_t hi,
                                                          uint64_t tid, uint64_t nthr) {
  pr_ff_t<MODE> dangling{};
  if constexpr (MODE == PR_DELTA_RESIDUAL || MODE == PR_DELTA_PUSH) {
    float* cw = a.contrib + (uint64_t)p * a.n;
    for (uint64_t u = lo + tid; u < hi; u += nthr) {
      const uint32_t d = a.deg[u];
      cw[u] = d ? pr_ld<PERSIST>(a.rank + u) / (float)d : 0.f;
    }
  } else if constexpr (MODE == PR_NORM32) {
    const float* r = (p == 0) ? a.rank : a.comp;
    const float* rl = (p == 0) ? a.lo0 : a.lo1;
    float* cw = a.contrib;
    // the contribution is an FP32 quotient of the high word (the low word is below its
    // rounding); the low word enters the FP64 dangling sum and the residual
    for (uint64_t u = lo + tid; u < hi; u += nthr) {
      const uint32_t d = a.deg[u];
      const float rh = pr_ld<PERSIST>(r + u);
      cw[u] = d ? rh / (float)d : 0.f;
      if (!d) dangling = ff_add(dangling, FF{rh, pr_ld<PERSIST>(rl + u)});
    }
  } else if constexpr (MODE == PR_W32) {
    const float* r = (p == 0) ? a.rank : a.comp;
    const float* rl = (p == 0) ? a.lo0 : a.lo1;
    for (uint64_t u = lo + tid; u < hi; u += nthr) {
      const double s = a.wsum[u];
      const float rh = pr_ld<PERSIST>(r + u);
      a.contrib[u] = s > 0.0 ? rh / (float)s : 0.f;
      if (!(s > 0.0)) dangling += (double)rh + (double)pr_ld<PERSIST>(rl + u);
    }
  } else if constexpr (MODE == PR_W64) {
    const double* r = (p == 0) ? a.r64 : a.r64n;
    for (uint64_t u = lo + tid; u < hi; u += nthr) {
      const double s = a.wsum[u];
      const double rv = pr_ld<PERSIST>(r + u);
      a.contrib64[u] = s > 0.0 ? rv / s : 0.0;
      if (!(s > 0.0)) dangling += rv;
    }
  } else if constexpr (MODE == PR_ADJ32) {
    // gather source = lambda itself; the returned sum is t . lambda
    const float* l = (p == 0) ? a.rank : a.comp;
    const double tu = 1.0 / (double)a.n;
    for (uint64_t u = lo + tid; u < hi; u += nthr) {
      const float lv = pr_ld<PERSIST>(l + u);
      a.contrib[u] = lv;
      dangling += (a.tele ? a.tele[u] : tu) * (double)lv;
    }
  } else if constexpr (MODE == PR_ADJ64) {
    const double* l = (p == 0) ? a.r64 : a.r64n;
    const double tu = 1.0 / (double)a.n;
    for (uint64_t u = lo + tid; u < hi; u += nthr) {
      const double lv = pr_ld<PERSIST>(l + u);
      a.contrib64[u] = lv;
      dangling += (a.tele ? a.tele[u] : tu) * lv;
    }
  } else {
    const double* r = (p == 0) ? a.r64 : a.r64n;
    double* cw = a.contrib64;
    for (uint64_t u = lo + tid; u < hi; u += nthr) {
      const uint32_t d = a.deg[u];
      const double rv = pr_ld<PERSIST>(r + u);
      cw[u] = d ? rv / (double)d : 0.0;
      if (!d) dangling += rv;
    }
  }
  return dangling;
}

// Warp-reduced dangling mass into the loop state (every lane calls it).
template <int MODE>
__device__ __forceinline__ void pr_dangling_flush(LoopState* ls, unsigned p, pr_ff_t<MODE> dangling) {
  if constexpr (MODE == PR_NORM32) {
    // float-float warp sum; one conversion per warp
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
      dangling = ff_add(dangling, FF{__shfl_xor_sync(0xFFFFFFFFu, dangling.hi, o),
                                     __shfl_xor_sync(0xFFFFFFFFu, dangling.lo, o)});
    if ((threadIdx.x & 31) == 0 && dangling.hi != 0.f)
      atomicAdd(&ls->dangling[p], (double)dangling.hi + (double)dangling.lo);
  } else if constexpr (MODE >= PR_NORM32) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) dangling += __shfl_xor_sync(0xFFFFFFFFu, dangling, o);
    if ((threadIdx.x & 31) == 0 && dangling != 0.0) atomicAdd(&ls->dangling[p], dangling);
  }
}

// The round's dangling term as pr_finish takes it: D / n (normalised PageRank), D
// (weighted: scaled by t_v in pr_finish), t . lambda (adjoint), none (PageRank-delta).
template <int MODE, bool PERSIST>
__device__ __forceinline__ pr_ff_t<MODE> pr_dang_arg(const PrArgs& a, const LoopState* ls, unsigned p) {
  if constexpr (MODE == PR_NORM32) {
    return ff_mul(ff_from_double(pr_ld<PERSIST>(&ls->dangling[p])), a.inv_n_ff);
  } else {
    if (MODE < PR_NORM32) return 0.0;
    const double d = pr_ld<PERSIST>(&ls->dangling[p]);
    return MODE == PR_NORM64 ? d / (double)a.n : d;
  }
}

// The normalised forms' rank of v before the round (FP32: high and low word; FP64: d),
// loaded ahead of the sum by the batched executor's pulls.
struct PrOld {
  double d;
  float hi, lo;
};
template <int MODE, bool PERSIST>
__device__ __forceinline__ PrOld pr_load_old(const PrArgs& a, uint64_t v, unsigned p) {
  PrOld o{};
  if constexpr (MODE == PR_NORM32) {
    o.hi = pr_ld<PERSIST>(((p == 0) ? a.rank : a.comp) + v);
    o.lo = pr_ld<PERSIST>(((p == 0) ? a.lo0 : a.lo1) + v);
  } else {
    o.d = pr_ld<PERSIST>(((p == 0) ? a.r64 : a.r64n) + v);
  }
  return o;
}

// The update of target v (pr_finish); returns |change| for the FP64 residual.
template <int MODE, bool PERSIST>
__device__ __forceinline__ double pr_apply(const PrArgs& a, uint64_t v, double sum, unsigned p, double dang,
                                           double* rsum, unsigned* nact) {
  if (MODE == PR_W32 || MODE == PR_W64) {
    const double tv = a.tele ? a.tele[v] : 1.0 / (double)a.n;
    const double nv = tv * ((1.0 - a.alpha) + a.alpha * dang) + a.alpha * sum;
    if (MODE == PR_W32) {
      const float* r = (p == 0) ? a.rank : a.comp;
      const float* rl = (p == 0) ? a.lo0 : a.lo1;
      float* rn = (p == 0) ? a.comp : a.rank;
      float* rnl = (p == 0) ? a.lo1 : a.lo0;
      const float hi = (float)nv;
      rn[v] = hi;
      rnl[v] = (float)(nv - (double)hi);
      *rsum += nv;
      return fabs(nv - ((double)pr_ld<PERSIST>(r + v) + (double)pr_ld<PERSIST>(rl + v)));
    } else {
      const double* r = (p == 0) ? a.r64 : a.r64n;
      double* rn = (p == 0) ? a.r64n : a.r64;
      rn[v] = nv;
      *rsum += nv;
      return fabs(nv - pr_ld<PERSIST>(r + v));
    }
  } else if (MODE == PR_ADJ32 || MODE == PR_ADJ64) {
    // v is a source here: lambda'_v = c_v + alpha ((P^T lambda)_v + a_v (t . lambda))
    const double s = a.wsum[v];
    const double ptv = s > 0.0 ? sum / s : 0.0;
    const double nl = a.cvec[v] + a.alpha * (ptv + (s > 0.0 ? 0.0 : dang));
    if (MODE == PR_ADJ32) {
      const float* l = (p == 0) ? a.rank : a.comp;
      float* ln = (p == 0) ? a.comp : a.rank;
      const float nf = (float)nl;
      ln[v] = nf;
      a.pt[v] = (float)ptv;
      *rsum += (double)nf;
      return fabs((double)nf - (double)pr_ld<PERSIST>(l + v));
    } else {
      const double* l = (p == 0) ? a.r64 : a.r64n;
      double* ln = (p == 0) ? a.r64n : a.r64;
      ln[v] = nl;
      a.pt64[v] = ptv;
      *rsum += nl;
      return fabs(nl - pr_ld<PERSIST>(l + v));
    }
  } else {
    // PageRank-delta: residual round or delta round, rank += change (compensated)
    const float rank_v = pr_ld<PERSIST>(a.rank + v);
    const float comp_v = pr_ld<PERSIST>(a.comp + v);
    float change;
    if (MODE == PR_DELTA_RESIDUAL) {
      change = (float)((1.0 - a.alpha) + a.alpha * sum - (double)rank_v - (double)comp_v);
    } else {
      change = (sum == 0.0) ? 0.f : (float)(a.alpha * sum);
    }
    a.delta[v] = change;
    // Kahan: rank + comp carries the exact running sum of the changes
    const float y = change + comp_v;
    const float t = rank_v + y;
    a.comp[v] = y - (t - rank_v);
    a.rank[v] = t;
    *rsum += (double)change;
    // v stays active (contributes delta / outdeg next round) while |delta| > delta_param * rank
    const bool act = change != 0.f && (double)fabsf(change) > a.delta_param * (double)t;
    *nact += act ? 1u : 0u;
    const uint32_t dg = a.deg[v];
    a.contrib[(uint64_t)(p ^ 1u) * a.n + v] = (act && dg) ? change / (float)dg : 0.f;
    return fabs((double)change);
  }
}

// A thread's share of a round's totals: FP64 residual (sum of |change|), rank sum and
// the vertices activated for the next round (PageRank-delta). Flushed once per block
// (pr_tally_flush).
struct PrTally {
  double resid, rsum;
  FF fres;  // FP32-compensated form: the residual in float-float
  unsigned nact;
  __device__ __forceinline__ void init() { resid = rsum = 0.0, fres = FF{0.f, 0.f}, nact = 0u; }
};

// The normalised forms' update of v from its sum and its rank before the round; the
// residual share goes to the tally (the rank sum is not kept: their control step does
// not read it). FP32-compensated: nv = base + alpha (sum + D/n) in float-float, stored as
// its high and low words; FP64: the same in FP64.
template <int MODE>
__device__ __forceinline__ void pr_apply_norm(const PrArgs& a, uint64_t v, pr_ff_t<MODE> sum, unsigned p,
                                              pr_ff_t<MODE> dang, PrOld o, PrTally& t) {
  if constexpr (MODE == PR_NORM32) {
    float* rn = (p == 0) ? a.comp : a.rank;
    float* rnl = (p == 0) ? a.lo1 : a.lo0;
    const FF nv = ff_add(a.base_ff, ff_mul(a.alpha_ff, ff_add(sum, dang)));
    rn[v] = nv.hi;
    rnl[v] = nv.lo;
    t.fres = ff_add(t.fres, ff_abs(ff_add(nv, FF{-o.hi, -o.lo})));
  } else {
    double* rn = (p == 0) ? a.r64n : a.r64;
    const double nv = a.base + a.alpha * (sum + dang);
    rn[v] = nv;
    t.resid += fabs(nv - o.d);
  }
}

// Applies the finished sum of target v and adds its share to the tally. The fused form
// also writes v's contribution to the next round (half p^1), exactly as the
// contribution pass would compute it from the new delta.
template <int MODE, bool PERSIST>
__device__ __forceinline__ void pr_finish(const PrArgs& a, uint64_t v, pr_ff_t<MODE> sum, unsigned p,
                                          pr_ff_t<MODE> dang, PrTally& t) {
  if constexpr (MODE == PR_NORM32 || MODE == PR_NORM64)
    pr_apply_norm<MODE>(a, v, sum, p, dang, pr_load_old<MODE, PERSIST>(a, v, p), t);
  else
    t.resid += pr_apply<MODE, PERSIST>(a, v, sum, p, dang, &t.rsum, &t.nact);
}

// The block's tally into the loop state: one atomic per quantity and block (every
// thread of the block calls it). Residual and rank sum of round p; the next round's
// activations by parity p^1.
template <int MODE>
__device__ __forceinline__ void pr_tally_flush(LoopState* ls, unsigned p, PrTally t) {
  __shared__ double s_r[32], s_s[32];
  __shared__ unsigned s_n[32];
  constexpr bool kN = pr_fused<MODE>();  // activations (PageRank-delta)
  constexpr bool kS = MODE != PR_NORM32 && MODE != PR_NORM64;  // rank sum kept
  if (!kN) t.nact = 0u;
  if constexpr (MODE == PR_NORM32) {
    // float-float warp sum of the residual; one conversion per warp
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
      t.fres = ff_add(t.fres, FF{__shfl_xor_sync(0xFFFFFFFFu, t.fres.hi, o), __shfl_xor_sync(0xFFFFFFFFu, t.fres.lo, o)});
    t.resid = (double)t.fres.hi + (double)t.fres.lo;
  } else {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t.resid += __shfl_xor_sync(0xFFFFFFFFu, t.resid, o);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    if (kS) t.rsum += __shfl_xor_sync(0xFFFFFFFFu, t.rsum, o);
    if (kN) t.nact += __shfl_xor_sync(0xFFFFFFFFu, t.nact, o);
  }
  const unsigned w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  if ((threadIdx.x & 31) == 0) {
    s_r[w] = t.resid;
    s_s[w] = t.rsum;
    s_n[w] = t.nact;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double r = 0.0, sm = 0.0;
    unsigned na = 0;
    for (unsigned k = 0; k < nw; ++k) {
      r += s_r[k];
      sm += s_s[k];
      na += s_n[k];
    }
    if (r != 0.0) atomicAdd(&ls->resid[p], r);
    if (sm != 0.0) atomicAdd(&ls->rank_sum[p], sm);
    if (kN && na) atomicAdd(&ls->active[p ^ 1u], na);
  }
  __syncthreads();
}

// One lane's ordered sum of the in-edges e0, e0 + stride, ... below hi into acc: the
// source ids of B edges, then their B contributions in flight, the next B ids loaded
// while those contributions arrive (one dependent L2 round trip per B edges).
template <int MODE, bool PERSIST, int B, class Acc>
__device__ __forceinline__ void pr_lane_sum(const PrArgs& a, const pr_val_t<MODE>* cr, uint32_t e0, uint32_t hi,
                                            uint32_t stride, Acc& acc) {
  // 32-bit edge indices: the CSC holds fewer than 2^32 - 2^20 edges (build_csx), so
  // e + B * stride cannot wrap
  uint32_t id[B];
#pragma unroll
  for (int k = 0; k < B; ++k) {
    const uint32_t e = e0 + (uint32_t)k * stride;
    id[k] = e < hi ? __ldcs(a.csc_src + e) : 0u;  // streamed: keep L1 for the gathered contributions
  }
  for (uint32_t e = e0; e < hi; e += (uint32_t)B * stride) {
    pr_val_t<MODE> c[B];
#pragma unroll
    for (int k = 0; k < B; ++k) {
      const uint32_t ek = e + (uint32_t)k * stride;
      c[k] = ek < hi ? pr_cval<MODE, PERSIST>(a, cr, ek, id[k]) : (pr_val_t<MODE>)0;
    }
    const uint32_t en = e + (uint32_t)B * stride;
#pragma unroll
    for (int k = 0; k < B; ++k) {
      const uint32_t ek = en + (uint32_t)k * stride;
      id[k] = ek < hi ? __ldcs(a.csc_src + ek) : 0u;
    }
#pragma unroll
    for (int k = 0; k < B; ++k)
      if (e + (uint32_t)k * stride < hi) acc.add(c[k]);
  }
}

// A compensated FP32 sum as the update takes it: the float pair itself in the
// FP32-compensated form, s + e in FP64 in the other FP32 forms.
template <int MODE>
__device__ __forceinline__ pr_ff_t<MODE> pr_acc32_out(float s, float e) {
  if constexpr (MODE == PR_NORM32) return FF{s, e};
  else return (double)s + (double)e;
}

// Sum of target v's in-edge contributions by one thread (in-degree <= 4), in edge order.
template <int MODE, bool PERSIST>
__device__ __forceinline__ pr_ff_t<MODE> pr_sum_thread(const PrArgs& a, const pr_val_t<MODE>* cr, uint32_t v) {
  const uint32_t lo = a.csc_ptr[v], hi = a.csc_ptr[v + 1];
  if constexpr (pr_is64<MODE>()) {
    Acc64 acc;
    acc.init();
    pr_lane_sum<MODE, PERSIST, 4>(a, cr, lo, hi, 1u, acc);
    return acc.value();
  } else {
    Acc32 acc;
    acc.init();
    pr_lane_sum<MODE, PERSIST, 4>(a, cr, lo, hi, 1u, acc);
    return pr_acc32_out<MODE>(acc.s, acc.e);
  }
}

// The same by a group of VW lanes (lanes of one group are VW consecutive lanes of a
// warp; every lane of the warp calls it, an idle group with lo = hi): lane gl of the
// group sums edges lo+gl, lo+gl+VW, ... in order, then the group merges its lanes by an
// xor tree. Every lane of the group returns the sum.
template <int MODE, bool PERSIST, int VW>
__device__ __forceinline__ pr_ff_t<MODE> pr_sum_group(const PrArgs& a, const pr_val_t<MODE>* cr, uint32_t lo, uint32_t hi,
                                               unsigned gl) {
  constexpr int B = 4;
  if constexpr (pr_is64<MODE>()) {
    Acc64 acc;
    acc.init();
    pr_lane_sum<MODE, PERSIST, B>(a, cr, lo + gl, hi, VW, acc);
    double s = acc.s;
#pragma unroll
    for (int o = VW / 2; o > 0; o >>= 1) s += __shfl_xor_sync(0xFFFFFFFFu, s, o, VW);
    return s;
  } else {
    Acc32 acc;
    acc.init();
    pr_lane_sum<MODE, PERSIST, B>(a, cr, lo + gl, hi, VW, acc);
#pragma unroll
    for (int o = VW / 2; o > 0; o >>= 1) {
      const float s2 = __shfl_xor_sync(0xFFFFFFFFu, acc.s, o, VW);
      const float e2 = __shfl_xor_sync(0xFFFFFFFFu, acc.e, o, VW);
      acc.merge(s2, e2);
    }
    return pr_acc32_out<MODE>(acc.s, acc.e);
  }
}

// The same by a whole block (in-degree > 4096: RMAT hubs; up to 1024 threads); thread 0
// returns the sum. Every thread of the block calls it.
template <int MODE, bool PERSIST>
__device__ __forceinline__ pr_ff_t<MODE> pr_sum_block(const PrArgs& a, const pr_val_t<MODE>* cr, uint32_t v) {
  __shared__ float s_s[32], s_e[32];
  __shared__ double s_d[32];
  const unsigned lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const uint32_t lo = a.csc_ptr[v], hi = a.csc_ptr[v + 1];
  pr_ff_t<MODE> sum{};
  if constexpr (pr_is64<MODE>()) {
    Acc64 acc;
    acc.init();
    pr_lane_sum<MODE, PERSIST, 4>(a, cr, lo + threadIdx.x, hi, blockDim.x, acc);
    double s = acc.s;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xFFFFFFFFu, s, o);
    if (lane == 0) s_d[wid] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
      for (unsigned k = 0; k < nw; ++k) sum += s_d[k];
    }
  } else {
    Acc32 acc;
    acc.init();
    pr_lane_sum<MODE, PERSIST, 4>(a, cr, lo + threadIdx.x, hi, blockDim.x, acc);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const float s2 = __shfl_xor_sync(0xFFFFFFFFu, acc.s, o);
      const float e2 = __shfl_xor_sync(0xFFFFFFFFu, acc.e, o);
      acc.merge(s2, e2);
    }
    if (lane == 0) {
      s_s[wid] = acc.s;
      s_e[wid] = acc.e;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      Acc32 t;
      t.init();
      for (unsigned k = 0; k < nw; ++k) t.merge(s_s[k], s_e[k]);
      sum = pr_acc32_out<MODE>(t.s, t.e);
    }
  }
  __syncthreads();
  return sum;
}

// The loop state of a PageRank-family run before its first round (one thread); every
// round reads every stored edge once (teps[0] = edges).
__device__ __forceinline__ void pr_begin_state(LoopState* ls, unsigned max_iter, double tol, unsigned long long edges) {
  ls->iter = 0;
  ls->sel_rounds = 0;
  ls->apply_done = 0;
  ls->max_iter = max_iter;
  ls->cont = max_iter > 0 ? 1u : 0u;
  ls->err = 0;
  ls->active[0] = ls->active[1] = 0;
  ls->teps[0] = edges;
  ls->teps[1] = 0;
  ls->count_edges = 0;
  ls->edges_scanned = 0;
  ls->active_total = 0;
  ls->resid[0] = ls->resid[1] = 0.0;
  ls->rank_sum[0] = ls->rank_sum[1] = 0.0;
  ls->dangling[0] = ls->dangling[1] = 0.0;
  ls->tol = tol;
  ls->resid_final = 0.0;
  ls->base_sum = 0.0;
  ls->change_sum = 0.0;
  ls->best_resid = 1.0e300;
  ls->stall = 0;
}

// Ends a round: records the FP64 residual, decides whether to continue (one thread).
// Every value the step reads is loaded from L2 up front (one round trip; the other
// blocks' totals are complete and visible when it runs), then the new state is stored.
__device__ __forceinline__ unsigned pr_control_step(LoopState* ls, int mode) {
  if (__ldcg(&ls->cont) == 0u) return 0u;
  const unsigned iter = __ldcg(&ls->iter), max_iter = __ldcg(&ls->max_iter);
  const double resid_p[2] = {__ldcg(&ls->resid[0]), __ldcg(&ls->resid[1])};
  const double rsum_p[2] = {__ldcg(&ls->rank_sum[0]), __ldcg(&ls->rank_sum[1])};
  const unsigned act_p[2] = {__ldcg(&ls->active[0]), __ldcg(&ls->active[1])};
  const double change_sum = __ldcg(&ls->change_sum), base_sum = __ldcg(&ls->base_sum);
  const double tol = __ldcg(&ls->tol), best = __ldcg(&ls->best_resid);
  const unsigned long long active_total = __ldcg(&ls->active_total), count_edges = __ldcg(&ls->count_edges);
  const unsigned long long edges_scanned = __ldcg(&ls->edges_scanned), teps0 = __ldcg(&ls->teps[0]);
  const unsigned stall = __ldcg(&ls->stall);
  const bool delta_mode = mode == PR_DELTA_RESIDUAL || mode == PR_DELTA_PUSH;

  const unsigned p = iter & 1u, q = p ^ 1u;
  const double resid = resid_p[p];
  ls->resid_final = resid;
  double cs = change_sum;
  if (delta_mode) {
    cs = change_sum + rsum_p[p];
    ls->change_sum = cs;
    ls->active_total = active_total + act_p[q];
  }
  ls->count_edges = count_edges + teps0;
  ls->edges_scanned = edges_scanned + teps0;
  ls->iter = iter + 1u;
  bool more = iter + 1u < max_iter;
  if (delta_mode) {
    const double total = base_sum + cs;
    more = more && act_p[q] > 0;
    if (tol > 0.0) more = more && resid > tol * total;
  } else {
    more = more && resid > tol;
    // FP32 ranks cannot change by less than their rounding floor (about 6e-8 of the rank
    // mass per round); once the FP64-measured change stops shrinking, the run is done
    if (mode == PR_NORM32 || mode == PR_W32 || mode == PR_ADJ32) {
      if (resid < best * 0.999) {
        ls->best_resid = resid;
        ls->stall = 0;
      } else {
        ls->stall = stall + 1u;
        if (stall + 1u >= 4) more = false;
      }
    }
  }
  ls->resid[q] = 0.0;
  ls->dangling[q] = 0.0;
  ls->active[p] = 0;
  ls->rank_sum[q] = 0.0;
  ls->cont = more ? 1u : 0u;
  return more ? 1u : 0u;
}

}  // namespace cytom
