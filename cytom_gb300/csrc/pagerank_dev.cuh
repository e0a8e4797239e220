// pagerank_dev.cuh — device building blocks of one PageRank-family round, shared by the
// one-job kernels (exec_pagerank.cu) and the batched persistent executor (exec_batch.cu).
//
// A round: per-source contributions (and the dangling mass), then a pull over the
// target-sorted CSC — each target's in-edges summed in a fixed order with Neumaier
// compensation, one thread (in-degree <= 16), one warp (<= 4096) or one block (more)
// per target — then the control step (FP64 residual, convergence). PageRank-delta is
// examples/pagerank-delta.cc (pullGather :127-132, apply :142-174); PAGERANK is the
// normalised PageRank with dangling-mass redistribution.
//
// Load policy as in minprop_dev.cuh: PERSIST = the persistent kernel, which reads every
// value written in the same launch (ranks, contributions) through L2.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

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

struct PrArgs {
  const uint32_t* csc_src;
  const uint32_t* csc_ptr;
  const uint32_t* bins;     // targets grouped by in-degree bin (pr_bin_hi), bin after bin
  uint64_t bin_off, bin_count;
  const uint32_t* deg;      // out-degree used for contributions
  float* rank;
  float* comp;
  float* delta;
  float* contrib;
  double* r64;
  double* r64n;
  double* contrib64;
  uint32_t* fa2;            // 2 x nwords (PR_DELTA)
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
  uint64_t nwords;
  double alpha, delta_param, base;
};

template <bool PERSIST, class T>
__device__ __forceinline__ T pr_ld(const T* p) {
  if constexpr (PERSIST) return __ldcg(p);
  else return *p;
}

// Contribution of in-edge e with source s: contrib[s], times the edge's raw weight in
// the weighted modes (an FP32 product in the FP32 modes).
template <int MODE, bool PERSIST>
__device__ __forceinline__ float pr_c32(const PrArgs& a, uint32_t e, uint32_t s) {
  const float c = pr_ld<PERSIST>(a.contrib + s);
  if constexpr (pr_weighted<MODE>()) return c * a.csc_w[e];
  else return c;
}
template <int MODE, bool PERSIST>
__device__ __forceinline__ double pr_c64(const PrArgs& a, uint32_t e, uint32_t s) {
  const double c = pr_ld<PERSIST>(a.contrib64 + s);
  if constexpr (pr_weighted<MODE>()) return c * (double)a.csc_w[e];
  else return c;
}

// Contributions of the sources handled by this thread (u = lo + tid, lo + tid + nthr, ...
// below hi); for PageRank-delta also clears the next frontier's words [wlo, whi).
// Returns the thread's share of the dangling mass (PAGERANK).
template <int MODE, bool PERSIST>
__device__ __forceinline__ double pr_contrib_range(const PrArgs& a, unsigned p, uint64_t lo, uint64_t hi,
                                                   uint64_t wlo, uint64_t whi, uint64_t tid, uint64_t nthr) {
  double dangling = 0.0;
  if (MODE == PR_DELTA_RESIDUAL || MODE == PR_DELTA_PUSH) {
    const uint32_t* fa = a.fa2 + p * a.nwords;
    uint32_t* fn = a.fa2 + (p ^ 1u) * a.nwords;
    for (uint64_t w = wlo + tid; w < whi; w += nthr) fn[w] = 0;
    for (uint64_t u = lo + tid; u < hi; u += nthr) {
      const uint32_t d = a.deg[u];
      float v = 0.f;
      if (d) {
        if (MODE == PR_DELTA_RESIDUAL) v = pr_ld<PERSIST>(a.rank + u) / (float)d;
        else if ((pr_ld<PERSIST>(fa + (u >> 5)) >> (u & 31)) & 1u) v = pr_ld<PERSIST>(a.delta + u) / (float)d;
      }
      a.contrib[u] = v;
    }
  } else if (MODE == PR_NORM32) {
    const float* r = (p == 0) ? a.rank : a.comp;
    const float* rl = (p == 0) ? a.lo0 : a.lo1;
    // the contribution is an FP32 quotient of the high word (the low word is below its
    // rounding); the low word enters the FP64 dangling sum and the residual
    for (uint64_t u = lo + tid; u < hi; u += nthr) {
      const uint32_t d = a.deg[u];
      const float rh = pr_ld<PERSIST>(r + u);
      a.contrib[u] = d ? rh / (float)d : 0.f;
      if (!d) dangling += (double)rh + (double)pr_ld<PERSIST>(rl + u);
    }
  } else if (MODE == PR_W32) {
    const float* r = (p == 0) ? a.rank : a.comp;
    const float* rl = (p == 0) ? a.lo0 : a.lo1;
    for (uint64_t u = lo + tid; u < hi; u += nthr) {
      const double s = a.wsum[u];
      const float rh = pr_ld<PERSIST>(r + u);
      a.contrib[u] = s > 0.0 ? rh / (float)s : 0.f;
      if (!(s > 0.0)) dangling += (double)rh + (double)pr_ld<PERSIST>(rl + u);
    }
  } else if (MODE == PR_W64) {
    const double* r = (p == 0) ? a.r64 : a.r64n;
    for (uint64_t u = lo + tid; u < hi; u += nthr) {
      const double s = a.wsum[u];
      const double rv = pr_ld<PERSIST>(r + u);
      a.contrib64[u] = s > 0.0 ? rv / s : 0.0;
      if (!(s > 0.0)) dangling += rv;
    }
  } else if (MODE == PR_ADJ32) {
    // gather source = lambda itself; the returned sum is t . lambda
    const float* l = (p == 0) ? a.rank : a.comp;
    const double tu = 1.0 / (double)a.n;
    for (uint64_t u = lo + tid; u < hi; u += nthr) {
      const float lv = pr_ld<PERSIST>(l + u);
      a.contrib[u] = lv;
      dangling += (a.tele ? a.tele[u] : tu) * (double)lv;
    }
  } else if (MODE == PR_ADJ64) {
    const double* l = (p == 0) ? a.r64 : a.r64n;
    const double tu = 1.0 / (double)a.n;
    for (uint64_t u = lo + tid; u < hi; u += nthr) {
      const double lv = pr_ld<PERSIST>(l + u);
      a.contrib64[u] = lv;
      dangling += (a.tele ? a.tele[u] : tu) * lv;
    }
  } else {
    const double* r = (p == 0) ? a.r64 : a.r64n;
    for (uint64_t u = lo + tid; u < hi; u += nthr) {
      const uint32_t d = a.deg[u];
      const double rv = pr_ld<PERSIST>(r + u);
      a.contrib64[u] = d ? rv / (double)d : 0.0;
      if (!d) dangling += rv;
    }
  }
  return dangling;
}

// Warp-reduced dangling mass into the loop state (every lane calls it).
template <int MODE>
__device__ __forceinline__ void pr_dangling_flush(LoopState* ls, unsigned p, double dangling) {
  if (MODE >= PR_NORM32) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) dangling += __shfl_xor_sync(0xFFFFFFFFu, dangling, o);
    if ((threadIdx.x & 31) == 0 && dangling != 0.0) atomicAdd(&ls->dangling[p], dangling);
  }
}

// The round's dangling term as pr_finish takes it: D / n (normalised PageRank), D
// (weighted: scaled by t_v in pr_finish), t . lambda (adjoint), none (PageRank-delta).
template <int MODE, bool PERSIST>
__device__ __forceinline__ double pr_dang_arg(const LoopState* ls, unsigned p, uint64_t n) {
  if (MODE < PR_NORM32) return 0.0;
  const double d = pr_ld<PERSIST>(&ls->dangling[p]);
  return (MODE == PR_NORM32 || MODE == PR_NORM64) ? d / (double)n : d;
}

// Applies the finished sum of target v; returns |change| for the FP64 residual.
template <int MODE, bool PERSIST>
__device__ __forceinline__ double pr_finish(const PrArgs& a, uint64_t v, double sum, unsigned p, double dang,
                                            double* rsum) {
  if (MODE == PR_NORM32) {
    const float* r = (p == 0) ? a.rank : a.comp;
    const float* rl = (p == 0) ? a.lo0 : a.lo1;
    float* rn = (p == 0) ? a.comp : a.rank;
    float* rnl = (p == 0) ? a.lo1 : a.lo0;
    const double nv = a.base + a.alpha * (sum + dang);
    const float hi = (float)nv;
    const double d = fabs(nv - ((double)pr_ld<PERSIST>(r + v) + (double)pr_ld<PERSIST>(rl + v)));
    rn[v] = hi;
    rnl[v] = (float)(nv - (double)hi);
    *rsum += nv;
    return d;
  } else if (MODE == PR_NORM64) {
    const double* r = (p == 0) ? a.r64 : a.r64n;
    double* rn = (p == 0) ? a.r64n : a.r64;
    const double nv = a.base + a.alpha * (sum + dang);
    const double d = fabs(nv - pr_ld<PERSIST>(r + v));
    rn[v] = nv;
    *rsum += nv;
    return d;
  } else if (MODE == PR_W32 || MODE == PR_W64) {
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
    if (change != 0.f && (double)fabsf(change) > a.delta_param * (double)t) {
      uint32_t* fn = a.fa2 + (p ^ 1u) * a.nwords;
      atomicOr(&fn[v >> 5], 1u << (v & 31));
      atomicAdd(&a.ls->active[p ^ 1u], 1u);
    }
    return fabs((double)change);
  }
}

// Warp-reduced residual and rank sum into the loop state (every lane calls it).
__device__ __forceinline__ void pr_flush(LoopState* ls, unsigned p, double resid, double rsum) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    resid += __shfl_xor_sync(0xFFFFFFFFu, resid, o);
    rsum += __shfl_xor_sync(0xFFFFFFFFu, rsum, o);
  }
  if ((threadIdx.x & 31) == 0) {
    if (resid != 0.0) atomicAdd(&ls->resid[p], resid);
    if (rsum != 0.0) atomicAdd(&ls->rank_sum[p], rsum);
  }
}

// Sum of target v's in-edge contributions by one thread (in-degree <= 16): four
// independent gathers in flight, accumulated in edge order.
template <int MODE, bool PERSIST>
__device__ __forceinline__ double pr_sum_thread(const PrArgs& a, uint32_t v) {
  const uint32_t lo = a.csc_ptr[v], hi = a.csc_ptr[v + 1];
  if constexpr (pr_is64<MODE>()) {
    Acc64 acc;
    acc.init();
    uint32_t e = lo;
    for (; e + 4 <= hi; e += 4) {
      const uint32_t s0 = a.csc_src[e], s1 = a.csc_src[e + 1], s2 = a.csc_src[e + 2], s3 = a.csc_src[e + 3];
      const double c0 = pr_c64<MODE, PERSIST>(a, e, s0), c1 = pr_c64<MODE, PERSIST>(a, e + 1, s1),
                   c2 = pr_c64<MODE, PERSIST>(a, e + 2, s2), c3 = pr_c64<MODE, PERSIST>(a, e + 3, s3);
      acc.add(c0);
      acc.add(c1);
      acc.add(c2);
      acc.add(c3);
    }
    for (; e < hi; ++e) acc.add(pr_c64<MODE, PERSIST>(a, e, a.csc_src[e]));
    return acc.value();
  } else {
    Acc32 acc;
    acc.init();
    uint32_t e = lo;
    for (; e + 4 <= hi; e += 4) {
      const uint32_t s0 = a.csc_src[e], s1 = a.csc_src[e + 1], s2 = a.csc_src[e + 2], s3 = a.csc_src[e + 3];
      const float c0 = pr_c32<MODE, PERSIST>(a, e, s0), c1 = pr_c32<MODE, PERSIST>(a, e + 1, s1),
                  c2 = pr_c32<MODE, PERSIST>(a, e + 2, s2), c3 = pr_c32<MODE, PERSIST>(a, e + 3, s3);
      acc.add(c0);
      acc.add(c1);
      acc.add(c2);
      acc.add(c3);
    }
    for (; e < hi; ++e) acc.add(pr_c32<MODE, PERSIST>(a, e, a.csc_src[e]));
    return (double)acc.s + (double)acc.e;
  }
}

// The same by a group of VW lanes (lanes of one group are VW consecutive lanes of a
// warp; every lane of the warp calls it, an idle group with lo = hi): lane gl of the
// group sums edges lo+gl, lo+gl+VW, ... in order, then the group merges its lanes by an
// xor tree. Every lane of the group returns the sum.
template <int MODE, bool PERSIST, int VW>
__device__ __forceinline__ double pr_sum_group(const PrArgs& a, uint32_t lo, uint32_t hi, unsigned gl) {
  if constexpr (pr_is64<MODE>()) {
    double s = 0.0;
    uint32_t e = lo + gl;
    for (; e + 3 * VW < hi; e += 4 * VW) {
      const uint32_t s0 = a.csc_src[e], s1 = a.csc_src[e + VW], s2 = a.csc_src[e + 2 * VW], s3 = a.csc_src[e + 3 * VW];
      const double c0 = pr_c64<MODE, PERSIST>(a, e, s0), c1 = pr_c64<MODE, PERSIST>(a, e + VW, s1),
                   c2 = pr_c64<MODE, PERSIST>(a, e + 2 * VW, s2), c3 = pr_c64<MODE, PERSIST>(a, e + 3 * VW, s3);
      s += c0;
      s += c1;
      s += c2;
      s += c3;
    }
    for (; e < hi; e += VW) s += pr_c64<MODE, PERSIST>(a, e, a.csc_src[e]);
#pragma unroll
    for (int o = VW / 2; o > 0; o >>= 1) s += __shfl_xor_sync(0xFFFFFFFFu, s, o, VW);
    return s;
  } else {
    Acc32 acc;
    acc.init();
    uint32_t e = lo + gl;
    for (; e + 3 * VW < hi; e += 4 * VW) {
      const uint32_t s0 = a.csc_src[e], s1 = a.csc_src[e + VW], s2 = a.csc_src[e + 2 * VW], s3 = a.csc_src[e + 3 * VW];
      const float c0 = pr_c32<MODE, PERSIST>(a, e, s0), c1 = pr_c32<MODE, PERSIST>(a, e + VW, s1),
                  c2 = pr_c32<MODE, PERSIST>(a, e + 2 * VW, s2), c3 = pr_c32<MODE, PERSIST>(a, e + 3 * VW, s3);
      acc.add(c0);
      acc.add(c1);
      acc.add(c2);
      acc.add(c3);
    }
    for (; e < hi; e += VW) acc.add(pr_c32<MODE, PERSIST>(a, e, a.csc_src[e]));
#pragma unroll
    for (int o = VW / 2; o > 0; o >>= 1) {
      const float s2 = __shfl_xor_sync(0xFFFFFFFFu, acc.s, o, VW);
      const float e2 = __shfl_xor_sync(0xFFFFFFFFu, acc.e, o, VW);
      acc.merge(s2, e2);
    }
    return (double)acc.s + (double)acc.e;
  }
}

// The same by a block of PR_BLOCK_T threads (in-degree > 4096: RMAT hubs); thread 0
// returns the sum. Every thread of the block calls it.
template <int MODE, bool PERSIST>
__device__ __forceinline__ double pr_sum_block(const PrArgs& a, uint32_t v) {
  __shared__ float s_s[PR_BLOCK_T / 32], s_e[PR_BLOCK_T / 32];
  __shared__ double s_d[PR_BLOCK_T / 32];
  const unsigned lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const uint32_t lo = a.csc_ptr[v], hi = a.csc_ptr[v + 1];
  double sum = 0.0;
  if constexpr (pr_is64<MODE>()) {
    double s = 0.0;
    uint32_t e = lo + threadIdx.x;
    for (; e + 3 * PR_BLOCK_T < hi; e += 4 * PR_BLOCK_T) {
      const uint32_t s0 = a.csc_src[e], s1 = a.csc_src[e + PR_BLOCK_T], s2 = a.csc_src[e + 2 * PR_BLOCK_T],
                     s3 = a.csc_src[e + 3 * PR_BLOCK_T];
      const double c0 = pr_c64<MODE, PERSIST>(a, e, s0), c1 = pr_c64<MODE, PERSIST>(a, e + PR_BLOCK_T, s1),
                   c2 = pr_c64<MODE, PERSIST>(a, e + 2 * PR_BLOCK_T, s2),
                   c3 = pr_c64<MODE, PERSIST>(a, e + 3 * PR_BLOCK_T, s3);
      s += c0;
      s += c1;
      s += c2;
      s += c3;
    }
    for (; e < hi; e += PR_BLOCK_T) s += pr_c64<MODE, PERSIST>(a, e, a.csc_src[e]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xFFFFFFFFu, s, o);
    if (lane == 0) s_d[wid] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
      for (int k = 0; k < PR_BLOCK_T / 32; ++k) sum += s_d[k];
    }
  } else {
    Acc32 acc;
    acc.init();
    uint32_t e = lo + threadIdx.x;
    for (; e + 3 * PR_BLOCK_T < hi; e += 4 * PR_BLOCK_T) {
      const uint32_t s0 = a.csc_src[e], s1 = a.csc_src[e + PR_BLOCK_T], s2 = a.csc_src[e + 2 * PR_BLOCK_T],
                     s3 = a.csc_src[e + 3 * PR_BLOCK_T];
      const float c0 = pr_c32<MODE, PERSIST>(a, e, s0), c1 = pr_c32<MODE, PERSIST>(a, e + PR_BLOCK_T, s1),
                  c2 = pr_c32<MODE, PERSIST>(a, e + 2 * PR_BLOCK_T, s2),
                  c3 = pr_c32<MODE, PERSIST>(a, e + 3 * PR_BLOCK_T, s3);
      acc.add(c0);
      acc.add(c1);
      acc.add(c2);
      acc.add(c3);
    }
    for (; e < hi; e += PR_BLOCK_T) acc.add(pr_c32<MODE, PERSIST>(a, e, a.csc_src[e]));
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
      for (int k = 0; k < PR_BLOCK_T / 32; ++k) t.merge(s_s[k], s_e[k]);
      sum = (double)t.s + (double)t.e;
    }
  }
  __syncthreads();
  return sum;
}

// Ends a round: records the FP64 residual, decides whether to continue (one thread).
__device__ __forceinline__ unsigned pr_control_step(LoopState* ls_, int mode) {
  volatile LoopState* ls = ls_;
  if (ls->cont) {
    const unsigned p = ls->iter & 1u;
    const double resid = ls->resid[p];
    ls->resid_final = resid;
    if (mode == PR_DELTA_RESIDUAL || mode == PR_DELTA_PUSH) {
      ls->change_sum = ls->change_sum + ls->rank_sum[p];
      ls->active_total = ls->active_total + ls->active[p ^ 1u];
    }
    ls->count_edges = ls->count_edges + ls->teps[0];
    ls->edges_scanned = ls->edges_scanned + ls->teps[0];
    ls->iter = ls->iter + 1;
    const unsigned q = ls->iter & 1u;
    bool more = ls->iter < ls->max_iter;
    if (mode == PR_DELTA_RESIDUAL || mode == PR_DELTA_PUSH) {
      const double total = ls->base_sum + ls->change_sum;
      more = more && ls->active[q] > 0;
      if (ls->tol > 0.0) more = more && resid > ls->tol * total;
    } else {
      more = more && resid > ls->tol;
      // FP32 ranks cannot change by less than their rounding floor (about 6e-8 of the rank
      // mass per round); once the FP64-measured change stops shrinking, the run is done
      if (mode == PR_NORM32 || mode == PR_W32 || mode == PR_ADJ32) {
        if (resid < ls->best_resid * 0.999) {
          ls->best_resid = resid;
          ls->stall = 0;
        } else {
          ls->stall = ls->stall + 1;
          if (ls->stall >= 4) more = false;
        }
      }
    }
    ls->resid[q] = 0.0;
    ls->dangling[q] = 0.0;
    ls->active[q ^ 1u] = 0;
    ls->rank_sum[q] = 0.0;
    ls->cont = more ? 1u : 0u;
  }
  return ls->cont;
}

}  // namespace cytom
