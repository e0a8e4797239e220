// exec_pagerank.cu — PageRank-delta and normalised PageRank executors (pull).
//
// PageRank-delta is the reference's vertex program examples/pagerank-delta.cc:
// unnormalised ranks r = (1-alpha) + alpha * sum_{u->v} r_u / outdeg(u) (multiplicity
// out-degrees, the vertex store's), reached by pushing deltas from active vertices:
// round k gives delta_v = alpha * sum_{u->v, u active} delta_u / outdeg(u) and
// rank_v += delta_v (pagerank-delta.cc:127-174); a vertex stays active while
// |delta| > delta_param * rank. The first round of a run is a residual round:
// res_v = (1-alpha) + alpha * sum_{u->v} rank_u / outdeg(u) - rank_v, rank_v += res_v,
// delta_v = res_v. From rank = 1 this is exactly the reference's first iteration
// (rank = 0.15 + 0.85 * sum 1/outdeg, delta = rank - 1); after a batch it is the
// exact correction of the converged ranks to the new graph.
//
// PAGERANK is the normalised PageRank with dangling mass: r_v = (1-alpha)/n +
// alpha * (sum_{u->v} r_u / d_u + D / n), d_u = distinct out-edges, D = sum of r over
// vertices without out-edges; FP32 with compensated sums (kahan = 1) or FP64 plain.
//
// Both pull over a target-sorted CSC built from the tile store once per snapshot
// (radix sort of (tgt, src) keys): each target's in-edges are contiguous, so its sum is
// accumulated in a fixed order with Neumaier compensation -- deterministic and
// compensated, no float atomics. Targets are binned by in-degree: one thread (<= 16
// in-edges), one warp (<= 4096) or one block (more) per target. Residuals, dangling
// mass and rank sums are FP64 reductions.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cstdlib>
#include <cstring>

#include "engine.h"

namespace cytom {

constexpr uint32_t kBinSmall = 16;
constexpr uint32_t kBinMedium = 4096;
constexpr int PR_T = 256;
constexpr int PR_BLOCK_T = 512;

// CSC of the compacted store, per job (PageRank family).
struct Csc {
  uint32_t* src = nullptr;       // E: global source of each in-edge, grouped by target
  uint32_t* ptr = nullptr;       // n+1
  uint32_t* deg_out = nullptr;   // n: distinct out-degree (stored edges)
  uint32_t* bins = nullptr;      // n: targets, small | medium | large
  uint64_t nb[3] = {0, 0, 0};
  uint64_t E = 0;
  uint64_t cap = 0;
  uint64_t built_version = ~0ULL;
};

struct PrState {
  Csc csc;
  float* rank = nullptr;      // PR_DELTA: rank; PAGERANK fp32: r (double-buffered with rank_c)
  float* comp = nullptr;      // PR_DELTA: Kahan compensation of rank; PAGERANK fp32: r_next
  float* delta = nullptr;     // PR_DELTA: delta of the last round
  float* contrib = nullptr;   // per-source contribution of the round
  double* r64 = nullptr;      // PAGERANK fp64: r
  double* r64n = nullptr;     // PAGERANK fp64: r_next
  double* contrib64 = nullptr;
  uint32_t* fa2 = nullptr;    // PR_DELTA: frontier bitmaps by parity (2 x n/32)
  bool need_residual = true;
  uint64_t seen_version = ~0ULL;
};

// --------------------------------------------------------------------------
// Compensated accumulation (Neumaier): true sum ~= s + e.
// --------------------------------------------------------------------------
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

// --------------------------------------------------------------------------
// CSC construction from the tile store
// --------------------------------------------------------------------------
__global__ void csc_keys_kernel(const StoreDesc* __restrict__ sd, uint64_t* __restrict__ keys,
                                uint32_t* __restrict__ deg_out, uint32_t* __restrict__ in_cnt, uint32_t lg_n) {
  const uint64_t E = sd->E;
  const uint32_t lT = sd->lT, lvpt = sd->lvpt;
  const uint32_t ymask = (uint32_t)(sd->T - 1);
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; e < E; e += stride) {
    uint32_t t = sd->chunk_tile[e >> 7];
    while (sd->tile_ptr[t + 1] <= e) ++t;
    const uint32_t p = sd->edges[e];
    const uint32_t u = ((t >> lT) << lvpt) | (p >> 16);
    const uint32_t v = ((t & ymask) << lvpt) | (p & 0xFFFFu);
    keys[e] = ((uint64_t)v << lg_n) | u;
    atomicAdd(&deg_out[u], 1u);
    atomicAdd(&in_cnt[v], 1u);
  }
}

__global__ void csc_src_kernel(const uint64_t* __restrict__ keys, uint64_t E, uint32_t lg_n,
                               uint32_t* __restrict__ src) {
  const uint64_t mask = (1ULL << lg_n) - 1ULL;
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; e < E; e += stride)
    src[e] = (uint32_t)(keys[e] & mask);
}

// class of each target by in-degree: 0 small, 1 medium, 2 large (flags for three scans)
__global__ void csc_class_kernel(const uint32_t* __restrict__ in_cnt, uint64_t n, uint32_t* __restrict__ f0,
                                 uint32_t* __restrict__ f1, uint32_t* __restrict__ f2) {
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t v = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += stride) {
    const uint32_t d = in_cnt[v];
    f0[v] = d <= kBinSmall ? 1u : 0u;
    f1[v] = (d > kBinSmall && d <= kBinMedium) ? 1u : 0u;
    f2[v] = d > kBinMedium ? 1u : 0u;
  }
}

__global__ void csc_bins_kernel(const uint32_t* __restrict__ f0, const uint32_t* __restrict__ f1,
                                const uint32_t* __restrict__ f2, const uint32_t* __restrict__ p0,
                                const uint32_t* __restrict__ p1, const uint32_t* __restrict__ p2,
                                const uint32_t* __restrict__ tot, uint64_t n, uint32_t* __restrict__ bins) {
  const uint32_t n0 = tot[0], n1 = tot[1];
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t v = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += stride) {
    if (f0[v]) bins[p0[v]] = (uint32_t)v;
    else if (f1[v]) bins[n0 + p1[v]] = (uint32_t)v;
    else if (f2[v]) bins[n0 + n1 + p2[v]] = (uint32_t)v;
  }
}

static int grid_n(Ctx* c, uint64_t work, int threads = 256, int per_sm = 8) {
  uint64_t b = (work + threads - 1) / threads;
  uint64_t cap = (uint64_t)c->num_sms * per_sm;
  if (b > cap) b = cap;
  return (int)std::max<uint64_t>(b, 1);
}

static uint64_t store_version(Ctx* c) { return c->version; }

static int build_csc(Ctx* c, Csc& q) {
  const uint64_t n = c->n, E = c->E;
  uint32_t lg_n = 0;
  while ((1ULL << lg_n) < n) ++lg_n;
  if (E > 0xFFFFFFFFULL) return set_err(c, CYTOM_ERR_RANGE, "PageRank CSC holds at most 2^32 edges");
  if (E > q.cap || !q.src) {
    cudaFree(q.src);
    q.cap = std::max<uint64_t>(E + E / 4, 1024);
    if (cudaMalloc(&q.src, q.cap * 4) != cudaSuccess) return set_err(c, CYTOM_ERR_OOM, "CSC");
  }
  if (!q.ptr) {
    if (cudaMalloc(&q.ptr, (n + 1) * 4) != cudaSuccess || cudaMalloc(&q.deg_out, n * 4) != cudaSuccess ||
        cudaMalloc(&q.bins, n * 4) != cudaSuccess)
      return set_err(c, CYTOM_ERR_OOM, "CSC index");
  }
  char* tmp = nullptr;
  const size_t kbytes = std::max<uint64_t>(E, 1) * 8;
  const size_t nbytes = n * 4;
  if (cudaMallocAsync((void**)&tmp, 2 * kbytes + 7 * nbytes + 64, c->stream) != cudaSuccess)
    return set_err(c, CYTOM_ERR_OOM, "CSC temporaries");
  uint64_t* k0 = (uint64_t*)tmp;
  uint64_t* k1 = (uint64_t*)(tmp + kbytes);
  uint32_t* in_cnt = (uint32_t*)(tmp + 2 * kbytes);
  uint32_t* f0 = in_cnt + n;
  uint32_t* f1 = f0 + n;
  uint32_t* f2 = f1 + n;
  uint32_t* p0 = f2 + n;
  uint32_t* p1 = p0 + n;
  uint32_t* p2 = p1 + n;
  uint32_t* tot = p2 + n;  // 3 totals + 1
  cudaMemsetAsync(q.deg_out, 0, n * 4, c->stream);
  cudaMemsetAsync(in_cnt, 0, n * 4, c->stream);
  int rc = CYTOM_OK;
  if (E) {
    csc_keys_kernel<<<grid_n(c, E), 256, 0, c->stream>>>(c->dsd, k0, q.deg_out, in_cnt, lg_n);
    c->launches++;
    bool alt = false;
    rc = radix_sort_pairs(c, k0, k1, nullptr, nullptr, E, (int)(2 * lg_n), &alt);
    if (rc) return rc;
    csc_src_kernel<<<grid_n(c, E), 256, 0, c->stream>>>(alt ? k1 : k0, E, lg_n, q.src);
    c->launches++;
  }
  rc = exclusive_scan_u32(c, in_cnt, q.ptr, n, q.ptr + n);
  if (rc) return rc;
  csc_class_kernel<<<grid_n(c, n), 256, 0, c->stream>>>(in_cnt, n, f0, f1, f2);
  c->launches++;
  rc = exclusive_scan_u32(c, f0, p0, n, tot + 0);
  if (!rc) rc = exclusive_scan_u32(c, f1, p1, n, tot + 1);
  if (!rc) rc = exclusive_scan_u32(c, f2, p2, n, tot + 2);
  if (rc) return rc;
  csc_bins_kernel<<<grid_n(c, n), 256, 0, c->stream>>>(f0, f1, f2, p0, p1, p2, tot, n, q.bins);
  c->launches++;
  uint32_t ht[3];
  cudaMemcpyAsync(ht, tot, 12, cudaMemcpyDeviceToHost, c->stream);
  cudaFreeAsync(tmp, c->stream);
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_err(c, e, "CSC build");
  q.nb[0] = ht[0];
  q.nb[1] = ht[1];
  q.nb[2] = ht[2];
  q.E = E;
  return CYTOM_OK;
}

// --------------------------------------------------------------------------
// Round kernels
// --------------------------------------------------------------------------
enum PrMode { PR_DELTA_RESIDUAL = 0, PR_DELTA_PUSH = 1, PR_NORM32 = 2, PR_NORM64 = 3 };

struct PrArgs {
  const uint32_t* csc_src;
  const uint32_t* csc_ptr;
  const uint32_t* bins;
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
  LoopState* ls;
  uint64_t n;
  uint64_t nwords;
  double alpha, delta_param, base;
};

// Per-vertex contribution of the round and the dangling mass (PAGERANK).
template <int MODE>
__global__ void pr_contrib_kernel(PrArgs a) {
  LoopState* ls = a.ls;
  if (!ls->cont) return;
  const unsigned p = ls->iter & 1u;
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  double dangling = 0.0;
  if (MODE == PR_DELTA_RESIDUAL || MODE == PR_DELTA_PUSH) {
    const uint32_t* fa = a.fa2 + p * a.nwords;
    uint32_t* fn = a.fa2 + (p ^ 1u) * a.nwords;
    for (uint64_t w = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; w < a.nwords; w += stride) fn[w] = 0;
    for (uint64_t u = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; u < a.n; u += stride) {
      const uint32_t d = a.deg[u];
      float v = 0.f;
      if (d) {
        if (MODE == PR_DELTA_RESIDUAL) v = a.rank[u] / (float)d;
        else if ((fa[u >> 5] >> (u & 31)) & 1u) v = a.delta[u] / (float)d;
      }
      a.contrib[u] = v;
    }
  } else if (MODE == PR_NORM32) {
    const float* r = (p == 0) ? a.rank : a.comp;
    for (uint64_t u = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; u < a.n; u += stride) {
      const uint32_t d = a.deg[u];
      const float rv = r[u];
      a.contrib[u] = d ? rv / (float)d : 0.f;
      if (!d) dangling += (double)rv;
    }
  } else {
    const double* r = (p == 0) ? a.r64 : a.r64n;
    for (uint64_t u = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; u < a.n; u += stride) {
      const uint32_t d = a.deg[u];
      const double rv = r[u];
      a.contrib64[u] = d ? rv / (double)d : 0.0;
      if (!d) dangling += rv;
    }
  }
  if (MODE == PR_NORM32 || MODE == PR_NORM64) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) dangling += __shfl_xor_sync(0xFFFFFFFFu, dangling, o);
    if ((threadIdx.x & 31) == 0 && dangling != 0.0) atomicAdd(&ls->dangling[p], dangling);
  }
}

// Applies the finished sum of target v; returns |change| for the FP64 residual.
template <int MODE>
__device__ __forceinline__ double pr_finish(const PrArgs& a, uint64_t v, double sum, unsigned p, double dang,
                                            double* rsum) {
  if (MODE == PR_NORM32) {
    const float* r = (p == 0) ? a.rank : a.comp;
    float* rn = (p == 0) ? a.comp : a.rank;
    const float nv = (float)(a.base + a.alpha * (sum + dang));
    const double d = fabs((double)nv - (double)r[v]);
    rn[v] = nv;
    *rsum += (double)nv;
    return d;
  } else if (MODE == PR_NORM64) {
    const double* r = (p == 0) ? a.r64 : a.r64n;
    double* rn = (p == 0) ? a.r64n : a.r64;
    const double nv = a.base + a.alpha * (sum + dang);
    const double d = fabs(nv - r[v]);
    rn[v] = nv;
    *rsum += nv;
    return d;
  } else {
    // PageRank-delta: residual round or delta round, rank += change (compensated)
    float change;
    if (MODE == PR_DELTA_RESIDUAL) {
      change = (float)((1.0 - a.alpha) + a.alpha * sum - (double)a.rank[v] - (double)a.comp[v]);
    } else {
      change = (sum == 0.0) ? 0.f : (float)(a.alpha * sum);
    }
    a.delta[v] = change;
    // Kahan: rank + comp carries the exact running sum of the changes
    const float y = change + a.comp[v];
    const float t = a.rank[v] + y;
    a.comp[v] = y - (t - a.rank[v]);
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

template <int MODE>
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

template <int MODE>
__device__ __forceinline__ auto pr_load(const PrArgs& a, uint32_t u) {
  if constexpr (MODE == PR_NORM64) return a.contrib64[u];
  else return a.contrib[u];
}

// One thread per target (in-degree <= 16).
template <int MODE>
__global__ void __launch_bounds__(PR_T) pr_pull_small(PrArgs a) {
  LoopState* ls = a.ls;
  if (!ls->cont) return;
  const unsigned p = ls->iter & 1u;
  const double dang = (MODE == PR_NORM32 || MODE == PR_NORM64) ? ls->dangling[p] / (double)a.n : 0.0;
  double resid = 0.0, rsum = 0.0;
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t base = (uint64_t)blockIdx.x * blockDim.x; base < a.bin_count; base += stride) {
    const uint64_t i = base + threadIdx.x;
    if (i < a.bin_count) {
      const uint32_t v = a.bins[a.bin_off + i];
      const uint32_t lo = a.csc_ptr[v], hi = a.csc_ptr[v + 1];
      double sum;
      // four independent gathers in flight, accumulated in edge order
      if constexpr (MODE == PR_NORM64) {
        Acc64 acc;
        acc.init();
        uint32_t e = lo;
        for (; e + 4 <= hi; e += 4) {
          const uint32_t s0 = a.csc_src[e], s1 = a.csc_src[e + 1], s2 = a.csc_src[e + 2], s3 = a.csc_src[e + 3];
          const double c0 = a.contrib64[s0], c1 = a.contrib64[s1], c2 = a.contrib64[s2], c3 = a.contrib64[s3];
          acc.add(c0);
          acc.add(c1);
          acc.add(c2);
          acc.add(c3);
        }
        for (; e < hi; ++e) acc.add(a.contrib64[a.csc_src[e]]);
        sum = acc.value();
      } else {
        Acc32 acc;
        acc.init();
        uint32_t e = lo;
        for (; e + 4 <= hi; e += 4) {
          const uint32_t s0 = a.csc_src[e], s1 = a.csc_src[e + 1], s2 = a.csc_src[e + 2], s3 = a.csc_src[e + 3];
          const float c0 = a.contrib[s0], c1 = a.contrib[s1], c2 = a.contrib[s2], c3 = a.contrib[s3];
          acc.add(c0);
          acc.add(c1);
          acc.add(c2);
          acc.add(c3);
        }
        for (; e < hi; ++e) acc.add(a.contrib[a.csc_src[e]]);
        sum = (double)acc.s + (double)acc.e;
      }
      resid += pr_finish<MODE>(a, v, sum, p, dang, &rsum);
    }
  }
  pr_flush<MODE>(ls, p, resid, rsum);
}

// One warp per target (16 < in-degree <= 4096).
template <int MODE>
__global__ void __launch_bounds__(PR_T) pr_pull_medium(PrArgs a) {
  LoopState* ls = a.ls;
  if (!ls->cont) return;
  const unsigned p = ls->iter & 1u;
  const double dang = (MODE == PR_NORM32 || MODE == PR_NORM64) ? ls->dangling[p] / (double)a.n : 0.0;
  const unsigned lane = threadIdx.x & 31;
  const uint64_t warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  double resid = 0.0, rsum = 0.0;
  for (uint64_t i = warp; i < a.bin_count; i += nwarps) {
    const uint32_t v = a.bins[a.bin_off + i];
    const uint32_t lo = a.csc_ptr[v], hi = a.csc_ptr[v + 1];
    double sum;
    if constexpr (MODE == PR_NORM64) {
      double s = 0.0;
      uint32_t e = lo + lane;
      for (; e + 96 < hi; e += 128) {
        const uint32_t s0 = a.csc_src[e], s1 = a.csc_src[e + 32], s2 = a.csc_src[e + 64], s3 = a.csc_src[e + 96];
        const double c0 = a.contrib64[s0], c1 = a.contrib64[s1], c2 = a.contrib64[s2], c3 = a.contrib64[s3];
        s += c0;
        s += c1;
        s += c2;
        s += c3;
      }
      for (; e < hi; e += 32) s += a.contrib64[a.csc_src[e]];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xFFFFFFFFu, s, o);
      sum = s;
    } else {
      Acc32 acc;
      acc.init();
      uint32_t e = lo + lane;
      for (; e + 96 < hi; e += 128) {
        const uint32_t s0 = a.csc_src[e], s1 = a.csc_src[e + 32], s2 = a.csc_src[e + 64], s3 = a.csc_src[e + 96];
        const float c0 = a.contrib[s0], c1 = a.contrib[s1], c2 = a.contrib[s2], c3 = a.contrib[s3];
        acc.add(c0);
        acc.add(c1);
        acc.add(c2);
        acc.add(c3);
      }
      for (; e < hi; e += 32) acc.add(a.contrib[a.csc_src[e]]);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const float s2 = __shfl_xor_sync(0xFFFFFFFFu, acc.s, o);
        const float e2 = __shfl_xor_sync(0xFFFFFFFFu, acc.e, o);
        acc.merge(s2, e2);
      }
      sum = (double)acc.s + (double)acc.e;
    }
    if (lane == 0) resid += pr_finish<MODE>(a, v, sum, p, dang, &rsum);
  }
  pr_flush<MODE>(ls, p, resid, rsum);
}

// One block per target (in-degree > 4096: RMAT hubs).
template <int MODE>
__global__ void __launch_bounds__(PR_BLOCK_T) pr_pull_large(PrArgs a) {
  LoopState* ls = a.ls;
  if (!ls->cont) return;
  const unsigned p = ls->iter & 1u;
  const double dang = (MODE == PR_NORM32 || MODE == PR_NORM64) ? ls->dangling[p] / (double)a.n : 0.0;
  __shared__ float s_s[PR_BLOCK_T / 32], s_e[PR_BLOCK_T / 32];
  __shared__ double s_d[PR_BLOCK_T / 32];
  const unsigned lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  double resid = 0.0, rsum = 0.0;
  for (uint64_t i = blockIdx.x; i < a.bin_count; i += gridDim.x) {
    const uint32_t v = a.bins[a.bin_off + i];
    const uint32_t lo = a.csc_ptr[v], hi = a.csc_ptr[v + 1];
    double sum = 0.0;
    if constexpr (MODE == PR_NORM64) {
      double s = 0.0;
      uint32_t e = lo + threadIdx.x;
      for (; e + 3 * PR_BLOCK_T < hi; e += 4 * PR_BLOCK_T) {
        const uint32_t s0 = a.csc_src[e], s1 = a.csc_src[e + PR_BLOCK_T], s2 = a.csc_src[e + 2 * PR_BLOCK_T],
                       s3 = a.csc_src[e + 3 * PR_BLOCK_T];
        const double c0 = a.contrib64[s0], c1 = a.contrib64[s1], c2 = a.contrib64[s2], c3 = a.contrib64[s3];
        s += c0;
        s += c1;
        s += c2;
        s += c3;
      }
      for (; e < hi; e += PR_BLOCK_T) s += a.contrib64[a.csc_src[e]];
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
        const float c0 = a.contrib[s0], c1 = a.contrib[s1], c2 = a.contrib[s2], c3 = a.contrib[s3];
        acc.add(c0);
        acc.add(c1);
        acc.add(c2);
        acc.add(c3);
      }
      for (; e < hi; e += PR_BLOCK_T) acc.add(a.contrib[a.csc_src[e]]);
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
    if (threadIdx.x == 0) resid += pr_finish<MODE>(a, v, sum, p, dang, &rsum);
    __syncthreads();
  }
  pr_flush<MODE>(ls, p, resid, rsum);
}

// Ends the round: records the FP64 residual, decides whether to continue.
__global__ void pr_control_kernel(LoopState* ls, int mode, cudaGraphConditionalHandle h, int use_handle) {
  if (ls->cont) {
    const unsigned p = ls->iter & 1u;
    const double resid = ls->resid[p];
    ls->resid_final = resid;
    if (mode == PR_DELTA_RESIDUAL || mode == PR_DELTA_PUSH) {
      ls->change_sum += ls->rank_sum[p];
      ls->active_total += ls->active[p ^ 1u];
    }
    ls->count_edges += ls->teps[0];
    ls->edges_scanned += ls->teps[0];
    ls->iter += 1;
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
      if (mode == PR_NORM32) {
        if (resid < ls->best_resid * 0.999) {
          ls->best_resid = resid;
          ls->stall = 0;
        } else if (++ls->stall >= 4) {
          more = false;
        }
      }
    }
    ls->resid[q] = 0.0;
    ls->dangling[q] = 0.0;
    ls->active[q ^ 1u] = 0;
    ls->rank_sum[q] = 0.0;
    ls->cont = more ? 1u : 0u;
  }
  if (use_handle) cudaGraphSetConditional(h, ls->cont);
}

// --------------------------------------------------------------------------
// Job plumbing
// --------------------------------------------------------------------------
__global__ void pr_fill_kernel(float* a, float v, uint64_t n) {
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) a[i] = v;
}
__global__ void pr_fill64_kernel(double* a, double v, uint64_t n) {
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) a[i] = v;
}
__global__ void pr_to_float_kernel(const double* a, float* b, uint64_t n) {
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) b[i] = (float)a[i];
}
// Sum of the current ranks (FP64), stored where the control kernel reads it.
__global__ void pr_rank_sum_kernel(const float* r, uint64_t n, LoopState* ls) {
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  double s = 0.0;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) s += (double)r[i];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xFFFFFFFFu, s, o);
  if ((threadIdx.x & 31) == 0 && s != 0.0) atomicAdd(&ls->base_sum, s);
}
__global__ void pr_begin_kernel(LoopState* ls, unsigned max_iter, double tol, unsigned long long edges) {
  ls->iter = 0;
  ls->max_iter = max_iter;
  ls->cont = max_iter > 0 ? 1u : 0u;
  ls->err = 0;
  ls->active[0] = ls->active[1] = 0;
  ls->teps[0] = edges;  // every round reads every stored edge once
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

static PrState* prs(Job* j) { return reinterpret_cast<PrState*>(j->ext); }

int pagerank_alloc(Ctx* c, Job* j) {
  PrState* s = new (std::nothrow) PrState();
  if (!s) return set_err(c, CYTOM_ERR_OOM, "PageRank state");
  j->ext = s;
  const uint64_t n = c->n;
  const uint64_t nwords = (n + 31) / 32;
  bool ok = true;
  if (j->algo == CYTOM_ALGO_PR_DELTA) {
    ok = ok && cudaMalloc(&s->rank, n * 4) == cudaSuccess;
    ok = ok && cudaMalloc(&s->comp, n * 4) == cudaSuccess;
    ok = ok && cudaMalloc(&s->delta, n * 4) == cudaSuccess;
    ok = ok && cudaMalloc(&s->contrib, n * 4) == cudaSuccess;
    ok = ok && cudaMalloc(&s->fa2, 2 * nwords * 4) == cudaSuccess;
  } else if (j->params.kahan) {
    ok = ok && cudaMalloc(&s->rank, n * 4) == cudaSuccess;
    ok = ok && cudaMalloc(&s->comp, n * 4) == cudaSuccess;
    ok = ok && cudaMalloc(&s->contrib, n * 4) == cudaSuccess;
  } else {
    ok = ok && cudaMalloc(&s->r64, n * 8) == cudaSuccess;
    ok = ok && cudaMalloc(&s->r64n, n * 8) == cudaSuccess;
    ok = ok && cudaMalloc(&s->contrib64, n * 8) == cudaSuccess;
    ok = ok && cudaMalloc(&s->rank, n * 4) == cudaSuccess;  // float copy for results
  }
  if (!ok) {
    cudaGetLastError();
    return set_err(c, CYTOM_ERR_OOM, "PageRank state");
  }
  return CYTOM_OK;
}

void pagerank_free(Job* j) {
  PrState* s = prs(j);
  if (!s) return;
  void* ptrs[] = {s->csc.src, s->csc.ptr, s->csc.deg_out, s->csc.bins, s->rank, s->comp, s->delta,
                  s->contrib, s->r64, s->r64n, s->contrib64, s->fa2};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  delete s;
  j->ext = nullptr;
}

int pagerank_init(Ctx* c, Job* j) {
  PrState* s = prs(j);
  const uint64_t n = c->n;
  int g = grid_n(c, n);
  if (j->algo == CYTOM_ALGO_PR_DELTA) {
    // reference init_vertices: rank 0 with delta 1 everywhere; here rank = 1 and the
    // residual round reproduces the reference's first iteration
    pr_fill_kernel<<<g, 256, 0, c->stream>>>(s->rank, 1.0f, n);
    cudaMemsetAsync(s->comp, 0, n * 4, c->stream);
    cudaMemsetAsync(s->delta, 0, n * 4, c->stream);
    cudaMemsetAsync(s->fa2, 0xFF, 2 * ((n + 31) / 32) * 4, c->stream);
    c->launches++;
  } else if (j->params.kahan) {
    pr_fill_kernel<<<g, 256, 0, c->stream>>>(s->rank, (float)(1.0 / (double)n), n);
    c->launches++;
  } else {
    pr_fill64_kernel<<<g, 256, 0, c->stream>>>(s->r64, 1.0 / (double)n, n);
    c->launches++;
  }
  s->need_residual = true;
  return cuda_err(c, cudaGetLastError(), "pagerank init");
}

int pagerank_seed(Ctx* c, Job* j, const uint32_t*, const uint32_t*, const uint32_t*, uint64_t) {
  // the next run starts with a residual round over the new snapshot
  prs(j)->need_residual = true;
  (void)c;
  return CYTOM_OK;
}

template <int MODE>
static int launch_round(Ctx* c, Job* j, const PrArgs& base_args) {
  PrState* s = prs(j);
  PrArgs a = base_args;
  pr_contrib_kernel<MODE><<<grid_n(c, c->n), 256, 0, c->stream>>>(a);
  a.bin_off = 0;
  a.bin_count = s->csc.nb[0];
  if (a.bin_count) pr_pull_small<MODE><<<grid_n(c, a.bin_count, PR_T), PR_T, 0, c->stream>>>(a);
  a.bin_off = s->csc.nb[0];
  a.bin_count = s->csc.nb[1];
  if (a.bin_count) pr_pull_medium<MODE><<<grid_n(c, a.bin_count * 32, PR_T), PR_T, 0, c->stream>>>(a);
  a.bin_off = s->csc.nb[0] + s->csc.nb[1];
  a.bin_count = s->csc.nb[2];
  if (a.bin_count)
    pr_pull_large<MODE><<<(unsigned)std::min<uint64_t>(a.bin_count, (uint64_t)c->num_sms * 4), PR_BLOCK_T, 0,
                          c->stream>>>(a);
  pr_control_kernel<<<1, 1, 0, c->stream>>>(a.ls, MODE, 0, 0);
  c->launches += 2 + (s->csc.nb[0] ? 1 : 0) + (s->csc.nb[1] ? 1 : 0) + (s->csc.nb[2] ? 1 : 0);
  return cuda_err(c, cudaGetLastError(), "pagerank round");
}

template <int MODE>
static int run_rounds(Ctx* c, Job* j, const PrArgs& a, uint64_t max_rounds) {
  for (uint64_t r = 0; r < max_rounds;) {
    for (int k = 0; k < 8 && r < max_rounds; ++k, ++r) {
      int slot = prof_begin(c, KC_PAGERANK);
      int rc = launch_round<MODE>(c, j, a);
      prof_end(c, slot, -1.0);
      if (rc) return rc;
    }
    cudaError_t e = cudaMemcpyAsync(c->h_pinned, &j->ls->cont, 4, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_err(c, e, "pagerank loop");
    if (*(unsigned*)c->h_pinned == 0) break;
  }
  return CYTOM_OK;
}

int pagerank_run(Ctx* c, Job* j) {
  PrState* s = prs(j);
  const uint64_t ver = store_version(c);
  if (s->csc.built_version != ver) {
    int rc = build_csc(c, s->csc);
    if (rc) return rc;
    s->csc.built_version = ver;
  }
  if (s->seen_version != ver) {
    s->need_residual = true;
    s->seen_version = ver;
  }
  const uint64_t n = c->n;
  PrArgs a{};
  a.csc_src = s->csc.src;
  a.csc_ptr = s->csc.ptr;
  a.bins = s->csc.bins;
  a.rank = s->rank;
  a.comp = s->comp;
  a.delta = s->delta;
  a.contrib = s->contrib;
  a.r64 = s->r64;
  a.r64n = s->r64n;
  a.contrib64 = s->contrib64;
  a.fa2 = s->fa2;
  a.ls = j->ls;
  a.n = n;
  a.nwords = (n + 31) / 32;
  a.alpha = j->params.alpha;
  a.delta_param = j->params.delta;
  a.base = (1.0 - j->params.alpha) / (double)n;
  unsigned max_iter = (unsigned)std::min<uint64_t>(j->params.max_iterations, 0xFFFFFFFFu);
  pr_begin_kernel<<<1, 1, 0, c->stream>>>(j->ls, max_iter, j->params.tolerance, (unsigned long long)s->csc.E);
  c->launches++;
  j->last_run_graph = false;
  if (j->algo == CYTOM_ALGO_PR_DELTA) {
    a.deg = c->out_deg;  // multiplicity out-degrees, as the reference's vertex store
    // rank sum before the run (relative stopping rule)
    pr_rank_sum_kernel<<<grid_n(c, n), 256, 0, c->stream>>>(s->rank, n, j->ls);
    c->launches++;
    // Every run opens with the residual round (all sources contribute rank / outdeg):
    // exact after any change of the graph, and a no-op correction when nothing changed.
    int rc = run_rounds<PR_DELTA_RESIDUAL>(c, j, a, 1);
    if (rc) return rc;
    s->need_residual = false;
    return run_rounds<PR_DELTA_PUSH>(c, j, a, max_iter);
  }
  a.deg = s->csc.deg_out;
  if (j->params.kahan) {
    int rc = run_rounds<PR_NORM32>(c, j, a, max_iter);
    return rc;
  }
  return run_rounds<PR_NORM64>(c, j, a, max_iter);
}

int pagerank_result(Ctx* c, Job* j, void* out, int where) {
  PrState* s = prs(j);
  const uint64_t n = c->n;
  const float* src = s->rank;
  LoopState ls;
  cudaMemcpyAsync(&ls, j->ls, sizeof(ls), cudaMemcpyDeviceToHost, c->stream);
  cudaStreamSynchronize(c->stream);
  const unsigned p = ls.iter & 1u;  // buffer holding the newest ranks
  if (j->algo == CYTOM_ALGO_PAGERANK) {
    if (j->params.kahan) {
      src = (p == 0) ? s->rank : s->comp;
    } else {
      const double* r = (p == 0) ? s->r64 : s->r64n;
      pr_to_float_kernel<<<grid_n(c, n), 256, 0, c->stream>>>(r, s->rank, n);
      c->launches++;
      src = s->rank;
    }
  }
  cudaMemcpyKind k = where == CYTOM_PTR_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
  cudaError_t e = cudaMemcpyAsync(out, src, n * 4, k, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  return cuda_err(c, e, "pagerank result");
}

int pagerank_result64(Ctx* c, Job* j, double* out, int where) {
  PrState* s = prs(j);
  if (j->algo != CYTOM_ALGO_PAGERANK || j->params.kahan) return set_err(c, CYTOM_ERR_INVAL, "not an FP64 job");
  LoopState ls;
  cudaMemcpyAsync(&ls, j->ls, sizeof(ls), cudaMemcpyDeviceToHost, c->stream);
  cudaStreamSynchronize(c->stream);
  const double* r = ((ls.iter & 1u) == 0) ? s->r64 : s->r64n;
  cudaMemcpyKind k = where == CYTOM_PTR_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
  cudaError_t e = cudaMemcpyAsync(out, r, c->n * 8, k, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  return cuda_err(c, e, "pagerank result64");
}

}  // namespace cytom
