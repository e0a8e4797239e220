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
// compensated, no float atomics. Targets are binned by in-degree: one thread (<= 4
// in-edges), 4 lanes (<= 32), 8 lanes (<= 256), a warp (<= 4096) or a block (more) per
// target, all bins in one launch. Residuals, dangling mass and rank sums are FP64
// reductions.
//
// A round of PageRank-delta is that one launch: each finished target also writes its
// contribution to the next round (contributions by round parity), and the last block to
// finish runs the control step and, in a captured loop, sets the loop condition. Only the
// run's residual round has a contribution pass before the pull. The other forms run
// contributions -> pull -> control.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cstdlib>
#include <cstring>

#include "engine.h"
#include "pagerank_dev.cuh"

namespace cytom {

// The pulls of one round, every in-degree bin in one launch: bin k owns the virtual
// blocks [first[k], first[k] + nblk[k]) and walks its targets with pr_bin_vw(k) lanes per
// target (1: one thread, 0: one whole block). The heaviest bins take the lowest ids, so
// their long-running blocks start first. The layout lives in device memory (one per CSC,
// rewritten by each build) and the launch has a fixed grid that strides over the
// virtual blocks, so a captured round loop stays valid when the bins change.
struct PrBinLaunch {
  uint64_t off[kPrBins], count[kPrBins];
  uint32_t first[kPrBins], nblk[kPrBins];
  uint32_t blocks;  // virtual blocks
};

// CSC of the compacted store, per job (PageRank family).
struct Csc {
  uint32_t* src = nullptr;       // E: global source of each in-edge, grouped by target
  uint32_t* src_alt = nullptr;   // the merge's output (merge_csc_stage), swapped with src
  uint64_t cap_alt = 0;
  uint32_t* ptr = nullptr;       // n+1
  uint32_t* deg_out = nullptr;   // n: distinct out-degree (stored edges)
  uint32_t* bins = nullptr;      // n: targets, small | medium | large
  uint64_t nb[kPrBins] = {};
  PrBinLaunch* dbl = nullptr;    // the pull's bin layout (device)
  uint64_t E = 0;
  uint64_t cap = 0;
  uint64_t built_version = ~0ULL;
  // A build or merge in flight on the context's stream writes its bin sizes here (pinned)
  // and sets `pending`; csc_settle waits for it and takes nb and the bin layout from them.
  uint32_t* htot = nullptr;
  bool pending = false;
};

struct PrState {
  Csc* csc = nullptr;         // the context's CSC, shared by its PageRank-family jobs
  float* rank = nullptr;      // PR_DELTA: rank; PAGERANK fp32: r (double-buffered with rank_c)
  float* comp = nullptr;      // PR_DELTA: Kahan compensation of rank; PAGERANK fp32: r_next
  float* delta = nullptr;     // PR_DELTA: delta of the last round
  float* contrib = nullptr;   // per-source contributions (PR_DELTA: 2 x n by round parity)
  double* r64 = nullptr;      // PAGERANK fp64: r
  double* r64n = nullptr;     // PAGERANK fp64: r_next
  double* contrib64 = nullptr;
  float* lo = nullptr;        // PAGERANK / WPAGERANK fp32: low words of the ranks (2 x n)
  bool need_residual = true;
  uint64_t seen_version = ~0ULL;
  // WPAGERANK
  double* tele = nullptr;     // teleport vector (NULL = uniform 1/n)
  // WPAGERANK adjoint (allocated by the first adjoint call)
  float* lam = nullptr;       // FP32: lambda, double-buffered (2 x n)
  double* lam64 = nullptr;    // FP64: lambda, double-buffered (2 x n)
  float* pt = nullptr;        // (P^T lambda) of the last round
  double* pt64 = nullptr;
  double* cvec = nullptr;     // loss weights c
  LoopState* adj_ls = nullptr;
  // captured round loops (one per round kind), rebuilt when their launch arguments change
  cudaGraphExec_t loop_exec[8] = {};
  PrArgs loop_args[8] = {};
  const PrBinLaunch* loop_bl[8] = {};
  unsigned loop_grid[8] = {};
};

// Weighted graph of a context (WPAGERANK): CSC by target and CSR by source, both with
// the raw FP32 weights, and every vertex's out-weight sum (FP64, summed in CSR order).
struct WGraph {
  Csc in, out;
  float* in_w = nullptr;
  float* out_w = nullptr;
  uint64_t in_wcap = 0, out_wcap = 0;
  double* wsum = nullptr;
  uint64_t built_version = ~0ULL;
};

// --------------------------------------------------------------------------
// CSC construction from the tile store
// --------------------------------------------------------------------------
// Sort keys of every stored edge u -> v in the renumbered ids u' = perm[u], v' = perm[v]:
// (v', u') for the target-major CSC, (u', v') for the source-major CSR (by_source); the
// edge's weight bits ride along (vals, weighted stores). deg_out (target-major CSC): the
// distinct out-degree of each source, one atomic per source and warp (store order keeps
// a tile's edges grouped by source).
__global__ void csc_keys_kernel(const StoreDesc* __restrict__ sd, const uint32_t* __restrict__ perm,
                                uint64_t* __restrict__ keys, uint32_t* __restrict__ vals,
                                uint32_t* __restrict__ deg_out, uint32_t lg_n, int by_source) {
  const uint64_t E = sd->E;
  const uint32_t lT = sd->lT, lvpt = sd->lvpt;
  const uint32_t ymask = (uint32_t)(sd->T - 1);
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; e < E; e += stride) {
    uint32_t t = sd->chunk_tile[e >> 7];
    while (sd->tile_ptr[t + 1] <= e) ++t;
    const uint32_t p = sd->edges[e];
    const uint32_t u = perm[((t >> lT) << lvpt) | (p >> 16)];
    const uint32_t v = perm[((t & ymask) << lvpt) | (p & 0xFFFFu)];
    keys[e] = by_source ? (((uint64_t)u << lg_n) | v) : (((uint64_t)v << lg_n) | u);
    if (vals) vals[e] = sd->wts[e];
    if (deg_out) {
      const unsigned m = __match_any_sync(__activemask(), u);
      if ((threadIdx.x & 31u) == (unsigned)(__ffs(m) - 1)) atomicAdd(&deg_out[u], (unsigned)__popc(m));
    }
  }
}

// src[e] = the minor id of sorted key e; seg_lo / seg_hi[major] = the major's key range
// [lo, hi), written by the range's first and last key (both stay 0 for a major without
// keys) -- segment lengths without per-edge counters.
__global__ void csc_src_kernel(const uint64_t* __restrict__ keys, uint64_t E, uint32_t lg_n,
                               uint32_t* __restrict__ src, uint32_t* __restrict__ seg_lo,
                               uint32_t* __restrict__ seg_hi) {
  const uint64_t mask = (1ULL << lg_n) - 1ULL;
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; e < E; e += stride) {
    const uint64_t k = keys[e];
    const uint64_t mj = k >> lg_n;
    src[e] = (uint32_t)(k & mask);
    if (e == 0 || (keys[e - 1] >> lg_n) != mj) seg_lo[mj] = (uint32_t)e;
    if (e + 1 == E || (keys[e + 1] >> lg_n) != mj) seg_hi[mj] = (uint32_t)(e + 1);
  }
}

// Per vertex v: cnt[v] = its segment length, binkey[v] = its in-degree bin (pr_bin_hi) and
// vid[v] = v (vid may be seg_lo: each element is read before its own thread overwrites
// it); tot[k] += the bin sizes (one atomic per bin and block).
__global__ void csc_cnt_bins_kernel(const uint32_t* seg_lo, const uint32_t* __restrict__ seg_hi, uint64_t n,
                                    uint32_t* __restrict__ cnt, uint64_t* __restrict__ binkey, uint32_t* vid,
                                    uint32_t* __restrict__ tot) {
  __shared__ unsigned s_tot[kPrBins];
  if (threadIdx.x < kPrBins) s_tot[threadIdx.x] = 0;
  __syncthreads();
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t v = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += stride) {
    const uint32_t d = seg_hi[v] - seg_lo[v];
    int k = 0;
    while (k + 1 < kPrBins && d > pr_bin_hi(k)) ++k;
    cnt[v] = d;
    binkey[v] = (uint64_t)k;
    vid[v] = (uint32_t)v;
    const unsigned m = __match_any_sync(__activemask(), k);
    if ((threadIdx.x & 31u) == (unsigned)(__ffs(m) - 1)) atomicAdd(&s_tot[k], (unsigned)__popc(m));
  }
  __syncthreads();
  if (threadIdx.x < kPrBins && s_tot[threadIdx.x]) atomicAdd(&tot[threadIdx.x], s_tot[threadIdx.x]);
}

// ---- incremental CSC: one compaction's kept edges merged in ------------------------
// Renumbered (target, source) keys of the kept edges (csc_keys_kernel's key, by target).
__global__ void csc_delta_keys_kernel(const uint32_t* __restrict__ nloc, const uint32_t* __restrict__ ntile,
                                      uint64_t kept, const uint32_t* __restrict__ perm, uint32_t lg_n, uint32_t lT,
                                      uint32_t lvpt, uint64_t* __restrict__ keys) {
  const uint32_t ymask = (1u << lT) - 1u;
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < kept; i += stride) {
    const uint32_t t = ntile[i], p = nloc[i];
    const uint32_t u = perm[((t >> lT) << lvpt) | (p >> 16)];
    const uint32_t v = perm[((t & ymask) << lvpt) | (p & 0xFFFFu)];
    keys[i] = ((uint64_t)v << lg_n) | u;
  }
}

// Per target: the new keys it receives (cnt; the keys are sorted by target, so a warp
// adds each target's run with one atomic), and each new key's source gains an out-edge.
__global__ void csc_delta_count_kernel(const uint64_t* __restrict__ keys, uint64_t kept, uint32_t lg_n,
                                       uint32_t* __restrict__ cnt, uint32_t* __restrict__ deg_out) {
  const uint64_t mask = (1ULL << lg_n) - 1ULL;
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < kept; i += stride) {
    const uint64_t k = keys[i];
    const uint32_t t = (uint32_t)(k >> lg_n);
    const unsigned m = __match_any_sync(__activemask(), t);
    if ((threadIdx.x & 31u) == (unsigned)(__ffs(m) - 1)) atomicAdd(&cnt[t], (unsigned)__popc(m));
    atomicAdd(&deg_out[(uint32_t)(k & mask)], 1u);
  }
}

// np[v] = ptr[v] + dx[v]: the merged segment offsets (dx = new keys before target v).
__global__ void csc_new_ptr_kernel(const uint32_t* __restrict__ ptr, const uint32_t* __restrict__ dx, uint64_t n,
                                   uint32_t* __restrict__ np) {
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t v = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; v <= n; v += stride) np[v] = ptr[v] + dx[v];
}

// New keys: key j of target t lands at ptr[t] + j plus the number of t's old in-edges
// with a smaller source (ptr[t] + dx[t] + (j - dx[t]) + that count); at[j] = ptr[t] + that
// count, the old edge the key is placed before. The keys are sorted by (target, source),
// so at[] ascends.
__global__ void csc_merge_new_kernel(const uint32_t* __restrict__ ptr, const uint32_t* __restrict__ src,
                                     const uint64_t* __restrict__ keys, uint64_t kept, uint32_t lg_n,
                                     uint32_t* __restrict__ nsrc, uint32_t* __restrict__ at) {
  const uint64_t mask = (1ULL << lg_n) - 1ULL;
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; j < kept; j += stride) {
    const uint64_t k = keys[j];
    const uint32_t t = (uint32_t)(k >> lg_n), sv = (uint32_t)(k & mask);
    uint32_t a = ptr[t], b = ptr[t + 1];
    while (a < b) {
      const uint32_t m = (a + b) >> 1;
      if (src[m] < sv) a = m + 1;
      else b = m;
    }
    nsrc[(uint64_t)a + j] = sv;
    at[j] = a;
  }
}

// The old edges move in blocks of CSC_MB; jb[b] = the new keys placed before block b's
// first edge (at[j] < b * CSC_MB).
constexpr uint32_t CSC_MB = 2048;
__global__ void csc_block_keys_kernel(const uint32_t* __restrict__ at, uint64_t kept, uint32_t nblk,
                                      uint32_t* __restrict__ jb) {
  const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b > nblk) return;
  const uint64_t e = (uint64_t)b * CSC_MB;
  uint64_t lo = 0, hi = kept;
  while (lo < hi) {
    const uint64_t m = (lo + hi) >> 1;
    if ((uint64_t)at[m] < e) lo = m + 1;
    else hi = m;
  }
  jb[b] = (uint32_t)lo;
}

// Old edge e moves up by the new keys placed at or before it: jb[b] plus those of the
// block's keys with at <= e, counted by a search of the block's at[] (staged in shared
// memory when it fits). Consecutive threads take consecutive edges.
__global__ void __launch_bounds__(256) csc_merge_old_kernel(const uint32_t* __restrict__ src, uint64_t E,
                                                            const uint32_t* __restrict__ at,
                                                            const uint32_t* __restrict__ jb,
                                                            uint32_t* __restrict__ nsrc) {
  __shared__ uint32_t s_at[CSC_MB];
  const uint64_t base = (uint64_t)blockIdx.x * CSC_MB;
  const uint32_t jlo = jb[blockIdx.x], jhi = jb[blockIdx.x + 1];
  const uint32_t nk = jhi - jlo;
  const bool staged = nk <= CSC_MB;
  if (staged)
    for (uint32_t i = threadIdx.x; i < nk; i += blockDim.x) s_at[i] = at[jlo + i];
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < CSC_MB; i += blockDim.x) {
    const uint64_t e = base + i;
    if (e >= E) break;
    uint32_t a = 0, b = nk;  // keys of the block with at <= e
    while (a < b) {
      const uint32_t m = (a + b) >> 1;
      const uint32_t v = staged ? s_at[m] : at[jlo + m];
      if ((uint64_t)v <= e) a = m + 1;
      else b = m;
    }
    nsrc[e + jlo + a] = src[e];
  }
}

static int grid_n(Ctx* c, uint64_t work, int threads = 256, int per_sm = 8) {
  uint64_t b = (work + threads - 1) / threads;
  uint64_t cap = (uint64_t)c->num_sms * per_sm;
  if (b > cap) b = cap;
  return (int)std::max<uint64_t>(b, 1);
}

static uint64_t store_version(Ctx* c) { return c->version; }

// Builds a CSC (by_source = 0: each target's in-edges, `src` = their sources) or a CSR
// (by_source = 1: each source's out-edges, `src` = their targets) of the compacted store
// by one radix sort of (major, minor) keys; minor ids ascend inside each segment. With
// w != NULL the edges' weights are sorted along into *w (grown to hold E). Vertices are
// binned by segment length for the pull (small / medium / large).
static int pr_ensure_perm(Ctx* c);
static PrBinLaunch bin_launch(Ctx* c, const uint64_t* nb);

static int csc_settle(Ctx* c, Csc& q);

static int build_csx_stage(Ctx* c, Csc& q, int by_source, float** w, uint64_t* wcap) {
  int prc = pr_ensure_perm(c);
  if (prc) return prc;
  const uint64_t n = c->n, E = c->E;
  uint32_t lg_n = 0;
  while ((1ULL << lg_n) < n) ++lg_n;
  if (E > 0xFFFFFFFFULL - (1ULL << 20)) return set_err(c, CYTOM_ERR_RANGE, "PageRank CSC holds fewer than 2^32 - 2^20 edges");
  if (E > q.cap || !q.src) {
    cudaFree(q.src);
    q.cap = std::max<uint64_t>(E + E / 4, 1024);
    if (cy_malloc(&q.src, q.cap * 4) != cudaSuccess) return set_err(c, CYTOM_ERR_OOM, "CSC");
  }
  if (w && (E > *wcap || !*w)) {
    cudaFree(*w);
    *wcap = std::max<uint64_t>(E + E / 4, 1024);
    if (cy_malloc(w, *wcap * 4) != cudaSuccess) return set_err(c, CYTOM_ERR_OOM, "CSC weights");
  }
  if (!q.ptr) {
    if (cy_malloc(&q.ptr, (n + 1) * 4) != cudaSuccess || cy_malloc(&q.deg_out, n * 4) != cudaSuccess ||
        cy_malloc(&q.bins, n * 4) != cudaSuccess)
      return set_err(c, CYTOM_ERR_OOM, "CSC index");
  }
  if ((!q.htot && cy_malloc_host(&q.htot, 64) != cudaSuccess) ||
      (!q.dbl && cy_malloc(&q.dbl, sizeof(PrBinLaunch)) != cudaSuccess))
    return set_err(c, CYTOM_ERR_OOM, "CSC bins");
  char* tmp = nullptr;
  const size_t kbytes = std::max<uint64_t>(std::max<uint64_t>(E, n), 1) * 8;
  const size_t vbytes = w ? std::max<uint64_t>(E, 1) * 4 : 0;
  const size_t nbytes = n * 4;
  if (cy_malloc_async((void**)&tmp, 2 * kbytes + 2 * vbytes + 3 * nbytes + 64, c->stream) != cudaSuccess)
    return set_err(c, CYTOM_ERR_OOM, "CSC temporaries");
  uint64_t* k0 = (uint64_t*)tmp;
  uint64_t* k1 = (uint64_t*)(tmp + kbytes);
  uint32_t* v0 = w ? (uint32_t*)(tmp + 2 * kbytes) : nullptr;
  uint32_t* v1 = w ? (uint32_t*)(tmp + 2 * kbytes + vbytes) : nullptr;
  uint32_t* cnt = (uint32_t*)(tmp + 2 * kbytes + 2 * vbytes);
  uint32_t* seg_lo = cnt + n;  // then the vertex ids the bin sort moves
  uint32_t* seg_hi = seg_lo + n;
  uint32_t* tot = seg_hi + n;  // kPrBins totals
  cudaMemsetAsync(q.deg_out, 0, n * 4, c->stream);
  cudaMemsetAsync(seg_lo, 0, 2 * nbytes + 64, c->stream);
  int rc = CYTOM_OK;
  if (E) {
    csc_keys_kernel<<<grid_n(c, E), 256, 0, c->stream>>>(c->dsd, c->pr_perm, k0, v0, by_source ? nullptr : q.deg_out,
                                                         lg_n, by_source);
    c->launches++;
    bool alt = false;
    rc = radix_sort_pairs(c, k0, k1, v0, v1, E, (int)(2 * lg_n), &alt);
    if (rc) return rc;
    csc_src_kernel<<<grid_n(c, E), 256, 0, c->stream>>>(alt ? k1 : k0, E, lg_n, q.src, seg_lo, seg_hi);
    c->launches++;
    if (w) cudaMemcpyAsync(*w, alt ? v1 : v0, E * 4, cudaMemcpyDeviceToDevice, c->stream);
  }
  // segment lengths and bin keys, then the offsets and one stable 3-bit sort of the
  // vertices by bin (vertex order kept inside each bin)
  csc_cnt_bins_kernel<<<grid_n(c, n), 256, 0, c->stream>>>(seg_lo, seg_hi, n, cnt, k0, seg_lo, tot);
  c->launches++;
  rc = exclusive_scan_u32(c, cnt, q.ptr, n, q.ptr + n);
  if (rc) return rc;
  bool balt = false;
  rc = radix_sort_pairs(c, k0, k1, seg_lo, q.bins, n, 3, &balt);
  if (rc) return rc;
  if (!balt) cudaMemcpyAsync(q.bins, seg_lo, nbytes, cudaMemcpyDeviceToDevice, c->stream);
  cudaMemcpyAsync(q.htot, tot, kPrBins * 4, cudaMemcpyDeviceToHost, c->stream);
  cudaFreeAsync(tmp, c->stream);
  q.E = E;
  q.pending = true;
  return cuda_err(c, cudaGetLastError(), "CSC build");
}

// Waits for the build or merge in flight (if any) and installs its bin sizes and layout.
static int csc_settle(Ctx* c, Csc& q) {
  if (!q.pending) return CYTOM_OK;
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_err(c, e, "CSC build");
  q.pending = false;
  for (int k = 0; k < kPrBins; ++k) q.nb[k] = q.htot[k];
  const PrBinLaunch hb = bin_launch(c, q.nb);
  // pageable source: the call returns once the bytes are staged
  e = cudaMemcpyAsync(q.dbl, &hb, sizeof(hb), cudaMemcpyHostToDevice, c->stream);
  return e == cudaSuccess ? CYTOM_OK : cuda_err(c, e, "CSC bins");
}

static int build_csx(Ctx* c, Csc& q, int by_source, float** w, uint64_t* wcap) {
  int rc = build_csx_stage(c, q, by_source, w, wcap);
  return rc ? rc : csc_settle(c, q);
}

static int build_csc_stage(Ctx* c, Csc& q) { return build_csx_stage(c, q, 0, nullptr, nullptr); }

// Called by the compaction once it knows its kept edges (nloc / ntile, `kept` of them):
// while the context's CSC matches the store before this compaction, the edges are saved
// as CSC keys for merge_csc_stage. Without room for them the next build re-sorts.
int pagerank_note_kept(Ctx* c, const uint32_t* nloc, const uint32_t* ntile, uint64_t kept) {
  c->pr_delta_version = ~0ULL;
  const Csc* q = reinterpret_cast<const Csc*>(c->pr_csc);
  if (!q || !q->src || !c->pr_perm || q->built_version != c->version) return CYTOM_OK;
  if (kept > c->pr_delta_cap || !c->pr_delta_keys) {
    cudaFree(c->pr_delta_keys);
    c->pr_delta_keys = nullptr;
    c->pr_delta_cap = 0;
    const uint64_t cap = std::max<uint64_t>(kept + kept / 2, 1024);
    if (cy_malloc(&c->pr_delta_keys, cap * 8) != cudaSuccess) {
      cudaGetLastError();
      return CYTOM_OK;
    }
    c->pr_delta_cap = cap;
  }
  uint32_t lg_n = 0;
  while ((1ULL << lg_n) < c->n) ++lg_n;
  if (kept) {
    csc_delta_keys_kernel<<<grid_n(c, kept), 256, 0, c->stream>>>(nloc, ntile, kept, c->pr_perm, lg_n, c->lT, c->lvpt,
                                                                  c->pr_delta_keys);
    c->launches++;
  }
  c->pr_delta_count = kept;
  c->pr_delta_version = c->version + 1;
  return cuda_err(c, cudaGetLastError(), "CSC delta keys");
}

// The CSC after one compaction that only added edges: the saved keys sorted, counted
// per target and merged into the old segments (csc_merge_old_kernel, csc_merge_new_kernel) -- the same CSC,
// offsets, out-degrees and bins a full build of the new store gives, without re-sorting
// the old edges.
static int merge_csc_stage(Ctx* c, Csc& q) {
  const uint64_t n = c->n, K = c->pr_delta_count, E = q.E + K;
  if (E != c->E || E > 0xFFFFFFFFULL - (1ULL << 20)) return build_csc_stage(c, q);
  uint32_t lg_n = 0;
  while ((1ULL << lg_n) < n) ++lg_n;
  if (E > q.cap_alt || !q.src_alt) {
    cudaFree(q.src_alt);
    q.src_alt = nullptr;
    q.cap_alt = 0;
    const uint64_t cap = std::max<uint64_t>(E + E / 4, 1024);
    if (cy_malloc(&q.src_alt, cap * 4) != cudaSuccess) {
      cudaGetLastError();
      return build_csc_stage(c, q);
    }
    q.cap_alt = cap;
  }
  const size_t kb = std::max<uint64_t>(K, 1) * 8, nb8 = std::max<uint64_t>(n, 1) * 8, n4 = (n + 1) * 4;
  const size_t ab = std::max<uint64_t>(K, 1) * 4 + ((q.E + CSC_MB - 1) / CSC_MB + 2) * 4;
  char* tmp = nullptr;
  if (cy_malloc_async((void**)&tmp, kb + 2 * nb8 + 4 * n4 + 64 + ab, c->stream) != cudaSuccess)
    return set_err(c, CYTOM_ERR_OOM, "CSC merge temporaries");
  uint64_t* kalt = (uint64_t*)tmp;
  uint64_t* bk0 = (uint64_t*)(tmp + kb);
  uint64_t* bk1 = (uint64_t*)(tmp + kb + nb8);
  uint32_t* cnt = (uint32_t*)(tmp + kb + 2 * nb8);
  uint32_t* dx = cnt + (n + 1);
  uint32_t* np = dx + (n + 1);
  uint32_t* vid = np + (n + 1);
  uint32_t* tot = vid + (n + 1);
  uint32_t* at = tot + 16;  // the old edge each new key is placed before
  uint32_t* jb = at + std::max<uint64_t>(K, 1);  // new keys before each block of the merge
  bool alt = false;
  int rc = radix_sort_pairs(c, c->pr_delta_keys, kalt, nullptr, nullptr, K, (int)(2 * lg_n), &alt);
  if (rc) {
    cudaFreeAsync(tmp, c->stream);
    return rc;
  }
  const uint64_t* keys = alt ? kalt : c->pr_delta_keys;
  cudaMemsetAsync(cnt, 0, n4, c->stream);
  cudaMemsetAsync(tot, 0, 64, c->stream);
  if (K) {
    csc_delta_count_kernel<<<grid_n(c, K), 256, 0, c->stream>>>(keys, K, lg_n, cnt, q.deg_out);
    c->launches++;
  }
  rc = exclusive_scan_u32(c, cnt, dx, n, dx + n);
  if (rc) {
    cudaFreeAsync(tmp, c->stream);
    return rc;
  }
  csc_new_ptr_kernel<<<grid_n(c, n + 1), 256, 0, c->stream>>>(q.ptr, dx, n, np);
  const uint64_t Eo = q.E;
  const uint32_t mblk = (uint32_t)((Eo + CSC_MB - 1) / CSC_MB);
  if (K) csc_merge_new_kernel<<<grid_n(c, K), 256, 0, c->stream>>>(q.ptr, q.src, keys, K, lg_n, q.src_alt, at);
  csc_block_keys_kernel<<<(mblk + 1 + 255) / 256, 256, 0, c->stream>>>(at, K, mblk, jb);
  if (mblk) csc_merge_old_kernel<<<mblk, 256, 0, c->stream>>>(q.src, Eo, at, jb, q.src_alt);
  c->launches += 4;
  // bins of the new in-degrees, as build_csx makes them
  csc_cnt_bins_kernel<<<grid_n(c, n), 256, 0, c->stream>>>(np, np + 1, n, cnt, bk0, vid, tot);
  c->launches++;
  bool balt = false;
  rc = radix_sort_pairs(c, bk0, bk1, vid, q.bins, n, 3, &balt);
  if (rc) {
    cudaFreeAsync(tmp, c->stream);
    return rc;
  }
  if (!balt) cudaMemcpyAsync(q.bins, vid, n * 4, cudaMemcpyDeviceToDevice, c->stream);
  cudaMemcpyAsync(q.ptr, np, n4, cudaMemcpyDeviceToDevice, c->stream);
  cudaMemcpyAsync(q.htot, tot, kPrBins * 4, cudaMemcpyDeviceToHost, c->stream);
  cudaFreeAsync(tmp, c->stream);
  std::swap(q.src, q.src_alt);  // later work on the stream reads the merged array
  std::swap(q.cap, q.cap_alt);
  q.E = E;
  q.pending = true;
  return cuda_err(c, cudaGetLastError(), "CSC merge");
}

constexpr uint64_t kCscMergeMinEdges = 1ULL << 21;

// The CSC for the current store, enqueued on the context's stream: merged from the
// previous one when exactly one compaction (that saved its kept edges) lies between
// them, rebuilt otherwise. csc_settle completes it.
static int update_csc_stage(Ctx* c, Csc& q) {
  int rc = csc_settle(c, q);  // the merge reads the previous bins
  if (rc) return rc;
  // below about 2 M edges a full sort is as fast as the merge's extra passes (RMAT-16
  // PageRank-delta stream: 1.30 ms per update with full builds, 1.37 with merges)
  if (q.src && q.dbl && q.built_version != ~0ULL && q.built_version + 1 == c->version &&
      c->pr_delta_version == c->version && q.E >= kCscMergeMinEdges)
    rc = merge_csc_stage(c, q);
  else
    rc = build_csc_stage(c, q);
  if (!rc) q.built_version = c->version;
  return rc;
}

static int update_csc(Ctx* c, Csc& q) {
  int rc = q.built_version == c->version ? CYTOM_OK : update_csc_stage(c, q);
  return rc ? rc : csc_settle(c, q);
}

// The batched executor enqueues every snapshot's CSC update before it waits for any, so
// the updates of several contexts run side by side.
int pagerank_csc_stage(Ctx* c) {
  Csc* q = reinterpret_cast<Csc*>(c->pr_csc);
  if (!q || q->built_version == c->version) return CYTOM_OK;
  return update_csc_stage(c, *q);
}

// ---- renumbering by out-degree ---------------------------------------------------
__global__ void perm_keys_kernel(const uint32_t* __restrict__ deg, uint64_t n, uint32_t lg_n,
                                 uint64_t* __restrict__ keys) {
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t v = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += stride)
    keys[v] = ((uint64_t)(0xFFFFFFFFu - deg[v]) << lg_n) | v;  // descending degree, then id
}
__global__ void perm_from_keys_kernel(const uint64_t* __restrict__ keys, uint64_t n, uint32_t lg_n,
                                      uint32_t* __restrict__ perm, uint32_t* __restrict__ inv) {
  const uint64_t mask = (lg_n >= 64) ? ~0ULL : ((1ULL << lg_n) - 1ULL);
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const uint32_t v = (uint32_t)(keys[i] & mask);
    inv[i] = v;
    perm[v] = (uint32_t)i;
  }
}
// out[perm[v]] = in[v] (to the renumbering) or out[v] = in[perm[v]] (back), any 4- or 8-byte type
template <typename T>
__global__ void permute_kernel(const T* __restrict__ in, const uint32_t* __restrict__ perm, uint64_t n,
                               int to_renumbered, T* __restrict__ out) {
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t v = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += stride) {
    if (to_renumbered) out[perm[v]] = in[v];
    else out[v] = in[perm[v]];
  }
}

// The renumbering, made once per context from the out-degrees of the graph at that time
// (a later graph keeps it: any numbering gives the same results, this one only packs
// the sources most edges read into few cache lines).
static int pr_ensure_perm(Ctx* c) {
  if (c->pr_perm) return CYTOM_OK;
  const uint64_t n = c->n;
  uint32_t lg_n = 0;
  while ((1ULL << lg_n) < n) ++lg_n;
  uint64_t* k = nullptr;
  uint32_t *perm = nullptr, *inv = nullptr;
  if (cy_malloc_async((void**)&k, 2 * n * 8, c->stream) != cudaSuccess || cy_malloc(&perm, n * 4) != cudaSuccess ||
      cy_malloc(&inv, n * 4) != cudaSuccess) {
    cudaGetLastError();
    if (k) cudaFreeAsync(k, c->stream);
    if (perm) cudaFree(perm);
    return set_err(c, CYTOM_ERR_OOM, "vertex renumbering");
  }
  c->pr_perm = perm;
  c->pr_inv = inv;
  perm_keys_kernel<<<grid_n(c, n), 256, 0, c->stream>>>(c->out_deg, n, lg_n, k);
  bool alt = false;
  int rc = radix_sort_pairs(c, k, k + n, nullptr, nullptr, n, (int)(32 + lg_n), &alt);
  if (rc) return rc;
  perm_from_keys_kernel<<<grid_n(c, n), 256, 0, c->stream>>>(alt ? k + n : k, n, lg_n, c->pr_perm, c->pr_inv);
  c->launches += 2;
  cudaFreeAsync(k, c->stream);
  return cuda_err(c, cudaGetLastError(), "vertex renumbering");
}

// Multiplicity out-degrees in the renumbering (PageRank-delta), per graph version.
static int pr_deg_mult(Ctx* c) {
  int rc = pr_ensure_perm(c);
  if (rc) return rc;
  if (c->pr_deg_mult && c->pr_deg_mult_version == c->version) return CYTOM_OK;
  if (!c->pr_deg_mult && cy_malloc(&c->pr_deg_mult, c->n * 4) != cudaSuccess)
    return set_err(c, CYTOM_ERR_OOM, "degrees");
  permute_kernel<uint32_t><<<grid_n(c, c->n), 256, 0, c->stream>>>(c->out_deg, c->pr_perm, c->n, 1, c->pr_deg_mult);
  c->launches++;
  c->pr_deg_mult_version = c->version;
  return cuda_err(c, cudaGetLastError(), "degrees");
}

// --------------------------------------------------------------------------
// Round kernels
// --------------------------------------------------------------------------
// Per-vertex contribution of the round and the dangling mass (PAGERANK).
template <int MODE>
__global__ void pr_contrib_kernel(PrArgs a) {
  LoopState* ls = a.ls;
  if (!ls->cont) return;
  const unsigned p = ls->iter & 1u;
  const pr_ff_t<MODE> dangling = pr_contrib_range<MODE, false>(a, p, 0, a.n, (uint64_t)blockIdx.x * blockDim.x + threadIdx.x,
                                                        (uint64_t)gridDim.x * blockDim.x);
  pr_dangling_flush<MODE>(ls, p, dangling);
}

template <int MODE>
__device__ __forceinline__ void pull_small_body(const PrArgs& a, const pr_val_t<MODE>* cr, unsigned p, pr_ff_t<MODE> dang,
                                                uint64_t bid, uint64_t nblk, PrTally& t) {
  const uint64_t stride = nblk * blockDim.x;
  for (uint64_t base = bid * blockDim.x; base < a.bin_count; base += stride) {
    const uint64_t i = base + threadIdx.x;
    if (i < a.bin_count) {
      const uint32_t v = a.bins[a.bin_off + i];
      const pr_ff_t<MODE> sum = pr_sum_thread<MODE, false>(a, cr, v);
      pr_finish<MODE, false>(a, v, sum, p, dang, t);
    }
  }
}

template <int MODE, int VW>
__device__ __forceinline__ void pull_group_body(const PrArgs& a, const pr_val_t<MODE>* cr, unsigned p, pr_ff_t<MODE> dang,
                                                uint64_t bid, uint64_t nblk, PrTally& t) {
  constexpr uint64_t GPW = 32 / VW;  // groups per warp
  const unsigned gl = threadIdx.x & (VW - 1);
  const uint64_t gid = (bid * blockDim.x + threadIdx.x) / VW;
  const uint64_t ngroups = (nblk * blockDim.x) / VW;
  // warp-uniform trip count: every lane stays in the loop for the group shuffles
  const uint64_t gbase = gid - (gid % GPW);
  for (uint64_t b = gbase; b < a.bin_count; b += ngroups) {
    const uint64_t i = b + (gid - gbase);
    uint32_t v = 0, lo = 0, hi = 0;
    if (i < a.bin_count) {
      v = a.bins[a.bin_off + i];
      lo = a.csc_ptr[v];
      hi = a.csc_ptr[v + 1];
    }
    const pr_ff_t<MODE> sum = pr_sum_group<MODE, false, VW>(a, cr, lo, hi, gl);
    if (gl == 0 && i < a.bin_count) pr_finish<MODE, false>(a, v, sum, p, dang, t);
  }
}

template <int MODE>
__device__ __forceinline__ void pull_large_body(const PrArgs& a, const pr_val_t<MODE>* cr, unsigned p, pr_ff_t<MODE> dang,
                                                uint64_t bid, uint64_t nblk, PrTally& t) {
  for (uint64_t i = bid; i < a.bin_count; i += nblk) {
    const uint32_t v = a.bins[a.bin_off + i];
    const pr_ff_t<MODE> sum = pr_sum_block<MODE, false>(a, cr, v);
    if (threadIdx.x == 0) pr_finish<MODE, false>(a, v, sum, p, dang, t);
  }
}

// Ends the round: records the FP64 residual, decides whether to continue. In a captured
// loop it also sets the loop condition, and bounds the loop by its own count of rounds
// (max_iter + 2; beyond it the run stops with err = 2).
__device__ __forceinline__ void pr_loop_control(LoopState* ls, int mode, cudaGraphConditionalHandle h,
                                                int use_handle) {
  unsigned cont = pr_control_step(ls, mode);
  if (use_handle) {
    const unsigned started = ls->sel_rounds + 1;
    ls->sel_rounds = started;
    if ((unsigned long long)started > (unsigned long long)ls->max_iter + 2ULL) {
      ls->err = 2u;
      ls->cont = 0u;
      cont = 0u;
    }
    cudaGraphSetConditional(h, cont);
  }
}

// Fused forms: the control step and loop condition of the round, run by the last block
// of the pull to finish (every block counts itself in after its results are visible;
// the wrapping increment leaves the counter at 0 for the next round).
__device__ __forceinline__ void pr_round_end(LoopState* ls, int mode, cudaGraphConditionalHandle h, int use_handle) {
  __shared__ unsigned s_last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) s_last = atomicInc(&ls->apply_done, gridDim.x - 1u) == gridDim.x - 1u ? 1u : 0u;
  __syncthreads();
  if (s_last && threadIdx.x == 0) {
    __threadfence();
    pr_loop_control(ls, mode, h, use_handle);
  }
}

// Every block takes part in the round end of the fused forms, whether or not the run
// still continues (a captured loop's condition is only set here).
// The virtual blocks of the bin layout from blockIdx.x on, gridDim.x apart.
template <int MODE>
__device__ __forceinline__ void pull_vblocks(PrArgs& a, const pr_val_t<MODE>* cr, unsigned p, pr_ff_t<MODE> dang,
                                             const PrBinLaunch* __restrict__ blp, uint32_t total, PrTally& t) {
  for (uint32_t vb = blockIdx.x; vb < total; vb += gridDim.x) {
    int k = 0;
    while (k < kPrBins && !(vb >= blp->first[k] && vb - blp->first[k] < blp->nblk[k])) ++k;
    if (k == kPrBins) continue;
    const uint64_t bid = vb - blp->first[k], nblk = blp->nblk[k];
    a.bin_off = blp->off[k];
    a.bin_count = blp->count[k];
    switch (pr_bin_vw(k)) {
      case 1: pull_small_body<MODE>(a, cr, p, dang, bid, nblk, t); break;
      case 4: pull_group_body<MODE, 4>(a, cr, p, dang, bid, nblk, t); break;
      case 8: pull_group_body<MODE, 8>(a, cr, p, dang, bid, nblk, t); break;
      case 32: pull_group_body<MODE, 32>(a, cr, p, dang, bid, nblk, t); break;
      default: pull_large_body<MODE>(a, cr, p, dang, bid, nblk, t);
    }
  }
}

template <int MODE>
__global__ void __launch_bounds__(PR_T) pr_pull_kernel(PrArgs a, const PrBinLaunch* __restrict__ blp,
                                                       cudaGraphConditionalHandle h, int use_handle) {
  LoopState* ls = a.ls;
  const bool live = ls->cont != 0;
  if (!live && !pr_fused<MODE>()) return;
  const unsigned p = ls->iter & 1u;
  PrTally t;
  t.init();
  const uint32_t total = live ? blp->blocks : 0u;
  const pr_ff_t<MODE> dang = pr_dang_arg<MODE, false>(a, ls, p);
  const pr_val_t<MODE>* cr = pr_cread<MODE>(a, p);
  pull_vblocks<MODE>(a, cr, p, dang, blp, total, t);
  if (live) pr_tally_flush<MODE>(ls, p, t);
  if constexpr (pr_fused<MODE>()) pr_round_end(ls, MODE, h, use_handle);
}



// The control step as its own launch (the forms without a fused round end).
__global__ void pr_control_kernel(LoopState* ls, int mode, cudaGraphConditionalHandle h, int use_handle) {
  pr_loop_control(ls, mode, h, use_handle);
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
  pr_begin_state(ls, max_iter, tol, edges);
}

static PrState* prs(Job* j) { return reinterpret_cast<PrState*>(j->ext); }

// One CSC per context (per snapshot), rebuilt when the store changed, shared by every
// PageRank-family job of the context.
static Csc* ctx_csc(Ctx* c) {
  if (!c->pr_csc) c->pr_csc = new (std::nothrow) Csc();
  return reinterpret_cast<Csc*>(c->pr_csc);
}

static void csc_free(Csc* q) {
  void* ptrs[] = {q->src, q->src_alt, q->ptr, q->deg_out, q->bins, q->dbl};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (q->htot) cudaFreeHost(q->htot);
}

static WGraph* ctx_wgraph(Ctx* c) {
  if (!c->pr_wgraph) c->pr_wgraph = new (std::nothrow) WGraph();
  return reinterpret_cast<WGraph*>(c->pr_wgraph);
}

void pagerank_ctx_free(Ctx* c) {
  void* pp[] = {c->pr_perm, c->pr_inv, c->pr_deg_mult, c->pr_delta_keys};
  for (void* p : pp)
    if (p) cudaFree(p);
  c->pr_perm = c->pr_inv = c->pr_deg_mult = nullptr;
  c->pr_delta_keys = nullptr;
  c->pr_delta_cap = 0;
  c->pr_delta_version = ~0ULL;
  Csc* q = reinterpret_cast<Csc*>(c->pr_csc);
  if (q) {
    csc_free(q);
    delete q;
    c->pr_csc = nullptr;
  }
  WGraph* g = reinterpret_cast<WGraph*>(c->pr_wgraph);
  if (g) {
    csc_free(&g->in);
    csc_free(&g->out);
    void* ptrs[] = {g->in_w, g->out_w, g->wsum};
    for (void* p : ptrs)
      if (p) cudaFree(p);
    delete g;
    c->pr_wgraph = nullptr;
  }
}

int pagerank_alloc(Ctx* c, Job* j) {
  PrState* s = new (std::nothrow) PrState();
  if (!s) return set_err(c, CYTOM_ERR_OOM, "PageRank state");
  j->ext = s;
  s->csc = ctx_csc(c);
  if (!s->csc) return set_err(c, CYTOM_ERR_OOM, "PageRank CSC");
  const uint64_t n = c->n;
  bool ok = true;
  if (j->algo == CYTOM_ALGO_PR_DELTA) {
    ok = ok && cy_malloc(&s->rank, n * 4) == cudaSuccess;
    ok = ok && cy_malloc(&s->comp, n * 4) == cudaSuccess;
    ok = ok && cy_malloc(&s->delta, n * 4) == cudaSuccess;
    ok = ok && cy_malloc(&s->contrib, 2 * n * 4) == cudaSuccess;
  } else if (j->params.kahan) {
    ok = ok && cy_malloc(&s->rank, n * 4) == cudaSuccess;
    ok = ok && cy_malloc(&s->comp, n * 4) == cudaSuccess;
    ok = ok && cy_malloc(&s->lo, 2 * n * 4) == cudaSuccess;
    ok = ok && cy_malloc(&s->contrib, n * 4) == cudaSuccess;
  } else {
    ok = ok && cy_malloc(&s->r64, n * 8) == cudaSuccess;
    ok = ok && cy_malloc(&s->r64n, n * 8) == cudaSuccess;
    ok = ok && cy_malloc(&s->contrib64, n * 8) == cudaSuccess;
    ok = ok && cy_malloc(&s->rank, n * 4) == cudaSuccess;  // float copy for results
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
  for (auto& g : s->loop_exec)
    if (g) cudaGraphExecDestroy(g);
  void* ptrs[] = {s->rank, s->comp, s->delta, s->contrib, s->r64,  s->r64n, s->contrib64, s->lo,
                  s->tele, s->lam,  s->lam64, s->pt,      s->pt64, s->cvec, s->adj_ls};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  delete s;
  j->ext = nullptr;
}

int pagerank_init(Ctx* c, Job* j) {
  PrState* s = prs(j);
  int prc = pr_ensure_perm(c);
  if (prc) return prc;
  const uint64_t n = c->n;
  int g = grid_n(c, n);
  if (j->algo == CYTOM_ALGO_PR_DELTA) {
    // reference init_vertices: rank 0 with delta 1 everywhere; here rank = 1 and the
    // residual round reproduces the reference's first iteration
    pr_fill_kernel<<<g, 256, 0, c->stream>>>(s->rank, 1.0f, n);
    cudaMemsetAsync(s->comp, 0, n * 4, c->stream);
    cudaMemsetAsync(s->delta, 0, n * 4, c->stream);
    c->launches++;
  } else if (j->algo == CYTOM_ALGO_WPAGERANK && s->tele) {
    if (j->params.kahan) pr_to_float_kernel<<<g, 256, 0, c->stream>>>(s->tele, s->rank, n);
    else cudaMemcpyAsync(s->r64, s->tele, n * 8, cudaMemcpyDeviceToDevice, c->stream);
    c->launches++;
  } else if (j->params.kahan) {
    pr_fill_kernel<<<g, 256, 0, c->stream>>>(s->rank, (float)(1.0 / (double)n), n);
    c->launches++;
  } else {
    pr_fill64_kernel<<<g, 256, 0, c->stream>>>(s->r64, 1.0 / (double)n, n);
    c->launches++;
  }
  if (s->lo) cudaMemsetAsync(s->lo, 0, 2 * n * 4, c->stream);
  s->need_residual = true;
  return cuda_err(c, cudaGetLastError(), "pagerank init");
}

int pagerank_seed(Ctx* c, Job* j, const uint32_t*, const uint32_t*, const uint32_t*, uint64_t) {
  // the next run starts with a residual round over the new snapshot
  prs(j)->need_residual = true;
  (void)c;
  return CYTOM_OK;
}

// Blocks per bin of the one-launch pull, heaviest bin first (as the bins' own launches
// would use).
static PrBinLaunch bin_launch(Ctx* c, const uint64_t* nb) {
  PrBinLaunch bl{};
  uint64_t off = 0;
  for (int k = 0; k < kPrBins; ++k) {
    bl.off[k] = off;
    bl.count[k] = nb[k];
    off += nb[k];
  }
  uint64_t blocks = 0;
  for (int k = kPrBins - 1; k >= 0; --k) {
    uint64_t b = 0;
    if (nb[k]) {
      switch (pr_bin_vw(k)) {
        case 1: b = grid_n(c, nb[k], PR_T); break;
        case 4: b = grid_n(c, nb[k] * 4, PR_T); break;
        case 8: b = grid_n(c, nb[k] * 8, PR_T); break;
        case 32: b = grid_n(c, nb[k] * 32, PR_T); break;
        default: b = std::min<uint64_t>(nb[k], (uint64_t)c->num_sms * 4);
      }
    }
    bl.first[k] = (uint32_t)blocks;
    bl.nblk[k] = (uint32_t)b;
    blocks += b;
  }
  bl.blocks = (uint32_t)blocks;
  return bl;
}

// The pull's grid. Fused form: as many blocks as fit on the device at once, striding
// over the virtual blocks (a captured loop outlives changes of the bins; at least one
// block, so the round end always runs). The others: one block per virtual block, which
// the hardware balances (a persistent grid lost 5-10 % on RMAT-26 PageRank).
template <int MODE>
static unsigned pull_grid(Ctx* c, const Csc& q) {
  if (!pr_fused<MODE>()) return std::max<uint32_t>(bin_launch(c, q.nb).blocks, 1u);
  static int per_sm = -1;
  if (per_sm < 0) {
    int b = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, pr_pull_kernel<MODE>, PR_T, 0) != cudaSuccess) {
      cudaGetLastError();
      b = 4;
    }
    per_sm = std::max(b, 1);
  }
  return (unsigned)(c->num_sms * per_sm);
}

// Whether a round of this form opens with a contribution pass: every round of the
// unfused forms, PageRank-delta's residual round (its delta rounds take the previous
// pull's contributions).
template <int MODE>
static constexpr bool pr_opens_with_contrib() {
  return !pr_fused<MODE>() || MODE == PR_DELTA_RESIDUAL;
}

// One round (first: the run's first round). Fused form: the pull alone (its last block
// runs the control step), after the residual round's contribution pass; the others:
// contributions -> pull -> control.
template <int MODE>
static int launch_round(Ctx* c, const PrArgs& base_args, const Csc& q, bool first) {
  PrArgs a = base_args;
  int launched = 0;
  if (!pr_fused<MODE>() || (first && pr_opens_with_contrib<MODE>())) {
    pr_contrib_kernel<MODE><<<grid_n(c, c->n), 256, 0, c->stream>>>(a);
    ++launched;
  }
  cudaGraphConditionalHandle h{};
  pr_pull_kernel<MODE><<<pull_grid<MODE>(c, q), PR_T, 0, c->stream>>>(a, q.dbl, h, 0);
  ++launched;
  if (!pr_fused<MODE>()) {
    pr_control_kernel<<<1, 1, 0, c->stream>>>(a.ls, MODE, h, 0);
    ++launched;
  }
  c->launches += launched;
  return cuda_err(c, cudaGetLastError(), "pagerank round");
}

static cudaError_t pr_add_kernel(cudaGraph_t g, cudaGraphNode_t* node, const cudaGraphNode_t* deps, size_t ndeps,
                                 void* fn, dim3 grid, dim3 block, void** args) {
  cudaKernelNodeParams kp{};
  kp.func = fn;
  kp.gridDim = grid;
  kp.blockDim = block;
  kp.kernelParams = args;
  return cudaGraphAddKernelNode(node, g, deps, ndeps, &kp);
}

// The round loop as one CUDA graph; a run is one graph launch. Fused form: while(cont)
// { pull, whose last block sets the condition }; the others: while(cont) { contributions
// -> pull -> control, which sets the condition }.
template <int MODE>
static int build_round_graph(Ctx* c, const PrArgs& base, const Csc& q, cudaGraphExec_t* out) {
  constexpr bool F = pr_fused<MODE>();
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaGraphCreate(&g, 0);
  if (e != cudaSuccess) return cuda_err(c, e, "graph create");
  PrArgs a = base;
  void* a_c[] = {(void*)&a};
  cudaGraphNode_t n_pre;
  const bool pre = F && pr_opens_with_contrib<MODE>();
  if (pre)
    e = pr_add_kernel(g, &n_pre, nullptr, 0, (void*)pr_contrib_kernel<MODE>, dim3(grid_n(c, c->n)), dim3(256), a_c);
  cudaGraphConditionalHandle h;
  if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault);
  cudaGraphNodeParams cp{};
  cp.type = cudaGraphNodeTypeConditional;
  cp.conditional.handle = h;
  cp.conditional.type = cudaGraphCondTypeWhile;
  cp.conditional.size = 1;
  cudaGraphNode_t wnode;
  if (e == cudaSuccess) e = cudaGraphAddNode(&wnode, g, pre ? &n_pre : nullptr, nullptr, pre ? 1 : 0, &cp);
  if (e == cudaSuccess) {
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    const PrBinLaunch* blp = q.dbl;
    const dim3 pg(pull_grid<MODE>(c, q));
    LoopState* ls = base.ls;
    int mode = MODE, one = 1;
    void* a_p[] = {(void*)&a, (void*)&blp, (void*)&h, (void*)&one};
    if (F) {
      cudaGraphNode_t n_p;
      e = pr_add_kernel(body, &n_p, nullptr, 0, (void*)pr_pull_kernel<MODE>, pg, dim3(PR_T), a_p);
    } else {
      cudaGraphNode_t n_c, n_p, n_ctl;
      int zero = 0;
      void* a_p0[] = {(void*)&a, (void*)&blp, (void*)&h, (void*)&zero};
      e = pr_add_kernel(body, &n_c, nullptr, 0, (void*)pr_contrib_kernel<MODE>, dim3(grid_n(c, c->n)), dim3(256), a_c);
      if (e == cudaSuccess)
        e = pr_add_kernel(body, &n_p, &n_c, 1, (void*)pr_pull_kernel<MODE>, pg, dim3(PR_T), a_p0);
      void* a_ctl[] = {(void*)&ls, (void*)&mode, (void*)&h, (void*)&one};
      if (e == cudaSuccess)
        e = pr_add_kernel(body, &n_ctl, &n_p, 1, (void*)pr_control_kernel, dim3(1), dim3(1), a_ctl);
    }
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(out, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) {
    cudaGetLastError();
    *out = nullptr;
    return CYTOM_ERR_CUDA;
  }
  return CYTOM_OK;
}

static bool pr_use_graphs() {
  static int v = -1;
  if (v < 0) {
    const char* s = getenv("CYTOM_NO_GRAPH");
    v = (s && s[0] == '1') ? 0 : 1;
  }
  return v == 1;
}

template <int MODE>
static int run_rounds(Ctx* c, Job* j, const PrArgs& a, uint64_t max_rounds, const Csc& q) {
  if (max_rounds > 1 && !c->profiling && pr_use_graphs()) {
    PrState* s = prs(j);
    cudaGraphExec_t& gx = s->loop_exec[MODE];
    const unsigned grid = pull_grid<MODE>(c, q);
    if (gx && (memcmp(&s->loop_args[MODE], &a, sizeof(PrArgs)) != 0 || s->loop_bl[MODE] != q.dbl ||
               s->loop_grid[MODE] != grid)) {
      cudaGraphExecDestroy(gx);
      gx = nullptr;
    }
    if (!gx && build_round_graph<MODE>(c, a, q, &gx) == CYTOM_OK) {
      memcpy(&s->loop_args[MODE], &a, sizeof(PrArgs));
      s->loop_bl[MODE] = q.dbl;
      s->loop_grid[MODE] = grid;
    }
    if (gx) {
      cudaError_t e = cudaGraphLaunch(gx, c->stream);
      c->launches += 1;
      return cuda_err(c, e, "pagerank graph launch");
    }
  }
  for (uint64_t r = 0; r < max_rounds;) {
    for (int k = 0; k < 8 && r < max_rounds; ++k, ++r) {
      int slot = prof_begin(c, KC_PAGERANK);
      int rc = launch_round<MODE>(c, a, q, r == 0);
      prof_end(c, slot, -1.0);
      if (rc) return rc;
    }
    if (r >= max_rounds) break;  // the last round: nothing to check
    cudaError_t e = cudaMemcpyAsync(c->h_pinned, &a.ls->cont, 4, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_err(c, e, "pagerank loop");
    if (*(unsigned*)c->h_pinned == 0) break;
  }
  return CYTOM_OK;
}

static int wpagerank_run(Ctx* c, Job* j);

int pagerank_run(Ctx* c, Job* j) {
  if (j->algo == CYTOM_ALGO_WPAGERANK) return wpagerank_run(c, j);
  PrState* s = prs(j);
  const uint64_t ver = store_version(c);
  {
    int rc = update_csc(c, *s->csc);
    if (rc) return rc;
  }
  if (s->seen_version != ver) {
    s->need_residual = true;
    s->seen_version = ver;
  }
  const uint64_t n = c->n;
  PrArgs a{};
  a.csc_src = s->csc->src;
  a.csc_ptr = s->csc->ptr;
  a.bins = s->csc->bins;
  a.rank = s->rank;
  a.comp = s->comp;
  a.lo0 = s->lo;
  a.lo1 = s->lo ? s->lo + c->n : nullptr;
  a.delta = s->delta;
  a.contrib = s->contrib;
  a.r64 = s->r64;
  a.r64n = s->r64n;
  a.contrib64 = s->contrib64;
  a.ls = j->ls;
  a.n = n;
  a.alpha = j->params.alpha;
  a.delta_param = j->params.delta;
  a.base = (1.0 - j->params.alpha) / (double)n;
  pr_args_ff(a);
  unsigned max_iter = (unsigned)std::min<uint64_t>(j->params.max_iterations, 0xFFFFFFFFu);
  pr_begin_kernel<<<1, 1, 0, c->stream>>>(j->ls, max_iter, j->params.tolerance, (unsigned long long)s->csc->E);
  c->launches++;
  j->last_run_graph = false;
  if (j->algo == CYTOM_ALGO_PR_DELTA) {
    int drc = pr_deg_mult(c);
    if (drc) return drc;
    a.deg = c->pr_deg_mult;  // multiplicity out-degrees, as the reference's vertex store
    // rank sum before the run (relative stopping rule)
    pr_rank_sum_kernel<<<grid_n(c, n), 256, 0, c->stream>>>(s->rank, n, j->ls);
    c->launches++;
    // Every run opens with the residual round (all sources contribute rank / outdeg):
    // exact after any change of the graph, and a no-op correction when nothing changed.
    int rc = run_rounds<PR_DELTA_RESIDUAL>(c, j, a, 1, *s->csc);
    if (rc) return rc;
    s->need_residual = false;
    return run_rounds<PR_DELTA_PUSH>(c, j, a, max_iter, *s->csc);
  }
  a.deg = s->csc->deg_out;
  if (j->params.kahan) {
    int rc = run_rounds<PR_NORM32>(c, j, a, max_iter, *s->csc);
    return rc;
  }
  return run_rounds<PR_NORM64>(c, j, a, max_iter, *s->csc);
}

// Prepares a run of the batched executor: the snapshot's CSC, the loop state (and for
// PageRank-delta the rank sum before the run), the round arguments, the bin sizes and
// the mode of the first round.
// Prepares a PageRank-family job of the batched executor. A PAGERANK job's loop state is
// reset by the batch's begin kernel (*begin_edges = the edges a round reads); a
// PageRank-delta job's here, before its rank sum.
int pagerank_batch_prep(Ctx* c, Job* j, PrArgs* out, uint64_t* nb, int* first_mode, uint64_t* begin_edges) {
  if (j->algo == CYTOM_ALGO_WPAGERANK)
    return set_err(c, CYTOM_ERR_UNIMPLEMENTED, "weighted PageRank runs through cytom_run only");
  PrState* s = prs(j);
  const uint64_t ver = store_version(c);
  {
    int rc = update_csc(c, *s->csc);
    if (rc) return rc;
  }
  s->seen_version = ver;
  const uint64_t n = c->n;
  PrArgs a{};
  a.csc_src = s->csc->src;
  a.csc_ptr = s->csc->ptr;
  a.bins = s->csc->bins;
  a.rank = s->rank;
  a.comp = s->comp;
  a.lo0 = s->lo;
  a.lo1 = s->lo ? s->lo + c->n : nullptr;
  a.delta = s->delta;
  a.contrib = s->contrib;
  a.r64 = s->r64;
  a.r64n = s->r64n;
  a.contrib64 = s->contrib64;
  a.ls = j->ls;
  a.n = n;
  a.alpha = j->params.alpha;
  a.delta_param = j->params.delta;
  a.base = (1.0 - j->params.alpha) / (double)n;
  pr_args_ff(a);
  unsigned max_iter = (unsigned)std::min<uint64_t>(j->params.max_iterations, 0xFFFFFFFFu);
  *begin_edges = s->csc->E;
  if (j->algo == CYTOM_ALGO_PR_DELTA) {
    pr_begin_kernel<<<1, 1, 0, c->stream>>>(j->ls, max_iter, j->params.tolerance, (unsigned long long)s->csc->E);
    c->launches++;
    int drc = pr_deg_mult(c);
    if (drc) return drc;
    a.deg = c->pr_deg_mult;
    pr_rank_sum_kernel<<<grid_n(c, n), 256, 0, c->stream>>>(s->rank, n, j->ls);
    c->launches++;
    *first_mode = PR_DELTA_RESIDUAL;
    s->need_residual = false;
  } else {
    a.deg = s->csc->deg_out;
    *first_mode = j->params.kahan ? PR_NORM32 : PR_NORM64;
  }
  for (int k = 0; k < kPrBins; ++k) nb[k] = s->csc->nb[k];
  *out = a;
  return cuda_err(c, cudaGetLastError(), "batch prep");
}

// Copies a renumbered vertex vector out in vertex order (host or device destination).
template <typename T>
static int unpermute_out(Ctx* c, const T* src, void* out, int where, const char* what) {
  const uint64_t n = c->n;
  T* dst = (T*)out;
  T* tmp = nullptr;
  if (where != CYTOM_PTR_DEVICE) {
    if (cy_malloc_async((void**)&tmp, n * sizeof(T), c->stream) != cudaSuccess) return set_err(c, CYTOM_ERR_OOM, what);
    dst = tmp;
  }
  permute_kernel<T><<<grid_n(c, n), 256, 0, c->stream>>>(src, c->pr_perm, n, 0, dst);
  c->launches++;
  cudaError_t e = cudaSuccess;
  if (tmp) {
    e = cudaMemcpyAsync(out, tmp, n * sizeof(T), cudaMemcpyDeviceToHost, c->stream);
    cudaFreeAsync(tmp, c->stream);
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  return cuda_err(c, e, what);
}

int pagerank_result(Ctx* c, Job* j, void* out, int where) {
  PrState* s = prs(j);
  const uint64_t n = c->n;
  const float* src = s->rank;
  LoopState ls;
  cudaMemcpyAsync(&ls, j->ls, sizeof(ls), cudaMemcpyDeviceToHost, c->stream);
  cudaStreamSynchronize(c->stream);
  const unsigned p = ls.iter & 1u;  // buffer holding the newest ranks
  if (j->algo == CYTOM_ALGO_PAGERANK || j->algo == CYTOM_ALGO_WPAGERANK) {
    if (j->params.kahan) {
      src = (p == 0) ? s->rank : s->comp;
    } else {
      const double* r = (p == 0) ? s->r64 : s->r64n;
      pr_to_float_kernel<<<grid_n(c, n), 256, 0, c->stream>>>(r, s->rank, n);
      c->launches++;
      src = s->rank;
    }
  }
  return unpermute_out<float>(c, src, out, where, "pagerank result");
}

// PageRank-delta rank and last delta in vertex order (host buffers), for the results dump.
int pagerank_delta_out(Ctx* c, Job* j, float* rank, float* delta) {
  PrState* s = prs(j);
  if (j->algo != CYTOM_ALGO_PR_DELTA) return set_err(c, CYTOM_ERR_INVAL, "not a PageRank-delta job");
  if (!c->pr_perm) {
    // never run: the initial state (rank 1, delta 0)
    for (uint64_t v = 0; v < c->n; ++v) {
      rank[v] = 1.f;
      delta[v] = 0.f;
    }
    return CYTOM_OK;
  }
  int rc = unpermute_out<float>(c, s->rank, rank, CYTOM_PTR_HOST, "pagerank-delta rank");
  if (!rc) rc = unpermute_out<float>(c, s->delta, delta, CYTOM_PTR_HOST, "pagerank-delta delta");
  return rc;
}

int pagerank_result64(Ctx* c, Job* j, double* out, int where) {
  PrState* s = prs(j);
  if ((j->algo != CYTOM_ALGO_PAGERANK && j->algo != CYTOM_ALGO_WPAGERANK) || j->params.kahan)
    return set_err(c, CYTOM_ERR_INVAL, "not an FP64 job");
  LoopState ls;
  cudaMemcpyAsync(&ls, j->ls, sizeof(ls), cudaMemcpyDeviceToHost, c->stream);
  cudaStreamSynchronize(c->stream);
  const double* r = ((ls.iter & 1u) == 0) ? s->r64 : s->r64n;
  return unpermute_out<double>(c, r, out, where, "pagerank result64");
}


// --------------------------------------------------------------------------
// Weighted PageRank (WPAGERANK) and its adjoint
// --------------------------------------------------------------------------

// s_u = sum of u's out-weights, one warp per source in CSR order (deterministic).
__global__ void wsum_kernel(const uint32_t* __restrict__ ptr, const float* __restrict__ w, uint64_t n,
                            double* __restrict__ wsum) {
  const unsigned lane = threadIdx.x & 31;
  const uint64_t warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  for (uint64_t u = warp; u < n; u += nwarps) {
    double s = 0.0;
    for (uint32_t e = ptr[u] + lane; e < ptr[u + 1]; e += 32) s += (double)w[e];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xFFFFFFFFu, s, o);
    if (lane == 0) wsum[u] = s;
  }
}

static int build_wgraph(Ctx* c, WGraph& g) {
  if (g.built_version == c->version) return CYTOM_OK;
  int rc = build_csx(c, g.in, 0, &g.in_w, &g.in_wcap);
  if (!rc) rc = build_csx(c, g.out, 1, &g.out_w, &g.out_wcap);
  if (rc) return rc;
  if (!g.wsum && cy_malloc(&g.wsum, c->n * 8) != cudaSuccess) return set_err(c, CYTOM_ERR_OOM, "weight sums");
  wsum_kernel<<<grid_n(c, c->n * 32), 256, 0, c->stream>>>(g.out.ptr, g.out_w, c->n, g.wsum);
  c->launches++;
  g.built_version = c->version;
  return cuda_err(c, cudaGetLastError(), "weight sums");
}

static PrArgs wargs(Ctx* c, Job* j, const WGraph& g) {
  PrState* s = prs(j);
  PrArgs a{};
  a.csc_src = g.in.src;
  a.csc_ptr = g.in.ptr;
  a.bins = g.in.bins;
  a.csc_w = g.in_w;
  a.wsum = g.wsum;
  a.tele = s->tele;
  a.rank = s->rank;
  a.comp = s->comp;
  a.lo0 = s->lo;
  a.lo1 = s->lo ? s->lo + c->n : nullptr;
  a.contrib = s->contrib;
  a.r64 = s->r64;
  a.r64n = s->r64n;
  a.contrib64 = s->contrib64;
  a.ls = j->ls;
  a.n = c->n;
  a.alpha = j->params.alpha;
  pr_args_ff(a);
  return a;
}

static int wpagerank_run(Ctx* c, Job* j) {
  WGraph* g = ctx_wgraph(c);
  if (!g) return set_err(c, CYTOM_ERR_OOM, "weighted graph");
  int rc = build_wgraph(c, *g);
  if (rc) return rc;
  PrArgs a = wargs(c, j, *g);
  unsigned max_iter = (unsigned)std::min<uint64_t>(j->params.max_iterations, 0xFFFFFFFFu);
  pr_begin_kernel<<<1, 1, 0, c->stream>>>(j->ls, max_iter, j->params.tolerance, (unsigned long long)g->in.E);
  c->launches++;
  j->last_run_graph = false;
  return j->params.kahan ? run_rounds<PR_W32>(c, j, a, max_iter, g->in)
                         : run_rounds<PR_W64>(c, j, a, max_iter, g->in);
}

int pagerank_set_teleport(Ctx* c, Job* j, const double* t, int where) {
  PrState* s = prs(j);
  if (j->algo != CYTOM_ALGO_WPAGERANK) return set_err(c, CYTOM_ERR_INVAL, "teleport vectors are for WPAGERANK jobs");
  if (!t) {
    if (s->tele) {
      cudaStreamSynchronize(c->stream);
      cudaFree(s->tele);
    }
    s->tele = nullptr;
    return CYTOM_OK;
  }
  int prc = pr_ensure_perm(c);
  if (prc) return prc;
  if (!s->tele && cy_malloc(&s->tele, c->n * 8) != cudaSuccess) return set_err(c, CYTOM_ERR_OOM, "teleport");
  // kept in the renumbering
  double* tmp = nullptr;
  if (cy_malloc_async((void**)&tmp, c->n * 8, c->stream) != cudaSuccess) return set_err(c, CYTOM_ERR_OOM, "teleport");
  cudaError_t e = cudaMemcpyAsync(tmp, t, c->n * 8,
                                  where == CYTOM_PTR_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                                  c->stream);
  permute_kernel<double><<<grid_n(c, c->n), 256, 0, c->stream>>>(tmp, c->pr_perm, c->n, 1, s->tele);
  c->launches++;
  cudaFreeAsync(tmp, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  return cuda_err(c, e, "teleport upload");
}

__global__ void adj_init_kernel(const double* __restrict__ cvec, uint64_t n, float* lam32, double* lam64,
                                LoopState* ls) {
  double l1 = 0.0;
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t v = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += stride) {
    const double cv = cvec[v];
    if (lam32) lam32[v] = (float)cv;
    if (lam64) lam64[v] = cv;
    l1 += fabs(cv);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) l1 += __shfl_xor_sync(0xFFFFFFFFu, l1, o);
  if ((threadIdx.x & 31) == 0 && l1 != 0.0) atomicAdd(&ls->base_sum, l1);
}

// The adjoint stops at an L1 change <= rel * |c|_1.
__global__ void adj_tol_kernel(LoopState* ls, double rel) { ls->tol = rel * ls->base_sum; }

// D = sum of r over vertices without out-weight.
template <typename T>
__global__ void dangling_sum_kernel(const T* __restrict__ r, const double* __restrict__ wsum, uint64_t n,
                                    double* out) {
  double d = 0.0;
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t v = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += stride)
    if (!(wsum[v] > 0.0)) d += (double)r[v];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) d += __shfl_xor_sync(0xFFFFFFFFu, d, o);
  if ((threadIdx.x & 31) == 0 && d != 0.0) atomicAdd(out, d);
}

// dL/dw of every stored edge u -> k, in store order:
// alpha * r_u / s_u * (lambda_k - (P^T lambda)_u), evaluated in FP64.
template <typename T>
__global__ void grad_w_kernel(const StoreDesc* __restrict__ sd, const uint32_t* __restrict__ perm,
                              const T* __restrict__ r, const T* __restrict__ lam, const T* __restrict__ pt,
                              const double* __restrict__ wsum, double alpha, float* __restrict__ gw) {
  const uint64_t E = sd->E;
  const uint32_t lT = sd->lT, lvpt = sd->lvpt;
  const uint32_t ymask = (uint32_t)(sd->T - 1);
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; e < E; e += stride) {
    uint32_t t = sd->chunk_tile[e >> 7];
    while (sd->tile_ptr[t + 1] <= e) ++t;
    const uint32_t p = sd->edges[e];
    const uint32_t u = perm[((t >> lT) << lvpt) | (p >> 16)];
    const uint32_t k = perm[((t & ymask) << lvpt) | (p & 0xFFFFu)];
    gw[e] = (float)(alpha * (double)r[u] / wsum[u] * ((double)lam[k] - (double)pt[u]));
  }
}

// dL/dt_v = ((1 - alpha) + alpha * D) * lambda_v.
template <typename T>
__global__ void grad_t_kernel(const T* __restrict__ lam, const uint32_t* __restrict__ perm, uint64_t n,
                              const double* __restrict__ dang, double alpha, float* __restrict__ gt) {
  const double f = (1.0 - alpha) + alpha * dang[0];
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t v = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += stride)
    gt[v] = (float)(f * (double)lam[perm[v]]);
}

// Adjoint of L = c . r at the converged ranks of WPAGERANK job j: solves
// lambda = c + alpha (P^T lambda + a (t . lambda)) over the source-major CSR (the same
// edges in reverse orientation), then writes dL/dw (every stored edge, store order) and
// dL/dt. Only the converged rank vector of the forward run is used (no per-round state).
int pagerank_adjoint(Ctx* c, Job* j, const double* cv, int cwhere, float* d_w, float* d_t, int owhere,
                     cytom_run_stats* st) {
  PrState* s = prs(j);
  if (j->algo != CYTOM_ALGO_WPAGERANK) return set_err(c, CYTOM_ERR_INVAL, "the adjoint needs a WPAGERANK job");
  WGraph* g = ctx_wgraph(c);
  if (j->fresh || !g || g->built_version != c->version || c->A)
    return set_err(c, CYTOM_ERR_INVAL, "run the forward PageRank on the current graph first");
  const uint64_t n = c->n, E = c->E;
  const bool f32 = j->params.kahan != 0;
  cudaError_t e = cudaSuccess;
  if (!s->adj_ls) e = cy_malloc(&s->adj_ls, sizeof(LoopState));
  if (e == cudaSuccess && !s->cvec) e = cy_malloc(&s->cvec, n * 8);
  if (f32) {
    if (e == cudaSuccess && !s->lam) e = cy_malloc(&s->lam, 2 * n * 4);
    if (e == cudaSuccess && !s->pt) e = cy_malloc(&s->pt, n * 4);
  } else {
    if (e == cudaSuccess && !s->lam64) e = cy_malloc(&s->lam64, 2 * n * 8);
    if (e == cudaSuccess && !s->pt64) e = cy_malloc(&s->pt64, n * 8);
  }
  if (e != cudaSuccess) {
    cudaGetLastError();
    return set_err(c, CYTOM_ERR_OOM, "adjoint state");
  }
  // the forward's newest ranks
  LoopState fls;
  e = cudaMemcpyAsync(&fls, j->ls, sizeof(LoopState), cudaMemcpyDeviceToHost, c->stream);
  double* ctmp = nullptr;
  if (e == cudaSuccess && cy_malloc_async((void**)&ctmp, n * 8, c->stream) != cudaSuccess)
    return set_err(c, CYTOM_ERR_OOM, "adjoint setup");
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(ctmp, cv, n * 8, cwhere == CYTOM_PTR_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                        c->stream);
  if (e == cudaSuccess) {
    permute_kernel<double><<<grid_n(c, n), 256, 0, c->stream>>>(ctmp, c->pr_perm, n, 1, s->cvec);
    c->launches++;
  }
  if (ctmp) cudaFreeAsync(ctmp, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_err(c, e, "adjoint setup");
  const unsigned pf = fls.iter & 1u;
  const float* r32 = f32 ? ((pf == 0) ? s->rank : s->comp) : nullptr;
  const double* r64 = f32 ? nullptr : ((pf == 0) ? s->r64 : s->r64n);

  cudaEventRecord(c->run_a, c->stream);
  unsigned max_iter = (unsigned)std::min<uint64_t>(j->params.max_iterations, 0xFFFFFFFFu);
  pr_begin_kernel<<<1, 1, 0, c->stream>>>(s->adj_ls, max_iter, 0.0, (unsigned long long)g->out.E);
  adj_init_kernel<<<grid_n(c, n), 256, 0, c->stream>>>(s->cvec, n, f32 ? s->lam : nullptr, f32 ? nullptr : s->lam64,
                                                        s->adj_ls);
  adj_tol_kernel<<<1, 1, 0, c->stream>>>(s->adj_ls, j->params.tolerance);
  c->launches += 3;
  PrArgs a{};
  a.csc_src = g->out.src;
  a.csc_ptr = g->out.ptr;
  a.bins = g->out.bins;
  a.csc_w = g->out_w;
  a.wsum = g->wsum;
  a.tele = s->tele;
  a.cvec = s->cvec;
  a.pt = s->pt;
  a.pt64 = s->pt64;
  a.rank = f32 ? s->lam : nullptr;
  a.comp = f32 ? s->lam + n : nullptr;
  a.r64 = f32 ? nullptr : s->lam64;
  a.r64n = f32 ? nullptr : s->lam64 + n;
  a.contrib = s->contrib;  // the forward's contribution buffer is free once it has converged
  a.contrib64 = s->contrib64;
  a.ls = s->adj_ls;
  a.n = n;
  a.alpha = j->params.alpha;
  pr_args_ff(a);
  int rc = f32 ? run_rounds<PR_ADJ32>(c, j, a, max_iter, g->out) : run_rounds<PR_ADJ64>(c, j, a, max_iter, g->out);
  if (rc) return rc;
  LoopState als;
  e = cudaMemcpyAsync(&als, s->adj_ls, sizeof(LoopState), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_err(c, e, "adjoint run");
  const unsigned pa = als.iter & 1u;  // buffer holding the newest lambda
  // gradients into device scratch, then to the caller
  // layout (256-byte aligned regions): D (one double), dL/dw (E floats), dL/dt (n floats)
  char* tmp = nullptr;
  auto align256 = [](size_t b) { return (b + 255) & ~(size_t)255; };
  const size_t wbytes = align256(std::max<uint64_t>(E, 1) * 4), tbytes = align256(n * 4);
  if (cy_malloc_async((void**)&tmp, 256 + wbytes + tbytes, c->stream) != cudaSuccess)
    return set_err(c, CYTOM_ERR_OOM, "adjoint outputs");
  double* dang = (double*)tmp;
  float* gw = (owhere == CYTOM_PTR_DEVICE && d_w) ? d_w : (float*)(tmp + 256);
  float* gt = (owhere == CYTOM_PTR_DEVICE && d_t) ? d_t : (float*)(tmp + 256 + wbytes);
  cudaMemsetAsync(dang, 0, 8, c->stream);
  if (f32) {
    const float* lam = (pa == 0) ? s->lam : s->lam + n;
    dangling_sum_kernel<float><<<grid_n(c, n), 256, 0, c->stream>>>(r32, g->wsum, n, dang);
    if (E)
      grad_w_kernel<float><<<grid_n(c, E), 256, 0, c->stream>>>(c->dsd, c->pr_perm, r32, lam, s->pt, g->wsum, a.alpha, gw);
    grad_t_kernel<float><<<grid_n(c, n), 256, 0, c->stream>>>(lam, c->pr_perm, n, dang, a.alpha, gt);
  } else {
    const double* lam = (pa == 0) ? s->lam64 : s->lam64 + n;
    dangling_sum_kernel<double><<<grid_n(c, n), 256, 0, c->stream>>>(r64, g->wsum, n, dang);
    if (E)
      grad_w_kernel<double><<<grid_n(c, E), 256, 0, c->stream>>>(c->dsd, c->pr_perm, r64, lam, s->pt64, g->wsum, a.alpha, gw);
    grad_t_kernel<double><<<grid_n(c, n), 256, 0, c->stream>>>(lam, c->pr_perm, n, dang, a.alpha, gt);
  }
  c->launches += 3;
  cudaEventRecord(c->run_b, c->stream);
  if (owhere != CYTOM_PTR_DEVICE) {
    if (d_w && E) cudaMemcpyAsync(d_w, gw, E * 4, cudaMemcpyDeviceToHost, c->stream);
    if (d_t) cudaMemcpyAsync(d_t, gt, n * 4, cudaMemcpyDeviceToHost, c->stream);
  }
  cudaFreeAsync(tmp, c->stream);
  e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_err(c, e, "adjoint gradients");
  if (st) {
    memset(st, 0, sizeof(*st));
    st->iterations = als.iter;
    st->count_edges = als.count_edges;
    st->edges_scanned = als.edges_scanned;
    st->converged = als.cont == 0 ? 1 : 0;
    st->residual = als.resid_final;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, c->run_a, c->run_b);
    st->elapsed_ms = ms;
  }
  return CYTOM_OK;
}

}  // namespace cytom
