// ingest.cu — edge sources, streaming insert and compaction of the tile store.
//
// Replaces, for one GPU:
//   RMATContext::getEdge / rMatIterative   (src/include/edge-inserter/rmat-context.h:39-73)
//   Jobs GridGraph reader                  (src/include/core/jobs.h:53-64, 111-118)
//   MetaTileManager::insertEdge + TileManager::insertEdge
//                                          (meta-tile-manager.h:112-125, tile-manager.h:136-163)
//   TileManager::compactStorage / fillCSR  (tile-manager.h:192-291, 518-565)
//
// Compaction is a global merge: the append region is radix-sorted by the
// composite key (x, y, src_local, tgt_local), deduplicated within itself and
// against the compacted store (binary search in the tile's segment), and the
// survivors are merged into a new buffer by output-position ranking. Every
// compacted tile is then exactly the reference's sorted, deduplicated CSR.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <vector>

#include "engine.h"
#include "radix.cuh"

namespace cytom {

// --------------------------------------------------------------------------
// Hash (Ligra 64-bit, src/include/util/util.h:188-196)
// --------------------------------------------------------------------------
__host__ __device__ __forceinline__ uint64_t hash64(uint64_t a) {
  a = (a + 0x7ed55d166bef7a1dULL) + (a << 12);
  a = (a ^ 0xc761c23c510fa2ddULL) ^ (a >> 9);
  a = (a + 0x165667b183a9c0e1ULL) + (a << 59);
  a = (a + 0xd3a2646cab3487e3ULL) ^ (a << 49);
  a = (a + 0xfd7046c5ef9ab54cULL) + (a << 3);
  a = (a ^ 0xb55a4f090dd4a67bULL) ^ (a >> 32);
  return a;
}

// --------------------------------------------------------------------------
// RMAT
// --------------------------------------------------------------------------
// util::hashDouble(i) = (double)hash(i) / (double)UINT64_MAX, and (double)UINT64_MAX
// is exactly 2^64, so `hashDouble(i) < t` <=> `(double)hash(i) < t * 2^64`. Because
// the u64 -> double rounding is monotone, that is `hash(i) < H` for the least H
// whose double value reaches t * 2^64. The kernel compares integers against H;
// the host derives H once from the double thresholds a, a+b, a+b+c.
struct RmatThr {
  unsigned long long h[3];
  int all[3];  // 1 when every hash is below the threshold
};

static void rmat_threshold(double t, unsigned long long* h, int* all) {
  const double two64 = 18446744073709551616.0;
  double A = t * two64;
  *all = 0;
  if (!(A > 0.0)) {  // also NaN
    *h = 0;
    return;
  }
  if (A > (double)UINT64_MAX) {  // (double)UINT64_MAX == 2^64
    *all = 1;
    *h = 0;
    return;
  }
  // A < 2^64 here or A == 2^64 (handled above); search H in a window around A.
  unsigned long long guess = (A >= two64)                     ? UINT64_MAX
                             : (A >= 9223372036854775808.0) ? (unsigned long long)(A)
                                                            : (unsigned long long)std::ceil(A);
  unsigned long long lo = guess > 8192 ? guess - 8192 : 0;
  unsigned long long hi = guess < UINT64_MAX - 8192 ? guess + 8192 : UINT64_MAX;
  // predicate p(h) = ((double)h >= A) is monotone; find the least h with p(h).
  if ((double)hi < A) {  // all values in range below A: every hash < A
    *all = 1;
    *h = 0;
    return;
  }
  while (lo < hi) {
    unsigned long long mid = lo + (hi - lo) / 2;
    if ((double)mid >= A) hi = mid;
    else lo = mid + 1;
  }
  *h = lo;
}

__device__ __forceinline__ bool below(uint64_t v, const RmatThr& t, int k) {
  return t.all[k] ? true : (v < t.h[k]);
}

__global__ void rmat_kernel(RmatThr thr, uint32_t scale, uint64_t hseed, uint64_t first,
                            uint64_t count, uint32_t* __restrict__ src, uint32_t* __restrict__ tgt,
                            uint32_t* __restrict__ w, uint64_t wseed_h, uint32_t wmin,
                            uint64_t wspan) {
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < count; k += stride) {
    uint64_t index = first + k;
    uint64_t rs = hash64(2ULL * index * hseed);
    uint64_t st = hash64((2ULL * index + 1ULL) * hseed);
    // bit j (value 2^j) uses hash(rs + (scale-1-j)*st): the most significant bit
    // uses hash(rs), as rMatIterative walks back from the finest level.
    uint32_t es = 0, et = 0;
    uint64_t r = rs;
    for (int j = (int)scale - 1; j >= 0; --j) {
      uint64_t h = hash64(r);
      r += st;
      uint32_t bit = 1u << j;
      if (below(h, thr, 0)) {
      } else if (below(h, thr, 1)) {
        et |= bit;
      } else if (below(h, thr, 2)) {
        es |= bit;
      } else {
        es |= bit;
        et |= bit;
      }
    }
    src[k] = es;
    tgt[k] = et;
    if (w) {
      uint64_t key = wseed_h ^ (((uint64_t)es << 32) | (uint64_t)et);
      w[k] = wmin + (uint32_t)(hash64(key) % wspan);
    }
  }
}

static int grid_for(Ctx* c, uint64_t work, int threads, int per_sm = 8) {
  uint64_t blocks = (work + threads - 1) / threads;
  uint64_t cap = (uint64_t)c->num_sms * per_sm;
  if (blocks > cap) blocks = cap;
  if (blocks == 0) blocks = 1;
  return (int)blocks;
}

int rmat_generate(Ctx* c, const cytom_rmat_params* p, uint64_t first, uint64_t count,
                  uint32_t* src, uint32_t* tgt, uint32_t* w) {
  if (count == 0) return CYTOM_OK;
  RmatThr thr;
  double a_ = p->a, ab_ = p->a + p->b, abc_ = p->a + p->b + p->c;
  rmat_threshold(a_, &thr.h[0], &thr.all[0]);
  rmat_threshold(ab_, &thr.h[1], &thr.all[1]);
  rmat_threshold(abc_, &thr.h[2], &thr.all[2]);
  uint64_t hseed = hash64(p->seed);
  uint64_t wspan = (uint64_t)p->wmax - (uint64_t)p->wmin + 1ULL;
  int slot = prof_begin(c, KC_RMAT);
  rmat_kernel<<<grid_for(c, count, 256, 16), 256, 0, c->stream>>>(
      thr, p->scale, hseed, first, count, src, tgt, (p->wmax > 0) ? w : nullptr,
      hash64(p->weight_seed), p->wmin, wspan);
  c->launches++;
  prof_end(c, slot, (double)count * ((p->wmax > 0) ? 12.0 : 8.0));
  return cuda_err(c, cudaGetLastError(), "rmat_kernel");
}

// --------------------------------------------------------------------------
// GridGraph decode
// --------------------------------------------------------------------------
__global__ void gridgraph_decode_kernel(const int2* __restrict__ rec, uint64_t m, uint64_t n,
                                        uint32_t* __restrict__ src, uint32_t* __restrict__ tgt,
                                        unsigned int* bad) {
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  unsigned int nb = 0;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += stride) {
    int2 r = rec[i];
    bool ok = r.x >= 0 && r.y >= 0 && (uint64_t)r.x < n && (uint64_t)r.y < n;
    nb += ok ? 0 : 1;
    src[i] = ok ? (uint32_t)r.x : 0u;
    tgt[i] = ok ? (uint32_t)r.y : 0u;
  }
  if (nb) atomicAdd(bad, nb);
}

int gridgraph_decode(Ctx* c, const void* dbytes, uint64_t m, uint32_t* src, uint32_t* tgt) {
  if (m == 0) return CYTOM_OK;
  cudaError_t e = cudaMemsetAsync(c->d_flag, 0, sizeof(unsigned int), c->stream);
  if (e != cudaSuccess) return cuda_err(c, e, "memset");
  int slot = prof_begin(c, KC_INSERT);
  gridgraph_decode_kernel<<<grid_for(c, m, 256), 256, 0, c->stream>>>(
      (const int2*)dbytes, m, c->n, src, tgt, c->d_flag);
  c->launches++;
  prof_end(c, slot, (double)m * 16.0);
  e = cudaMemcpyAsync(c->h_pinned, c->d_flag, sizeof(unsigned int), cudaMemcpyDeviceToHost,
                      c->stream);
  if (e != cudaSuccess) return cuda_err(c, e, "memcpy");
  e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_err(c, e, "gridgraph_decode");
  unsigned int bad = *(unsigned int*)c->h_pinned;
  if (bad) return set_err(c, CYTOM_ERR_RANGE, "gridgraph record with a negative id or an id >= vertex count");
  return CYTOM_OK;
}

// --------------------------------------------------------------------------
// Insert
// --------------------------------------------------------------------------
__global__ void validate_kernel(const uint32_t* __restrict__ src, const uint32_t* __restrict__ tgt,
                                uint64_t count, uint64_t n, unsigned int* bad) {
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  unsigned int nb = 0;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += stride)
    nb += (src[i] >= n || tgt[i] >= n) ? 1u : 0u;
  if (nb) atomicAdd(bad, nb);
}

// Composite key: [x : lT][y : lT][src_local : lvpt][tgt_local : lvpt].
__device__ __forceinline__ uint64_t make_key(uint32_t s, uint32_t t, uint32_t lvpt, uint32_t lT) {
  uint64_t m = (1ULL << lvpt) - 1ULL;
  uint64_t x = (uint64_t)s >> lvpt, y = (uint64_t)t >> lvpt;
  uint64_t tile = (x << lT) | y;
  return (tile << (2 * lvpt)) | (((uint64_t)s & m) << lvpt) | ((uint64_t)t & m);
}

// Appends one batch to the append region and counts degrees. Degree increments
// are warp-aggregated: lanes holding the same vertex elect one leader that adds
// the group's size (RMAT hubs repeat often within a warp).
// Appends the batch and counts its degrees -- unless validate_kernel, earlier on the same
// stream, found an endpoint out of range: then the whole batch is rejected and nothing
// is written, so the host reads the verdict once, after both kernels.
__global__ void append_kernel(const uint32_t* __restrict__ src, const uint32_t* __restrict__ tgt,
                              const uint32_t* __restrict__ w, uint64_t count,
                              uint64_t* __restrict__ keys, uint32_t* __restrict__ kw,
                              uint32_t* __restrict__ out_deg, uint32_t* __restrict__ in_deg,
                              uint32_t lvpt, uint32_t lT, const unsigned int* __restrict__ bad) {
  if (*bad) return;
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  const unsigned lane = threadIdx.x & 31;
  for (uint64_t base = (uint64_t)blockIdx.x * blockDim.x; base < count; base += stride) {
    uint64_t i = base + threadIdx.x;
    bool valid = i < count;
    unsigned vmask = __ballot_sync(0xFFFFFFFFu, valid);
    if (!valid) continue;
    uint32_t s = src[i], t = tgt[i];
    keys[i] = make_key(s, t, lvpt, lT);
    if (w) kw[i] = w[i];
    unsigned ps = __match_any_sync(vmask, s);
    if ((__ffs(ps) - 1) == (int)lane) atomicAdd(&out_deg[s], (uint32_t)__popc(ps));
    unsigned pt = __match_any_sync(vmask, t);
    if ((__ffs(pt) - 1) == (int)lane) atomicAdd(&in_deg[t], (uint32_t)__popc(pt));
  }
}

// ---- dynamic compaction (TileManager::insertEdge, tile-manager.h:117, 150-161) ----
// Appended edges per tile (one atomic per tile and warp).
__global__ void dyn_count_kernel(const uint64_t* __restrict__ keys, uint64_t count, uint32_t lvpt,
                                 uint32_t* __restrict__ pending) {
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += stride) {
    const uint32_t t = (uint32_t)(keys[i] >> (2 * lvpt));
    const unsigned m = __match_any_sync(__activemask(), t);
    if ((threadIdx.x & 31u) == (unsigned)(__ffs(m) - 1)) atomicAdd(&pending[t], (unsigned)__popc(m));
  }
}
// A tile whose edges (stored + appended) reached its threshold raises the flag; the
// threshold doubles past the count, as one doubling per crossing would leave it.
__global__ void dyn_check_kernel(const unsigned long long* __restrict__ tile_ptr, const uint32_t* __restrict__ pending,
                                 uint64_t ntiles, unsigned long long* __restrict__ next, unsigned* __restrict__ flag) {
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < ntiles; t += stride) {
    const unsigned long long total = (tile_ptr[t + 1] - tile_ptr[t]) + pending[t];
    unsigned long long nx = next[t];
    if (total >= nx) {
      while (nx <= total) nx *= 2;
      next[t] = nx;
      atomicOr(flag, 1u);
    }
  }
}
__global__ void dyn_init_kernel(unsigned long long* __restrict__ next, uint64_t ntiles) {
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < ntiles; t += stride) next[t] = 4096;
}

// After an insert with dynamic compaction on: counts the batch's edges per tile and
// compacts the store when some tile reached its threshold.
static int dynamic_compaction(Ctx* c, uint64_t first, uint64_t count) {
  const uint64_t nt = c->ntiles;
  if (!c->dyn_pending) {
    if (cy_malloc(&c->dyn_pending, nt * 4) != cudaSuccess || cy_malloc(&c->dyn_next, nt * 8) != cudaSuccess) {
      cudaGetLastError();
      return set_err(c, CYTOM_ERR_OOM, "dynamic compaction counters");
    }
    cudaMemsetAsync(c->dyn_pending, 0, nt * 4, c->stream);
    dyn_init_kernel<<<grid_for(c, nt, 256), 256, 0, c->stream>>>(c->dyn_next, nt);
    c->launches++;
    // edges appended before the counters existed
    if (first) {
      dyn_count_kernel<<<grid_for(c, first, 256), 256, 0, c->stream>>>(c->app_keys, first, c->lvpt, c->dyn_pending);
      c->launches++;
    }
  }
  dyn_count_kernel<<<grid_for(c, count, 256), 256, 0, c->stream>>>(c->app_keys + first, count, c->lvpt,
                                                                    c->dyn_pending);
  cudaMemsetAsync(c->d_flag, 0, sizeof(unsigned int), c->stream);
  dyn_check_kernel<<<grid_for(c, nt, 256), 256, 0, c->stream>>>(c->tile_ptr, c->dyn_pending, nt, c->dyn_next,
                                                                c->d_flag);
  c->launches += 2;
  cudaError_t e = cudaMemcpyAsync(c->h_pinned, c->d_flag, sizeof(unsigned int), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_err(c, e, "dynamic compaction check");
  if (!*(unsigned int*)c->h_pinned) return CYTOM_OK;
  c->dyn_compactions++;
  return compact(c);
}

int insert_device(Ctx* c, const uint32_t* src, const uint32_t* tgt, const uint32_t* w,
                  uint64_t count) {
  if (count == 0) return CYTOM_OK;
  if (c->wtype != CYTOM_UNWEIGHTED && w == nullptr)
    return set_err(c, CYTOM_ERR_INVAL, "weighted store needs a weight per edge");
  cudaError_t e = cudaMemsetAsync(c->d_flag, 0, sizeof(unsigned int), c->stream);
  if (e != cudaSuccess) return cuda_err(c, e, "memset");
  int rc = ensure_app_capacity(c, c->A + count);
  if (rc) return rc;
  int slot = prof_begin(c, KC_INSERT);
  validate_kernel<<<grid_for(c, count, 256), 256, 0, c->stream>>>(src, tgt, count, c->n, c->d_flag);
  c->launches++;
  prof_end(c, slot, (double)count * 8.0);
  const uint32_t* wuse = (c->wtype != CYTOM_UNWEIGHTED) ? w : nullptr;
  slot = prof_begin(c, KC_INSERT);
  append_kernel<<<grid_for(c, count, 256), 256, 0, c->stream>>>(
      src, tgt, wuse, count, c->app_keys + c->A, wuse ? c->app_w + c->A : nullptr, c->out_deg,
      c->in_deg, c->lvpt, c->lT, c->d_flag);
  c->launches++;
  prof_end(c, slot, (double)count * (wuse ? 28.0 : 24.0));
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_err(c, e, "append_kernel");
  // one wait: the batch's copies (host path), validation and append
  e = cudaMemcpyAsync(c->h_pinned, c->d_flag, sizeof(unsigned int), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_err(c, e, "insert");
  if (*(unsigned int*)c->h_pinned)
    return set_err(c, CYTOM_ERR_RANGE, "edge endpoint >= vertex count; batch rejected");
  // the jobs are seeded by these edges when the compaction installs them
  c->A += count;
  if (c->cfg.use_dynamic_compaction) return dynamic_compaction(c, c->A - count, count);
  return CYTOM_OK;
}

// --------------------------------------------------------------------------
// Device-wide exclusive scan (u32), three phases with recursion on block sums.
// --------------------------------------------------------------------------
constexpr int SCAN_T = 256, SCAN_IPT = 16, SCAN_TILE = SCAN_T * SCAN_IPT;

__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t v) {
  const unsigned lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(0xFFFFFFFFu, v, o);
    if (lane >= (unsigned)o) v += y;
  }
  return v;
}

// Returns the exclusive block prefix of `v`; *total receives the block sum.
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t* total) {
  __shared__ uint32_t wsum[SCAN_T / 32];
  __shared__ uint32_t tot_s;
  const unsigned lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  uint32_t inc = warp_incl_scan(v);
  if (lane == 31) wsum[wid] = inc;
  __syncthreads();
  if (wid == 0) {
    uint32_t s = (lane < SCAN_T / 32) ? wsum[lane] : 0u;
    uint32_t si = warp_incl_scan(s);
    if (lane < SCAN_T / 32) wsum[lane] = si - s;
    if (lane == SCAN_T / 32 - 1) tot_s = si;
  }
  __syncthreads();
  uint32_t r = wsum[wid] + inc - v;
  *total = tot_s;
  __syncthreads();
  return r;
}

__global__ void scan_reduce_kernel(const uint32_t* __restrict__ in, uint64_t n,
                                   uint32_t* __restrict__ sums) {
  uint64_t base = (uint64_t)blockIdx.x * SCAN_TILE + (uint64_t)threadIdx.x * SCAN_IPT;
  uint32_t s = 0;
#pragma unroll
  for (int k = 0; k < SCAN_IPT; ++k) {
    uint64_t i = base + k;
    s += (i < n) ? in[i] : 0u;
  }
  uint32_t t;
  block_excl_scan(s, &t);
  if (threadIdx.x == 0) sums[blockIdx.x] = t;
}

__global__ void scan_down_kernel(const uint32_t* __restrict__ in, uint32_t* __restrict__ out,
                                 uint64_t n, const uint32_t* __restrict__ offs,
                                 uint32_t* total_out) {
  uint64_t base = (uint64_t)blockIdx.x * SCAN_TILE + (uint64_t)threadIdx.x * SCAN_IPT;
  uint32_t v[SCAN_IPT];
  uint32_t s = 0;
#pragma unroll
  for (int k = 0; k < SCAN_IPT; ++k) {
    uint64_t i = base + k;
    v[k] = (i < n) ? in[i] : 0u;
    s += v[k];
  }
  uint32_t t;
  const uint32_t boff = offs ? offs[blockIdx.x] : 0u;
  uint32_t p = block_excl_scan(s, &t) + boff;
#pragma unroll
  for (int k = 0; k < SCAN_IPT; ++k) {
    uint64_t i = base + k;
    if (i < n) out[i] = p;
    p += v[k];
  }
  if (total_out && blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) *total_out = boff + t;
}

// Words of scratch a scan of n values needs for its per-tile sums and their offsets,
// every recursion level together.
static uint64_t scan_scratch_words(uint64_t n) {
  const uint64_t nb = (n + SCAN_TILE - 1) / SCAN_TILE;
  return nb <= 1 ? 0 : 2 * nb + scan_scratch_words(nb);
}

// The scan on scratch the caller provides (scan_scratch_words(n) words): launches only.
static int scan_into(Ctx* c, const uint32_t* in, uint32_t* out, uint64_t n, uint32_t* total_dev,
                     uint32_t* scratch) {
  if (n == 0) return CYTOM_OK;
  const uint64_t nb = (n + SCAN_TILE - 1) / SCAN_TILE;
  if (nb == 1) {
    scan_down_kernel<<<1, SCAN_T, 0, c->stream>>>(in, out, n, nullptr, total_dev);
    c->launches++;
    return cuda_err(c, cudaGetLastError(), "scan_down");
  }
  uint32_t* sums = scratch;
  uint32_t* soffs = scratch + nb;
  scan_reduce_kernel<<<(unsigned)nb, SCAN_T, 0, c->stream>>>(in, n, sums);
  c->launches++;
  int rc = scan_into(c, sums, soffs, nb, nullptr, scratch + 2 * nb);
  if (rc) return rc;
  scan_down_kernel<<<(unsigned)nb, SCAN_T, 0, c->stream>>>(in, out, n, soffs, total_dev);
  c->launches++;
  return cuda_err(c, cudaGetLastError(), "scan");
}

int exclusive_scan_u32(Ctx* c, const uint32_t* in, uint32_t* out, uint64_t n, uint32_t* total_dev) {
  const uint64_t words = scan_scratch_words(n);
  if (words == 0) return scan_into(c, in, out, n, total_dev, nullptr);
  uint32_t* scratch = nullptr;
  if (cy_malloc_async((void**)&scratch, words * 4, c->stream) != cudaSuccess)
    return set_err(c, CYTOM_ERR_OOM, "scan temp");
  const int rc = scan_into(c, in, out, n, total_dev, scratch);
  cudaFreeAsync(scratch, c->stream);
  return rc;
}

// --------------------------------------------------------------------------
// LSD radix sort of (u64 key, u32 value) pairs, 8-bit digits, stable.
// Upsweep: per-block digit histogram (digit-major). Scan. Downsweep: warps rank
// items with __match_any_sync in input order and scatter.
// --------------------------------------------------------------------------

int radix_sort_pairs(Ctx* c, uint64_t* keys, uint64_t* keys_alt, uint32_t* vals, uint32_t* vals_alt,
                     uint64_t n, int bits, bool* result_in_alt) {
  *result_in_alt = false;
  if (n <= 1 || bits <= 0) return CYTOM_OK;
  const bool small = n < (1ULL << 24);
  const uint64_t tile = (uint64_t)RS_T * (small ? RS_IPT_SMALL : RS_IPT_LARGE);
  uint64_t nb = (n + tile - 1) / tile;
  uint32_t* hist = nullptr;
  // histogram, its scan and the scan's scratch in one allocation for every pass
  const uint64_t sw = scan_scratch_words(nb * 256);
  cudaError_t e = cy_malloc_async((void**)&hist, (nb * 256 * 2 + sw) * 4, c->stream);
  if (e != cudaSuccess) return set_err(c, CYTOM_ERR_OOM, "radix histogram");
  uint32_t* offs = hist + nb * 256;
  uint32_t* sscr = offs + nb * 256;
  uint64_t *kin = keys, *kout = keys_alt;
  uint32_t *vin = vals, *vout = vals_alt;
  bool alt = false;
  for (int shift = 0; shift < bits; shift += 8) {
    int slot = prof_begin(c, KC_SORT);
    if (small) radix_upsweep_kernel<RS_IPT_SMALL><<<(unsigned)nb, RS_T, 0, c->stream>>>(kin, n, shift, hist, (uint32_t)nb);
    else radix_upsweep_kernel<RS_IPT_LARGE><<<(unsigned)nb, RS_T, 0, c->stream>>>(kin, n, shift, hist, (uint32_t)nb);
    c->launches++;
    int rc = scan_into(c, hist, offs, nb * 256, nullptr, sscr);
    if (rc) {
      cudaFreeAsync(hist, c->stream);
      return rc;
    }
    if (small)
      radix_downsweep_kernel<RS_IPT_SMALL><<<(unsigned)nb, RS_T, 0, c->stream>>>(kin, vin, n, shift, offs, (uint32_t)nb,
                                                                               kout, vout);
    else
      radix_downsweep_kernel<RS_IPT_LARGE><<<(unsigned)nb, RS_T, 0, c->stream>>>(kin, vin, n, shift, offs, (uint32_t)nb,
                                                                               kout, vout);
    c->launches++;
    prof_end(c, slot, (double)n * (vals ? 12.0 : 8.0) * 3.0);
    e = cudaGetLastError();
    if (e != cudaSuccess) {
      cudaFreeAsync(hist, c->stream);
      return cuda_err(c, e, "radix");
    }
    std::swap(kin, kout);
    std::swap(vin, vout);
    alt = !alt;
  }
  cudaFreeAsync(hist, c->stream);
  *result_in_alt = alt;
  return CYTOM_OK;
}

// --------------------------------------------------------------------------
// Compaction
// --------------------------------------------------------------------------
__device__ __forceinline__ uint64_t lower_bound_u32(const uint32_t* a, uint64_t lo, uint64_t hi,
                                                    uint32_t v) {
  while (lo < hi) {
    uint64_t mid = lo + ((hi - lo) >> 1);
    if (a[mid] < v) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// For each sorted appended key: first of its run? present in the compacted tile?
// keep[i] = 1 for a new distinct edge; lb[i] = its insertion index in the old store;
// wsel[i] = the least weight of its run. A weight that undercuts the stored copy of
// an existing edge lowers that copy in place.
constexpr unsigned long long kNoFix = ~0ULL, kFixFlag = 1ULL << 62;

__global__ void dedupe_lookup_kernel(const uint64_t* __restrict__ K, const uint32_t* __restrict__ W,
                                     uint64_t A, const uint32_t* __restrict__ edges,
                                     const uint32_t* __restrict__ wts,
                                     const unsigned long long* __restrict__ tile_ptr,
                                     uint32_t lvpt, uint32_t* __restrict__ keep,
                                     unsigned long long* __restrict__ lb,
                                     uint32_t* __restrict__ wsel) {
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  const uint64_t m = (1ULL << lvpt) - 1ULL;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < A; i += stride) {
    uint64_t key = K[i];
    if (i > 0 && K[i - 1] == key) {
      keep[i] = 0;
      lb[i] = kNoFix;
      continue;
    }
    uint32_t wmin = 0;
    if (W) {
      wmin = W[i];
      for (uint64_t j = i + 1; j < A && K[j] == key; ++j) wmin = min(wmin, W[j]);
    }
    uint64_t tile = key >> (2 * lvpt);
    uint32_t local = (uint32_t)((((key >> lvpt) & m) << 16) | (key & m));
    uint64_t lo = tile_ptr[tile], hi = tile_ptr[tile + 1];
    // fillCSR starts its duplicate filter at (UINT16_MAX, UINT16_MAX)
    // (tile-manager.h:519-541): when that edge is the first in its tile's sorted
    // list -- an otherwise empty tile -- the reference drops it.
    if (local == 0xFFFFFFFFu && lo == hi && (i == 0 || (K[i - 1] >> (2 * lvpt)) != tile)) {
      keep[i] = 0;
      lb[i] = kNoFix;
      continue;
    }
    uint64_t pos = lower_bound_u32(edges, lo, hi, local);
    bool found = pos < hi && edges[pos] == local;
    if (found) {
      // a lower weight for a stored edge is applied to the merged copy (fixup_weights_kernel):
      // the store itself may still be read by runs of the previous batch
      keep[i] = 0;
      lb[i] = (W && wmin < wts[pos]) ? (kFixFlag | pos) : kNoFix;
      wsel[i] = wmin;
    } else {
      keep[i] = 1;
      lb[i] = pos;
      wsel[i] = wmin;
    }
  }
}

// Also sets the column-mask bit (StoreDesc::cmask) of every appended key's source and
// tile column, once per run of keys with the same (tile, source); duplicates and dropped
// corner edges only add bits that are allowed to be spare.
__global__ void pack_kept_kernel(const uint64_t* __restrict__ K, uint64_t A,
                                 const uint32_t* __restrict__ keep, const uint32_t* __restrict__ P,
                                 const unsigned long long* __restrict__ lb,
                                 const uint32_t* __restrict__ wsel, uint32_t lvpt,
                                 unsigned long long* __restrict__ q, uint32_t* __restrict__ nloc,
                                 uint32_t* __restrict__ nw, uint32_t* __restrict__ ntile,
                                 unsigned long long* __restrict__ cmask, uint32_t lT, uint32_t cshift) {
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  const uint64_t m = (1ULL << lvpt) - 1ULL;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < A; i += stride) {
    if (cmask) {
      const uint64_t ts = K[i] >> lvpt;  // (tile, local source)
      if (i == 0 || (K[i - 1] >> lvpt) != ts) {
        const uint64_t tile = ts >> lvpt;
        const uint64_t u = ((tile >> lT) << lvpt) | (ts & m);
        atomicOr(cmask + u, 1ULL << ((tile & ((1ULL << lT) - 1ULL)) >> cshift));
      }
    }
    if (!keep[i]) continue;
    uint64_t key = K[i];
    uint32_t p = P[i];
    q[p] = lb[i] + p;
    nloc[p] = (uint32_t)((((key >> lvpt) & m) << 16) | (key & m));
    if (nw) nw[p] = wsel[i];
    ntile[p] = (uint32_t)(key >> (2 * lvpt));
  }
}

// Weight of a stored edge lowered by the batch, on the merged copy: the old edge at pos
// moved by the kept new edges inserted at or before pos (q[p] - p <= pos).
__global__ void fixup_weights_kernel(const unsigned long long* __restrict__ lb, const uint32_t* __restrict__ wsel,
                                     uint64_t A, const unsigned long long* __restrict__ q,
                                     const uint32_t* __restrict__ Kdev, uint32_t* __restrict__ ow) {
  const uint64_t K = *Kdev;
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < A; i += stride) {
    const unsigned long long v = lb[i];
    if (v == kNoFix || !(v & kFixFlag)) continue;
    const uint64_t pos = v & ~kFixFlag;
    uint64_t lo = 0, hi = K;
    while (lo < hi) {
      const uint64_t mid = (lo + hi) >> 1;
      if (q[mid] - mid <= pos) lo = mid + 1;
      else hi = mid;
    }
    atomicMin(ow + pos + lo, wsel[i]);
  }
}

__device__ __forceinline__ uint64_t lower_bound_tile(const uint32_t* a, uint64_t n, uint32_t v) {
  uint64_t lo = 0, hi = n;
  while (lo < hi) {
    uint64_t mid = lo + ((hi - lo) >> 1);
    if (a[mid] < v) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

__global__ void new_tile_ptr_kernel(const unsigned long long* __restrict__ tile_ptr,
                                    uint64_t ntiles, const uint32_t* __restrict__ ntile,
                                    const uint32_t* __restrict__ Kdev,
                                    unsigned long long* __restrict__ out) {
  uint64_t K = *Kdev;
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t <= ntiles; t += stride) {
    uint64_t add = (t == ntiles) ? K : lower_bound_tile(ntile, K, (uint32_t)t);
    out[t] = tile_ptr[t] + add;
  }
}

// Output position o of the merged store holds kept batch element b when q[b] == o,
// otherwise old store element o - (number of q below o). One warp produces 32
// consecutive outputs per step, 1024 per span. merge_spans_kernel gives every span its
// first new element (sb) and the tile of its first output (ts) by binary searches that
// all run at once. When a span holds at most 64 new elements (the usual case: new edges
// are sparse in the store) they sit in two registers per lane and each step finds its
// candidates by shuffles, so the sources of MG steps are known without memory round
// trips and their loads issue together; a span with more new elements loads its
// candidates step by step. Stores are coalesced 128-byte warp writes.
//
// The store is streamed with evict-first loads and stores, leaving L2 to the jobs that
// run on the installed snapshot meanwhile (the pipelined stream).
// The same pass writes the chunk table of the new store and, when the context keeps a
// source directory, its per-edge entries (the work of dir_edges_kernel): each output
// knows its tile (walked from the span's first tile) and the edge before it.
constexpr int MERGE_STEPS = 32;  // 1024 outputs per warp span
constexpr uint64_t MERGE_SPAN = 32ULL * MERGE_STEPS;
constexpr int MG = 8;            // steps whose loads are issued together

__global__ void merge_spans_kernel(const unsigned long long* __restrict__ q, const uint32_t* __restrict__ Kdev,
                                   uint64_t E, const unsigned long long* __restrict__ tp, uint64_t ntiles,
                                   uint64_t nsp, uint32_t* __restrict__ sb, uint32_t* __restrict__ ts,
                                   uint32_t* __restrict__ chunk_tile) {
  const uint64_t K = *Kdev;
  const uint64_t total = E + K;
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  const uint64_t gid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (gid == 0) chunk_tile[(total + kChunk - 1) / kChunk] = (uint32_t)(ntiles - 1);
  for (uint64_t sp = gid; sp <= nsp; sp += stride) {
    const uint64_t target = sp * MERGE_SPAN;
    uint64_t lo = 0, hi = K;
    while (lo < hi) {
      uint64_t mid = lo + ((hi - lo) >> 1);
      if (q[mid] < target) lo = mid + 1;
      else hi = mid;
    }
    sb[sp] = (uint32_t)lo;
    // the last tile t with tp[t] <= target
    lo = 0;
    hi = ntiles - 1;
    while (lo < hi) {
      const uint64_t mid = (lo + hi + 1) >> 1;
      if (tp[mid] <= target) lo = mid;
      else hi = mid - 1;
    }
    ts[sp] = (uint32_t)lo;
  }
}

// Per output (offsets relative to the span start): its tile, walked forward from the
// warp's tile state (tile t; toff turns a span offset into an offset within the tile;
// tend = the span offset where the tile ends), the chunk-table entry at every 128th
// output, and the directory entries of the 32-source blocks that start at this edge.
// The tile state of lane 31 carries over to the next step.
__device__ __forceinline__ void merge_index_step(uint32_t o, uint32_t nout, uint32_t ev, uint32_t pv, uint32_t& t,
                                                 uint32_t& toff, uint32_t& tend, uint64_t wbase,
                                                 const unsigned long long* __restrict__ tp,
                                                 uint32_t* __restrict__ ctb, uint32_t* __restrict__ dir,
                                                 uint32_t nbw) {
  uint32_t lt = t, loff = toff, lend = tend;
  if (o < nout) {
    while (o >= lend) {
      ++lt;
      loff = 0u - lend;
      const unsigned long long nx = tp[lt + 1] - wbase;
      lend = nx > 0xFFFFFFFFULL ? 0xFFFFFFFFu : (uint32_t)nx;
    }
    if ((o & (kChunk - 1)) == 0) ctb[o / kChunk] = lt;
    if (dir) {
      const uint32_t off = o + loff;
      const int bk = (int)(ev >> 21);
      const int bprev = off == 0 ? -1 : (int)(pv >> 21);
      if (bk != bprev) {
        uint32_t* dt = dir + (uint64_t)lt * (nbw + 1);
        for (int bb = bprev + 1; bb <= bk; ++bb) dt[bb] = off;
      }
    }
  }
  t = __shfl_sync(0xFFFFFFFFu, lt, 31);
  toff = __shfl_sync(0xFFFFFFFFu, loff, 31);
  tend = __shfl_sync(0xFFFFFFFFu, lend, 31);
}

__global__ void merge_gather_kernel(const uint32_t* __restrict__ edges, const uint32_t* __restrict__ wts,
                                    uint64_t E, const unsigned long long* __restrict__ q,
                                    const uint32_t* __restrict__ nloc, const uint32_t* __restrict__ nw,
                                    const uint32_t* __restrict__ Kdev, const uint32_t* __restrict__ sb,
                                    const uint32_t* __restrict__ ts, uint64_t nsp,
                                    const unsigned long long* __restrict__ tp, uint32_t* __restrict__ chunk_tile,
                                    uint32_t* __restrict__ dir, uint32_t nbw, uint32_t* __restrict__ oe,
                                    uint32_t* __restrict__ ow) {
  const uint64_t K = *Kdev;
  const uint64_t total = E + K;
  const unsigned lane = threadIdx.x & 31;
  const uint64_t warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  const unsigned lt = (1u << lane) - 1u;
  for (uint64_t sp = warp; sp < nsp; sp += nwarps) {
    const uint64_t wbase = sp * MERGE_SPAN;
    if (wbase >= total) break;
    const uint32_t nout = (uint32_t)(total - wbase < MERGE_SPAN ? total - wbase : MERGE_SPAN);
    const uint64_t b0 = sb[sp];
    const uint32_t cnt = sb[sp + 1] - (uint32_t)b0;
    // span-relative views: output x preceded by y new elements of the span comes from
    // eb[x - y] (old) or nb[y] (new)
    const uint32_t* eb = edges + (wbase - b0);
    const uint32_t* wb = wts ? wts + (wbase - b0) : nullptr;
    const uint32_t* nb = nloc + b0;
    const uint32_t* nwb = nw ? nw + b0 : nullptr;
    uint32_t* oeb = oe + wbase;
    uint32_t* owb = ow ? ow + wbase : nullptr;
    uint32_t* ctb = chunk_tile + wbase / kChunk;
    uint32_t t = ts[sp];
    uint32_t toff = (uint32_t)(wbase - tp[t]);
    uint32_t tend;
    {
      const unsigned long long nx = tp[t + 1] - wbase;
      tend = nx > 0xFFFFFFFFULL ? 0xFFFFFFFFu : (uint32_t)nx;
    }
    // the edge before the span (the first output's predecessor)
    uint32_t plast = 0;
    if (lane == 0 && wbase > 0) {
      if (b0 > 0 && q[b0 - 1] == wbase - 1) plast = nloc[b0 - 1];
      else plast = edges[wbase - 1 - b0];
    }
    plast = __shfl_sync(0xFFFFFFFFu, plast, 0);
    if (cnt <= 64) {
      const uint32_t qa = (lane < cnt) ? (uint32_t)(q[b0 + lane] - wbase) : 0xFFFFFFFFu;
      const uint32_t qb = (32 + lane < cnt) ? (uint32_t)(q[b0 + 32 + lane] - wbase) : 0xFFFFFFFFu;
      uint32_t r = 0;  // new elements consumed so far in this span
      for (int g = 0; g < MERGE_STEPS; g += MG) {
        if ((uint32_t)g * 32 >= nout) break;
        uint32_t src[MG];
        unsigned isnew = 0;
#pragma unroll
        for (int k = 0; k < MG; ++k) {
          const uint32_t o_start = (uint32_t)(g + k) * 32;
          const uint32_t idx = r + lane;
          const uint32_t ca = __shfl_sync(0xFFFFFFFFu, qa, idx & 31);
          const uint32_t cb = __shfl_sync(0xFFFFFFFFu, qb, idx & 31);
          const uint32_t rel = (idx < 32 ? ca : (idx < 64 ? cb : 0xFFFFFFFFu)) - o_start;
          const unsigned mask = __reduce_or_sync(0xFFFFFFFFu, rel < 32u ? (1u << rel) : 0u);
          const uint32_t y = r + __popc(mask & lt);
          if ((mask >> lane) & 1u) {
            isnew |= 1u << k;
            src[k] = y;
          } else {
            src[k] = o_start + lane - y;
          }
          r += __popc(mask);
        }
        uint32_t ev[MG], wv[MG];
#pragma unroll
        for (int k = 0; k < MG; ++k) {
          const uint32_t o = (uint32_t)(g + k) * 32 + lane;
          ev[k] = 0;
          wv[k] = 0;
          if (o < nout) {
            if ((isnew >> k) & 1u) {
              ev[k] = nb[src[k]];
              if (owb) wv[k] = nwb[src[k]];
            } else {
              ev[k] = __ldcs(eb + src[k]);
              if (owb) wv[k] = __ldcs(wb + src[k]);
            }
          }
        }
#pragma unroll
        for (int k = 0; k < MG; ++k) {
          const uint32_t o = (uint32_t)(g + k) * 32 + lane;
          if (o < nout) {
            __stcs(oeb + o, ev[k]);
            if (owb) __stcs(owb + o, wv[k]);
          }
          uint32_t pv = __shfl_up_sync(0xFFFFFFFFu, ev[k], 1);
          if (lane == 0) pv = plast;
          merge_index_step(o, nout, ev[k], pv, t, toff, tend, wbase, tp, ctb, dir, nbw);
          plast = __shfl_sync(0xFFFFFFFFu, ev[k], 31);
        }
      }
      continue;
    }
    uint32_t r = 0;
    for (int st = 0; st < MERGE_STEPS; ++st) {
      const uint32_t o_start = (uint32_t)st * 32;
      if (o_start >= nout) break;
      const uint32_t cand = (r + lane < cnt) ? (uint32_t)(q[b0 + r + lane] - wbase) : 0xFFFFFFFFu;
      const uint32_t rel = cand - o_start;
      const unsigned mask = __reduce_or_sync(0xFFFFFFFFu, rel < 32u ? (1u << rel) : 0u);
      const uint32_t o = o_start + lane;
      uint32_t ev = 0, wv = 0;
      if (o < nout) {
        const uint32_t y = r + __popc(mask & lt);
        if ((mask >> lane) & 1u) {
          ev = nb[y];
          if (owb) wv = nwb[y];
        } else {
          ev = __ldcs(eb + (o - y));
          if (owb) wv = __ldcs(wb + (o - y));
        }
        __stcs(oeb + o, ev);
        if (owb) __stcs(owb + o, wv);
      }
      uint32_t pv = __shfl_up_sync(0xFFFFFFFFu, ev, 1);
      if (lane == 0) pv = plast;
      merge_index_step(o, nout, ev, pv, t, toff, tend, wbase, tp, ctb, dir, nbw);
      plast = __shfl_sync(0xFFFFFFFFu, ev, 31);
      r += __popc(mask);
    }
  }
}

__global__ void chunk_tile_kernel(const unsigned long long* __restrict__ tile_ptr, uint64_t ntiles,
                                  uint64_t nchunks, uint32_t* __restrict__ chunk_tile) {
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t cix = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; cix <= nchunks; cix += stride) {
    if (cix == nchunks) {
      chunk_tile[cix] = (uint32_t)(ntiles - 1);
      continue;
    }
    unsigned long long e = (unsigned long long)cix * kChunk;
    // last tile t with tile_ptr[t] <= e
    uint64_t lo = 0, hi = ntiles;  // search in tile_ptr[0..ntiles]
    while (lo < hi) {
      uint64_t mid = lo + ((hi - lo + 1) >> 1);
      if (tile_ptr[mid] <= e) lo = mid;
      else hi = mid - 1;
    }
    if (lo >= ntiles) lo = ntiles - 1;
    chunk_tile[cix] = (uint32_t)lo;
  }
}

static int grow_store(Ctx* c, uint64_t need) {
  if (need <= c->cap) return CYTOM_OK;
  join_runs(c);  // the old buffers are freed below
  uint64_t ncap = std::max<uint64_t>(need + need / 2, 1 << 16);
  ncap = (ncap + kChunk - 1) / kChunk * kChunk + kChunk;
  uint32_t *ne = nullptr, *nea = nullptr, *nw = nullptr, *nwa = nullptr;
  cudaError_t e = cy_malloc(&ne, ncap * 4);
  if (e == cudaSuccess) e = cy_malloc(&nea, ncap * 4);
  if (e == cudaSuccess && c->wtype) e = cy_malloc(&nw, ncap * 4);
  if (e == cudaSuccess && c->wtype) e = cy_malloc(&nwa, ncap * 4);
  if (e != cudaSuccess) {
    cudaGetLastError();
    cudaFree(ne);
    cudaFree(nea);
    cudaFree(nw);
    cudaFree(nwa);
    return set_err(c, CYTOM_ERR_OOM, "tile store growth");
  }
  if (c->E) {
    cudaMemcpyAsync(ne, c->edges, c->E * 4, cudaMemcpyDeviceToDevice, c->stream);
    if (c->wtype) cudaMemcpyAsync(nw, c->wts, c->E * 4, cudaMemcpyDeviceToDevice, c->stream);
  }
  cudaStreamSynchronize(c->stream);
  cudaFree(c->edges);
  cudaFree(c->edges_alt);
  cudaFree(c->wts);
  cudaFree(c->wts_alt);
  c->edges = ne;
  c->edges_alt = nea;
  c->wts = nw;
  c->wts_alt = nwa;
  c->cap = ncap;
  uint64_t nch = ncap / kChunk + 2;
  if (nch > c->chunk_cap) {
    uint32_t *ct = nullptr, *cta = nullptr;
    if (cy_malloc(&ct, nch * 4) != cudaSuccess || cy_malloc(&cta, nch * 4) != cudaSuccess) {
      cudaGetLastError();
      cudaFree(ct);
      return set_err(c, CYTOM_ERR_OOM, "chunk table");
    }
    cudaMemcpyAsync(ct, c->chunk_tile, c->chunk_cap * 4, cudaMemcpyDeviceToDevice, c->stream);
    cudaStreamSynchronize(c->stream);
    cudaFree(c->chunk_tile);
    cudaFree(c->chunk_tile_alt);
    c->chunk_tile = ct;
    c->chunk_tile_alt = cta;
    c->chunk_cap = nch;
  }
  return CYTOM_OK;
}

int ensure_app_capacity(Ctx* c, uint64_t need) {
  if (need <= c->app_cap) return CYTOM_OK;
  uint64_t ncap = std::max<uint64_t>(need + need / 2, 1 << 16);
  uint64_t *k = nullptr, *ka = nullptr;
  uint32_t *w = nullptr, *wa = nullptr;
  cudaError_t e = cy_malloc(&k, ncap * 8);
  if (e == cudaSuccess) e = cy_malloc(&ka, ncap * 8);
  if (e == cudaSuccess && c->wtype) e = cy_malloc(&w, ncap * 4);
  if (e == cudaSuccess && c->wtype) e = cy_malloc(&wa, ncap * 4);
  if (e != cudaSuccess) {
    cudaGetLastError();
    cudaFree(k);
    cudaFree(ka);
    cudaFree(w);
    cudaFree(wa);
    return set_err(c, CYTOM_ERR_OOM, "append region growth");
  }
  if (c->A) {
    cudaMemcpyAsync(k, c->app_keys, c->A * 8, cudaMemcpyDeviceToDevice, c->stream);
    if (c->wtype) cudaMemcpyAsync(w, c->app_w, c->A * 4, cudaMemcpyDeviceToDevice, c->stream);
  }
  cudaStreamSynchronize(c->stream);
  cudaFree(c->app_keys);
  cudaFree(c->app_keys_alt);
  cudaFree(c->app_w);
  cudaFree(c->app_w_alt);
  c->app_keys = k;
  c->app_keys_alt = ka;
  c->app_w = w;
  c->app_w_alt = wa;
  c->app_cap = ncap;
  return CYTOM_OK;
}

__global__ void dir_tiles_kernel(const StoreDesc* __restrict__ sd, uint32_t* __restrict__ dir, uint32_t nbw);

int compact(Ctx* c) {
  if (c->A == 0) return CYTOM_OK;
  const uint64_t A = c->A;
  const bool wt = c->wtype != CYTOM_UNWEIGHTED;
  bool in_alt = false;
  int rc = radix_sort_pairs(c, c->app_keys, c->app_keys_alt, wt ? c->app_w : nullptr,
                            wt ? c->app_w_alt : nullptr, A, (int)(2 * (c->lvpt + c->lT)), &in_alt);
  if (rc) return rc;
  const uint64_t* K = in_alt ? c->app_keys_alt : c->app_keys;
  const uint32_t* W = wt ? (in_alt ? c->app_w_alt : c->app_w) : nullptr;
  rc = grow_store(c, c->E + A);
  if (rc) return rc;
  // temporaries
  const uint64_t nsp = (c->E + A + MERGE_SPAN - 1) / MERGE_SPAN;  // merge spans (upper bound)
  size_t bytes = A * (4 + 4 + 8 + 4 + 8 + 4 + 4 + 4) + 64 + 2 * (nsp + 1) * 4;
  char* tmp = nullptr;
  cudaError_t e = cy_malloc_async((void**)&tmp, bytes, c->stream);
  if (e != cudaSuccess) return set_err(c, CYTOM_ERR_OOM, "compaction temporaries");
  unsigned long long* lb = (unsigned long long*)tmp;
  unsigned long long* q = lb + A;
  uint32_t* keep = (uint32_t*)(q + A);
  uint32_t* P = keep + A;
  uint32_t* wsel = P + A;
  uint32_t* nloc = wsel + A;
  uint32_t* nw = nloc + A;
  uint32_t* ntile = nw + A;
  uint32_t* Kdev = ntile + A;
  uint32_t* sb = Kdev + 16;
  uint32_t* ts = sb + (nsp + 1);
  int slot = prof_begin(c, KC_MERGE);
  dedupe_lookup_kernel<<<grid_for(c, A, 256), 256, 0, c->stream>>>(
      K, W, A, c->edges, c->wts, c->tile_ptr, c->lvpt, keep, lb, wsel);
  c->launches++;
  rc = exclusive_scan_u32(c, keep, P, A, Kdev);
  if (rc) return rc;
  pack_kept_kernel<<<grid_for(c, A, 256), 256, 0, c->stream>>>(K, A, keep, P, lb, wsel, c->lvpt, q,
                                                               nloc, wt ? nw : nullptr, ntile, c->cmask, c->lT,
                                                               c->lT > 6 ? c->lT - 6 : 0u);
  c->launches++;
  new_tile_ptr_kernel<<<grid_for(c, c->ntiles + 1, 256), 256, 0, c->stream>>>(
      c->tile_ptr, c->ntiles, ntile, Kdev, c->tile_ptr_alt);
  c->launches++;
  // The merge writes only the alternate buffers (store, tile offsets, chunk table and,
  // once the context keeps one, the source directory), so it may overlap runs that still
  // read the installed snapshot.
  uint32_t* mdir = nullptr;
  if (c->dir && !c->dir_disabled) {
    if (!c->dir_alt && cy_malloc(&c->dir_alt, c->dir_entries * 4) != cudaSuccess) {
      cudaGetLastError();
      c->dir_alt = nullptr;
    }
    mdir = c->dir_alt;
  }
  merge_spans_kernel<<<grid_for(c, nsp + 1, 256), 256, 0, c->stream>>>(q, Kdev, c->E, c->tile_ptr_alt, c->ntiles,
                                                                       nsp, sb, ts, c->chunk_tile_alt);
  merge_gather_kernel<<<(unsigned)std::max<uint64_t>(1, std::min<uint64_t>((nsp + 7) / 8, (uint64_t)c->num_sms * 8)),
                        256, 0, c->stream>>>(c->edges, c->wts, c->E, q, nloc, nw, Kdev, sb, ts, nsp, c->tile_ptr_alt,
                                             c->chunk_tile_alt, mdir, (uint32_t)(c->vpt / 32), c->edges_alt,
                                             wt ? c->wts_alt : nullptr);
  c->launches += 2;
  e = cudaMemcpyAsync(c->h_pinned, Kdev, 4, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) {
    cudaFreeAsync(tmp, c->stream);
    return cuda_err(c, e, "compaction");
  }
  uint64_t Kn = *(uint32_t*)c->h_pinned;
  prof_end(c, slot, (double)A * (wt ? 44.0 : 36.0) + (double)(c->E + Kn) * (wt ? 16.0 : 8.0));
  rc = pagerank_note_kept(c, nloc, ntile, Kn);  // the PageRank CSC's next build merges these in
  if (rc) {
    cudaFreeAsync(tmp, c->stream);
    return rc;
  }
  // Installing the merged snapshot: runs on the previous one must have finished. The jobs
  // are then seeded by the merged edges (edgeChanged(INSERT)) and lowered weights of
  // stored edges are applied to the merged copy.
  join_runs(c);
  {
    std::vector<Job*> mp;
    for (Job* j : c->jobs) {
      if (!j || j->fresh) continue;
      if (j->algo == CYTOM_ALGO_BFS || j->algo == CYTOM_ALGO_CC || j->algo == CYTOM_ALGO_SSSP ||
          j->algo == CYTOM_ALGO_SSWP)
        mp.push_back(j);
      else
        rc = job_seed_keys(c, j, K, W, A);  // the PageRank family: a residual round next time
      if (rc) break;
    }
    if (!rc && !mp.empty()) rc = minprop_seed_keys_many(c, mp.data(), (int)mp.size(), K, W, A);
    if (rc) {
      cudaFreeAsync(tmp, c->stream);
      return rc;
    }
  }
  if (wt) {
    fixup_weights_kernel<<<grid_for(c, A, 256), 256, 0, c->stream>>>(lb, wsel, A, q, Kdev, c->wts_alt);
    c->launches++;
  }
  cudaFreeAsync(tmp, c->stream);
  if (c->dyn_pending) cudaMemsetAsync(c->dyn_pending, 0, c->ntiles * 4, c->stream);  // nothing appended now
  std::swap(c->edges, c->edges_alt);
  std::swap(c->wts, c->wts_alt);
  std::swap(c->tile_ptr, c->tile_ptr_alt);
  std::swap(c->chunk_tile, c->chunk_tile_alt);
  if (mdir) std::swap(c->dir, c->dir_alt);
  c->E += Kn;
  c->A = 0;
  c->version++;
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_err(c, e, "merge");
  if (mdir) c->dir_version = c->version;  // completed below, before any later launch reads it
  int urc = upload_store_desc(c);
  if (urc || !mdir) return urc;
  // the merge wrote every directory entry up to each tile's last source block
  dir_tiles_kernel<<<grid_for(c, c->ntiles * 32, 256), 256, 0, c->stream>>>(c->dsd, c->dir, (uint32_t)(c->vpt / 32));
  c->launches++;
  return cuda_err(c, cudaGetLastError(), "directory");
}

// Compact-vs-sparse flag per tile: distinct sources >= vpt / 2 (tile-manager.h:261-263).
__global__ void count_sources_kernel(const uint32_t* __restrict__ edges,
                                     const unsigned long long* __restrict__ tile_ptr,
                                     uint64_t ntiles, uint64_t vpt, uint8_t* __restrict__ flags) {
  // one warp per tile
  const unsigned lane = threadIdx.x & 31;
  uint64_t warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  for (uint64_t t = warp; t < ntiles; t += nwarps) {
    uint64_t lo = tile_ptr[t], hi = tile_ptr[t + 1];
    uint32_t cnt = 0;
    for (uint64_t i = lo + lane; i < hi; i += 32) {
      uint32_t s = edges[i] >> 16;
      uint32_t prev = (i == lo) ? 0xFFFFFFFFu : (edges[i - 1] >> 16);
      cnt += (s != prev) ? 1u : 0u;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xFFFFFFFFu, cnt, o);
    if (lane == 0) flags[t] = (hi > lo) ? (uint8_t)(cnt >= vpt / 2 ? 1 : 0) : 2;  // 2 = empty
  }
}

// Source directory for sparse rounds. Per edge: the 32-source blocks from just after
// the previous edge's block up to its own start at this edge. Per tile: the blocks after
// the last edge's block (all blocks of an empty tile) hold the tile size.
__global__ void dir_edges_kernel(const StoreDesc* __restrict__ sd, uint32_t* __restrict__ dir, uint32_t nbw) {
  // one warp per 128-edge chunk, four edges per lane; a chunk inside one tile (nearly
  // all of them) takes a 32-bit fast path
  const uint64_t E = sd->E, nchunks = sd->nchunks;
  const unsigned lane = threadIdx.x & 31;
  const uint64_t warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  for (uint64_t c = warp; c < nchunks; c += nwarps) {
    const uint64_t cbase = c * kChunk;
    const uint64_t e0 = cbase + (uint64_t)lane * 4;
    const uint4 q = *reinterpret_cast<const uint4*>(sd->edges + e0);  // the store has kChunk slack
    uint32_t prev0 = __shfl_up_sync(0xFFFFFFFFu, q.w, 1);
    if (lane == 0) prev0 = cbase > 0 ? sd->edges[cbase - 1] : 0u;
    const uint32_t ev[5] = {prev0, q.x, q.y, q.z, q.w};
    uint32_t t = sd->chunk_tile[c];
    unsigned long long tlo = sd->tile_ptr[t], thi = sd->tile_ptr[t + 1];
    const uint64_t cend = cbase + kChunk < E ? cbase + kChunk : E;
    if (tlo <= cbase && cend <= thi) {
      uint32_t* dt = dir + (uint64_t)t * (nbw + 1);
      const uint32_t r0 = (uint32_t)(e0 - tlo);
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        if (e0 + k >= E) break;
        const int b = (int)(ev[k + 1] >> 21);
        const int bprev = (r0 + k == 0) ? -1 : (int)(ev[k] >> 21);
        for (int bb = bprev + 1; bb <= b; ++bb) dt[bb] = r0 + k;
      }
      continue;
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const uint64_t e = e0 + k;
      if (e >= E) break;
      while (thi <= e) {
        ++t;
        tlo = thi;
        thi = sd->tile_ptr[t + 1];
      }
      const int b = (int)((ev[k + 1] >> 16) >> 5);
      const int bprev = (e == tlo) ? -1 : (int)((ev[k] >> 16) >> 5);
      if (b == bprev) continue;
      uint32_t* dt = dir + (uint64_t)t * (nbw + 1);
      for (int bb = bprev + 1; bb <= b; ++bb) dt[bb] = (uint32_t)(e - tlo);
    }
  }
}

__global__ void dir_tiles_kernel(const StoreDesc* __restrict__ sd, uint32_t* __restrict__ dir, uint32_t nbw) {
  const uint64_t ntiles = sd->ntiles;
  const unsigned lane = threadIdx.x & 31;
  const uint64_t warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  for (uint64_t t = warp; t < ntiles; t += nwarps) {
    const uint64_t lo = sd->tile_ptr[t], hi = sd->tile_ptr[t + 1];
    const int blast = (hi > lo) ? (int)((sd->edges[hi - 1] >> 16) >> 5) : -1;
    uint32_t* dt = dir + t * (nbw + 1);
    for (int bb = blast + 1 + (int)lane; bb <= (int)nbw; bb += 32) dt[bb] = (uint32_t)(hi - lo);
  }
}

// Column-mask bits of every stored edge (a full directory build): one atomic per run of
// edges with the same source in a tile.
__global__ void cmask_all_kernel(const StoreDesc* __restrict__ sd, unsigned long long* __restrict__ cmask,
                                 uint32_t cshift) {
  const uint64_t E = sd->E, T = sd->T;
  const uint32_t lT = sd->lT, lvpt = sd->lvpt;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; e < E; e += stride) {
    uint64_t t = sd->chunk_tile[e / kChunk];
    while (sd->tile_ptr[t + 1] <= e) ++t;
    const uint32_t src = sd->edges[e] >> 16;
    if (e > sd->tile_ptr[t] && (sd->edges[e - 1] >> 16) == src) continue;
    atomicOr(cmask + (((t >> lT) << lvpt) | src), 1ULL << ((t & (T - 1)) >> cshift));
  }
}

int build_directory(Ctx* c) {
  if (c->dir_version == c->version || c->dir_disabled) return CYTOM_OK;
  const char* env = getenv("CYTOM_SPARSE");  // "0": dense rounds only
  if (c->lvpt < 5 || !c->cfg.enable_adaptive_scheduling || (env && env[0] == '0')) {
    c->dir_disabled = true;
    return upload_store_desc(c);
  }
  const uint64_t nbw = c->vpt / 32;
  const uint64_t entries = c->T * (nbw + 1) * c->T;
  // the directory is worth its memory only while it is small next to the edges
  if (entries * 4 > (4ULL << 30)) {
    c->dir_disabled = true;
    return upload_store_desc(c);
  }
  if (!c->dir) {
    if (cy_malloc(&c->dir, entries * 4) != cudaSuccess) {
      cudaGetLastError();
      c->dir_disabled = true;
      return upload_store_desc(c);
    }
    c->dir_entries = entries;
  }
  // column masks: without memory for them sparse rounds read every item's directory entry
  if (!c->cmask) {
    if (cy_malloc(&c->cmask, c->n * 8) != cudaSuccess) {
      cudaGetLastError();
      c->cmask = nullptr;
    } else {
      cudaMemsetAsync(c->cmask, 0, c->n * 8, c->stream);
    }
  }
  int slot = prof_begin(c, KC_MERGE);
  if (c->E) {
    dir_edges_kernel<<<grid_for(c, (c->E + 3) / 4, 256), 256, 0, c->stream>>>(c->dsd, c->dir, (uint32_t)nbw);
    c->launches++;
    if (c->cmask) {
      cmask_all_kernel<<<grid_for(c, c->E, 256), 256, 0, c->stream>>>(c->dsd, c->cmask, c->lT > 6 ? c->lT - 6 : 0u);
      c->launches++;
    }
  }
  dir_tiles_kernel<<<grid_for(c, c->ntiles * 32, 256), 256, 0, c->stream>>>(c->dsd, c->dir, (uint32_t)nbw);
  c->launches++;
  prof_end(c, slot, (double)c->E * 8.0 + (double)entries * 4.0);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_err(c, e, "directory");
  c->dir_version = c->version;
  return upload_store_desc(c);
}

int compute_compact_flags(Ctx* c, uint8_t* dflags) {
  count_sources_kernel<<<grid_for(c, c->ntiles * 32, 256), 256, 0, c->stream>>>(
      c->edges, c->tile_ptr, c->ntiles, c->vpt, dflags);
  c->launches++;
  return cuda_err(c, cudaGetLastError(), "count_sources");
}


// Deletion of stored edges: the store side of TileManager::deleteEdge and of the
// deleted-edge filter of compactStorage / fillCSR (tile-manager.h:165-173, 249-253,
// 532-535), applied at once instead of kept as a deleted set. Request i finds
// (src[i], tgt[i]) in its tile (binary search over the sorted packed edges); the request
// that sets the edge's kill bit first drops out_deg[src] and in_deg[tgt] by one and
// appends (src, tgt, weight) to the deleted list. A pair that is not stored is skipped.
__global__ void delete_mark_kernel(const StoreDesc* __restrict__ sd, const uint32_t* __restrict__ src,
                                   const uint32_t* __restrict__ tgt, uint64_t count, uint32_t* kill,
                                   uint32_t* out_deg, uint32_t* in_deg, uint32_t* dsrc, uint32_t* dtgt,
                                   uint32_t* dw, unsigned long long* ndel) {
  const uint32_t lvpt = sd->lvpt, lT = sd->lT;
  const uint32_t lmask = (1u << lvpt) - 1u;
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += stride) {
    const uint32_t u = src[i], v = tgt[i];
    if ((uint64_t)u >= sd->n || (uint64_t)v >= sd->n) continue;
    const uint64_t t = ((uint64_t)(u >> lvpt) << lT) | (v >> lvpt);
    const uint32_t key = ((u & lmask) << 16) | (v & lmask);
    const uint64_t end = sd->tile_ptr[t + 1];
    uint64_t lo = sd->tile_ptr[t], hi = end;
    while (lo < hi) {
      const uint64_t mid = (lo + hi) >> 1;
      if (sd->edges[mid] < key) lo = mid + 1;
      else hi = mid;
    }
    if (lo >= end || sd->edges[lo] != key) continue;
    const uint32_t bit = 1u << (lo & 31);
    if (atomicOr(kill + (lo >> 5), bit) & bit) continue;  // another request took it
    atomicSub(out_deg + u, 1u);
    atomicSub(in_deg + v, 1u);
    const unsigned long long k = atomicAdd(ndel, 1ULL);
    dsrc[k] = u;
    dtgt[k] = v;
    if (dw) dw[k] = sd->wts[lo];
  }
}

// Kept edges per 32-edge word of the kill bitmap; word nw (one past the last) counts 0,
// so the exclusive scan's entry nw is the new edge count.
__global__ void keep_count_kernel(const uint32_t* __restrict__ kill, uint64_t E, uint64_t nw,
                                  uint32_t* __restrict__ cnt) {
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t w = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; w <= nw; w += stride) {
    if (w == nw) {
      cnt[w] = 0;
      continue;
    }
    const unsigned r = (unsigned)(E - w * 32);
    const uint32_t valid = r >= 32 ? 0xFFFFFFFFu : ((1u << r) - 1u);
    cnt[w] = __popc(~kill[w] & valid);
  }
}

// New position of old position p: kept edges before p.
__device__ __forceinline__ uint64_t kept_before(const uint32_t* kill, const uint32_t* P, uint64_t p) {
  const uint64_t w = p >> 5;
  const unsigned b = (unsigned)(p & 31);
  return (uint64_t)P[w] + (b ? (uint64_t)__popc(~kill[w] & ((1u << b) - 1u)) : 0ULL);
}

// Order-preserving gather of the kept edges (each tile stays sorted).
__global__ void delete_gather_kernel(const uint32_t* __restrict__ edges, const uint32_t* __restrict__ wts,
                                     uint64_t E, const uint32_t* __restrict__ kill, const uint32_t* __restrict__ P,
                                     uint32_t* __restrict__ oe, uint32_t* __restrict__ ow) {
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < E; i += stride) {
    const uint32_t k = kill[i >> 5];
    const unsigned b = (unsigned)(i & 31);
    if ((k >> b) & 1u) continue;
    const uint64_t o = (uint64_t)P[i >> 5] + __popc(~k & ((1u << b) - 1u));
    oe[o] = edges[i];
    if (ow) ow[o] = wts[i];
  }
}

__global__ void delete_tile_ptr_kernel(const unsigned long long* __restrict__ tile_ptr, uint64_t ntiles,
                                       const uint32_t* __restrict__ kill, const uint32_t* __restrict__ P,
                                       unsigned long long* __restrict__ out) {
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t <= ntiles; t += stride)
    out[t] = kept_before(kill, P, tile_ptr[t]);
}

int minprop_delete_check(Ctx* c, Job* j, const uint32_t* dsrc, const uint32_t* dtgt, const uint32_t* dw,
                         uint64_t count, unsigned* tight);

// Removes the stored (src, tgt) pairs listed (device pointers) after compacting pending
// inserts. The store is rewritten without them in one order-preserving pass; BFS / CC /
// SSSP / SSWP jobs restart only if a deleted edge was tight for them, the PageRank
// family re-converges on the new snapshot (its first round is a residual round).
int delete_edges(Ctx* c, const uint32_t* src, const uint32_t* tgt, uint64_t count, uint64_t* removed) {
  if (removed) *removed = 0;
  int rc = compact(c);
  if (rc) return rc;
  const uint64_t E = c->E;
  if (E == 0 || count == 0) return CYTOM_OK;
  const bool wt = c->wtype != CYTOM_UNWEIGHTED;
  const uint64_t nw = (E + 31) / 32;
  std::vector<Job*> mp;
  for (Job* j : c->jobs)
    if (j && !j->fresh && (j->algo == CYTOM_ALGO_BFS || j->algo == CYTOM_ALGO_CC || j->algo == CYTOM_ALGO_SSSP ||
                           j->algo == CYTOM_ALGO_SSWP))
      mp.push_back(j);
  // temporaries: kill[nw+1], cnt[nw+1], P[nw+1], total, deleted list 3 x count, ndel, tight flags
  const uint64_t words = 3 * (nw + 1) + 1 + 3 * count;
  const size_t bytes = ((words * 4 + 15) / 16) * 16 + 8 + (mp.size() + 1) * 4;
  char* tmp = nullptr;
  cudaError_t e = cy_malloc_async((void**)&tmp, bytes, c->stream);
  if (e != cudaSuccess) return set_err(c, CYTOM_ERR_OOM, "deletion temporaries");
  uint32_t* kill = (uint32_t*)tmp;
  uint32_t* cnt = kill + (nw + 1);
  uint32_t* P = cnt + (nw + 1);
  uint32_t* total = P + (nw + 1);
  uint32_t* dsrc = total + 1;
  uint32_t* dtgt = dsrc + count;
  uint32_t* dw = dtgt + count;
  unsigned long long* ndel = (unsigned long long*)(tmp + ((words * 4 + 15) / 16) * 16);
  unsigned* tight = (unsigned*)(ndel + 1);
  cudaMemsetAsync(kill, 0, (nw + 1) * 4, c->stream);
  cudaMemsetAsync(ndel, 0, 8 + (mp.size() + 1) * 4, c->stream);
  int slot = prof_begin(c, KC_MERGE);
  delete_mark_kernel<<<grid_for(c, count, 256), 256, 0, c->stream>>>(c->dsd, src, tgt, count, kill, c->out_deg,
                                                                       c->in_deg, dsrc, dtgt, wt ? dw : nullptr, ndel);
  c->launches++;
  e = cudaMemcpyAsync(c->h_pinned, ndel, 8, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) {
    cudaFreeAsync(tmp, c->stream);
    return cuda_err(c, e, "deletion");
  }
  const uint64_t nd = *(unsigned long long*)c->h_pinned;
  if (nd == 0) {
    cudaFreeAsync(tmp, c->stream);
    prof_end(c, slot, (double)count * 8.0);
    return CYTOM_OK;
  }
  keep_count_kernel<<<grid_for(c, nw + 1, 256), 256, 0, c->stream>>>(kill, E, nw, cnt);
  c->launches++;
  rc = exclusive_scan_u32(c, cnt, P, nw + 1, total);
  if (rc) return rc;
  delete_gather_kernel<<<grid_for(c, E, 256, 16), 256, 0, c->stream>>>(c->edges, c->wts, E, kill, P, c->edges_alt,
                                                                       wt ? c->wts_alt : nullptr);
  c->launches++;
  delete_tile_ptr_kernel<<<grid_for(c, c->ntiles + 1, 256), 256, 0, c->stream>>>(c->tile_ptr, c->ntiles, kill, P,
                                                                                  c->tile_ptr_alt);
  c->launches++;
  for (size_t k = 0; k < mp.size(); ++k) {
    rc = minprop_delete_check(c, mp[k], dsrc, dtgt, wt ? dw : nullptr, nd, tight + k);
    if (rc) return rc;
  }
  std::vector<unsigned> tflags(mp.size() + 1, 0);
  e = cudaMemcpyAsync(tflags.data(), tight, (mp.size() + 1) * 4, cudaMemcpyDeviceToHost, c->stream);
  cudaFreeAsync(tmp, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_err(c, e, "deletion");
  prof_end(c, slot, (double)count * 8.0 + (double)E * (wt ? 16.0 : 8.0));
  std::swap(c->edges, c->edges_alt);
  std::swap(c->wts, c->wts_alt);
  std::swap(c->tile_ptr, c->tile_ptr_alt);
  c->E = E - nd;
  c->version++;
  for (size_t k = 0; k < mp.size(); ++k)
    if (tflags[k]) mp[k]->fresh = true;
  if (removed) *removed = nd;
  const uint64_t nch = (c->E + kChunk - 1) / kChunk;
  chunk_tile_kernel<<<grid_for(c, nch + 1, 256), 256, 0, c->stream>>>(c->tile_ptr, c->ntiles, nch, c->chunk_tile);
  c->launches++;
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_err(c, e, "chunk_tile");
  return upload_store_desc(c);
}

// Random deletion picks (the reference's deletion_percentage mode,
// meta-tile-manager.h:201-231, with TileManager::deleteRandomEdge, tile-manager.h:175-190):
// pick i chooses a tile uniformly by hash64(hash64(seed) + 2i) and one of its edges
// uniformly by hash64(hash64(seed) + 2i + 1); an empty tile yields no edge (UINT32_MAX
// twice, which the deletion skips).
__global__ void pick_random_kernel(const StoreDesc* __restrict__ sd, uint64_t ntiles, uint64_t count,
                                   uint64_t hs, uint32_t* __restrict__ src, uint32_t* __restrict__ tgt) {
  const uint32_t lvpt = sd->lvpt, lT = sd->lT;
  const uint64_t tmask = (1ULL << lT) - 1ULL;
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += stride) {
    const uint64_t t = hash64(hs + 2 * i) % ntiles;
    const uint64_t lo = sd->tile_ptr[t], len = sd->tile_ptr[t + 1] - lo;
    if (len == 0) {
      src[i] = tgt[i] = 0xFFFFFFFFu;
      continue;
    }
    const uint32_t e = sd->edges[lo + hash64(hs + 2 * i + 1) % len];
    src[i] = (uint32_t)((t >> lT) << lvpt) | (e >> 16);
    tgt[i] = (uint32_t)((t & tmask) << lvpt) | (e & 0xFFFFu);
  }
}

int delete_random(Ctx* c, uint64_t count, uint64_t seed, uint32_t* src, uint32_t* tgt, uint64_t* removed) {
  if (removed) *removed = 0;
  int rc = compact(c);
  if (rc || count == 0) return rc;
  pick_random_kernel<<<grid_for(c, count, 256), 256, 0, c->stream>>>(c->dsd, c->ntiles, count, hash64(seed), src,
                                                                     tgt);
  c->launches++;
  rc = cuda_err(c, cudaGetLastError(), "random picks");
  if (rc) return rc;
  return delete_edges(c, src, tgt, count, removed);
}

// Weight update of stored edges: update i finds (src[i], tgt[i]) in its tile (binary
// search over the tile's sorted packed edges) and overwrites its weight; an edge that
// is not stored sets *missing.
__global__ void set_weights_kernel(const StoreDesc* __restrict__ sd, const uint32_t* __restrict__ src,
                                   const uint32_t* __restrict__ tgt, const uint32_t* __restrict__ w, uint64_t count,
                                   uint32_t* wts, unsigned* missing) {
  const uint32_t lvpt = sd->lvpt, lT = sd->lT;
  const uint32_t lmask = (1u << lvpt) - 1u;
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += stride) {
    const uint32_t u = src[i], v = tgt[i];
    if ((uint64_t)u >= sd->n || (uint64_t)v >= sd->n) {
      atomicOr(missing, 1u);
      continue;
    }
    const uint64_t t = ((uint64_t)(u >> lvpt) << lT) | (v >> lvpt);
    const uint32_t key = ((u & lmask) << 16) | (v & lmask);
    uint64_t lo = sd->tile_ptr[t], hi = sd->tile_ptr[t + 1];
    while (lo < hi) {
      const uint64_t mid = (lo + hi) >> 1;
      if (sd->edges[mid] < key) lo = mid + 1;
      else hi = mid;
    }
    if (lo < sd->tile_ptr[t + 1] && sd->edges[lo] == key) wts[lo] = w[i];
    else atomicOr(missing, 1u);
  }
}

int set_edge_weights(Ctx* c, const uint32_t* src, const uint32_t* tgt, const uint32_t* w, uint64_t count) {
  int rc = compact(c);
  if (rc) return rc;
  cudaMemsetAsync(c->d_flag, 0, 4, c->stream);
  if (count) {
    set_weights_kernel<<<grid_for(c, count, 256), 256, 0, c->stream>>>(c->dsd, src, tgt, w, count, c->wts,
                                                                          c->d_flag);
    c->launches++;
  }
  unsigned missing = 0;
  cudaError_t e = cudaMemcpyAsync(&missing, c->d_flag, 4, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_err(c, e, "weight update");
  // every weight-dependent structure is rebuilt; SSSP and SSWP jobs restart (a changed
  // weight can worsen a path, which min- or max-propagation cannot undo)
  c->version++;
  rc = upload_store_desc(c);
  if (rc) return rc;
  for (Job* j : c->jobs)
    if (j && (j->algo == CYTOM_ALGO_SSSP || j->algo == CYTOM_ALGO_SSWP)) j->fresh = true;
  if (missing) return set_err(c, CYTOM_ERR_RANGE, "weight update of an edge that is not stored");
  return CYTOM_OK;
}

}  // namespace cytom
