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

#include "engine.h"

namespace cytom {

constexpr int GATHER_T = 256;
constexpr int APPLY_T = 256;

__device__ __forceinline__ unsigned long long row_edges(const StoreDesc* sd, uint64_t x) {
  return sd->tile_ptr[(x + 1) << sd->lT] - sd->tile_ptr[x << sd->lT];
}

// Clears both parities of the row flags and the loop counters before a run.
__global__ void begin_kernel(const JobDesc* __restrict__ jd, const StoreDesc* __restrict__ sd,
                             unsigned max_iter) {
  LoopState* ls = jd->ls;
  const uint64_t T = sd->T;
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < 2 * T; i += stride)
    jd->rows[i] = 0;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    ls->iter = 0;
    ls->max_iter = max_iter;
    ls->cont = 1;
    ls->err = 0;
    ls->active[0] = ls->active[1] = 0;
    ls->teps[0] = ls->teps[1] = 0;
    ls->count_edges = 0;
    ls->edges_scanned = 0;
    ls->active_total = 0;
  }
}

// Apply: `initial` = the seeding apply before round 0 (writes parity 0).
__global__ void __launch_bounds__(APPLY_T) apply_minprop_kernel(const JobDesc* __restrict__ jd,
                                                                const StoreDesc* __restrict__ sd,
                                                                int initial) {
  LoopState* ls = jd->ls;
  if (!ls->cont) return;
  const unsigned pw = initial ? 0u : ((ls->iter & 1u) ^ 1u);
  const uint64_t n = sd->n, T = sd->T;
  const uint32_t lvpt = sd->lvpt;
  const uint64_t nwords = (n + 31) >> 5;
  unsigned* rows_w = jd->rows + pw * T;
  uint32_t* __restrict__ ch = jd->ch;
  uint32_t* __restrict__ fa = jd->fa;
  uint32_t* __restrict__ cur = jd->cur;
  const uint32_t* __restrict__ next = jd->next;
  unsigned cnt = 0;
  unsigned long long teps = 0;
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nwords; i += stride) {
    uint32_t w = ch[i];
    fa[i] = w;
    if (w == 0) continue;
    ch[i] = 0;
    cnt += __popc(w);
    uint32_t bits = w;
    while (bits) {
      int b = __ffs(bits) - 1;
      bits &= bits - 1;
      uint64_t v = (i << 5) + b;
      cur[v] = next[v];
      if (lvpt < 5 || b == __ffs(w) - 1) {
        uint64_t x = v >> lvpt;
        if (rows_w[x] == 0 && atomicExch(&rows_w[x], 1u) == 0) teps += row_edges(sd, x);
      }
    }
  }
  // block reduction
  __shared__ unsigned s_cnt[APPLY_T / 32];
  __shared__ unsigned long long s_teps[APPLY_T / 32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    cnt += __shfl_xor_sync(0xFFFFFFFFu, cnt, o);
    teps += __shfl_xor_sync(0xFFFFFFFFu, teps, o);
  }
  const unsigned lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) {
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
}

__global__ void control_kernel(const JobDesc* __restrict__ jd, cudaGraphConditionalHandle h,
                               int initial, int use_handle) {
  LoopState* ls = jd->ls;
  if (ls->cont) {
    unsigned p;
    if (initial) {
      p = 0;
    } else {
      ls->iter += 1;
      p = ls->iter & 1u;
    }
    unsigned a = ls->active[p];
    ls->active_total += a;
    ls->cont = (a > 0 && ls->iter < ls->max_iter) ? 1u : 0u;
  }
  if (use_handle) cudaGraphSetConditional(h, ls->cont);
}

// Gather for BFS (ALGO 0), CC (1), SSSP (2). A warp owns a 128-edge chunk: lane l
// loads edges [4l, 4l+4) of it with one 128-bit load. The tile of an edge is found
// from the chunk's first tile and tile_ptr (edges are tile-major).
template <int ALGO>
__global__ void __launch_bounds__(GATHER_T) gather_minprop_kernel(const JobDesc* __restrict__ jd,
                                                                  const StoreDesc* __restrict__ sd,
                                                                  int adaptive) {
  LoopState* ls = jd->ls;
  if (!ls->cont) return;
  const unsigned p = ls->iter & 1u;
  const uint64_t T = sd->T;
  const unsigned* __restrict__ rows_cur = jd->rows + p * T;
  unsigned* rows_nxt = jd->rows + (p ^ 1u) * T;
  {
    uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < T; i += stride)
      rows_nxt[i] = 0;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      ls->active[p ^ 1u] = 0;
      ls->teps[p ^ 1u] = 0;
      ls->count_edges += adaptive ? ls->teps[p] : sd->E;
    }
  }
  const uint32_t* __restrict__ edges = sd->edges;
  const uint32_t* __restrict__ wts = sd->wts;
  const unsigned long long* __restrict__ tile_ptr = sd->tile_ptr;
  const uint32_t* __restrict__ chunk_tile = sd->chunk_tile;
  const uint32_t* __restrict__ fa = jd->fa;
  const uint32_t* __restrict__ cur = jd->cur;
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
    if (ALGO == 2) wv = *reinterpret_cast<const uint4*>(wts + e0);
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
      const uint32_t uv = cur[u];
      if (uv == kInf) continue;
      uint32_t cand;
      if (ALGO == 0) {
        cand = uv + 1;
      } else if (ALGO == 1) {
        cand = uv;
      } else {
        unsigned long long s = (unsigned long long)uv + wvk[k];
        if (s >= kInf) continue;
        cand = (uint32_t)s;
      }
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
    uint32_t cand;
    if (ALGO == 0) cand = uv + 1;
    else if (ALGO == 1) cand = uv;
    else {
      unsigned long long s = (unsigned long long)uv + (w ? w[i] : 1u);
      if (s >= kInf) continue;
      cand = (uint32_t)s;
    }
    if (cand < __ldcg(next + v)) {
      uint32_t old = atomicMin(next + v, cand);
      if (cand < old) atomicOr(ch + (v >> 5), 1u << (v & 31));
    }
  }
}

static int grid_persistent(Ctx* c, int per_sm) { return c->num_sms * per_sm; }

static bool is_minprop(int algo) {
  return algo == CYTOM_ALGO_BFS || algo == CYTOM_ALGO_CC || algo == CYTOM_ALGO_SSSP;
}

int minprop_alloc(Ctx* c, Job* j) {
  const uint64_t n = c->n;
  const uint64_t nwords = (n + 31) / 32;
  JobDesc& h = j->h;
  cudaError_t e = cudaMalloc(&h.cur, n * 4);
  if (e == cudaSuccess) e = cudaMalloc(&h.next, n * 4);
  if (e == cudaSuccess) e = cudaMalloc(&h.fa, nwords * 4);
  if (e == cudaSuccess) e = cudaMalloc(&h.ch, nwords * 4);
  if (e == cudaSuccess) e = cudaMalloc(&h.rows, 2 * c->T * 4);
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
    default: seed_minprop_kernel<2><<<g, 256, 0, c->stream>>>(j->d, src, tgt, w, count); break;
  }
  c->launches++;
  prof_end(c, slot, (double)count * 16.0);
  return cuda_err(c, cudaGetLastError(), "seed_minprop");
}

static void* gather_fn(int algo) {
  switch (algo) {
    case CYTOM_ALGO_BFS: return (void*)gather_minprop_kernel<0>;
    case CYTOM_ALGO_CC: return (void*)gather_minprop_kernel<1>;
    default: return (void*)gather_minprop_kernel<2>;
  }
}

static int launch_gather(Ctx* c, Job* j, int adaptive) {
  int g = grid_persistent(c, 8);
  switch (j->algo) {
    case CYTOM_ALGO_BFS: gather_minprop_kernel<0><<<g, GATHER_T, 0, c->stream>>>(j->d, c->dsd, adaptive); break;
    case CYTOM_ALGO_CC: gather_minprop_kernel<1><<<g, GATHER_T, 0, c->stream>>>(j->d, c->dsd, adaptive); break;
    default: gather_minprop_kernel<2><<<g, GATHER_T, 0, c->stream>>>(j->d, c->dsd, adaptive); break;
  }
  c->launches++;
  return cuda_err(c, cudaGetLastError(), "gather");
}

static cudaError_t add_kernel(cudaGraph_t g, cudaGraphNode_t* node, const cudaGraphNode_t* deps,
                              size_t ndeps, void* fn, dim3 grid, dim3 block, void** args) {
  cudaKernelNodeParams kp{};
  kp.func = fn;
  kp.gridDim = grid;
  kp.blockDim = block;
  kp.sharedMemBytes = 0;
  kp.kernelParams = args;
  kp.extra = nullptr;
  return cudaGraphAddKernelNode(node, g, deps, ndeps, &kp);
}

// Graph: begin -> seeding apply -> control(initial) -> while(cond) { gather -> apply -> control }.
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
  int gper = grid_persistent(c, 8);
  cudaGraphNode_t n_begin, n_apply0, n_ctl0, n_while, b_gather, b_apply, b_ctl;
  void* a_begin[] = {(void*)&jd, (void*)&sd, (void*)&max_iter};
  if (e == cudaSuccess)
    e = add_kernel(g, &n_begin, nullptr, 0, (void*)begin_kernel, dim3(std::max(1, c->num_sms)), dim3(256), a_begin);
  void* a_apply0[] = {(void*)&jd, (void*)&sd, (void*)&one};
  if (e == cudaSuccess)
    e = add_kernel(g, &n_apply0, &n_begin, 1, (void*)apply_minprop_kernel, dim3(gper), dim3(APPLY_T), a_apply0);
  void* a_ctl0[] = {(void*)&jd, (void*)&h, (void*)&one, (void*)&one};
  if (e == cudaSuccess)
    e = add_kernel(g, &n_ctl0, &n_apply0, 1, (void*)control_kernel, dim3(1), dim3(1), a_ctl0);
  cudaGraphNodeParams cp{};
  cp.type = cudaGraphNodeTypeConditional;
  cp.conditional.handle = h;
  cp.conditional.type = cudaGraphCondTypeWhile;
  cp.conditional.size = 1;
  if (e == cudaSuccess) e = cudaGraphAddNode(&n_while, g, &n_ctl0, nullptr, 1, &cp);
  if (e == cudaSuccess) {
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    void* a_g[] = {(void*)&jd, (void*)&sd, (void*)&adaptive};
    e = add_kernel(body, &b_gather, nullptr, 0, gather_fn(j->algo), dim3(gper), dim3(GATHER_T), a_g);
    void* a_a[] = {(void*)&jd, (void*)&sd, (void*)&zero};
    if (e == cudaSuccess)
      e = add_kernel(body, &b_apply, &b_gather, 1, (void*)apply_minprop_kernel, dim3(gper), dim3(APPLY_T), a_a);
    void* a_c[] = {(void*)&jd, (void*)&h, (void*)&zero, (void*)&one};
    if (e == cudaSuccess)
      e = add_kernel(body, &b_ctl, &b_apply, 1, (void*)control_kernel, dim3(1), dim3(1), a_c);
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

int minprop_run(Ctx* c, Job* j) {
  int adaptive = c->cfg.enable_adaptive_scheduling;
  unsigned max_iter = (unsigned)std::min<uint64_t>(j->params.max_iterations, 0xFFFFFFFFu);
  if (!c->profiling && use_graphs() && !j->graph_failed) {
    if (!j->loop_exec) build_minprop_graph(c, j);
    if (j->loop_exec) {
      j->last_run_graph = true;
      cudaError_t e = cudaGraphLaunch(j->loop_exec, c->stream);
      c->launches += 3;  // per-round launches are counted from the loop state afterwards
      if (e != cudaSuccess) return cuda_err(c, e, "graph launch");
      return CYTOM_OK;
    }
  }
  // host-driven loop (profiling mode or no graph support)
  j->last_run_graph = false;
  int gper = grid_persistent(c, 8);
  begin_kernel<<<std::max(1, c->num_sms), 256, 0, c->stream>>>(j->d, c->dsd, max_iter);
  apply_minprop_kernel<<<gper, APPLY_T, 0, c->stream>>>(j->d, c->dsd, 1);
  control_kernel<<<1, 1, 0, c->stream>>>(j->d, 0, 1, 0);
  c->launches += 3;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_err(c, e, "run prologue");
  for (uint64_t round = 0; round < max_iter;) {
    // launch a few rounds before checking: kernels are no-ops once the run ended
    int batch = 4;
    for (int k = 0; k < batch && round < max_iter; ++k, ++round) {
      int s1 = prof_begin(c, KC_GATHER);
      int rc = launch_gather(c, j, adaptive);
      if (rc) return rc;
      prof_end(c, s1, -1.0);
      int s2 = prof_begin(c, KC_APPLY);
      apply_minprop_kernel<<<gper, APPLY_T, 0, c->stream>>>(j->d, c->dsd, 0);
      prof_end(c, s2, -1.0);
      control_kernel<<<1, 1, 0, c->stream>>>(j->d, 0, 0, 0);
      c->launches += 2;
    }
    e = cudaMemcpyAsync(c->h_pinned, &j->ls->cont, 4, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_err(c, e, "run loop");
    if (*(unsigned*)c->h_pinned == 0) break;
  }
  return CYTOM_OK;
}

}  // namespace cytom
