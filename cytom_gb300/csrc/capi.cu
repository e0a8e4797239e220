// capi.cu — the C ABI (include/cytom_gpu.h): contexts, buffers, jobs, statistics.
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <new>
#include <string>
#include <vector>

#include "engine.h"

namespace cytom {

int minprop_alloc(Ctx* c, Job* j);
int minprop_init(Ctx* c, Job* j);
int minprop_seed(Ctx* c, Job* j, const uint32_t* src, const uint32_t* tgt, const uint32_t* w,
                 uint64_t count);
int minprop_run(Ctx* c, Job* j);
int pagerank_alloc(Ctx* c, Job* j);
int pagerank_init(Ctx* c, Job* j);
int pagerank_seed(Ctx* c, Job* j, const uint32_t* src, const uint32_t* tgt, const uint32_t* w,
                  uint64_t count);
int pagerank_run(Ctx* c, Job* j);
int pagerank_result(Ctx* c, Job* j, void* out, int where);
int pagerank_result64(Ctx* c, Job* j, double* out, int where);
int pagerank_set_teleport(Ctx* c, Job* j, const double* t, int where);
int pagerank_adjoint(Ctx* c, Job* j, const double* cv, int cwhere, float* d_w, float* d_t, int owhere,
                     cytom_run_stats* st);
int set_edge_weights(Ctx* c, const uint32_t* src, const uint32_t* tgt, const uint32_t* w, uint64_t count);
int delete_edges(Ctx* c, const uint32_t* src, const uint32_t* tgt, uint64_t count, uint64_t* removed);
int delete_random(Ctx* c, uint64_t count, uint64_t seed, uint32_t* src, uint32_t* tgt, uint64_t* removed);
void pagerank_free(Job* j);

__global__ void complement_kernel(const uint32_t* __restrict__ in, uint64_t n, uint32_t* __restrict__ out) {
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) out[i] = ~in[i];
}

// Fault injection: the allocation that turns the countdown from 1 to 0 fails.
static std::atomic<uint64_t> g_alloc_countdown{0};

bool alloc_fault_fires() {
  uint64_t v = g_alloc_countdown.load(std::memory_order_relaxed);
  while (v != 0) {
    if (g_alloc_countdown.compare_exchange_weak(v, v - 1, std::memory_order_relaxed)) return v == 1;
  }
  return false;
}

int set_err(Ctx* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  return code;
}

int cuda_err(Ctx* c, cudaError_t e, const char* what) {
  if (e == cudaSuccess) return CYTOM_OK;
  if (c) c->err = std::string(what) + ": " + cudaGetErrorString(e);
  if (e == cudaErrorMemoryAllocation) return CYTOM_ERR_OOM;
  return CYTOM_ERR_CUDA;
}

// ---- profiling: CUDA events around launches --------------------------------
static const char* kClassNames[CYTOM_KERNEL_CLASSES] = {"rmat", "insert", "sort", "merge",
                                                        "gather", "apply", "pagerank", "gather_sparse"};

int prof_begin(Ctx* c, int cls) {
  if (!c->profiling) return -1;
  cudaEvent_t a, b;
  if (c->ev_pool.size() >= 2) {
    a = c->ev_pool.back();
    c->ev_pool.pop_back();
    b = c->ev_pool.back();
    c->ev_pool.pop_back();
  } else {
    cudaEventCreate(&a);
    cudaEventCreate(&b);
  }
  cudaEventRecord(a, c->stream);
  c->pending.push_back({cls, a, b, 0.0});
  return (int)c->pending.size() - 1;
}

void prof_end(Ctx* c, int slot, double bytes) {
  if (slot < 0 || !c->profiling) return;
  cudaEventRecord(c->pending[slot].b, c->stream);
  c->pending[slot].bytes = bytes;
}

int prof_flush(Ctx* c) {
  if (c->pending.empty()) return CYTOM_OK;
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_err(c, e, "profiling sync");
  for (auto& p : c->pending) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, p.a, p.b);
    c->kstats.launches[p.cls] += 1;
    c->kstats.total_ms[p.cls] += ms;
    if (p.bytes > 0) c->kstats.algo_bytes[p.cls] += p.bytes;
    c->ev_pool.push_back(p.a);
    c->ev_pool.push_back(p.b);
  }
  c->pending.clear();
  return CYTOM_OK;
}

int upload_store_desc(Ctx* c) {
  StoreDesc& h = c->hsd;
  h.edges = c->edges;
  h.wts = c->wts;
  h.tile_ptr = c->tile_ptr;
  h.chunk_tile = c->chunk_tile;
  h.out_deg = c->out_deg;
  h.in_deg = c->in_deg;
  h.E = c->E;
  h.nchunks = (c->E + kChunk - 1) / kChunk;
  h.n = c->n;
  h.T = c->T;
  h.ntiles = c->ntiles;
  h.lvpt = c->lvpt;
  h.lT = c->lT;
  h.wtype = c->wtype;
  h.adaptive = c->cfg.enable_adaptive_scheduling;
  h.dir = c->dir;
  h.nbw = c->lvpt >= 5 ? (uint32_t)(c->vpt / 32) : 0u;
  h.dir_ok = (c->dir && c->dir_version == c->version && !c->dir_disabled) ? 1 : 0;
  h.cmask = h.dir_ok ? c->cmask : nullptr;
  h.cshift = c->lT > 6 ? c->lT - 6 : 0u;
  h.traversal = (uint32_t)c->cfg.traversal;
  h.xst = c->xs_stage;
  h.xcum = c->xs_cum;
  h.xcolcum = c->xs_colcum;
  h.xnst = c->xs_tmp ? c->xs_tmp + 2 * (c->ntiles + 1) : nullptr;
  {
    static int div = -1;
    if (div < 0) {
      const char* ev = getenv("CYTOM_SPARSE_DIV");
      div = (ev && atoi(ev) > 0) ? atoi(ev) : 8;
    }
    h.sparse_div = (uint32_t)div;
  }
  // pageable source: the copy is staged before the call returns, so h may change later
  cudaError_t e = cudaMemcpyAsync(c->dsd, &h, sizeof(StoreDesc), cudaMemcpyHostToDevice, c->stream);
  return cuda_err(c, e, "store descriptor upload");
}

static uint32_t ilog2(uint64_t v) {
  uint32_t r = 0;
  while ((1ULL << r) < v) ++r;
  return r;
}

// ---- jobs -----------------------------------------------------------------
static bool is_minprop(int a) {
  return a == CYTOM_ALGO_BFS || a == CYTOM_ALGO_CC || a == CYTOM_ALGO_SSSP || a == CYTOM_ALGO_SSWP;
}

int job_alloc(Ctx* c, Job* j) {
  cudaError_t e = cy_malloc(&j->ls, sizeof(LoopState));
  if (e != cudaSuccess) return set_err(c, CYTOM_ERR_OOM, "loop state");
  cudaMemsetAsync(j->ls, 0, sizeof(LoopState), c->stream);
  j->h.ls = j->ls;
  j->h.algo = j->algo;
  j->h.kahan = j->params.kahan;
  j->h.async = j->async ? 1 : 0;
  j->h.alpha = j->params.alpha;
  j->h.delta_param = j->params.delta;
  j->h.start = j->params.start_vertex;
  int rc = is_minprop(j->algo) ? minprop_alloc(c, j) : pagerank_alloc(c, j);
  if (rc) return rc;
  e = cy_malloc(&j->d, sizeof(JobDesc));
  if (e != cudaSuccess) return set_err(c, CYTOM_ERR_OOM, "job descriptor");
  e = cudaMemcpyAsync(j->d, &j->h, sizeof(JobDesc), cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  return cuda_err(c, e, "job descriptor upload");
}

void job_free(Ctx* c, Job* j) {
  (void)c;
  if (j->loop_exec) cudaGraphExecDestroy(j->loop_exec);
  if (j->ext) pagerank_free(j);
  void* ptrs[] = {j->h.spq, j->h.aw, j->h.awm, j->h.cur, j->h.next, j->h.fa, j->h.ch, j->h.rows, j->h.rank, j->h.rank_c,
                  j->h.delta, j->h.dsum, j->h.contrib, j->h.rank64, j->h.dsum64, j->h.deg_distinct,
                  j->ls, j->d};
  for (void* p : ptrs)
    if (p) cudaFree(p);
}

// Chunk queue of a job's sparse rounds: queued items are longer than 32 edges (at most
// E / 32 of them) and give one chunk per 256 edges, so E / 32 + E / 256 entries always
// fit. Without a queue (allocation failed) heavy items are walked as light ones.
int ensure_job_queue(Ctx* c, Job* j) {
  const uint64_t need = c->E / 32 + c->E / 256 + 1024;
  if (need <= j->h.spq_cap) return CYTOM_OK;
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_err(c, e, "queue resize");
  if (j->h.spq) cudaFree(j->h.spq);
  j->h.spq = nullptr;
  j->h.spq_cap = 0;
  const uint64_t cap = need + need / 2;
  if (cy_malloc(&j->h.spq, cap * sizeof(uint2)) == cudaSuccess) {
    j->h.spq_cap = cap;
  } else {
    cudaGetLastError();
    j->h.spq = nullptr;
  }
  // pageable source: the copy is staged before the call returns
  e = cudaMemcpyAsync(j->d, &j->h, sizeof(JobDesc), cudaMemcpyHostToDevice, c->stream);
  return cuda_err(c, e, "job descriptor upload");
}

int job_init_state(Ctx* c, Job* j) {
  return is_minprop(j->algo) ? minprop_init(c, j) : pagerank_init(c, j);
}

int job_seed(Ctx* c, Job* j, const uint32_t* src, const uint32_t* tgt, const uint32_t* w,
             uint64_t count) {
  return is_minprop(j->algo) ? minprop_seed(c, j, src, tgt, w, count)
                             : pagerank_seed(c, j, src, tgt, w, count);
}

// edgeChanged(INSERT) for the edges merged by a compaction, PageRank family (the
// min-propagation jobs are seeded together by minprop_seed_keys_many).
int job_seed_keys(Ctx* c, Job* j, const uint64_t* K, const uint32_t* W, uint64_t count) {
  (void)K;
  (void)W;
  return pagerank_seed(c, j, nullptr, nullptr, nullptr, count);
}

// The streaming gather is tuned once per context, on the first run at >= 2^20 edges
// (cytom_autotune re-tunes on demand; CYTOM_AUTOTUNE=0 keeps the default shapes).
static bool autotune_due(Ctx* c) {
  static int env = -1;
  if (env < 0) {
    const char* s = getenv("CYTOM_AUTOTUNE");
    env = (s && s[0] == '0') ? 0 : 1;
  }
  return env && !c->profiling && c->tune_E == 0 && c->E >= (1ULL << 20);
}

// Everything a run needs before its loop: pending edges merged, the source directory,
// the job's sparse queue, the one-time shape tuning, and the initial state of a fresh job.
static int job_prepare(Ctx* c, Job* j) {
  int rc = compact(c);
  if (rc) return rc;
  if (is_minprop(j->algo)) {
    rc = build_directory(c);
    if (!rc) rc = ensure_job_queue(c, j);
    if (!rc && autotune_due(c)) rc = minprop_autotune(c);
    if (!rc && tiles_in_use(c, j->algo)) rc = build_tile_stages(c);
    if (rc) return rc;
    // the tuned sparse-round threshold of the job's class, read by its control step
    const uint32_t div = c->tune_div[(j->algo == CYTOM_ALGO_SSSP || j->algo == CYTOM_ALGO_SSWP) ? 1 : 0];
    if (div != j->h.sparse_div) {
      j->h.sparse_div = div;
      cudaError_t e = cudaMemcpyAsync(j->d, &j->h, sizeof(JobDesc), cudaMemcpyHostToDevice, c->stream);
      if (e != cudaSuccess) return cuda_err(c, e, "job descriptor upload");
    }
  }
  if (j->fresh) {
    rc = job_init_state(c, j);
    if (rc) return rc;
    j->fresh = false;
  }
  return CYTOM_OK;
}

// Statistics of a finished run from its loop state; ev_a / ev_b bracket its launches.
static int job_finish(Ctx* c, Job* j, const LoopState& ls, cudaEvent_t ev_a, cudaEvent_t ev_b,
                      cytom_run_stats* st) {
  if (ls.err) return set_err(c, CYTOM_ERR_TIMEOUT, "a bounded device wait gave up");
  if (j->last_run_graph) c->launches += 4ULL * ls.iter;  // per round: two gathers, chunk pass, apply
  if (st) {
    memset(st, 0, sizeof(*st));
    st->iterations = ls.iter;
    st->count_edges = ls.count_edges;
    st->edges_scanned = ls.edges_scanned;
    st->active_vertices = ls.active_total;
    st->converged = (ls.cont == 0 && ls.iter < ls.max_iter) ? 1 : (ls.cont == 0 ? 1 : 0);
    st->residual = ls.resid_final;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ev_a, ev_b);
    st->elapsed_ms = ms;
  }
  return CYTOM_OK;
}

int job_run(Ctx* c, Job* j, cytom_run_stats* st) {
  int rc = job_prepare(c, j);
  if (rc) return rc;
  cudaEventRecord(c->run_a, c->stream);
  rc = is_minprop(j->algo) ? minprop_run(c, j) : pagerank_run(c, j);
  if (rc) return rc;
  cudaEventRecord(c->run_b, c->stream);
  LoopState ls;
  cudaError_t e = cudaMemcpyAsync(&ls, j->ls, sizeof(LoopState), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_err(c, e, "run");
  rc = prof_flush(c);
  if (rc) return rc;
  return job_finish(c, j, ls, c->run_a, c->run_b, st);
}

void join_runs(Ctx* c) {
  if (!c->runs_unjoined) return;
  for (size_t k = 0; k < c->async_jobs.size(); ++k) cudaStreamWaitEvent(c->stream, c->conc[k].done, 0);
  c->runs_unjoined = false;
}

// Several jobs of one context: BFS / CC / SSSP / SSWP jobs are independent once the
// snapshot is prepared, as the reference's jobs are (one thread per job), so after a
// shared preparation each job's captured loop is launched on its own stream and they
// overlap (the small, latency-bound rounds of one job fill the GPU around another's).
// The caller's stream waits for all of them. Other jobs, and profiling runs, run in turn.
static int collect_runs(Ctx* c, cytom_run_stats* stats);

void settle_runs(Ctx* c) {
  if (!c->async_jobs.empty()) collect_runs(c, nullptr);
  c->sync_jobs.clear();
  c->sync_stats.clear();
}

// Launches the jobs' loops on their streams after the shared preparation; the context's
// stream is not made to wait for them (join_runs does that).
static int launch_many(Ctx* c, Job** jobs, int count) {
  for (int k = 0; k < count; ++k) {
    int rc = job_prepare(c, jobs[k]);
    if (rc) return rc;
  }
  while ((int)c->conc.size() < count) {
    ConcSlot slot{};
    cudaError_t e = cudaStreamCreateWithFlags(&slot.stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&slot.a);
    if (e == cudaSuccess) e = cudaEventCreate(&slot.b);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&slot.done, cudaEventDisableTiming);
    if (e != cudaSuccess) return cuda_err(c, e, "job streams");
    c->conc.push_back(slot);
  }
  if (!c->fork_ev && cudaEventCreateWithFlags(&c->fork_ev, cudaEventDisableTiming) != cudaSuccess)
    return set_err(c, CYTOM_ERR_CUDA, "fork event");
  cudaEventRecord(c->fork_ev, c->stream);
  cudaStream_t home = c->stream;
  int rc = CYTOM_OK;
  c->async_jobs.clear();
  for (int k = 0; k < count && !rc; ++k) {
    ConcSlot& sl = c->conc[k];
    cudaStreamWaitEvent(sl.stream, c->fork_ev, 0);
    cudaEventRecord(sl.a, sl.stream);
    c->stream = sl.stream;  // the job's launches go to its own stream
    rc = minprop_run(c, jobs[k]);
    c->stream = home;
    cudaEventRecord(sl.b, sl.stream);
    cudaEventRecord(sl.done, sl.stream);
    c->async_jobs.push_back(jobs[k]);
  }
  c->runs_unjoined = true;
  if (rc) {
    join_runs(c);
    cudaStreamSynchronize(home);
    c->async_jobs.clear();
  }
  return rc;
}

// Joins the last asynchronous launch and returns its statistics (stats: one entry per
// job of that launch, or NULL).
static int collect_runs(Ctx* c, cytom_run_stats* stats) {
  join_runs(c);
  const int count = (int)c->async_jobs.size();
  std::vector<LoopState> ls(count);
  cudaError_t e = cudaSuccess;
  for (int k = 0; k < count && e == cudaSuccess; ++k)
    e = cudaMemcpyAsync(&ls[k], c->async_jobs[k]->ls, sizeof(LoopState), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_err(c, e, "run");
  int rc = CYTOM_OK;
  for (int k = 0; k < count && !rc; ++k)
    rc = job_finish(c, c->async_jobs[k], ls[k], c->conc[k].a, c->conc[k].b, stats ? stats + k : nullptr);
  c->async_jobs.clear();
  return rc;
}

static bool runs_concurrently(const Ctx* c, Job** jobs, int count) {
  bool conc = count > 1 && !c->profiling;
  for (int k = 0; k < count && conc; ++k) conc = is_minprop(jobs[k]->algo);
  return conc;
}

int job_run_many(Ctx* c, Job** jobs, int count, cytom_run_stats* stats) {
  if (!runs_concurrently(c, jobs, count)) {
    for (int k = 0; k < count; ++k) {
      int rc = job_run(c, jobs[k], stats ? stats + k : nullptr);
      if (rc) return rc;
    }
    return CYTOM_OK;
  }
  int rc = launch_many(c, jobs, count);
  if (rc) return rc;
  return collect_runs(c, stats);
}

}  // namespace cytom

using namespace cytom;

extern "C" {

void cytom_config_default(cytom_config* cfg) {
  if (!cfg) return;
  memset(cfg, 0, sizeof(*cfg));
  cfg->max_vertices = 1ULL << 16;
  cfg->vertices_per_tile = 65536;  // VERTICES_PER_TILE, src/scripts/config.py:91
  cfg->weight_type = CYTOM_UNWEIGHTED;
  cfg->enable_adaptive_scheduling = 1;
  cfg->edge_capacity_hint = 0;
  cfg->stream = nullptr;
  cfg->traversal = CYTOM_TRAVERSAL_ROW_FIRST;  // TRAVERSAL, src/scripts/config.py:62
}

void cytom_rmat_default(cytom_rmat_params* p) {
  if (!p) return;
  memset(p, 0, sizeof(*p));
  p->scale = 16;
  p->a = (double)0.57f;  // RMAT_A, src/include/util/datatypes.h:17
  p->b = (double)0.19f;
  p->c = (double)0.19f;
  p->seed = 2;  // RMAT_SEED, datatypes.h:20
  p->weight_seed = 0;
  p->wmin = 1;
  p->wmax = 0;
}

void cytom_job_params_default(cytom_job_params* p) {
  if (!p) return;
  memset(p, 0, sizeof(*p));
  p->start_vertex = 1;  // DEFAULT_ALGORITHM_START_VERTEX, src/scripts/config.py:107
  p->max_iterations = 100;  // MAX_ITERATIONS, config.py:46
  p->delta = 0.01;  // DEFAULT_DELTA, config.py:105
  p->alpha = 0.85;  // ALPHA, examples/pagerank-delta.cc:19
  p->tolerance = 0.0;
  p->kahan = 1;
}

int cytom_create(const cytom_config* cfg, cytom_ctx** out) {
  if (!cfg || !out) return CYTOM_ERR_INVAL;
  *out = nullptr;
  Ctx* c = new (std::nothrow) Ctx();
  if (!c) return CYTOM_ERR_OOM;
  c->cfg = *cfg;
  uint64_t n = 1;
  while (n < cfg->max_vertices) n <<= 1;  // Config::normalizeConfig rounds up to 2^k
  uint64_t vpt = cfg->vertices_per_tile;
  if (cfg->max_vertices == 0 || vpt == 0 || (vpt & (vpt - 1)) || vpt > 65536 || vpt > n ||
      n > (1ULL << 32) || (cfg->weight_type < 0 || cfg->weight_type > 2) || cfg->traversal < 0 ||
      cfg->traversal > CYTOM_TRAVERSAL_HILBERT) {
    delete c;
    return CYTOM_ERR_INVAL;  // the reference gets 0 tiles when vpt > vertices (config.cc:18-19)
  }
  c->n = n;
  c->vpt = vpt;
  c->T = n / vpt;
  c->ntiles = c->T * c->T;
  c->lvpt = ilog2(vpt);
  c->lT = ilog2(c->T);
  c->wtype = cfg->weight_type;
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0) {
    delete c;
    return CYTOM_ERR_CUDA;
  }
  cudaGetDevice(&c->device);
  cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, c->device);
  if (cfg->stream) {
    c->stream = (cudaStream_t)cfg->stream;
  } else {
    e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    c->own_stream = true;
  }
  // keep stream-ordered temporaries cached in the pool
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, c->device) == cudaSuccess) {
    uint64_t thr = UINT64_MAX;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
  }
  bool ok = e == cudaSuccess;
  ok = ok && cy_malloc(&c->out_deg, n * 4) == cudaSuccess;
  ok = ok && cy_malloc(&c->in_deg, n * 4) == cudaSuccess;
  ok = ok && cy_malloc(&c->tile_ptr, (c->ntiles + 1) * 8) == cudaSuccess;
  ok = ok && cy_malloc(&c->tile_ptr_alt, (c->ntiles + 1) * 8) == cudaSuccess;
  ok = ok && cy_malloc(&c->dsd, sizeof(StoreDesc)) == cudaSuccess;
  ok = ok && cy_malloc(&c->d_flag, 64) == cudaSuccess;
  ok = ok && cy_malloc_host(&c->h_pinned, 64) == cudaSuccess;
  ok = ok && cudaEventCreate(&c->run_a) == cudaSuccess;
  ok = ok && cudaEventCreate(&c->run_b) == cudaSuccess;
  if (!ok) {
    cudaGetLastError();
    cytom_destroy((cytom_ctx*)c);
    return CYTOM_ERR_OOM;
  }
  cudaMemsetAsync(c->out_deg, 0, n * 4, c->stream);
  cudaMemsetAsync(c->in_deg, 0, n * 4, c->stream);
  cudaMemsetAsync(c->tile_ptr, 0, (c->ntiles + 1) * 8, c->stream);
  cudaMemsetAsync(c->tile_ptr_alt, 0, (c->ntiles + 1) * 8, c->stream);
  for (int k = 0; k < CYTOM_KERNEL_CLASSES; ++k)
    snprintf(c->kstats.name[k], sizeof(c->kstats.name[k]), "%s", kClassNames[k]);
  int rc = CYTOM_OK;
  uint64_t hint = std::max<uint64_t>(cfg->edge_capacity_hint, 1024);
  (void)hint;
  // the store starts empty with a small capacity; chunk table for zero edges
  c->cap = 0;
  c->chunk_cap = 0;
  {
    uint32_t* ct = nullptr;
    if (cy_malloc(&ct, 2 * 4) != cudaSuccess) rc = CYTOM_ERR_OOM;
    c->chunk_tile = ct;
    c->chunk_cap = 2;
    if (ct) cudaMemsetAsync(ct, 0, 8, c->stream);
  }
  if (!rc) rc = upload_store_desc(c);
  if (!rc && cudaStreamSynchronize(c->stream) != cudaSuccess) rc = CYTOM_ERR_CUDA;
  if (rc) {
    cytom_destroy((cytom_ctx*)c);
    return rc;
  }
  *out = (cytom_ctx*)c;
  return CYTOM_OK;
}

int cytom_destroy(cytom_ctx* ctx) {
  Ctx* c = (Ctx*)ctx;
  if (c) join_runs(c);
  if (!c) return CYTOM_ERR_INVAL;
  if (c->stream) cudaStreamSynchronize(c->stream);
  for (Job* j : c->jobs)
    if (j) {
      job_free(c, j);
      delete j;
    }
  batch_free(c);
  pagerank_ctx_free(c);
  edge_log_close(c);
  void* ptrs[] = {c->dir, c->dir_alt, c->cmask, c->edges, c->wts, c->edges_alt, c->wts_alt, c->tile_ptr, c->tile_ptr_alt,
                  c->chunk_tile, c->chunk_tile_alt, c->app_keys, c->app_keys_alt, c->app_w, c->app_w_alt,
                  c->out_deg, c->in_deg, c->dsd, c->scratch, c->d_flag, c->xs_stage, c->xs_cum,
                  c->xs_colcum, c->xs_tmp, c->pr_pair, c->dyn_pending, c->dyn_next};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (c->h_pinned) cudaFreeHost(c->h_pinned);
  for (auto& p : c->pending) {
    cudaEventDestroy(p.a);
    cudaEventDestroy(p.b);
  }
  for (auto ev : c->ev_pool) cudaEventDestroy(ev);
  if (c->run_a) cudaEventDestroy(c->run_a);
  if (c->run_b) cudaEventDestroy(c->run_b);
  for (auto& sl : c->conc) {
    cudaStreamSynchronize(sl.stream);
    cudaEventDestroy(sl.a);
    cudaEventDestroy(sl.b);
    cudaEventDestroy(sl.done);
    cudaStreamDestroy(sl.stream);
  }
  if (c->fork_ev) cudaEventDestroy(c->fork_ev);
  if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
  delete c;
  return CYTOM_OK;
}

const char* cytom_last_error(const cytom_ctx* ctx) {
  const Ctx* c = (const Ctx*)ctx;
  return c ? c->err.c_str() : "null context";
}

int cytom_geometry(const cytom_ctx* ctx, uint64_t* vertices, uint64_t* vpt, uint64_t* tpd) {
  const Ctx* c = (const Ctx*)ctx;
  if (!c) return CYTOM_ERR_INVAL;
  if (vertices) *vertices = c->n;
  if (vpt) *vpt = c->vpt;
  if (tpd) *tpd = c->T;
  return CYTOM_OK;
}

// Device staging for host inputs.
struct Staging {
  void* p = nullptr;
  cudaStream_t s = nullptr;
  ~Staging() {
    if (p) cudaFreeAsync(p, s);
  }
};

int cytom_rmat_generate(cytom_ctx* ctx, const cytom_rmat_params* p, uint64_t first, uint64_t count,
                        uint32_t* src, uint32_t* tgt, uint32_t* w, int where) {
  Ctx* c = (Ctx*)ctx;
  if (!c || !p || !src || !tgt) return CYTOM_ERR_INVAL;
  if (p->scale == 0 || p->scale > 32 || (p->wmax > 0 && (p->wmin > p->wmax || !w)))
    return set_err(c, CYTOM_ERR_INVAL, "bad rmat parameters");
  if (count == 0) return CYTOM_OK;
  if (where == CYTOM_PTR_DEVICE) {
    int rc = rmat_generate(c, p, first, count, src, tgt, w);
    if (rc) return rc;
    return cuda_err(c, cudaStreamSynchronize(c->stream), "rmat");
  }
  Staging st;
  st.s = c->stream;
  size_t per = (p->wmax > 0) ? 12 : 8;
  if (cy_malloc_async(&st.p, count * per, c->stream) != cudaSuccess)
    return set_err(c, CYTOM_ERR_OOM, "rmat staging");
  uint32_t* ds = (uint32_t*)st.p;
  uint32_t* dt = ds + count;
  uint32_t* dw = (p->wmax > 0) ? dt + count : nullptr;
  int rc = rmat_generate(c, p, first, count, ds, dt, dw);
  if (rc) return rc;
  cudaMemcpyAsync(src, ds, count * 4, cudaMemcpyDeviceToHost, c->stream);
  cudaMemcpyAsync(tgt, dt, count * 4, cudaMemcpyDeviceToHost, c->stream);
  if (dw) cudaMemcpyAsync(w, dw, count * 4, cudaMemcpyDeviceToHost, c->stream);
  return cuda_err(c, cudaStreamSynchronize(c->stream), "rmat copy");
}

int cytom_gridgraph_decode(cytom_ctx* ctx, const void* bytes, uint64_t size, uint32_t* src,
                           uint32_t* tgt, int where, uint64_t* count) {
  Ctx* c = (Ctx*)ctx;
  if (!c || (!bytes && size)) return CYTOM_ERR_INVAL;
  uint64_t m = size / 8;
  if (count) *count = m;
  if (m == 0) return CYTOM_OK;
  Staging st;
  st.s = c->stream;
  size_t need = m * 8 + (where == CYTOM_PTR_HOST ? m * 8 : 0);
  if (cy_malloc_async(&st.p, need, c->stream) != cudaSuccess)
    return set_err(c, CYTOM_ERR_OOM, "gridgraph staging");
  void* drec = st.p;
  cudaMemcpyAsync(drec, bytes, m * 8, cudaMemcpyHostToDevice, c->stream);
  uint32_t *ds = src, *dt = tgt;
  if (where == CYTOM_PTR_HOST) {
    ds = (uint32_t*)((char*)st.p + m * 8);
    dt = ds + m;
  }
  int rc = gridgraph_decode(c, drec, m, ds, dt);
  if (rc) return rc;
  if (where == CYTOM_PTR_HOST) {
    cudaMemcpyAsync(src, ds, m * 4, cudaMemcpyDeviceToHost, c->stream);
    cudaMemcpyAsync(tgt, dt, m * 4, cudaMemcpyDeviceToHost, c->stream);
  }
  return cuda_err(c, cudaStreamSynchronize(c->stream), "gridgraph copy");
}

int cytom_insert_batch(cytom_ctx* ctx, const uint32_t* src, const uint32_t* tgt, const uint32_t* w,
                       uint64_t count, int where) {
  Ctx* c = (Ctx*)ctx;
  if (!c || (count && (!src || !tgt))) return CYTOM_ERR_INVAL;
  if (count == 0) return CYTOM_OK;
  if (where == CYTOM_PTR_DEVICE) {
    int rc = insert_device(c, src, tgt, w, count);  // returns once the batch is appended
    if (rc) return rc;
    return edge_log_append(c, src, tgt, w, count, CYTOM_PTR_DEVICE);
  }
  Staging st;
  st.s = c->stream;
  bool wt = c->wtype != CYTOM_UNWEIGHTED && w;
  if (cy_malloc_async(&st.p, count * (wt ? 12 : 8), c->stream) != cudaSuccess)
    return set_err(c, CYTOM_ERR_OOM, "insert staging");
  uint32_t* ds = (uint32_t*)st.p;
  uint32_t* dt = ds + count;
  uint32_t* dw = wt ? dt + count : nullptr;
  cudaMemcpyAsync(ds, src, count * 4, cudaMemcpyHostToDevice, c->stream);
  cudaMemcpyAsync(dt, tgt, count * 4, cudaMemcpyHostToDevice, c->stream);
  if (dw) cudaMemcpyAsync(dw, w, count * 4, cudaMemcpyHostToDevice, c->stream);
  int rc = insert_device(c, ds, dt, dw, count);  // returns once the batch is appended
  if (rc) return rc;
  return edge_log_append(c, src, tgt, w, count, CYTOM_PTR_HOST);
}

int cytom_load_gridgraph(cytom_ctx* ctx, const char* path, uint64_t batch, uint64_t* count) {
  Ctx* c = (Ctx*)ctx;
  if (!c || !path) return CYTOM_ERR_INVAL;
  if (c->wtype != CYTOM_UNWEIGHTED)
    return set_err(c, CYTOM_ERR_INVAL, "GridGraph files carry no weights; use an unweighted store");
  FILE* f = fopen(path, "rb");
  if (!f) return set_err(c, CYTOM_ERR_IO, std::string("cannot open ") + path);
  if (batch == 0) batch = 1ULL << 20;
  std::vector<char> buf(batch * 8);
  uint64_t total = 0;
  int rc = CYTOM_OK;
  void* dev = nullptr;
  if (cy_malloc(&dev, batch * 16) != cudaSuccess) {
    fclose(f);
    return set_err(c, CYTOM_ERR_OOM, "gridgraph staging");
  }
  uint32_t* ds = (uint32_t*)((char*)dev + batch * 8);
  uint32_t* dt = ds + batch;
  while (true) {
    size_t got = fread(buf.data(), 1, batch * 8, f);
    uint64_t m = got / 8;
    if (m == 0) break;
    cudaMemcpyAsync(dev, buf.data(), m * 8, cudaMemcpyHostToDevice, c->stream);
    rc = gridgraph_decode(c, dev, m, ds, dt);
    if (rc) break;
    rc = insert_device(c, ds, dt, nullptr, m);
    if (rc) break;
    rc = cuda_err(c, cudaStreamSynchronize(c->stream), "gridgraph insert");
    if (rc) break;
    total += m;
    if (got < batch * 8) break;
  }
  fclose(f);
  cudaFree(dev);
  if (count) *count = total;
  return rc;
}

int cytom_compact(cytom_ctx* ctx) {
  Ctx* c = (Ctx*)ctx;
  if (!c) return CYTOM_ERR_INVAL;
  int rc = compact(c);
  if (rc) return rc;
  rc = cuda_err(c, cudaStreamSynchronize(c->stream), "compact");
  if (rc) return rc;
  return prof_flush(c);
}

int cytom_clear(cytom_ctx* ctx) {
  Ctx* c = (Ctx*)ctx;
  if (!c) return CYTOM_ERR_INVAL;
  settle_runs(c);
  cudaError_t e = cudaMemsetAsync(c->out_deg, 0, c->n * 4, c->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(c->in_deg, 0, c->n * 4, c->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(c->tile_ptr, 0, (c->ntiles + 1) * 8, c->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(c->tile_ptr_alt, 0, (c->ntiles + 1) * 8, c->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(c->chunk_tile, 0, 2 * 4, c->stream);
  if (e == cudaSuccess && c->cmask) e = cudaMemsetAsync(c->cmask, 0, c->n * 8, c->stream);
  if (e != cudaSuccess) return cuda_err(c, e, "clear");
  c->E = 0;
  c->A = 0;
  if (c->dyn_pending) {  // dynamic compaction starts over: no appended edges, thresholds 4096
    cudaFree(c->dyn_pending);
    cudaFree(c->dyn_next);
    c->dyn_pending = nullptr;
    c->dyn_next = nullptr;
  }
  c->version++;  // directory, PageRank structures and degree copies are rebuilt on use
  for (Job* j : c->jobs)
    if (j) j->fresh = true;
  int rc = upload_store_desc(c);
  if (rc) return rc;
  return cuda_err(c, cudaStreamSynchronize(c->stream), "clear");
}

int cytom_count_edges(const cytom_ctx* ctx, uint64_t* compacted, uint64_t* pending) {
  const Ctx* c = (const Ctx*)ctx;
  if (!c) return CYTOM_ERR_INVAL;
  if (compacted) *compacted = c->E;
  if (pending) *pending = c->A;
  return CYTOM_OK;
}

int cytom_get_tiles(cytom_ctx* ctx, uint64_t* tile_ptr, uint32_t* edges, uint32_t* weights,
                    uint8_t* compact_flags) {
  Ctx* c = (Ctx*)ctx;
  if (c) join_runs(c);
  if (!c) return CYTOM_ERR_INVAL;
  cudaError_t e = cudaSuccess;
  if (tile_ptr)
    e = cudaMemcpyAsync(tile_ptr, c->tile_ptr, (c->ntiles + 1) * 8, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess && edges && c->E)
    e = cudaMemcpyAsync(edges, c->edges, c->E * 4, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess && weights && c->E && c->wtype)
    e = cudaMemcpyAsync(weights, c->wts, c->E * 4, cudaMemcpyDeviceToHost, c->stream);
  if (e != cudaSuccess) return cuda_err(c, e, "get_tiles");
  if (compact_flags) {
    uint8_t* d = nullptr;
    if (cy_malloc(&d, c->ntiles) != cudaSuccess) return set_err(c, CYTOM_ERR_OOM, "flags");
    int rc = compute_compact_flags(c, d);
    if (!rc) e = cudaMemcpyAsync(compact_flags, d, c->ntiles, cudaMemcpyDeviceToHost, c->stream);
    cudaStreamSynchronize(c->stream);
    cudaFree(d);
    if (rc) return rc;
    for (uint64_t t = 0; t < c->ntiles; ++t)
      if (compact_flags[t] == 2) compact_flags[t] = 0;  // empty tile: storage flag stays false
  }
  return cuda_err(c, cudaStreamSynchronize(c->stream), "get_tiles");
}

int cytom_get_degrees(cytom_ctx* ctx, uint32_t* out_degree, uint32_t* in_degree) {
  Ctx* c = (Ctx*)ctx;
  if (c) join_runs(c);
  if (!c) return CYTOM_ERR_INVAL;
  if (out_degree) cudaMemcpyAsync(out_degree, c->out_deg, c->n * 4, cudaMemcpyDeviceToHost, c->stream);
  if (in_degree) cudaMemcpyAsync(in_degree, c->in_deg, c->n * 4, cudaMemcpyDeviceToHost, c->stream);
  return cuda_err(c, cudaStreamSynchronize(c->stream), "get_degrees");
}

int cytom_job_create(cytom_ctx* ctx, int algo, const cytom_job_params* params, int* job_id) {
  Ctx* c = (Ctx*)ctx;
  if (!c || !job_id || algo < CYTOM_ALGO_BFS || algo > CYTOM_ALGO_CC_ASYNC) return CYTOM_ERR_INVAL;
  Job* j = new (std::nothrow) Job();
  if (!j) return CYTOM_ERR_OOM;
  if (algo == CYTOM_ALGO_BFS_ASYNC || algo == CYTOM_ALGO_CC_ASYNC) {
    // the same program as BFS / CC with the asynchronous pull
    j->async = true;
    algo = algo == CYTOM_ALGO_BFS_ASYNC ? CYTOM_ALGO_BFS : CYTOM_ALGO_CC;
  }
  j->algo = algo;
  if (params) j->params = *params;
  else cytom_job_params_default(&j->params);
  if ((algo == CYTOM_ALGO_BFS || algo == CYTOM_ALGO_SSSP || algo == CYTOM_ALGO_SSWP) &&
      j->params.start_vertex >= c->n) {
    delete j;
    return set_err(c, CYTOM_ERR_RANGE, "start vertex >= vertex count");
  }
  if ((algo == CYTOM_ALGO_SSSP || algo == CYTOM_ALGO_SSWP) && c->wtype != CYTOM_WEIGHT_U32) {
    delete j;
    return set_err(c, CYTOM_ERR_INVAL, "SSSP and SSWP need a store with uint32 weights");
  }
  if (algo == CYTOM_ALGO_WPAGERANK && c->wtype != CYTOM_WEIGHT_F32) {
    delete j;
    return set_err(c, CYTOM_ERR_INVAL, "weighted PageRank needs a store with float weights");
  }
  int rc = job_alloc(c, j);
  if (rc) {
    job_free(c, j);
    delete j;
    return rc;
  }
  j->id = (int)c->jobs.size();
  c->jobs.push_back(j);
  *job_id = j->id;
  return CYTOM_OK;
}

static Job* get_job(Ctx* c, int id) {
  if (!c || id < 0 || id >= (int)c->jobs.size()) return nullptr;
  return c->jobs[id];
}

int cytom_job_destroy(cytom_ctx* ctx, int job_id) {
  Ctx* c = (Ctx*)ctx;
  if (c) settle_runs(c);
  Job* j = get_job(c, job_id);
  if (!j) return CYTOM_ERR_INVAL;
  cudaStreamSynchronize(c->stream);
  job_free(c, j);
  delete j;
  c->jobs[job_id] = nullptr;
  return CYTOM_OK;
}

int cytom_job_reset(cytom_ctx* ctx, int job_id) {
  Ctx* c = (Ctx*)ctx;
  if (c) settle_runs(c);
  Job* j = get_job(c, job_id);
  if (!j) return CYTOM_ERR_INVAL;
  j->fresh = true;
  return CYTOM_OK;
}

int cytom_run(cytom_ctx* ctx, int job_id, cytom_run_stats* stats) {
  Ctx* c = (Ctx*)ctx;
  if (c) settle_runs(c);
  Job* j = get_job(c, job_id);
  if (!j) return CYTOM_ERR_INVAL;
  return job_run(c, j, stats);
}

static int job_list(Ctx* c, const int* job_ids, int count, std::vector<Job*>* jobs) {
  if (count < 0 || (count > 0 && !job_ids)) return CYTOM_ERR_INVAL;
  jobs->resize(count);
  for (int k = 0; k < count; ++k) {
    (*jobs)[k] = get_job(c, job_ids[k]);
    if (!(*jobs)[k]) return CYTOM_ERR_INVAL;
    for (int i = 0; i < k; ++i)
      if ((*jobs)[i] == (*jobs)[k]) return set_err(c, CYTOM_ERR_INVAL, "a job listed twice");
  }
  return CYTOM_OK;
}

int cytom_run_many(cytom_ctx* ctx, const int* job_ids, int count, cytom_run_stats* stats) {
  Ctx* c = (Ctx*)ctx;
  if (!c) return CYTOM_ERR_INVAL;
  std::vector<Job*> jobs;
  int rc = job_list(c, job_ids, count, &jobs);
  if (rc) return rc;
  if (!c->async_jobs.empty()) {
    rc = collect_runs(c, nullptr);
    if (rc) return rc;
  }
  return job_run_many(c, jobs.data(), count, stats);
}

int cytom_run_many_async(cytom_ctx* ctx, const int* job_ids, int count) {
  Ctx* c = (Ctx*)ctx;
  if (!c) return CYTOM_ERR_INVAL;
  std::vector<Job*> jobs;
  int rc = job_list(c, job_ids, count, &jobs);
  if (rc) return rc;
  if (!c->async_jobs.empty()) return set_err(c, CYTOM_ERR_INVAL, "the previous asynchronous runs are not collected");
  if (!runs_concurrently(c, jobs.data(), count)) {
    // nothing to overlap: run now, collect later
    std::vector<cytom_run_stats> st(count);
    rc = job_run_many(c, jobs.data(), count, st.data());
    if (rc) return rc;
    c->sync_stats = st;
    c->sync_jobs = jobs;
    return CYTOM_OK;
  }
  return launch_many(c, jobs.data(), count);
}

int cytom_run_many_wait(cytom_ctx* ctx, cytom_run_stats* stats) {
  Ctx* c = (Ctx*)ctx;
  if (!c) return CYTOM_ERR_INVAL;
  if (!c->sync_jobs.empty()) {
    if (stats) memcpy(stats, c->sync_stats.data(), c->sync_stats.size() * sizeof(cytom_run_stats));
    c->sync_jobs.clear();
    c->sync_stats.clear();
    return CYTOM_OK;
  }
  if (c->async_jobs.empty()) return set_err(c, CYTOM_ERR_INVAL, "no asynchronous runs to collect");
  return collect_runs(c, stats);
}

int cytom_get_result(cytom_ctx* ctx, int job_id, void* out, int where) {
  Ctx* c = (Ctx*)ctx;
  if (c) join_runs(c);
  Job* j = get_job(c, job_id);
  if (!j || !out) return CYTOM_ERR_INVAL;
  if (!is_minprop(j->algo)) return pagerank_result(c, j, out, where);
  cudaMemcpyKind k = where == CYTOM_PTR_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
  const uint32_t* src = j->h.next;
  uint32_t* tmp = nullptr;
  cudaError_t e = cudaSuccess;
  if (j->algo == CYTOM_ALGO_SSWP) {
    // SSWP runs on complemented values: widths = ~values
    if (cy_malloc_async((void**)&tmp, c->n * 4, c->stream) != cudaSuccess) return set_err(c, CYTOM_ERR_OOM, "result");
    complement_kernel<<<(unsigned)std::min<uint64_t>((c->n + 255) / 256, (uint64_t)c->num_sms * 8), 256, 0,
                        c->stream>>>(src, c->n, tmp);
    c->launches++;
    src = tmp;
  }
  e = cudaMemcpyAsync(out, src, c->n * 4, k, c->stream);
  if (tmp) cudaFreeAsync(tmp, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  return cuda_err(c, e, "get_result");
}

int cytom_job_set_teleport(cytom_ctx* ctx, int job_id, const double* teleport, int where) {
  Ctx* c = (Ctx*)ctx;
  if (c) join_runs(c);
  Job* j = get_job(c, job_id);
  if (!j) return CYTOM_ERR_INVAL;
  return pagerank_set_teleport(c, j, teleport, where);
}

int cytom_pagerank_adjoint(cytom_ctx* ctx, int job_id, const double* c_weights, int c_where,
                           float* d_weights, float* d_teleport, int out_where, cytom_run_stats* stats) {
  Ctx* c = (Ctx*)ctx;
  if (c) join_runs(c);
  Job* j = get_job(c, job_id);
  if (!j || !c_weights) return CYTOM_ERR_INVAL;
  return pagerank_adjoint(c, j, c_weights, c_where, d_weights, d_teleport, out_where, stats);
}

int cytom_set_edge_weights(cytom_ctx* ctx, const uint32_t* src, const uint32_t* tgt, const uint32_t* w,
                           uint64_t count, int where) {
  Ctx* c = (Ctx*)ctx;
  if (c) join_runs(c);
  if (!c || (count && (!src || !tgt || !w))) return CYTOM_ERR_INVAL;
  if (c->wtype == CYTOM_UNWEIGHTED) return set_err(c, CYTOM_ERR_INVAL, "the store has no weights");
  if (where == CYTOM_PTR_DEVICE || count == 0) return set_edge_weights(c, src, tgt, w, count);
  Staging st;
  st.s = c->stream;
  if (cy_malloc_async(&st.p, count * 12, c->stream) != cudaSuccess) return set_err(c, CYTOM_ERR_OOM, "staging");
  uint32_t* ds = (uint32_t*)st.p;
  cudaMemcpyAsync(ds, src, count * 4, cudaMemcpyHostToDevice, c->stream);
  cudaMemcpyAsync(ds + count, tgt, count * 4, cudaMemcpyHostToDevice, c->stream);
  cudaMemcpyAsync(ds + 2 * count, w, count * 4, cudaMemcpyHostToDevice, c->stream);
  return set_edge_weights(c, ds, ds + count, ds + 2 * count, count);
}

int cytom_delete_batch(cytom_ctx* ctx, const uint32_t* src, const uint32_t* tgt, uint64_t count, int where,
                       uint64_t* deleted) {
  Ctx* c = (Ctx*)ctx;
  if (c) join_runs(c);
  if (deleted) *deleted = 0;
  if (!c || (count && (!src || !tgt))) return CYTOM_ERR_INVAL;
  if (where == CYTOM_PTR_DEVICE || count == 0) return delete_edges(c, src, tgt, count, deleted);
  Staging st;
  st.s = c->stream;
  if (cy_malloc_async(&st.p, count * 8, c->stream) != cudaSuccess) return set_err(c, CYTOM_ERR_OOM, "staging");
  uint32_t* ds = (uint32_t*)st.p;
  cudaMemcpyAsync(ds, src, count * 4, cudaMemcpyHostToDevice, c->stream);
  cudaMemcpyAsync(ds + count, tgt, count * 4, cudaMemcpyHostToDevice, c->stream);
  return delete_edges(c, ds, ds + count, count, deleted);
}

int cytom_delete_random(cytom_ctx* ctx, uint64_t count, uint64_t seed, uint32_t* src, uint32_t* tgt, int where,
                        uint64_t* deleted) {
  Ctx* c = (Ctx*)ctx;
  if (c) join_runs(c);
  if (deleted) *deleted = 0;
  if (!c || (src && !tgt) || (!src && tgt)) return CYTOM_ERR_INVAL;
  if (count == 0) return delete_edges(c, nullptr, nullptr, 0, nullptr);
  if (src && where == CYTOM_PTR_DEVICE) return delete_random(c, count, seed, src, tgt, deleted);
  Staging st;
  st.s = c->stream;
  if (cy_malloc_async(&st.p, count * 8, c->stream) != cudaSuccess) return set_err(c, CYTOM_ERR_OOM, "staging");
  uint32_t* ds = (uint32_t*)st.p;
  int rc = delete_random(c, count, seed, ds, ds + count, deleted);
  if (rc || !src) return rc;
  cudaError_t e = cudaMemcpyAsync(src, ds, count * 4, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(tgt, ds + count, count * 4, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  return cuda_err(c, e, "random deletion picks");
}

static void fill_tune_report(const Ctx* c, cytom_tune_report* out) {
  memset(out, 0, sizeof(*out));
  int cnt = 0;
  sg_shapes(out->edges_per_thread, out->pipeline_depth, out->blocks_per_sm, &cnt);
  out->variants = cnt;
  out->chosen[0] = c->sg_variant[0];
  out->chosen[1] = c->sg_variant[1];
  for (int k = 0; k < 2; ++k)
    for (int v = 0; v < cnt && v < 8; ++v) out->us[k][v] = c->tune_us[k][v];
  out->tuned_edges = c->tune_E;
  for (int k = 0; k < 2; ++k) {
    out->sparse_div[k] = (int32_t)c->tune_div[k];
    for (int i = 0; i < 6; ++i) {
      out->dense_round_us[k][i] = c->tune_dense_us[k][i];
      out->sparse_round_us[k][i] = c->tune_sparse_us[k][i];
    }
  }
  const int32_t divs[6] = {128, 64, 32, 16, 8, 4};
  for (int i = 0; i < 6; ++i) out->div_candidates[i] = divs[i];
}

int cytom_autotune(cytom_ctx* ctx, cytom_tune_report* out) {
  Ctx* c = (Ctx*)ctx;
  if (c) join_runs(c);
  if (!c) return CYTOM_ERR_INVAL;
  int rc = compact(c);
  if (!rc) rc = minprop_autotune(c);
  if (rc) return rc;
  if (out) fill_tune_report(c, out);
  return CYTOM_OK;
}

int cytom_get_tune_report(const cytom_ctx* ctx, cytom_tune_report* out) {
  const Ctx* c = (const Ctx*)ctx;
  if (!c || !out) return CYTOM_ERR_INVAL;
  fill_tune_report(c, out);
  return CYTOM_OK;
}

int cytom_get_result_f64(cytom_ctx* ctx, int job_id, double* out, int where) {
  Ctx* c = (Ctx*)ctx;
  if (c) join_runs(c);
  Job* j = get_job(c, job_id);
  if (!j || !out) return CYTOM_ERR_INVAL;
  return pagerank_result64(c, j, out, where);
}

int cytom_set_profiling(cytom_ctx* ctx, int on) {
  Ctx* c = (Ctx*)ctx;
  if (!c) return CYTOM_ERR_INVAL;
  prof_flush(c);
  c->profiling = on != 0;
  return CYTOM_OK;
}

int cytom_get_kernel_stats(cytom_ctx* ctx, cytom_kernel_stats* out) {
  Ctx* c = (Ctx*)ctx;
  if (!c || !out) return CYTOM_ERR_INVAL;
  int rc = prof_flush(c);
  *out = c->kstats;
  return rc;
}

int cytom_reset_kernel_stats(cytom_ctx* ctx) {
  Ctx* c = (Ctx*)ctx;
  if (!c) return CYTOM_ERR_INVAL;
  prof_flush(c);
  for (int k = 0; k < CYTOM_KERNEL_CLASSES; ++k) {
    c->kstats.launches[k] = 0;
    c->kstats.total_ms[k] = 0;
    c->kstats.algo_bytes[k] = 0;
  }
  return CYTOM_OK;
}

int cytom_launch_count(const cytom_ctx* ctx, uint64_t* launches) {
  const Ctx* c = (const Ctx*)ctx;
  if (!c || !launches) return CYTOM_ERR_INVAL;
  *launches = c->launches;
  return CYTOM_OK;
}

int cytom_set_fault_injection(cytom_ctx* ctx, const cytom_fault_injection* f) {
  Ctx* c = (Ctx*)ctx;
  if (!c || !f) return CYTOM_ERR_INVAL;
  g_alloc_countdown.store(f->fail_alloc_after, std::memory_order_relaxed);
  c->inj_idle_limit = f->idle_poll_limit;
  c->inj_phantom_jobs = f->phantom_jobs;
  return CYTOM_OK;
}

int cytom_sync(cytom_ctx* ctx) {
  Ctx* c = (Ctx*)ctx;
  if (c) join_runs(c);
  if (!c) return CYTOM_ERR_INVAL;
  return cuda_err(c, cudaStreamSynchronize(c->stream), "sync");
}

}  // extern "C"
