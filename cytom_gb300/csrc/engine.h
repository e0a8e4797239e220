// engine.h — internal declarations of the GB300 evolving-graph engine.
//
// Layout in HBM (one context = one graph):
//   edges[E]      packed local edge (src_local << 16 | tgt_local), u32, sorted by
//                 (tile_x, tile_y, src_local, tgt_local), duplicates removed: the
//                 concatenation, in tile-id order (id = x*T + y), of every tile's CSR.
//   wts[E]        per-edge weight (u32 or f32 bits), weighted stores only.
//   tile_ptr[T*T+1]  u64 offsets of every tile's edges.
//   chunk_tile[E/128+1]  tile id of the first edge of every 128-edge chunk.
//   app_keys[A]   append region: u64 composite keys (x, y, src_l, tgt_l) of edges
//                 inserted since the last compaction (+ app_w weights).
//   out_deg / in_deg  u32 per vertex (multiplicity counts).
// Kernels read pointers and sizes from a StoreDesc in device memory, so a captured
// CUDA graph stays valid when the host swaps or grows buffers.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/cytom_gpu.h"

namespace cytom {

constexpr int kChunk = 128;  // edges per warp chunk (32 lanes x uint4)
constexpr uint32_t kInf = 0xFFFFFFFFu;

// One stage of the column-ordered dense round: `count` (<= 4096) consecutive edges of one
// tile, starting at edge e0 of the store.
struct TileStage {
  uint32_t tile;
  uint32_t count;
  unsigned long long e0;
};

struct StoreDesc {
  const uint32_t* edges;
  const uint32_t* wts;
  const unsigned long long* tile_ptr;
  const uint32_t* chunk_tile;
  const uint32_t* out_deg;
  const uint32_t* in_deg;
  unsigned long long E;        // compacted edges (written on the device by compaction)
  unsigned long long nchunks;  // ceil(E / kChunk)
  unsigned long long n;        // vertices
  unsigned long long T;        // tiles per dimension
  unsigned long long ntiles;
  uint32_t lvpt, lT;           // log2(vertices per tile), log2(T)
  int wtype;
  int adaptive;                // adaptive scheduling (skip inactive tile rows)
  // source directory: dir[t*(nbw+1) + b] = offset, inside tile t = x*T + y, of its
  // first edge with src_local >= 32*b (b = nbw: the tile size)
  const uint32_t* dir;
  uint32_t nbw;                // 32-source blocks per tile row (vpt / 32)
  int dir_ok;                  // directory current (sparse rounds allowed)
  uint32_t sparse_div;         // sparse round while non-zero frontier words * sparse_div <= all words
  uint32_t pad_sd;
  // column-ordered stages of the dense round (gather_tiles_kernel): stages of every tile in
  // column-major tile order (column y, then row x); xcum[i] = partition weight before
  // stage i in that order (edges + a fixed cost per stage; xcum[*xnst] = the total);
  // xcolcum[y] = the weight before column y (T + 1 entries)
  uint32_t traversal;          // tile order of the column-ordered stages (CYTOM_TRAVERSAL_*)
  uint32_t pad_tr;
  const TileStage* xst;
  const unsigned long long* xcum;
  const unsigned long long* xcolcum;
  const uint32_t* xnst;
  // source column masks: bit (y >> cshift) of cmask[u] is set when source u may have an
  // edge in tile column y (a superset: set for every stored edge, never cleared by
  // deletions); NULL when the context keeps none. Current whenever dir_ok is.
  const unsigned long long* cmask;
  uint32_t cshift;             // log2(T) - 6 above 64 tile columns, else 0
  uint32_t pad_cm;
};

// Loop state of one job run, in device memory. Kernels index the double-buffered
// per-iteration counters by the parity of `iter`.
struct LoopState {
  unsigned int iter;       // rounds executed in this run
  unsigned int max_iter;
  unsigned int cont;       // 1 while the run continues
  unsigned int err;
  unsigned int active[2];  // vertices activated for the next round (by parity)
  unsigned int nact_words[2];  // non-zero frontier words listed for the next round
  unsigned int mode;       // gather of the current round: 0 dense (stream), 1 sparse (directory)
  unsigned int spq_count;  // heavy-item chunks queued in this round
  unsigned long long teps[2];  // edges of newly active tile rows (by parity)
  unsigned long long count_edges;   // reference counting rule, summed
  unsigned long long edges_scanned; // edges this engine read
  unsigned long long active_total;
  double resid[2];          // PageRank: FP64 residual by parity
  double rank_sum[2];
  double dangling[2];
  double tol;
  double resid_final;
  double base_sum;          // PageRank-delta: rank sum at the start of the run
  double change_sum;        // PageRank-delta: sum of all rank changes of the run
  double best_resid;        // PageRank FP32: best residual so far (rounding-floor detection)
  unsigned int stall;       // rounds without a residual improvement
  unsigned int apply_done;  // blocks of the running apply that finished (last one runs control)
  unsigned int sel_rounds;  // rounds started by the captured loop (bounds it independently)
  unsigned int pad2;
  unsigned long long items_read;  // sparse rounds: (word, column) items whose directory was read
};

struct JobDesc {
  uint32_t* cur;      // current values (u32 for BFS/CC/SSSP)
  uint32_t* next;
  uint32_t* fa;       // frontier (active_current) bitmap, n/32 words
  uint32_t* ch;       // changed bitmap
  uint32_t* rows;     // 2 x T tile-row activity flags (by parity)
  uint32_t* aw;       // indices of the non-zero frontier words (sparse rounds)
  unsigned long long* awm;  // per listed word: OR of its active sources' column masks
  uint2* spq;         // sparse rounds: queue of (item, chunk) of heavy items
  unsigned long long spq_cap;
  float* rank;        // PageRank family
  float* rank_c;      // Kahan compensation of rank
  float* delta;
  float* dsum;
  float* contrib;
  double* rank64;     // FP64 plain PageRank
  double* dsum64;
  unsigned int* deg_distinct;
  LoopState* ls;
  int algo;
  int kahan;
  int async;          // BFS / CC asynchronous programs: sources read from next
  uint32_t sparse_div;  // tuned sparse-round threshold of the job's class (0: the store's)
  uint32_t pad_jd;
  double alpha, delta_param;
  unsigned long long start;
};

enum KernelClass { KC_RMAT = 0, KC_INSERT, KC_SORT, KC_MERGE, KC_GATHER, KC_APPLY, KC_PAGERANK, KC_OTHER };

struct Job {
  int id = -1;
  int algo = 0;
  cytom_job_params params{};
  bool fresh = true;          // next run starts from scratch
  bool async = false;         // asynchronous program (CYTOM_ALGO_BFS_ASYNC / CC_ASYNC)
  JobDesc h{};                // host copy of the descriptor
  JobDesc* d = nullptr;       // device copy
  LoopState* ls = nullptr;    // device
  // CUDA graph of the converge loop (while-conditional)
  cudaGraphExec_t loop_exec = nullptr;
  bool graph_failed = false;
  bool last_run_graph = false;  // the last run went through the graph (launch accounting)
  uint64_t graph_epoch = 0;     // tune epoch the captured graph was built with
  void* ext = nullptr;          // per-algorithm state (PageRank family)
};

// A stream of its own for one job of a concurrent run, and the events around its launches.
struct ConcSlot {
  cudaStream_t stream = nullptr;
  cudaEvent_t a = nullptr, b = nullptr, done = nullptr;
};

struct Ctx {
  cytom_config cfg{};
  std::string err;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  int device = 0;
  int num_sms = 1;
  // geometry
  uint64_t n = 0, vpt = 0, T = 0, ntiles = 0;
  uint32_t lvpt = 0, lT = 0;
  int wtype = 0;
  // store (host view of pointers)
  uint32_t *edges = nullptr, *wts = nullptr, *edges_alt = nullptr, *wts_alt = nullptr;
  unsigned long long *tile_ptr = nullptr, *tile_ptr_alt = nullptr;
  uint32_t* chunk_tile = nullptr;
  uint32_t* chunk_tile_alt = nullptr;  // written by the merge, swapped in with the store
  uint64_t cap = 0, chunk_cap = 0;
  uint64_t E = 0;  // exact after compaction
  uint64_t version = 0;  // bumped by every compaction that merged edges
  std::vector<ConcSlot> conc;      // concurrent runs: one stream per job
  cudaEvent_t fork_ev = nullptr;
  // runs launched by cytom_run_many_async that the context's stream has not waited for
  // yet; they read the installed snapshot and write only their jobs' state
  std::vector<Job*> async_jobs;    // jobs of the last asynchronous launch (slot k = job k)
  bool runs_unjoined = false;
  std::vector<Job*> sync_jobs;     // an asynchronous request that ran synchronously
  std::vector<cytom_run_stats> sync_stats;
  uint32_t* dir = nullptr;  // source directory (sparse rounds)
  unsigned long long* cmask = nullptr;  // per-source tile-column masks (StoreDesc::cmask)
  uint32_t* dir_alt = nullptr;  // written by the merge, swapped in with the store
  uint64_t dir_entries = 0;
  uint64_t dir_version = ~0ULL;
  bool dir_disabled = false;
  // dynamic compaction (cfg.use_dynamic_compaction): appended edges per tile since the
  // last compaction and each tile's next threshold (4096, doubling)
  uint32_t* dyn_pending = nullptr;
  unsigned long long* dyn_next = nullptr;
  uint64_t dyn_compactions = 0;
  uint64_t *app_keys = nullptr, *app_keys_alt = nullptr;
  uint32_t *app_w = nullptr, *app_w_alt = nullptr;
  uint64_t A = 0, app_cap = 0;
  uint32_t *out_deg = nullptr, *in_deg = nullptr;
  StoreDesc hsd{};
  StoreDesc* dsd = nullptr;
  // scratch
  void* scratch = nullptr;
  size_t scratch_bytes = 0;
  unsigned int* d_flag = nullptr;       // error / misc flags
  unsigned long long* d_count = nullptr;
  unsigned long long* h_pinned = nullptr;  // pinned host words for readbacks
  // jobs
  std::vector<Job*> jobs;
  // instrumentation
  bool profiling = false;
  uint64_t launches = 0;
  struct PendingEv { int cls; cudaEvent_t a, b; double bytes; };
  std::vector<PendingEv> pending;
  std::vector<cudaEvent_t> ev_pool;
  cytom_kernel_stats kstats{};
  cudaEvent_t run_a = nullptr, run_b = nullptr;
  // batched executor: device tables kept by the first context of a batch
  void* batch = nullptr;
  uint64_t batch_units = 0;
  // PageRank family: the snapshot's CSC, shared by the context's PageRank jobs
  // autotuner: streaming-gather variant per program class (0: BFS / CC, 1: SSSP),
  // the edge count it was tuned at, and an epoch that invalidates captured graphs
  int sg_variant[2] = {0, 0};
  uint64_t tune_E = 0;
  uint64_t tune_epoch = 0;
  double tune_us[2][8] = {};
  uint32_t tune_div[2] = {0, 0};   // tuned sparse-round threshold per class (0 = untuned)
  double tune_dense_us[2][6] = {};
  double tune_sparse_us[2][6] = {};
  // PageRank family: vertices renumbered by out-degree (hubs first) so the hot part of
  // the gathered contribution vector packs densely into L2. perm[v] = position of vertex
  // v, inv[position] = v; fixed once computed. deg_mult = multiplicity out-degrees in
  // that numbering (PageRank-delta), rebuilt when the graph changes.
  uint32_t* pr_perm = nullptr;
  uint32_t* pr_inv = nullptr;
  uint32_t* pr_deg_mult = nullptr;
  uint64_t pr_deg_mult_version = ~0ULL;
  void* pr_csc = nullptr;
  // The kept edges of the last compaction as renumbered (target, source) keys, saved
  // while the PageRank CSC was current, so that its next build merges them in instead of
  // re-sorting every edge (pr_delta_version: the store version they lead to).
  uint64_t* pr_delta_keys = nullptr;
  uint64_t pr_delta_cap = 0;
  uint64_t pr_delta_count = 0;
  uint64_t pr_delta_version = ~0ULL;
  void* pr_wgraph = nullptr;  // weighted PageRank: CSC + CSR with weights
  void* pr_pair = nullptr;    // batched executor: interleaved contributions of paired PageRank jobs
  size_t pr_pair_bytes = 0;
  void* edge_log = nullptr;   // open edge log (cytom_persist_edges)
  // column-ordered stage list of the dense round, rebuilt when the store version changes
  TileStage* xs_stage = nullptr;
  unsigned long long* xs_cum = nullptr;
  unsigned long long* xs_colcum = nullptr;
  uint32_t* xs_tmp = nullptr;       // counts, offsets and totals of the build
  uint64_t xs_cap = 0;              // stage entries allocated
  uint64_t xs_version = ~0ULL;
  // fault injection (tests): batched executor's idle-wait limit (0 = default) and
  // phantom unfinished jobs
  uint32_t inj_idle_limit = 0;
  uint32_t inj_phantom_jobs = 0;
};

// ---- allocation ----
// Every device and pinned-host allocation of the library goes through these, so a test
// can make the n-th one fail (cytom_set_fault_injection) without a real shortage.
bool alloc_fault_fires();
template <class T>
inline cudaError_t cy_malloc(T** p, size_t bytes) {
  if (alloc_fault_fires()) {
    *p = nullptr;
    return cudaErrorMemoryAllocation;
  }
  return cudaMalloc(reinterpret_cast<void**>(p), bytes);
}
template <class T>
inline cudaError_t cy_malloc_async(T** p, size_t bytes, cudaStream_t s) {
  if (alloc_fault_fires()) {
    *p = nullptr;
    return cudaErrorMemoryAllocation;
  }
  return cudaMallocAsync(reinterpret_cast<void**>(p), bytes, s);
}
template <class T>
inline cudaError_t cy_malloc_host(T** p, size_t bytes) {
  if (alloc_fault_fires()) {
    *p = nullptr;
    return cudaErrorMemoryAllocation;
  }
  return cudaMallocHost(reinterpret_cast<void**>(p), bytes);
}

// ---- helpers (capi.cu) ----
int set_err(Ctx* c, int code, const std::string& msg);
int cuda_err(Ctx* c, cudaError_t e, const char* what);
int prof_begin(Ctx* c, int cls);          // returns slot or -1
void prof_end(Ctx* c, int slot, double bytes);
int prof_flush(Ctx* c);
int upload_store_desc(Ctx* c);

// ---- ingest (ingest.cu) ----
int rmat_generate(Ctx* c, const cytom_rmat_params* p, uint64_t first, uint64_t count,
                  uint32_t* src, uint32_t* tgt, uint32_t* w);
int gridgraph_decode(Ctx* c, const void* dbytes, uint64_t m, uint32_t* src, uint32_t* tgt);
int insert_device(Ctx* c, const uint32_t* src, const uint32_t* tgt, const uint32_t* w,
                  uint64_t count);
int compact(Ctx* c);
int compute_compact_flags(Ctx* c, uint8_t* dflags);
int build_directory(Ctx* c);
int build_tile_stages(Ctx* c);
bool tiles_in_use(Ctx* c, int algo);
int ensure_app_capacity(Ctx* c, uint64_t need);

// device-wide utilities
int exclusive_scan_u32(Ctx* c, const uint32_t* in, uint32_t* out, uint64_t n, uint32_t* total_dev);
int radix_sort_pairs(Ctx* c, uint64_t* keys, uint64_t* keys_alt, uint32_t* vals, uint32_t* vals_alt,
                     uint64_t n, int bits, bool* result_in_alt);

// ---- executors ----
int job_alloc(Ctx* c, Job* j);
void job_free(Ctx* c, Job* j);
int job_init_state(Ctx* c, Job* j);
int job_seed(Ctx* c, Job* j, const uint32_t* src, const uint32_t* tgt, const uint32_t* w,
             uint64_t count);
int job_seed_keys(Ctx* c, Job* j, const uint64_t* K, const uint32_t* W, uint64_t count);
int pagerank_note_kept(Ctx* c, const uint32_t* nloc, const uint32_t* ntile, uint64_t kept);
int pagerank_csc_stage(Ctx* c);
// The context's stream waits for runs launched asynchronously (no host wait); every
// operation that touches the installed snapshot or job state comes after it.
void join_runs(Ctx* c);
constexpr int kMaxSeedJobs = 16;  // jobs seeded by one pass over a compaction's keys
int minprop_seed_keys_many(Ctx* c, Job* const* jobs, int njobs, const uint64_t* K, const uint32_t* W,
                           uint64_t count);
// Joins and drops the statistics of uncollected asynchronous runs (before jobs run again
// or are reset or destroyed).
void settle_runs(Ctx* c);
int job_run(Ctx* c, Job* j, cytom_run_stats* st);
int job_result(Ctx* c, Job* j, void* out, int where);
int ensure_job_queue(Ctx* c, Job* j);
int minprop_autotune(Ctx* c);
void sg_shapes(int* ept, int* nst, int* minb, int* count);
void batch_free(Ctx* c);
void pagerank_ctx_free(Ctx* c);
void edge_log_close(Ctx* c);
int edge_log_append(Ctx* c, const uint32_t* src, const uint32_t* tgt, const uint32_t* w, uint64_t count, int where);

}  // namespace cytom
