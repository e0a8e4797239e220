/*
 * cytom_gpu.h — C ABI of the GB300-native evolving-graph engine.
 *
 * One context (cytom_ctx) owns one graph on one GPU: a device-resident tile
 * store (edges grouped into vpt x vpt tiles, tile-major, sorted, deduplicated),
 * the vertex degrees, and any number of algorithm jobs (vertex programs) that
 * keep their vertex state on the device between runs. Plain pointers and sizes
 * only; no C++ or torch types cross this boundary.
 *
 * Every call returns CYTOM_OK (0) or a negative CYTOM_ERR_* code and never
 * aborts; cytom_last_error() gives the message of the last failure. A context is
 * single-threaded: callers serialise calls on one context. All device work of a
 * context runs on one CUDA stream (the caller's, if given). Input pointers are
 * borrowed for the duration of the call; output buffers belong to the caller.
 *
 * Citations name the reference interface each entry point replaces
 * (oslab-swrc/cytom, path inside that project).
 */
#ifndef CYTOM_GPU_H
#define CYTOM_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. The reference aborts through util::die (src/lib/util/util.cc:21-32)
 * and parseOption returns -EINVAL (src/include/main/execute.h:207). */
#define CYTOM_OK 0
#define CYTOM_ERR_INVAL (-1)         /* bad argument or configuration */
#define CYTOM_ERR_OOM (-2)           /* device or host allocation failed */
#define CYTOM_ERR_RANGE (-3)         /* vertex id >= vertex count, negative id */
#define CYTOM_ERR_TIMEOUT (-4)       /* a bounded device wait gave up */
#define CYTOM_ERR_CUDA (-5)          /* CUDA runtime error */
#define CYTOM_ERR_UNIMPLEMENTED (-6) /* not implemented by the library */
#define CYTOM_ERR_IO (-7)            /* file could not be read */

/* Pointer location flags for buffers passed in or out. */
#define CYTOM_PTR_HOST 0
#define CYTOM_PTR_DEVICE 1

/* Weight storage of a tile store. */
#define CYTOM_UNWEIGHTED 0
#define CYTOM_WEIGHT_U32 1 /* integer weights (SSSP) */
#define CYTOM_WEIGHT_F32 2 /* float weights, stored as their bit pattern (weighted PageRank) */

/* Vertex programs: examples/bfs.cc, cc.cc, sssp.cc, pagerank-delta.cc in the
 * reference (selected by template argument in execute<V, A, w>,
 * src/include/main/execute.h:534). PAGERANK is the normalised PageRank with
 * dangling-mass redistribution (FP32 + Kahan, FP64 residual). */
#define CYTOM_ALGO_BFS 0
#define CYTOM_ALGO_CC 1
#define CYTOM_ALGO_SSSP 2
#define CYTOM_ALGO_PR_DELTA 3
#define CYTOM_ALGO_PAGERANK 4
/* Weighted PageRank on a CYTOM_WEIGHT_F32 store (no counterpart in the reference, whose
 * pullGatherWeighted is "not applicable", examples/pagerank.cc:98): raw edge weights
 * normalised per source, teleport vector t (uniform unless set), dangling mass sent
 * along t: r = (1-alpha) t + alpha (P r + D t). FP32 + compensated sums (kahan = 1)
 * or FP64 plain; FP64 L1 residual. Differentiable: cytom_pagerank_adjoint. */
#define CYTOM_ALGO_WPAGERANK 5
/* Single-source widest path (examples/sswp.cc): value = the largest bottleneck weight of
 * a path from start_vertex (v = max(v, min(u, w)); 0 = unreached, UINT32_MAX at the start),
 * uint32 weights (a CYTOM_WEIGHT_U32 store; the reference's float values are exact for
 * them). */
#define CYTOM_ALGO_SSWP 6
/* Asynchronous BFS and CC (examples/bfs-async.cc, cc-async.cc: ASYNC = true): the pull
 * reads the freshest value of every source, next[src], instead of current[src]
 * (src/include/core/algorithm-executor.h:303-312, 332-340), so a value lowered early in a
 * round can travel further in the same round. Same fixed points as BFS and CC; round and
 * processed-edge counts depend on scheduling, as in the reference. */
#define CYTOM_ALGO_BFS_ASYNC 7
#define CYTOM_ALGO_CC_ASYNC 8

/* Tile visiting order of the column-ordered dense round (dense-round variant 4, see
 * cytom_tune_report), the reference's --traversal (src/include/util/config.h traversal_t;
 * src/lib/traversal/row_first.cc, column_first.cc, hilbert.cc; default row-first,
 * src/scripts/config.py:62). x = source tile, y = target tile, T tiles per dimension.
 * The work of a round is this sequence of tiles cut into equal contiguous ranges, one
 * per SM (the reference's meta-tiles of consecutive tiles, src/include/core/tile-distributor.h). */
#define CYTOM_TRAVERSAL_ROW_FIRST 0    /* d = y * T + x: all sources of a target tile column in a
                                          row; only this order reduces a column's targets in
                                          shared memory */
#define CYTOM_TRAVERSAL_COLUMN_FIRST 1 /* d = x * T + y: the store's tile-major order */
#define CYTOM_TRAVERSAL_HILBERT 2      /* d along the Hilbert curve over (x, y) (hilbert.cc) */

/* Context configuration: the subset of ConfigContext (src/include/util/config.h:529-567)
 * and its command-line flags (src/include/core/jobs.h:176-216) that the hot path uses. */
typedef struct cytom_config {
  uint64_t max_vertices;         /* --max-vertices; rounded up to a power of two
                                    (Config::normalizeConfig, src/lib/util/config.cc:10-13) */
  uint64_t vertices_per_tile;    /* --vertices-per-tile; power of two, <= 65536, <= vertices */
  int32_t weight_type;           /* CYTOM_UNWEIGHTED / CYTOM_WEIGHT_U32 / CYTOM_WEIGHT_F32 */
  int32_t enable_adaptive_scheduling; /* --enable-adaptive-scheduling (skip inactive tile rows) */
  uint64_t edge_capacity_hint;   /* initial edge capacity; the store grows on demand */
  void* stream;                  /* cudaStream_t to run on; NULL = the context's own stream */
  int32_t traversal;             /* --traversal: CYTOM_TRAVERSAL_* (default row-first) */
  int32_t use_dynamic_compaction; /* --use-dynamic-compaction (default 0, src/scripts/config.py:95):
                                     after an insert, when some tile holds at least its next
                                     threshold of edges (stored + appended; 4096 at first,
                                     doubling past each crossing, TileManager::insertEdge,
                                     tile-manager.h:117, 150-161), the store compacts -- every
                                     tile at once, one merge pass */
} cytom_config;

/* Fills *cfg with the reference defaults (src/scripts/config.py:45-109). */
void cytom_config_default(cytom_config* cfg);

typedef struct cytom_ctx cytom_ctx;

/* Replaces the per-job construction in execute<V,A,w> (src/include/main/execute.h:534-620):
 * Config::normalizeConfig, VertexStore::init (vertex-store.h:25-53) and TileStore::init
 * (tile-store.h:27-74). */
int cytom_create(const cytom_config* cfg, cytom_ctx** out);
/* Replaces VertexStore::destroy / TileStore::destroy (vertex-store.h:55-62, tile-store.h:228-241). */
int cytom_destroy(cytom_ctx* ctx);
const char* cytom_last_error(const cytom_ctx* ctx);
/* Vertex count (power of two) and tiles per dimension after normalisation. */
int cytom_geometry(const cytom_ctx* ctx, uint64_t* vertices, uint64_t* vertices_per_tile,
                   uint64_t* tiles_per_dim);

/* ---- Edge sources ------------------------------------------------------ */

/* RMAT parameters. The reference's RMATContext (src/include/edge-inserter/rmat-context.h:12-82)
 * never stores a, b, c or the vertex count (rmat-context.h:14-15); these are the
 * values it was meant to hold. Defaults: a,b,c = (double)0.57f, 0.19f, 0.19f
 * (RMAT_A/B/C, src/include/util/datatypes.h:17-19). */
typedef struct cytom_rmat_params {
  uint32_t scale;   /* vertices = 2^scale */
  double a, b, c;   /* quadrant probabilities */
  uint64_t seed;    /* RMATContext seed (hash_ = hash(seed)) */
  uint64_t weight_seed; /* weights: wmin + hash(hash(weight_seed) ^ (src<<32|tgt)) % (wmax-wmin+1) */
  uint32_t wmin, wmax;  /* wmax = 0: no weights generated */
} cytom_rmat_params;
void cytom_rmat_default(cytom_rmat_params* p);

/* RMATContext::getEdge(first .. first+count-1) (rmat-context.h:67-73) into src/tgt
 * (and w when p->wmax > 0), on the device (CYTOM_PTR_DEVICE) or copied to host
 * buffers (CYTOM_PTR_HOST). */
int cytom_rmat_generate(cytom_ctx* ctx, const cytom_rmat_params* p, uint64_t first,
                        uint64_t count, uint32_t* src, uint32_t* tgt, uint32_t* w, int where);

/* GridGraph binary reader (Jobs::Jobs + edge_reader_thread, src/include/core/jobs.h:53-64,
 * 111-118): `bytes` holds little-endian {int32 src; int32 tgt} records (no header,
 * src/scripts/convert_graph.py:15-16), size/8 edges. Decodes on the device into
 * src/tgt (device or host per `where`); a negative id or one >= the vertex count is
 * CYTOM_ERR_RANGE (the reference would index out of bounds). *count receives size/8. */
int cytom_gridgraph_decode(cytom_ctx* ctx, const void* bytes, uint64_t size, uint32_t* src,
                           uint32_t* tgt, int where, uint64_t* count);
/* Reads a GridGraph file from disk and inserts its edges in batches of `batch`. */
int cytom_load_gridgraph(cytom_ctx* ctx, const char* path, uint64_t batch, uint64_t* count);

/* ---- Tile store -------------------------------------------------------- */

/* Streaming insert of one batch (IEdgeProvider::processEdge -> MetaTileManager::insertEdge
 * -> TileManager::insertEdge + VertexStore::increment{Out,In}Degree,
 * src/include/edge-inserter/i-edge-provider.h:81-96, meta-tile-manager.h:112-125,
 * tile-manager.h:136-163). Edges join the append region; degrees count every
 * copy (duplicates included). Every live job is notified of every edge
 * (Algorithm::edgeChanged(INSERT), meta-tile-manager.h:192-197). `w` may be NULL
 * for an unweighted store. All ids are checked before anything is inserted. */
int cytom_insert_batch(cytom_ctx* ctx, const uint32_t* src, const uint32_t* tgt,
                       const uint32_t* w, uint64_t count, int where);

/* TileStore::doGlobalCompaction -> TileManager::compactStorage for every tile
 * (tile-store.h:144-172, tile-manager.h:192-291): merges the append region into the
 * sorted tiles and drops duplicate (src,tgt) (for weighted duplicates the minimum
 * weight is kept). Runs implicitly before an algorithm runs. */
int cytom_compact(cytom_ctx* ctx);

/* Drops every stored and pending edge and zeroes the degrees, keeping the context's
 * buffers (their capacity), its tuned kernel shapes and its jobs; every job restarts
 * from scratch on its next run. The reference builds new stores instead
 * (TileStore::init, src/include/core/tile-store.h:27-74; VertexStore::init,
 * vertex-store.h:25-53). */
int cytom_clear(cytom_ctx* ctx);

/* Edge counts: compacted (distinct) edges and edges still in the append region
 * (TileStore::countEdges, tile-store.h:174-185). */
int cytom_count_edges(const cytom_ctx* ctx, uint64_t* compacted, uint64_t* pending);

/* Bit-exact view of the compacted tiles (TileManager::getCounts / getIdCounts /
 * getTargets / getCSRWeights, tile-manager.h:459-467), flattened: tile_ptr[ntiles+1]
 * (host, u64), edges[E] packed (src_local << 16 | tgt_local) in CSR order,
 * weights[E] (NULL to skip) and compact[ntiles] (1 = compact counts_ storage,
 * chosen when distinct sources >= vpt/2, tile-manager.h:261-263; NULL to skip).
 * All outputs are host buffers sized from cytom_count_edges. */
int cytom_get_tiles(cytom_ctx* ctx, uint64_t* tile_ptr, uint32_t* edges, uint32_t* weights,
                    uint8_t* compact);
/* vertex_degree_t {in, out} per vertex (datatypes.h:119-122), host buffers. */
int cytom_get_degrees(cytom_ctx* ctx, uint32_t* out_degree, uint32_t* in_degree);

/* ---- Jobs (vertex programs) -------------------------------------------- */

/* Per-job parameters (ConfigContext::algorithm_config and friends). */
typedef struct cytom_job_params {
  uint64_t start_vertex;   /* --algo-start-id (BFS, SSSP) */
  uint64_t max_iterations; /* --algorithm-iterations per run (reference default 100) */
  double delta;            /* --delta: PR-delta activation threshold */
  double alpha;            /* damping (reference ALPHA 0.85) */
  double tolerance;        /* PageRank / PR-delta: stop when the FP64 L1 residual <= tolerance
                              (relative to the rank sum for PR_DELTA); 0 = reference rule only */
  int32_t kahan;           /* PAGERANK: 1 = FP32 with compensated accumulation, 0 = FP64 plain */
  int32_t reserved;
} cytom_job_params;
void cytom_job_params_default(cytom_job_params* p);

/* Creates a job with its own vertex state (VertexStore<V> + Algorithm::init_vertices,
 * e.g. examples/bfs.cc:170-197). The first run computes from scratch; later runs
 * continue from the previous state, seeded by the edges inserted in between. */
int cytom_job_create(cytom_ctx* ctx, int algo, const cytom_job_params* params, int* job_id);
int cytom_job_destroy(cytom_ctx* ctx, int job_id);
/* Re-initialises a job (ContinuousAlgorithmExecutor::initAlgorithm, continuous-algorithm-executor.h:342). */
int cytom_job_reset(cytom_ctx* ctx, int job_id);

/* Per-run statistics of one job (the counters of continuous-algorithm-executor.h:53-177). */
typedef struct cytom_run_stats {
  uint64_t iterations;     /* pull/apply rounds executed */
  uint64_t count_edges;    /* edges of tiles with an active source, summed over rounds
                              (the reference's processed-edge count, algorithm-executor.h:424-426) */
  uint64_t edges_scanned;  /* edges this engine actually read */
  uint64_t active_vertices;/* vertices activated, summed over rounds */
  int32_t converged;
  int32_t reserved;
  double residual;         /* PageRank: final FP64 L1 residual */
  double elapsed_ms;       /* device time of the run (CUDA events) */
} cytom_run_stats;

/* ContinuousAlgorithmExecutor::executeAlgorithm (continuous-algorithm-executor.h:49-249)
 * for one job: compacts pending edges, then iterates pull -> apply -> swap until no
 * vertex changes or max_iterations. */
int cytom_run(cytom_ctx* ctx, int job_id, cytom_run_stats* stats);
/* Runs several jobs of this context (each listed once), as the reference runs its jobs
 * side by side (one thread per job, src/include/core/jobs.h:79-83). After one shared
 * preparation (compaction, directory), BFS / CC / SSSP / SSWP jobs run concurrently, each
 * on a stream of its own that waits for the context's stream; the context's stream then
 * waits for all of them. Lists with other jobs run one after another. stats: `count`
 * entries or NULL. */
int cytom_run_many(cytom_ctx* ctx, const int* job_ids, int count, cytom_run_stats* stats);
/* The same launch without waiting: returns once the jobs' loops are queued. The next
 * batch may then be inserted and compacted while they run: insertion, sorting and the
 * merge into the alternate buffers overlap the runs, and the context's stream waits for
 * them only where the merged snapshot is installed (and before any call that reads or
 * changes job state). cytom_run_many_wait returns the statistics (`count` entries of the
 * last cytom_run_many_async, or NULL) and must come before the next asynchronous launch.
 * Lists that cannot run side by side run at once and are returned by the wait. */
int cytom_run_many_async(cytom_ctx* ctx, const int* job_ids, int count);
int cytom_run_many_wait(cytom_ctx* ctx, cytom_run_stats* stats);

/* Batched persistent executor. Runs `count` jobs -- job_ids[k] of context ctxs[k]; the
 * contexts (graph snapshots of any size) may differ but must share one device -- together
 * in ONE persistent kernel launch on ctxs[0]'s stream, each job continuing exactly as
 * cytom_run would continue it (same rounds, same results; integer programs bit-exact).
 * The reference runs one executor thread pool per job (Jobs::Jobs starts a thread per
 * job, src/include/core/jobs.h:79-83; each runs ContinuousAlgorithmExecutor::executeAlgorithm,
 * continuous-algorithm-executor.h:49-249); here every job keeps a work queue of units
 * for its current phase (edge stages, frontier-item groups, vertex ranges, target bins)
 * and the blocks of the one launch take units from all jobs. Pending edges of every
 * context are compacted first. stats[k] (may be NULL) as cytom_run; elapsed_ms is the
 * device time of the whole batch. A job may appear once per call. */
int cytom_run_batch(cytom_ctx* const* ctxs, const int* job_ids, int count, cytom_run_stats* stats);
/* Work units processed by batched launches whose first context was ctx (statistics). */
int cytom_batch_units(const cytom_ctx* ctx, uint64_t* units);

/* Result of a job (ResultsWriter dumps vertices_.next, results-writer.h:54-64):
 * BFS levels / CC labels / SSSP distances as uint32 (UINT32_MAX = unreached),
 * PR_DELTA and PAGERANK ranks as float. `out` holds vertices elements. */
int cytom_get_result(cytom_ctx* ctx, int job_id, void* out, int where);
/* FP64 ranks of a PAGERANK job run with kahan = 0 (the FP64 plain form). */
int cytom_get_result_f64(cytom_ctx* ctx, int job_id, double* out, int where);

/* ---- Weighted PageRank: teleport, adjoint, weight updates --------------- */

/* Sets the teleport vector of a WPAGERANK job (`vertices` doubles, host or device;
 * NULL restores the uniform 1/n). A fresh run starts from t. */
int cytom_job_set_teleport(cytom_ctx* ctx, int job_id, const double* teleport, int where);

/* Adjoint of L = sum_v c_v r_v at the converged ranks r of WPAGERANK job `job_id` (run it
 * first; its converged rank vector is the only state kept from the forward). Solves the
 * transposed fixed point lambda = c + alpha (P^T lambda + a (t . lambda)) (a_u = 1 for
 * vertices without out-weight) over the store's edges in source-major orientation, in
 * the job's precision, to an L1 change <= tolerance * |c|_1, then writes
 *   d_weights[e]  = dL/dw_e for every stored edge e = u->k, in the order of
 *                   cytom_get_tiles: alpha r_u / s_u (lambda_k - (P^T lambda)_u)
 *                   (w_e the raw weight, s_u = sum of u's out-weights);
 *   d_teleport[v] = dL/dt_v = ((1-alpha) + alpha D) lambda_v.
 * c: `vertices` doubles (c_where); outputs (out_where) may be NULL to skip.
 * stats: the adjoint's rounds, residual and device time. No counterpart in the reference. */
int cytom_pagerank_adjoint(cytom_ctx* ctx, int job_id, const double* c_weights, int c_where,
                           float* d_weights, float* d_teleport, int out_where, cytom_run_stats* stats);

/* Deletes the stored edges (src[i], tgt[i]) after compacting pending edges; replaces
 * TileManager::deleteEdge / deleteRandomEdge with the compactStorage filter
 * (src/include/tile-manager/tile-manager.h:165-186, 249-253, 532-535) and
 * MetaTileManager::deleteEdge (src/include/tile-manager/meta-tile-manager.h:127-131).
 * A pair listed twice is deleted once; a pair that is not stored is skipped. Each deleted
 * edge lowers out_degree[src] and in_degree[tgt] by one. BFS / CC / SSSP / SSWP jobs for
 * which a deleted edge was tight (it carried its target's value: the reference's
 * critical-neighbour test, meta-tile-manager.h:213-226) restart from scratch on their
 * next run; the others keep their values, which stay exact. PageRank jobs re-converge.
 * *deleted (may be NULL) = edges deleted. */
int cytom_delete_batch(cytom_ctx* ctx, const uint32_t* src, const uint32_t* tgt, uint64_t count, int where,
                       uint64_t* deleted);

/* Deletes `count` randomly picked stored edges: the reference's deletion_percentage mode
 * (src/include/tile-manager/meta-tile-manager.h:201-231 with TileManager::deleteRandomEdge,
 * tile-manager.h:175-190). After compacting pending edges, pick i takes a tile uniformly
 * (hash64(hash64(seed) + 2i) mod tiles, the hash of src/include/util/util.h:188-196) and
 * one of its edges uniformly (hash64(hash64(seed) + 2i + 1) mod its edge count); an empty
 * tile gives no edge. The picks are then deleted as by cytom_delete_batch (a pair picked
 * twice once). src / tgt (both NULL, or `count` words each on the `where` side) receive
 * the picks, UINT32_MAX for none. *deleted (may be NULL) = edges deleted. */
int cytom_delete_random(cytom_ctx* ctx, uint64_t count, uint64_t seed, uint32_t* src, uint32_t* tgt, int where,
                        uint64_t* deleted);

/* Overwrites the weights of stored edges (src[i], tgt[i]) with w[i] (uint32, or float
 * bits in a CYTOM_WEIGHT_F32 store), after compacting pending edges: the weight carried
 * by the reference's Edge (mutate_weight, src/include/edge-inserter/i-edge-provider.h:88)
 * changed in place. Weight-dependent state is rebuilt; SSSP jobs restart from scratch on
 * their next run. An edge that is not stored is CYTOM_ERR_RANGE (the others are updated). */
int cytom_set_edge_weights(cytom_ctx* ctx, const uint32_t* src, const uint32_t* tgt, const uint32_t* w,
                           uint64_t count, int where);

/* ---- On-disk formats --------------------------------------------------- */

/* Edge log (EdgesWriter, src/include/tile-manager/edges-writer.h:114-185): from this call
 * on, every inserted batch is appended to `path` in arrival order, duplicates included,
 * as packed edge_compact_t {u32 src; u32 tgt} records, or edge_compact_weighted_t
 * {u32 src; u32 tgt; float weight} for a weighted store (datatypes.h:55-64). The file is
 * created (truncated); NULL closes the log. */
int cytom_persist_edges(cytom_ctx* ctx, const char* path);
/* Reads an edge log written that way (EdgesWriter::readEdges, edges-writer.h:30-90) and
 * inserts its records in batches of `batch` (0 = 2^20); weighted records for a weighted
 * store. *count receives the records read. */
int cytom_read_edges(cytom_ctx* ctx, const char* path, uint64_t batch, uint64_t* count);
/* Results dump (ResultsWriter::run, src/include/core/results-writer.h:46-81): the job's
 * values as the reference's raw VertexType array, vertex by vertex -- uint32 (BFS, CC),
 * float (SSSP, SSWP; FLT_MAX = not reached / the widest-path start), the 12-byte
 * {float delta_sum; float rank; float delta} (PageRank-delta, examples/pagerank-delta.cc:30-33;
 * delta_sum = delta / alpha, the sum that produced the last delta), float (PageRank). */
int cytom_write_results(cytom_ctx* ctx, int job_id, const char* path);

/* ---- Allocation-free batch compaction ---------------------------------- */

/* No counterpart in the reference. For callers that cannot allocate device memory
 * (an application that owns the device heap through its own pool or arena, or a
 * stream that must not see an allocation): compacts ONE edge batch into the tile
 * store's form -- sorted by (x, y, src_local, tgt_local), duplicates removed (least
 * weight kept), exactly the tiles cytom_get_tiles returns after inserting the batch
 * into an empty store and compacting -- without a context and without allocating.
 * All pointers are device pointers except edge_count (host). tile_ptr holds
 * (T*T + 1) entries for T = vertices (rounded up to a power of two) / vertices_per_tile;
 * edges and weights hold `count` entries (weights only when w is given). count must
 * not exceed CYTOM_NOALLOC_MAX_EDGES (CYTOM_ERR_INVAL otherwise); an id >= vertices
 * rounded up to a power of two (the store's own vertex count, as cytom_create rounds it)
 * is CYTOM_ERR_RANGE and leaves the outputs undefined. Scratch lives in one static device
 * array of CYTOM_NOALLOC_SCRATCH_BYTES per GPU, held until exit and shared by every
 * call: calls that overlap on the GPU race. The first call on a device looks the
 * array up (cudaGetSymbolAddress) with that device current. Every call synchronises
 * `stream` before it returns, so no call can be captured in a CUDA graph. */
#define CYTOM_NOALLOC_MAX_EDGES (1u << 18)
#define CYTOM_NOALLOC_SCRATCH_BYTES ((size_t)9 << 20)
int cytom_tile_batch_noalloc(const uint32_t* src, const uint32_t* tgt, const uint32_t* w,
                             uint64_t count, uint64_t vertices, uint64_t vertices_per_tile,
                             unsigned long long* tile_ptr, uint32_t* edges, uint32_t* weights,
                             uint64_t* edge_count, void* stream);

/* ---- Autotuner ---------------------------------------------------------- */

/* Kernels of the dense round and their shapes (edges per thread, bulk-copy pipeline
 * depth, resident blocks per SM): variants 0-3 stream the tile-major edge array;
 * variant 4 (where vertices_per_tile >= 1024) walks the tiles column by column and
 * reduces each column's targets in shared memory. With the round time each took on the
 * context's graph, per program class (0 = BFS / CC, 1 = SSSP); chosen[k] is the variant
 * in use. No counterpart in the reference (its tile batching, algorithm-tile-batching,
 * is a fixed flag). */
typedef struct cytom_tune_report {
  int32_t variants;
  int32_t chosen[2];
  int32_t edges_per_thread[8];
  int32_t pipeline_depth[8];
  int32_t blocks_per_sm[8];
  int32_t reserved;
  double us[2][8];       /* best of three timed rounds; 0 = not measured */
  uint64_t tuned_edges;  /* edge count the choice was made at (0 = never tuned) */
  /* Sparse-round threshold: a round walks only the listed frontier words (the source
   * directory) while at most 1/sparse_div of the frontier words are non-zero, else it
   * streams every active tile row. Tuned per program class by timing both kinds of
   * round on frontiers with 1/div_candidates[k] of the words non-zero (one active
   * vertex each); sparse_div = the largest such density at which the sparse round was
   * faster. 0 = not tuned (the default 8, or CYTOM_SPARSE_DIV, applies). */
  int32_t sparse_div[2];
  int32_t div_candidates[6];
  double dense_round_us[2][6];
  double sparse_round_us[2][6];
} cytom_tune_report;
/* Times every shape on the current graph (compacting first) and keeps the fastest.
 * Runs by itself once per context, on a job's first run at >= 2^20 edges (environment
 * CYTOM_AUTOTUNE=0 disables that); call it again to re-tune a grown graph. `out` may be NULL. */
int cytom_autotune(cytom_ctx* ctx, cytom_tune_report* out);
int cytom_get_tune_report(const cytom_ctx* ctx, cytom_tune_report* out);

/* ---- Fault injection (tests of the failure paths) ----------------------- */

/* No counterpart in the reference, which aborts on any failure (util::die,
 * src/lib/util/util.cc:21-32). Makes the library's own failure paths run without a GPU
 * fault, so tests can check that they return their status and leave the context usable:
 *  - fail_alloc_after: n > 0 makes the n-th device or pinned-host allocation the library
 *    makes from this call on (any context of the process) fail, once, as
 *    CYTOM_ERR_OOM; 0 turns it off.
 *  - idle_poll_limit: empty polls of the batched executor's bounded idle wait before a
 *    block gives up (CYTOM_ERR_TIMEOUT), for batches whose first context is ctx;
 *    0 = the default, 2^22.
 *  - phantom_jobs: the batched executor counts this many further unfinished jobs that
 *    have no work, so its blocks find none until the idle wait gives up.
 * After a batched run that gave up, its jobs restart from scratch on their next run. */
typedef struct cytom_fault_injection {
  uint64_t fail_alloc_after;
  uint32_t idle_poll_limit;
  uint32_t phantom_jobs;
} cytom_fault_injection;
int cytom_set_fault_injection(cytom_ctx* ctx, const cytom_fault_injection* f);

/* ---- Instrumentation --------------------------------------------------- */

/* Per-kernel-class timing, recorded with CUDA events around each launch when
 * profiling is on (off by default; it serialises launches). */
#define CYTOM_KERNEL_CLASSES 8
typedef struct cytom_kernel_stats {
  char name[CYTOM_KERNEL_CLASSES][24];
  uint64_t launches[CYTOM_KERNEL_CLASSES];
  double total_ms[CYTOM_KERNEL_CLASSES];
  double algo_bytes[CYTOM_KERNEL_CLASSES]; /* algorithmic bytes moved, summed */
} cytom_kernel_stats;
int cytom_set_profiling(cytom_ctx* ctx, int on);
int cytom_get_kernel_stats(cytom_ctx* ctx, cytom_kernel_stats* out);
int cytom_reset_kernel_stats(cytom_ctx* ctx);
/* Number of this library's kernels launched since creation. */
int cytom_launch_count(const cytom_ctx* ctx, uint64_t* launches);
/* Waits for all work of the context's stream. */
int cytom_sync(cytom_ctx* ctx);

#ifdef __cplusplus
}
#endif
#endif
