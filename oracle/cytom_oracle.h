/*
 * cytom_oracle.h — CPU restatement of Cytom's hot path.
 *
 * TEST INFRASTRUCTURE ONLY. Nothing in the product (libcytom_gpu.so, the
 * cytom_gb300 package) links, loads or calls this code. Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg use it, as the
 * checker.
 *
 * Every function restates the reference algorithm it names (file:line inside
 * the oslab-swrc/cytom project). Where the reference is broken (bitmap byte
 * casts, zeroed CSR weights, SSSP source never initialised) this restatement
 * follows the reference with the fix applied, and says so.
 *
 * Parity pin: the restatement is checked against the reference's own
 * TileManager / ContinuousAlgorithmExecutor, compiled from its sources by
 * oracle/ref/Makefile into oracle/_ref/ (tests/test_oracle_pin.py).
 */
#ifndef CYTOM_ORACLE_H
#define CYTOM_ORACLE_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- RMAT generator (inc/edge-inserter/rmat-context.h:39-73) ---------- */
uint64_t orc_hash64(uint64_t a);            /* inc/util/util.h:188-196 */
double orc_hash_double(uint64_t i);         /* inc/util/util.h:198-200 */
void orc_rmat(uint32_t scale, double a, double b, double c, uint64_t seed,
              uint64_t first, uint64_t count, uint32_t* src, uint32_t* tgt);
/* Deterministic integer edge weight in [wmin, wmax] from (seed, src, tgt):
 * duplicates of one (src,tgt) carry one weight. */
uint32_t orc_edge_weight(uint64_t wseed, uint32_t src, uint32_t tgt,
                         uint32_t wmin, uint32_t wmax);
void orc_edge_weights(uint64_t wseed, uint32_t wmin, uint32_t wmax,
                      const uint32_t* src, const uint32_t* tgt, uint64_t count,
                      uint32_t* w);

/* ---- GridGraph binary format (inc/core/jobs.h:53-64, datatypes.h:41-44) */
/* Decodes little-endian int32 pairs; returns count of edges or -1 when an id
 * is negative or >= n (the reference would index out of range). */
int64_t orc_gridgraph_decode(const void* bytes, uint64_t size, uint64_t n,
                             uint32_t* src, uint32_t* tgt);

/* ---- Tile store (inc/core/tile-store.h, inc/tile-manager/tile-manager.h) */
typedef struct orc_store orc_store;
orc_store* orc_store_create(uint64_t n, uint64_t vpt, int weighted);
void orc_store_destroy(orc_store* s);
/* MetaTileManager::insertEdge (meta-tile-manager.h:112-125): overflow append
 * + degree increments (duplicates counted). Returns 0, or -1 on a bad id. */
int orc_store_insert(orc_store* s, const uint32_t* src, const uint32_t* tgt,
                     const uint32_t* w, uint64_t count);
/* TileStore::doGlobalCompaction -> TileManager::compactStorage per tile. */
void orc_store_compact(orc_store* s);
uint64_t orc_store_count_edges(const orc_store* s); /* CSR + overflow */
/* Removes stored (src, tgt) pairs after compacting; degrees drop by one per removed
 * edge. Returns the edges removed. */
uint64_t orc_store_delete(orc_store* s, const uint32_t* src, const uint32_t* tgt, uint64_t count);
/* Random deletion picks: uniform tile, then a uniform edge in it (none for an empty tile:
 * 0xFFFFFFFF twice), hash-seeded, from the compacted store. */
void orc_store_pick_random(orc_store* s, uint64_t count, uint64_t seed, uint32_t* src, uint32_t* tgt);
uint64_t orc_store_count_tiles(const orc_store* s);
/* Dump of the compacted CSR part in tile-id order (id = x*T + y):
 * tile_ptr[ntiles+1], packed edges (src_l<<16 | tgt_l), weights (nullable),
 * compact flags per tile (nullable). */
void orc_store_dump(const orc_store* s, uint64_t* tile_ptr, uint32_t* edges,
                    uint32_t* w, uint8_t* compact);
void orc_store_degrees(const orc_store* s, uint32_t* out_deg, uint32_t* in_deg);

/* ---- Executors (inc/core/continuous-algorithm-executor.h:49-249) ------- */
enum { ORC_BFS = 0, ORC_CC = 1, ORC_SSSP = 2, ORC_SSWP = 3 };
/* From-scratch run of BFS / CC / SSSP / SSWP with the reference's Jacobi iteration
 * (pull over tiles with an active source, reduce into next, apply changed,
 * swap active bitmaps). values[n] receives the result (UINT32_MAX = not
 * reached). Returns iterations executed; *converged and the reference's
 * per-run edge count (edges of active tiles, algorithm-executor.h:424-426)
 * are reported. */
uint64_t orc_run_minprop(const orc_store* s, int algo, uint64_t start,
                         uint64_t max_iter, int adaptive, uint32_t* values,
                         int* converged, uint64_t* count_edges);

/* PageRankDelta (examples/pagerank-delta.cc) in the reference's exact FP32
 * operation order for one executor thread with ATOMICS tile distribution,
 * RowFirst traversal and algorithm-tile-batching = batch. rank/delta/dsum
 * (n each) receive the final `next` fields. Returns iterations. */
uint64_t orc_run_prdelta_ref(const orc_store* s, uint64_t max_iter,
                             double delta, uint64_t batch, float* rank,
                             float* delta_out, int* converged,
                             uint64_t* count_edges);

/* FP64 fixed point of the unnormalised PageRank that PageRankDelta converges
 * to at delta = 0: r = (1-alpha) + alpha * sum_{u->v} r_u / outdeg(u), over
 * the store's edges (CSR + overflow) with multiplicity out-degrees. Returns
 * iterations; stops when the L1 change <= tol * sum(r). */
uint64_t orc_pagerank_unnorm_f64(const orc_store* s, double alpha, double tol,
                                 uint64_t max_iter, double* r);

/* Normalised PageRank with dangling mass redistributed uniformly, FP64:
 * r = (1-alpha)/n + alpha * (sum_{u->v} r_u/outdeg(u) + D/n), D = sum of r
 * over vertices with outdeg 0; L1 stop at tol. Edges: the compacted store
 * (deduplicated), out-degree = distinct out-edges. */
uint64_t orc_pagerank_norm_f64(const orc_store* s, double alpha, double tol,
                               uint64_t max_iter, double* r);

/* Weighted PageRank with teleport vector t (NULL = uniform 1/n), dangling mass sent
 * along t, FP64, over m edges given as arrays (raw weights w, normalised per source):
 * r = (1-alpha) t + alpha (P r + D t), P[v,u] = w_uv / s_u. Stops at an L1 change
 * <= tol. Returns iterations. The reference has no weighted PageRank. */
uint64_t orc_wpagerank_f64(uint64_t n, uint64_t m, const uint32_t* src, const uint32_t* tgt,
                           const double* w, const double* t, double alpha, double tol,
                           uint64_t max_iter, double* r);
/* Adjoint of L = c . r at the fixed point r: lambda = c + alpha (P^T lambda + a (t . lambda))
 * (L1 change <= tol * |c|_1), then dL/dw for every edge (g_w, in the arrays' order) and
 * dL/dt (g_t); either may be NULL. Returns iterations. */
uint64_t orc_wpagerank_adjoint_f64(uint64_t n, uint64_t m, const uint32_t* src, const uint32_t* tgt,
                                   const double* w, const double* t, double alpha, double tol,
                                   uint64_t max_iter, const double* r, const double* c,
                                   double* lambda, double* g_w, double* g_t);

#ifdef __cplusplus
}
#endif
#endif
