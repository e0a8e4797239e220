/*
 * cytom_oracle.c — CPU restatement of Cytom's hot path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA engine, never part of it.
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load
 * this library. Build: oracle/Makefile (gcc -O2 -ffp-contract=off).
 *
 * Each function names the reference code (oslab-swrc/cytom, path inside the
 * project) whose behaviour it restates. The restatement is pinned against the
 * reference itself, compiled from its sources into oracle/_ref/.
 */
#include "cytom_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------ */
/* RMAT                                                                      */
/* ------------------------------------------------------------------------ */

/* Ligra 64-bit mixing hash, src/include/util/util.h:188-196. */
uint64_t orc_hash64(uint64_t a) {
  a = (a + 0x7ed55d166bef7a1dULL) + (a << 12);
  a = (a ^ 0xc761c23c510fa2ddULL) ^ (a >> 9);
  a = (a + 0x165667b183a9c0e1ULL) + (a << 59);
  a = (a + 0xd3a2646cab3487e3ULL) ^ (a << 49);
  a = (a + 0xfd7046c5ef9ab54cULL) + (a << 3);
  a = (a ^ 0xb55a4f090dd4a67bULL) ^ (a >> 32);
  return a;
}

/* util::hashDouble, src/include/util/util.h:198-200: hash / (double)UINT64_MAX. */
double orc_hash_double(uint64_t i) {
  return (double)orc_hash64(i) / (double)UINT64_MAX;
}

/*
 * RMATContext::getEdge + rMatIterative, src/include/edge-inserter/rmat-context.h:39-73,
 * with the initialisation the reference constructor omits (rmat-context.h:14-15):
 * a_ = a, ab_ = a + b, abc_ = a + b + c, count_vertices_ = 2^scale, hash_ = hash(seed).
 * Edge i: rand_start = hash(2 i hash_), rand_stride = hash((2 i + 1) hash_);
 * the quadrant for bit j (value 2^j) is chosen by hashDouble(rand_start +
 * (scale-1-j) * rand_stride) against the thresholds a, a+b, a+b+c.
 */
void orc_rmat(uint32_t scale, double a, double b, double c, uint64_t seed,
              uint64_t first, uint64_t count, uint32_t* src, uint32_t* tgt) {
  const double a_ = a, ab_ = a + b, abc_ = a + b + c;
  const uint64_t n = 1ULL << scale;
  const uint64_t h = orc_hash64(seed);
  for (uint64_t k = 0; k < count; ++k) {
    uint64_t index = first + k;
    uint64_t rand_start = orc_hash64(2ULL * index * h);
    uint64_t rand_stride = orc_hash64((2ULL * index + 1ULL) * h);
    uint64_t local_n = n, local_rs = rand_start;
    while (local_n != 1) {
      local_n /= 2;
      local_rs += rand_stride;
    }
    uint64_t es = 0, et = 0;
    while (local_n != n) {
      local_n *= 2;
      local_rs -= rand_stride;
      double r = orc_hash_double(local_rs);
      if (r < a_) {
      } else if (r < ab_) {
        et += local_n / 2;
      } else if (r < abc_) {
        es += local_n / 2;
      } else {
        et += local_n / 2;
        es += local_n / 2;
      }
    }
    src[k] = (uint32_t)es;
    tgt[k] = (uint32_t)et;
  }
}

/* Weight rule for weighted RMAT streams: w = wmin + hash(hash(seed) ^ (src<<32|tgt)) mod
 * (wmax - wmin + 1). The reference draws weights from std::random_device
 * (i-edge-provider.h:86-90), which no run can reproduce; a pure function of
 * (src, tgt) keeps duplicates consistent, so the weight kept by compaction does
 * not depend on sort stability. */
uint32_t orc_edge_weight(uint64_t wseed, uint32_t src, uint32_t tgt, uint32_t wmin,
                         uint32_t wmax) {
  uint64_t k = orc_hash64(wseed) ^ (((uint64_t)src << 32) | (uint64_t)tgt);
  uint64_t span = (uint64_t)wmax - (uint64_t)wmin + 1ULL;
  return wmin + (uint32_t)(orc_hash64(k) % span);
}

void orc_edge_weights(uint64_t wseed, uint32_t wmin, uint32_t wmax, const uint32_t* src,
                      const uint32_t* tgt, uint64_t count, uint32_t* w) {
  for (uint64_t i = 0; i < count; ++i) w[i] = orc_edge_weight(wseed, src[i], tgt[i], wmin, wmax);
}

/* ------------------------------------------------------------------------ */
/* GridGraph binary reader                                                   */
/* ------------------------------------------------------------------------ */

/* Jobs::Jobs mmaps the file and reads count = size / sizeof(file_edge_t) records of
 * {int src; int tgt;} (src/include/core/jobs.h:53-64, datatypes.h:41-44); the
 * writer packs "<l" pairs (src/scripts/convert_graph.py:15-16). */
int64_t orc_gridgraph_decode(const void* bytes, uint64_t size, uint64_t n, uint32_t* src,
                             uint32_t* tgt) {
  const uint8_t* p = (const uint8_t*)bytes;
  uint64_t m = size / 8;
  for (uint64_t i = 0; i < m; ++i) {
    int32_t s, t;
    uint32_t us = (uint32_t)p[8 * i] | ((uint32_t)p[8 * i + 1] << 8) |
                  ((uint32_t)p[8 * i + 2] << 16) | ((uint32_t)p[8 * i + 3] << 24);
    uint32_t ut = (uint32_t)p[8 * i + 4] | ((uint32_t)p[8 * i + 5] << 8) |
                  ((uint32_t)p[8 * i + 6] << 16) | ((uint32_t)p[8 * i + 7] << 24);
    memcpy(&s, &us, 4);
    memcpy(&t, &ut, 4);
    if (s < 0 || t < 0 || (uint64_t)s >= n || (uint64_t)t >= n) return -1;
    src[i] = (uint32_t)s;
    tgt[i] = (uint32_t)t;
  }
  return (int64_t)m;
}

/* ------------------------------------------------------------------------ */
/* Tile store                                                                */
/* ------------------------------------------------------------------------ */

typedef struct {
  /* CSR part after the last compaction, expanded to packed (src<<16 | tgt) in
   * CSR order (TileManager::targets_ with counts_ or id_counts_). */
  uint32_t* csr;
  uint32_t* csr_w;
  uint64_t csr_len, csr_cap;
  /* overflow list edges_ / edges_weights_ in insertion order */
  uint32_t* ovf;
  uint32_t* ovf_w;
  uint64_t ovf_len, ovf_cap;
  uint8_t compact; /* compact_storage_ */
} orc_tile;

struct orc_store {
  uint64_t n, vpt, T, ntiles;
  int weighted;
  orc_tile* tiles;
  uint32_t* out_deg;
  uint32_t* in_deg;
};

orc_store* orc_store_create(uint64_t n, uint64_t vpt, int weighted) {
  if (n == 0 || vpt == 0 || (n & (n - 1)) || (vpt & (vpt - 1)) || vpt > 65536 || vpt > n)
    return NULL;
  orc_store* s = (orc_store*)calloc(1, sizeof(orc_store));
  s->n = n;
  s->vpt = vpt;
  s->T = n / vpt; /* Config::normalizeConfig, src/lib/util/config.cc:18-22 */
  s->ntiles = s->T * s->T;
  s->weighted = weighted;
  s->tiles = (orc_tile*)calloc(s->ntiles, sizeof(orc_tile));
  s->out_deg = (uint32_t*)calloc(n, 4);
  s->in_deg = (uint32_t*)calloc(n, 4);
  return s;
}

void orc_store_destroy(orc_store* s) {
  if (!s) return;
  for (uint64_t t = 0; t < s->ntiles; ++t) {
    free(s->tiles[t].csr);
    free(s->tiles[t].csr_w);
    free(s->tiles[t].ovf);
    free(s->tiles[t].ovf_w);
  }
  free(s->tiles);
  free(s->out_deg);
  free(s->in_deg);
  free(s);
}

static void push2(uint32_t** a, uint32_t** w, uint64_t* len, uint64_t* cap, uint32_t v,
                  uint32_t wv, int weighted) {
  if (*len == *cap) {
    uint64_t nc = *cap ? *cap * 2 : 16;
    *a = (uint32_t*)realloc(*a, nc * 4);
    if (weighted) *w = (uint32_t*)realloc(*w, nc * 4);
    *cap = nc;
  }
  (*a)[*len] = v;
  if (weighted) (*w)[*len] = wv;
  ++*len;
}

/* MetaTileManager::insertEdge (src/include/tile-manager/meta-tile-manager.h:112-125)
 * -> TileStore::getTileManager (tile-store.h:88-96: x = src / vpt, y = tgt / vpt)
 * -> TileManager::insertEdge (tile-manager.h:136-147: local = id & (vpt-1), append to
 * the overflow list) plus out/in-degree increments (vertex-store.h:64-70). */
int orc_store_insert(orc_store* s, const uint32_t* src, const uint32_t* tgt, const uint32_t* w,
                     uint64_t count) {
  for (uint64_t i = 0; i < count; ++i)
    if (src[i] >= s->n || tgt[i] >= s->n) return -1;
  const uint64_t mask = s->vpt - 1;
  for (uint64_t i = 0; i < count; ++i) {
    uint64_t x = src[i] / s->vpt, y = tgt[i] / s->vpt;
    orc_tile* t = &s->tiles[x * s->T + y];
    uint32_t packed = ((uint32_t)(src[i] & mask) << 16) | (uint32_t)(tgt[i] & mask);
    push2(&t->ovf, &t->ovf_w, &t->ovf_len, &t->ovf_cap, packed, w ? w[i] : 0, s->weighted);
    s->out_deg[src[i]]++;
    s->in_deg[tgt[i]]++;
  }
  return 0;
}

typedef struct {
  uint32_t e;
  uint32_t w;
} ew_t;

static int cmp_ew(const void* pa, const void* pb) {
  const ew_t* a = (const ew_t*)pa;
  const ew_t* b = (const ew_t*)pb;
  if (a->e != b->e) return a->e < b->e ? -1 : 1;
  if (a->w != b->w) return a->w < b->w ? -1 : 1;
  return 0;
}

/*
 * TileManager::compactStorage (src/include/tile-manager/tile-manager.h:192-291),
 * copyCSRToEdgeList (:484-516) and fillCSR (:518-565):
 *  - an empty tile returns early and keeps its storage flag;
 *  - CSR edges are appended behind the overflow list and everything is sorted by
 *    (src, tgt) (local_edge_t::operator<, datatypes.h:81-87);
 *  - count_sources = distinct sources of the sorted list; compact storage
 *    (counts_[vpt]) when count_sources >= vpt/2, else sparse id_counts_ runs;
 *  - fillCSR drops an edge equal to the previous one, where "previous" starts as
 *    (UINT16_MAX, UINT16_MAX): a tile whose only edge is (65535, 65535) therefore
 *    comes out empty, exactly as in the reference.
 * Weighted duplicates: the reference keeps whichever weight std::sort's unstable
 * order leaves first (util.h:227-234); this restatement sorts by (edge, weight) and
 * keeps the minimum. With the F2 fix (csr_weights_.reserve instead of resize,
 * tile-manager.h:283) the kept weights line up with the kept targets.
 */
void orc_store_compact(orc_store* s) {
  for (uint64_t ti = 0; ti < s->ntiles; ++ti) {
    orc_tile* t = &s->tiles[ti];
    uint64_t cnt = t->ovf_len + t->csr_len;
    if (cnt == 0) continue;
    ew_t* list = (ew_t*)malloc(cnt * sizeof(ew_t));
    uint64_t k = 0;
    for (uint64_t i = 0; i < t->ovf_len; ++i, ++k) {
      list[k].e = t->ovf[i];
      list[k].w = s->weighted ? t->ovf_w[i] : 0;
    }
    for (uint64_t i = 0; i < t->csr_len; ++i, ++k) {
      list[k].e = t->csr[i];
      list[k].w = s->weighted ? t->csr_w[i] : 0;
    }
    qsort(list, cnt, sizeof(ew_t), cmp_ew);
    uint64_t count_sources = 1;
    uint32_t cur_src = list[0].e >> 16;
    for (uint64_t i = 0; i < cnt; ++i) {
      if ((list[i].e >> 16) != cur_src) {
        cur_src = list[i].e >> 16;
        ++count_sources;
      }
    }
    t->compact = (count_sources >= s->vpt / 2) ? 1 : 0;
    t->csr_len = 0;
    uint32_t prev = 0xFFFFFFFFu; /* (UINT16_MAX, UINT16_MAX) */
    for (uint64_t i = 0; i < cnt; ++i) {
      if (list[i].e == prev) continue;
      prev = list[i].e;
      push2(&t->csr, &t->csr_w, &t->csr_len, &t->csr_cap, list[i].e, list[i].w, s->weighted);
    }
    t->ovf_len = 0;
    free(list);
  }
}

/* Deletion (the working part of TileManager::deleteEdge / compactStorage's deleted-edge
 * filter, tile-manager.h:165-173, 251, 534): pending edges are compacted first, then each
 * listed (src, tgt) is removed from its tile if stored; every removed edge decrements
 * out_deg[src] and in_deg[tgt] once; the compact flag follows the remaining sources.
 * Returns the edges removed (a pair listed twice is removed once). */
uint64_t orc_store_delete(orc_store* s, const uint32_t* src, const uint32_t* tgt, uint64_t count) {
  orc_store_compact(s);
  const uint64_t mask = s->vpt - 1;
  uint64_t removed = 0;
  uint8_t* touched = (uint8_t*)calloc(s->ntiles, 1);
  for (uint64_t i = 0; i < count; ++i) {
    if (src[i] >= s->n || tgt[i] >= s->n) continue;
    const uint64_t ti = (src[i] / s->vpt) * s->T + tgt[i] / s->vpt;
    orc_tile* t = &s->tiles[ti];
    const uint32_t key = ((uint32_t)(src[i] & mask) << 16) | (uint32_t)(tgt[i] & mask);
    uint64_t lo = 0, hi = t->csr_len;
    while (lo < hi) {
      const uint64_t mid = (lo + hi) / 2;
      if (t->csr[mid] < key) lo = mid + 1;
      else hi = mid;
    }
    if (lo >= t->csr_len || t->csr[lo] != key) continue;
    memmove(t->csr + lo, t->csr + lo + 1, (t->csr_len - lo - 1) * 4);
    if (s->weighted) memmove(t->csr_w + lo, t->csr_w + lo + 1, (t->csr_len - lo - 1) * 4);
    t->csr_len--;
    s->out_deg[src[i]]--;
    s->in_deg[tgt[i]]--;
    touched[ti] = 1;
    ++removed;
  }
  for (uint64_t ti = 0; ti < s->ntiles; ++ti) {
    if (!touched[ti]) continue;
    orc_tile* t = &s->tiles[ti];
    uint64_t sources = 0;
    for (uint64_t i = 0; i < t->csr_len; ++i)
      if (i == 0 || (t->csr[i] >> 16) != (t->csr[i - 1] >> 16)) ++sources;
    t->compact = (sources >= s->vpt / 2) ? 1 : 0;
  }
  free(touched);
  return removed;
}

/* Random deletion picks (the reference's deletion_percentage mode,
 * meta-tile-manager.h:201-231 with TileManager::deleteRandomEdge, tile-manager.h:175-190):
 * pick i chooses a tile uniformly (hash64(hash64(seed) + 2i) mod tiles) and, if the tile
 * holds edges, one of them uniformly (hash64(hash64(seed) + 2i + 1) mod its edge count);
 * an empty tile yields no edge (0xFFFFFFFF, 0xFFFFFFFF). Picks are taken from the store
 * after compaction, all from the same snapshot. */
void orc_store_pick_random(orc_store* s, uint64_t count, uint64_t seed, uint32_t* src, uint32_t* tgt) {
  orc_store_compact(s);
  const uint64_t hs = orc_hash64(seed);
  for (uint64_t i = 0; i < count; ++i) {
    const uint64_t ti = orc_hash64(hs + 2 * i) % s->ntiles;
    const orc_tile* t = &s->tiles[ti];
    if (t->csr_len == 0) {
      src[i] = tgt[i] = 0xFFFFFFFFu;
      continue;
    }
    const uint32_t e = t->csr[orc_hash64(hs + 2 * i + 1) % t->csr_len];
    src[i] = (uint32_t)((ti / s->T) * s->vpt) | (e >> 16);
    tgt[i] = (uint32_t)((ti % s->T) * s->vpt) | (e & 0xFFFFu);
  }
}

uint64_t orc_store_count_edges(const orc_store* s) {
  uint64_t c = 0;
  for (uint64_t t = 0; t < s->ntiles; ++t) c += s->tiles[t].csr_len + s->tiles[t].ovf_len;
  return c;
}

uint64_t orc_store_count_tiles(const orc_store* s) { return s->ntiles; }

void orc_store_dump(const orc_store* s, uint64_t* tile_ptr, uint32_t* edges, uint32_t* w,
                    uint8_t* compact) {
  uint64_t off = 0;
  for (uint64_t t = 0; t < s->ntiles; ++t) {
    tile_ptr[t] = off;
    const orc_tile* tl = &s->tiles[t];
    if (edges) memcpy(edges + off, tl->csr, tl->csr_len * 4);
    if (w && s->weighted) memcpy(w + off, tl->csr_w, tl->csr_len * 4);
    if (compact) compact[t] = tl->compact;
    off += tl->csr_len;
  }
  tile_ptr[s->ntiles] = off;
}

void orc_store_degrees(const orc_store* s, uint32_t* out_deg, uint32_t* in_deg) {
  if (out_deg) memcpy(out_deg, s->out_deg, s->n * 4);
  if (in_deg) memcpy(in_deg, s->in_deg, s->n * 4);
}

/* ------------------------------------------------------------------------ */
/* Executors                                                                 */
/* ------------------------------------------------------------------------ */

/* TileManager::isActive with the F1 fix (tile-manager.h:403-427: an 8-byte load
 * where the reference casts one byte): any active vertex in the tile's source range. */
static int row_active(const orc_store* s, const uint8_t* fa, uint64_t x) {
  const uint8_t* p = fa + x * s->vpt;
  for (uint64_t i = 0; i < s->vpt; ++i)
    if (p[i]) return 1;
  return 0;
}

/*
 * ContinuousAlgorithmExecutor::executeAlgorithm (continuous-algorithm-executor.h:72-218)
 * for BFS (examples/bfs.cc), CC (examples/cc.cc) and SSSP (examples/sssp.cc):
 *  pull: every tile with an active source (when adaptive scheduling is on) and at
 *    least one edge counts all its edges (algorithm-executor.h:401-429); each edge
 *    whose source is active (isEdgeActive) gathers from current[src]
 *    (executeAlgorithmSingleEdge[Weighted], :293-399) and the tile-local result is
 *    min-reduced into next, marking changed (applyTiles, :431-505);
 *  apply: BFS/CC over changed vertices, SSSP over all (USE_CHANGED=false): when
 *    next != current copy it and activate (bfs.cc:101-113, cc.cc:101-111,
 *    sssp.cc:323-335); converged when no apply reports a change;
 *  reset: clear active_current, swap with active_next, clear changed
 *    (reset_vertices + :193-215).
 * SSSP distances are the f32 sums of integer weights in the reference; with
 * integer weights < 2^24 they are exact, so this restatement keeps uint32.
 * F3: the SSSP source gets distance 0 (sssp.cc:197-202 commented out upstream).
 */
uint64_t orc_run_minprop(const orc_store* s, int algo, uint64_t start, uint64_t max_iter,
                         int adaptive, uint32_t* values, int* converged,
                         uint64_t* count_edges) {
  const uint64_t n = s->n;
  uint32_t* cur = (uint32_t*)malloc(n * 4);
  uint32_t* next = (uint32_t*)malloc(n * 4);
  uint8_t* fa = (uint8_t*)calloc(n, 1);
  uint8_t* fn = (uint8_t*)calloc(n, 1);
  uint8_t* ch = (uint8_t*)calloc(n, 1);
  /* SSWP (examples/sswp.cc): values start at 0 (unreached), the start vertex at FLT_MAX
   * (here UINT32_MAX); an edge offers max(v, min(u, w)) when u != 0 (pullGatherWeighted,
   * sswp.cc:45-53); reduce = max. */
  const int sswp = (algo == ORC_SSWP);
  for (uint64_t v = 0; v < n; ++v)
    cur[v] = next[v] = sswp ? 0u : ((algo == ORC_CC) ? (uint32_t)v : UINT32_MAX);
  if (algo == ORC_CC) {
    memset(fa, 1, n);
  } else {
    cur[start] = next[start] = sswp ? UINT32_MAX : 0u;
    fa[start] = 1;
  }
  uint64_t edges = 0, it = 0;
  int conv = 0;
  for (it = 0; it < max_iter; ++it) {
    for (uint64_t ti = 0; ti < s->ntiles; ++ti) {
      uint64_t x = ti / s->T, y = ti % s->T;
      const orc_tile* t = &s->tiles[ti];
      if (adaptive && !row_active(s, fa, x)) continue;
      if (t->csr_len + t->ovf_len == 0) continue;
      edges += t->csr_len + t->ovf_len;
      for (int part = 0; part < 2; ++part) {
        const uint32_t* e = part ? t->ovf : t->csr;
        const uint32_t* w = part ? t->ovf_w : t->csr_w;
        uint64_t len = part ? t->ovf_len : t->csr_len;
        for (uint64_t i = 0; i < len; ++i) {
          uint64_t u = x * s->vpt + (e[i] >> 16);
          uint64_t v = y * s->vpt + (e[i] & 0xFFFF);
          if (adaptive && !fa[u]) continue;
          uint32_t uv = cur[u];
          if (sswp) {
            if (uv == 0) continue;
            uint32_t cand = uv < w[i] ? uv : w[i];
            if (cand > next[v]) {
              next[v] = cand;
              ch[v] = 1;
            }
            continue;
          }
          if (uv == UINT32_MAX) continue;
          uint64_t cand;
          if (algo == ORC_BFS) cand = (uint64_t)uv + 1;
          else if (algo == ORC_CC) cand = uv;
          else cand = (uint64_t)uv + w[i];
          if (cand < next[v]) {
            next[v] = (uint32_t)cand;
            ch[v] = 1;
          }
        }
      }
    }
    conv = 1;
    for (uint64_t v = 0; v < n; ++v) {
      if (algo != ORC_SSSP && !sswp && !ch[v]) continue;
      if (next[v] != cur[v]) {
        cur[v] = next[v];
        fn[v] = 1;
        conv = 0;
      }
    }
    if (conv) {
      ++it;
      break;
    }
    memset(fa, 0, n);
    if (it != max_iter - 1) {
      uint8_t* tmp = fa;
      fa = fn;
      fn = tmp;
    }
    memset(ch, 0, n);
  }
  memcpy(values, next, n * 4);
  if (converged) *converged = conv;
  if (count_edges) *count_edges = edges;
  free(cur);
  free(next);
  free(fa);
  free(fn);
  free(ch);
  return it;
}

/*
 * PageRankDelta (examples/pagerank-delta.cc:30-311) driven by one AlgorithmExecutor
 * thread with ATOMICS distribution (algorithm-executor.h:532-557) over RowFirst
 * traversal ids (src/lib/traversal/row_first.cc: d = y*T + x), one ApplyExecutor,
 * adaptive scheduling on. The FP32 operation order is the reference's for that
 * configuration: per tile batch, tile-local delta_sum arrays per target column y in
 * first-use order (getLocalNextArray, :160-200), CSR edges then overflow edges,
 * then next.delta_sum = local + next for non-neutral locals (applyTiles,
 * reduceVertex :238-244). Apply follows pagerank-delta.cc:142-174 with ALPHA 0.85
 * in double, first iteration over all vertices, later ones over changed vertices.
 */
typedef struct {
  float delta_sum, rank, delta;
} prd_t;

uint64_t orc_run_prdelta_ref(const orc_store* s, uint64_t max_iter, double delta, uint64_t batch,
                             float* rank, float* delta_out, int* converged,
                             uint64_t* count_edges) {
  const double ALPHA = 0.85;
  const uint64_t n = s->n, T = s->T, vpt = s->vpt;
  prd_t* cur = (prd_t*)calloc(n, sizeof(prd_t));
  prd_t* next = (prd_t*)calloc(n, sizeof(prd_t));
  uint8_t* fa = (uint8_t*)malloc(n);
  uint8_t* fn = (uint8_t*)calloc(n, 1);
  uint8_t* ch = (uint8_t*)calloc(n, 1);
  memset(fa, 1, n);
  for (uint64_t v = 0; v < n; ++v) cur[v].delta = next[v].delta = 1.0f;
  if (batch == 0) batch = 256;
  float* local = (float*)malloc(batch * vpt * sizeof(float));
  uint64_t* local_y = (uint64_t*)malloc(batch * sizeof(uint64_t));
  int first = 1, conv = 0;
  uint64_t edges = 0, it;
  for (it = 0; it < max_iter; ++it) {
    for (uint64_t b0 = 0; b0 < s->ntiles; b0 += batch) {
      uint64_t b1 = b0 + batch < s->ntiles ? b0 + batch : s->ntiles;
      uint64_t used = 0;
      for (uint64_t d = b0; d < b1; ++d) {
        uint64_t y = d / T, x = d - y * T;
        const orc_tile* t = &s->tiles[x * T + y];
        if (!row_active(s, fa, x)) continue;
        if (t->csr_len + t->ovf_len == 0) continue;
        uint64_t slot = used;
        for (uint64_t q = 0; q < used; ++q)
          if (local_y[q] == y) {
            slot = q;
            break;
          }
        if (slot == used) {
          local_y[used++] = y;
          memset(local + slot * vpt, 0, vpt * sizeof(float));
        }
        float* lv = local + slot * vpt;
        edges += t->csr_len + t->ovf_len;
        for (int part = 0; part < 2; ++part) {
          const uint32_t* e = part ? t->ovf : t->csr;
          uint64_t len = part ? t->ovf_len : t->csr_len;
          for (uint64_t i = 0; i < len; ++i) {
            uint64_t u = x * vpt + (e[i] >> 16);
            if (!fa[u]) continue;
            float c = cur[u].delta / (float)s->out_deg[u];
            lv[e[i] & 0xFFFF] = lv[e[i] & 0xFFFF] + c;
          }
        }
      }
      for (uint64_t q = 0; q < used; ++q) {
        const float* lv = local + q * vpt;
        for (uint64_t j = 0; j < vpt; ++j) {
          if (lv[j] == 0.0f) continue;
          uint64_t g = local_y[q] * vpt + j;
          float nv = lv[j] + next[g].delta_sum;
          if (nv != next[g].delta_sum) {
            next[g].delta_sum = nv;
            ch[g] = 1;
          }
        }
      }
    }
    conv = 1;
    for (uint64_t v = 0; v < n; ++v) {
      if (!first && !ch[v]) continue;
      float ds = next[v].delta_sum;
      if (first) {
        next[v].delta = (float)((1. - ALPHA) + (ALPHA * ds));
        next[v].rank += next[v].delta;
        next[v].delta = (float)((double)next[v].delta - 1.0);
      } else {
        if (ds == 0.0f) {
          cur[v].delta = 0;
          next[v].delta = 0;
          continue;
        }
        next[v].delta = (float)(ALPHA * ds);
        next[v].rank += next[v].delta;
      }
      cur[v].delta = next[v].delta;
      next[v].delta_sum = 0.0f;
      if ((double)fabsf(next[v].delta) > delta * (double)next[v].rank) {
        fn[v] = 1;
        conv = 0;
      }
    }
    if (conv) {
      ++it;
      break;
    }
    first = 0;
    memset(fa, 0, n);
    if (it != max_iter - 1) {
      uint8_t* tmp = fa;
      fa = fn;
      fn = tmp;
    }
    memset(ch, 0, n);
  }
  for (uint64_t v = 0; v < n; ++v) {
    if (rank) rank[v] = next[v].rank;
    if (delta_out) delta_out[v] = next[v].delta;
  }
  if (converged) *converged = conv;
  if (count_edges) *count_edges = edges;
  free(cur);
  free(next);
  free(fa);
  free(fn);
  free(ch);
  free(local);
  free(local_y);
  return it;
}

/* FP64 fixed point of PageRankDelta's recurrence at delta = 0 (pagerank-delta.cc:127-174):
 * rank = (1-alpha) + alpha * sum over edges of rank[u] / out_degree[u], with the
 * vertex store's multiplicity out-degrees (meta-tile-manager.h:123). */
uint64_t orc_pagerank_unnorm_f64(const orc_store* s, double alpha, double tol, uint64_t max_iter,
                                 double* r) {
  const uint64_t n = s->n;
  double* acc = (double*)malloc(n * sizeof(double));
  for (uint64_t v = 0; v < n; ++v) r[v] = 1.0;
  uint64_t it;
  for (it = 0; it < max_iter; ++it) {
    memset(acc, 0, n * sizeof(double));
    for (uint64_t ti = 0; ti < s->ntiles; ++ti) {
      uint64_t x = ti / s->T, y = ti % s->T;
      const orc_tile* t = &s->tiles[ti];
      for (int part = 0; part < 2; ++part) {
        const uint32_t* e = part ? t->ovf : t->csr;
        uint64_t len = part ? t->ovf_len : t->csr_len;
        for (uint64_t i = 0; i < len; ++i) {
          uint64_t u = x * s->vpt + (e[i] >> 16);
          uint64_t v = y * s->vpt + (e[i] & 0xFFFF);
          acc[v] += r[u] / (double)s->out_deg[u];
        }
      }
    }
    double diff = 0.0, tot = 0.0;
    for (uint64_t v = 0; v < n; ++v) {
      double nv = (1.0 - alpha) + alpha * acc[v];
      diff += fabs(nv - r[v]);
      tot += nv;
      r[v] = nv;
    }
    if (diff <= tol * tot) {
      ++it;
      break;
    }
  }
  free(acc);
  return it;
}

uint64_t orc_pagerank_norm_f64(const orc_store* s, double alpha, double tol, uint64_t max_iter,
                               double* r) {
  const uint64_t n = s->n;
  double* acc = (double*)malloc(n * sizeof(double));
  uint32_t* deg = (uint32_t*)calloc(n, 4);
  for (uint64_t ti = 0; ti < s->ntiles; ++ti) {
    uint64_t x = ti / s->T;
    const orc_tile* t = &s->tiles[ti];
    for (uint64_t i = 0; i < t->csr_len; ++i) deg[x * s->vpt + (t->csr[i] >> 16)]++;
  }
  for (uint64_t v = 0; v < n; ++v) r[v] = 1.0 / (double)n;
  uint64_t it;
  for (it = 0; it < max_iter; ++it) {
    memset(acc, 0, n * sizeof(double));
    double dangling = 0.0;
    for (uint64_t v = 0; v < n; ++v)
      if (deg[v] == 0) dangling += r[v];
    for (uint64_t ti = 0; ti < s->ntiles; ++ti) {
      uint64_t x = ti / s->T, y = ti % s->T;
      const orc_tile* t = &s->tiles[ti];
      for (uint64_t i = 0; i < t->csr_len; ++i) {
        uint64_t u = x * s->vpt + (t->csr[i] >> 16);
        uint64_t v = y * s->vpt + (t->csr[i] & 0xFFFF);
        acc[v] += r[u] / (double)deg[u];
      }
    }
    double diff = 0.0;
    const double base = (1.0 - alpha) / (double)n + alpha * dangling / (double)n;
    for (uint64_t v = 0; v < n; ++v) {
      double nv = base + alpha * acc[v];
      diff += fabs(nv - r[v]);
      r[v] = nv;
    }
    if (diff <= tol) {
      ++it;
      break;
    }
  }
  free(acc);
  free(deg);
  return it;
}

/* ------------------------------------------------------------------------ */
/* Weighted PageRank and its adjoint (FP64). The reference has no weighted    */
/* PageRank (pullGatherWeighted is "not applicable", examples/pagerank.cc:98, */
/* examples/pagerank-delta.cc:134-140); this is a restatement of the model:   */
/*   r = (1-alpha) t + alpha (P r + D t),  P[v,u] = w_uv / s_u,               */
/*   s_u = sum of u's out-weights, D = sum of r over vertices with s_u = 0,   */
/* and of its adjoint for L = c . r (derivation in orc_wpagerank_adjoint_f64). */
/* ------------------------------------------------------------------------ */

static double* wsum_of(uint64_t n, uint64_t m, const uint32_t* src, const double* w) {
  double* s = (double*)calloc(n, sizeof(double));
  for (uint64_t e = 0; e < m; ++e) s[src[e]] += w[e];
  return s;
}

uint64_t orc_wpagerank_f64(uint64_t n, uint64_t m, const uint32_t* src, const uint32_t* tgt,
                           const double* w, const double* t, double alpha, double tol,
                           uint64_t max_iter, double* r) {
  double* s = wsum_of(n, m, src, w);
  double* acc = (double*)malloc(n * sizeof(double));
  const double tu = 1.0 / (double)n;
  for (uint64_t v = 0; v < n; ++v) r[v] = t ? t[v] : tu;
  uint64_t it;
  for (it = 0; it < max_iter; ++it) {
    memset(acc, 0, n * sizeof(double));
    double dang = 0.0;
    for (uint64_t u = 0; u < n; ++u)
      if (s[u] == 0.0) dang += r[u];
    for (uint64_t e = 0; e < m; ++e) acc[tgt[e]] += w[e] / s[src[e]] * r[src[e]];
    double diff = 0.0;
    for (uint64_t v = 0; v < n; ++v) {
      const double tv = t ? t[v] : tu;
      const double nv = (1.0 - alpha) * tv + alpha * (acc[v] + dang * tv);
      diff += fabs(nv - r[v]);
      r[v] = nv;
    }
    if (diff <= tol) {
      ++it;
      break;
    }
  }
  free(acc);
  free(s);
  return it;
}

/* With M = P + t a^T (a_u = 1 when s_u = 0), the fixed point is (I - alpha M) r =
 * (1-alpha) t, so for L = c . r:
 *   lambda = c + alpha M^T lambda = c + alpha (P^T lambda + a (t . lambda)),
 *   dL/dw_uk = alpha r_u / s_u (lambda_k - (P^T lambda)_u)   (edge u->k, raw weight),
 *   dL/dt_v  = ((1-alpha) + alpha D) lambda_v.
 * lambda is iterated to an L1 change <= tol * sum|c|. g_w[e] follows the edge arrays. */
uint64_t orc_wpagerank_adjoint_f64(uint64_t n, uint64_t m, const uint32_t* src, const uint32_t* tgt,
                                   const double* w, const double* t, double alpha, double tol,
                                   uint64_t max_iter, const double* r, const double* c,
                                   double* lambda, double* g_w, double* g_t) {
  double* s = wsum_of(n, m, src, w);
  double* pt = (double*)malloc(n * sizeof(double));
  const double tu = 1.0 / (double)n;
  double cn = 0.0;
  for (uint64_t v = 0; v < n; ++v) {
    lambda[v] = c[v];
    cn += fabs(c[v]);
  }
  uint64_t it;
  for (it = 0; it < max_iter; ++it) {
    memset(pt, 0, n * sizeof(double));
    double tl = 0.0;
    for (uint64_t v = 0; v < n; ++v) tl += (t ? t[v] : tu) * lambda[v];
    for (uint64_t e = 0; e < m; ++e) pt[src[e]] += w[e] / s[src[e]] * lambda[tgt[e]];
    double diff = 0.0;
    for (uint64_t u = 0; u < n; ++u) {
      const double nl = c[u] + alpha * (pt[u] + (s[u] == 0.0 ? tl : 0.0));
      diff += fabs(nl - lambda[u]);
      lambda[u] = nl;
    }
    if (diff <= tol * cn) {
      ++it;
      break;
    }
  }
  /* (P^T lambda) at the final lambda */
  memset(pt, 0, n * sizeof(double));
  for (uint64_t e = 0; e < m; ++e) pt[src[e]] += w[e] / s[src[e]] * lambda[tgt[e]];
  double dang = 0.0;
  for (uint64_t u = 0; u < n; ++u)
    if (s[u] == 0.0) dang += r[u];
  if (g_w)
    for (uint64_t e = 0; e < m; ++e) {
      const uint32_t u = src[e];
      g_w[e] = alpha * r[u] / s[u] * (lambda[tgt[e]] - pt[u]);
    }
  if (g_t)
    for (uint64_t v = 0; v < n; ++v) g_t[v] = ((1.0 - alpha) + alpha * dang) * lambda[v];
  free(pt);
  free(s);
  return it;
}
