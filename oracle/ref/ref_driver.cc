// ref_driver.cc — runs the reference's own hot-path code on an edge list.
//
// TEST INFRASTRUCTURE ONLY (the parity pin and the CPU baseline). It constructs the
// reference's VertexStore, TileStore/TileManager and ContinuousAlgorithmExecutor with
// the example vertex programs (examples/bfs.cc, cc.cc, sssp.cc, pagerank-delta.cc),
// compiled from the reference sources by oracle/ref/Makefile with fixes F1 (8-byte
// bitmap block loads) and F2 (csr_weights_.reserve) applied; F3 (SSSP source distance
// 0) is applied here after initAlgorithm.
//
// usage: ref_driver <mode> <n> <vpt> <edges.bin> <out.bin> <batch> <executors>
//                   <max_iter> <delta> <start> <adaptive>
//   mode: compact | bfs | cc | sssp | prdelta | stream | istream
//   edges.bin: u64 count, u32 weighted, u32[count] src, u32[count] tgt, [u32[count] w]
#include <float.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include <memory>
#include <string>
#include <vector>

#include "util/datatypes.h"
#include "util/config.h"
#include "core/vertex-store.h"
#include "tile-manager/tile-manager.h"
#include "core/tile-store.h"
#include "core/continuous-algorithm-executor.h"
#include "traversal/row_first.h"
#include "examples/bfs.cc"
#include "examples/cc.cc"
#include "examples/sssp.cc"
#include "examples/pagerank-delta.cc"

namespace evolving_graphs {
// The ring buffer moves nothing with ATOMICS tile distribution.
Ringbuffer::Ringbuffer() : rb_(nullptr) {}
Ringbuffer::Ringbuffer(const Ringbuffer& other) : rb_(other.rb_) {}
Ringbuffer::~Ringbuffer() {}
int Ringbuffer::create(size_t, size_t, bool, ring_buffer_reap_cb_t, void*) { return 0; }
void Ringbuffer::init() {}
void Ringbuffer::destroy() {}
int Ringbuffer::put(ring_buffer_req_t*) { return 0; }
int Ringbuffer::get(ring_buffer_req_t*) { return 0; }
void Ringbuffer::set_ready(ring_buffer_req_t*) {}
void Ringbuffer::set_ready(void*) {}
void Ringbuffer::set_done(ring_buffer_req_t*) {}
void Ringbuffer::set_done(void*) {}
int Ringbuffer::putNoLock(ring_buffer_req_t*) { return 0; }
int Ringbuffer::getNoLock(ring_buffer_req_t*) { return 0; }
bool Ringbuffer::isFull() { return false; }
bool Ringbuffer::isEmpty() { return true; }
size_t Ringbuffer::getFreeSpace() { return 0; }
int Ringbuffer::copyToBuffer(void*, const void*, size_t) { return 0; }
int Ringbuffer::copyFromBuffer(void*, const void*, size_t) { return 0; }
ring_buffer_t* Ringbuffer::rb() { return rb_; }

namespace util {
void __die(int rc, const char* func, int line) {
  fprintf(stderr, "reference died (%d) in %s:%d\n", rc, func, line);
  exit(3);
}
void sendMessage(Ringbuffer&, flatbuffers::FlatBufferBuilder&) {}
cpu_id_t& cpu_id_t::nextNearest(bool) { return *this; }
Runnable::Runnable() : cpu_id_(cpu_id_t::ANYWHERE, cpu_id_t::ANYWHERE, cpu_id_t::ANYWHERE) {}
Runnable::~Runnable() {}
void Runnable::setAffinity(cpu_id_t&) {}
void Runnable::setHighestPriority() {}
int Runnable::start() { return pthread_create(&t_, nullptr, &Runnable::threadMain, this); }
void Runnable::setName(const std::string&) {}
void Runnable::join() { pthread_join(t_, nullptr); }
void* Runnable::threadMain(void* arg) {
  static_cast<Runnable*>(arg)->run();
  return nullptr;
}
}  // namespace util
}  // namespace evolving_graphs

using namespace evolving_graphs;

struct Args {
  std::string mode;
  uint64_t n, vpt, batch, execs, max_iter, start;
  double delta;
  int adaptive;
  std::vector<uint32_t> src, tgt, w;
  bool weighted;
};

static double now_s() {
  timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return ts.tv_sec + ts.tv_nsec * 1e-9;
}

static std::shared_ptr<Config> make_config(const Args& a, uint64_t execs) {
  auto config = std::make_shared<Config>();
  ConfigContext& c = config->context_;
  c.max_count_vertices = a.n;
  c.tile_store_config.vertices_per_tile = a.vpt;
  c.tile_store_config.td_count_meta_tiles_per_dimension = 0;
  c.tile_store_config.td_count_tiles_per_meta_tiles_per_dimension = 1;
  c.tile_store_config.td_count_tiles_per_meta_tiles = 1;
  config->normalizeConfig();
  c.batch_insertion_count = a.batch;
  c.count_edges = a.src.size();
  c.count_parallel_compaction = 1;
  c.algorithm_tile_batching = 256;
  c.algorithm_iterations = a.max_iter;
  c.meta_tile_manager_count = 1;
  c.edge_inserters_count = 1;
  c.algorithm_executor_count = (uint8_t)execs;
  c.algorithm_appliers_count = (uint8_t)execs;
  c.use_dynamic_compaction = false;
  c.enable_static_algorithm_before_compaction = false;
  c.enable_static_algorithm_after_compaction = true;
  c.enable_dynamic_algorithm = false;
  c.enable_perf_event_collection = false;
  c.enable_edge_apis = true;
  c.enable_rewrite_ids = false;
  c.enable_lazy_algorithm = false;
  c.enable_adaptive_scheduling = a.adaptive != 0;
  c.enable_in_memory_ingestion = false;
  c.enable_algorithm_reexecution = false;
  c.enable_write_results = false;
  c.detailed_tile_stats = false;
  c.deletion_percentage = 0.0;
  c.traversal = traversal_t::ROW_FIRST;
  c.generator = edge_generator_t::BINARY_EDGES;
  c.tile_distribution = tile_distribution_t::ATOMICS;
  c.min_count_edges_algorithm = 0;
  c.algorithm_config.algo_start_id = a.start;
  c.algorithm_config.delta = a.delta;
  c.persistence_config.enable_writing_edges = false;
  c.persistence_config.enable_reading_edges = false;
  return config;
}

// One reference job: its own VertexStore and TileStore (execute<V,A,w> builds one per job).
template <typename V, class A, bool W>
struct Job {
  std::shared_ptr<Config> config;
  RowFirst traversal;
  std::shared_ptr<VertexStore<V>> vs;
  std::shared_ptr<TileStore<V, A, W>> ts;
  Job(const Args& a, uint64_t execs) {
    config = make_config(a, execs);
    vs = std::make_shared<VertexStore<V>>();
    vs->init(config->context_.max_count_vertices);
    ts = std::make_shared<TileStore<V, A, W>>(config);
    ts->init(&traversal, vs);
  }
  // MetaTileManager::insertEdge (meta-tile-manager.h:112-125) for edges [lo, hi)
  void insert(const Args& a, uint64_t lo, uint64_t hi) {
    for (uint64_t i = lo; i < hi; ++i) {
      Edge e(a.src[i], a.tgt[i], W ? (float)a.w[i] : 0.0f);
      ts->getTileManager(e)->insertEdge(e);
      vs->incrementOutDegree(a.src[i]);
      vs->incrementInDegree(a.tgt[i]);
    }
  }
  // ContinuousAlgorithmExecutor::initAlgorithm + executeAlgorithm on the current store.
  uint64_t run(const Args& a, bool* converged, double* secs) {
    auto algo = std::make_shared<A>(config, vs);
    auto pem = std::make_shared<perf_event::PerfEventManager>();
    Ringbuffer rb;
    ContinuousAlgorithmExecutor<V, A, W> cae(rb, &traversal, "ref", config, pem, algo, vs);
    cae.initAlgorithm();
    fix_start(a);
    cae.init(vs, ts, std::shared_ptr<MetaTileStore<V, A, W>>(), pem);
    uint64_t count = 0;
    double t0 = now_s();
    cae.executeAlgorithm(ts->countEdges(), converged, &count);
    *secs = now_s() - t0;
    cae.destroy();
    return count;
  }
  void fix_start(const Args& a);
};

template <typename V, class A, bool W>
void Job<V, A, W>::fix_start(const Args&) {}
template <>
void Job<float, algorithm::SSSP, true>::fix_start(const Args& a) {
  // F3: examples/sssp.cc:197-202 (commented out upstream) sets the source distance to 0.
  vs->vertices_.current[a.start] = 0.0f;
  vs->vertices_.next[a.start] = 0.0f;
}

// One reference job run incrementally, as the reference's EdgeInserter drives it with
// enable_edge_apis (src/include/edge-inserter/edge-inserter.h:129-184): every inserted
// edge goes through MetaTileManager::insertEdge (tile insert + degrees,
// meta-tile-manager.h:112-125) and then Algorithm::edgeChanged(INSERT)
// (meta-tile-manager.h:192-198); after the batch's compaction one executeAlgorithm call
// continues from the vertex state. One executor object lives across batches. Left out:
// the swap of the active bitmaps right before the run (edge-inserter.h:150-151), which
// moves the frontier edgeChanged seeded out of the first round so that the run stops
// after one round (fix F5).
template <typename V, class A, bool W>
struct IncJob {
  Job<V, A, W> base;
  std::shared_ptr<A> algo;
  std::shared_ptr<perf_event::PerfEventManager> pem;
  Ringbuffer rb;
  ContinuousAlgorithmExecutor<V, A, W>* cae = nullptr;
  IncJob(const Args& a, uint64_t execs) : base(a, execs) {
    algo = std::make_shared<A>(base.config, base.vs);
    pem = std::make_shared<perf_event::PerfEventManager>();
    cae = new ContinuousAlgorithmExecutor<V, A, W>(rb, &base.traversal, "ref", base.config, pem, algo, base.vs);
    cae->initAlgorithm();
    base.fix_start(a);
    cae->init(base.vs, base.ts, std::shared_ptr<MetaTileStore<V, A, W>>(), pem);
  }
  ~IncJob() {
    cae->destroy();
    delete cae;
  }
  void insert(const Args& a, uint64_t lo, uint64_t hi) {
    for (uint64_t i = lo; i < hi; ++i) {
      Edge e(a.src[i], a.tgt[i], W ? (float)a.w[i] : 0.0f);
      base.ts->getTileManager(e)->insertEdge(e);
      base.vs->incrementOutDegree(a.src[i]);
      base.vs->incrementInDegree(a.tgt[i]);
      algo->edgeChanged(e, EdgeChangeEvent::INSERT);
    }
  }
  uint64_t run(bool* converged) {
    uint64_t count = 0;
    cae->executeAlgorithm(base.ts->countEdges(), converged, &count);
    return count;
  }
};

template <class J>
static void insert_all(J& job, const Args& a) {
  uint64_t m = a.src.size();
  for (uint64_t lo = 0; lo < m; lo += a.batch) {
    uint64_t hi = lo + a.batch < m ? lo + a.batch : m;
    job.insert(a, lo, hi);
    job.ts->doGlobalCompaction();
  }
}

static void write_or_die(FILE* f, const void* p, size_t bytes) {
  if (bytes && fwrite(p, 1, bytes, f) != bytes) {
    perror("write");
    exit(2);
  }
}

int main(int argc, char** argv) {
  if (argc < 12) {
    fprintf(stderr, "usage: %s mode n vpt edges.bin out.bin batch executors max_iter delta start adaptive\n", argv[0]);
    return 1;
  }
  Args a;
  a.mode = argv[1];
  a.n = strtoull(argv[2], 0, 10);
  a.vpt = strtoull(argv[3], 0, 10);
  a.batch = strtoull(argv[6], 0, 10);
  a.execs = strtoull(argv[7], 0, 10);
  a.max_iter = strtoull(argv[8], 0, 10);
  a.delta = strtod(argv[9], 0);
  a.start = strtoull(argv[10], 0, 10);
  a.adaptive = atoi(argv[11]);
  FILE* f = fopen(argv[4], "rb");
  if (!f) return 2;
  uint64_t m = 0;
  uint32_t wflag = 0;
  if (fread(&m, 8, 1, f) != 1 || fread(&wflag, 4, 1, f) != 1) return 2;
  a.weighted = wflag != 0;
  a.src.resize(m);
  a.tgt.resize(m);
  if (fread(a.src.data(), 4, m, f) != m || fread(a.tgt.data(), 4, m, f) != m) return 2;
  if (a.weighted) {
    a.w.resize(m);
    if (fread(a.w.data(), 4, m, f) != m) return 2;
  }
  fclose(f);
  if (a.batch == 0) a.batch = m ? m : 1;
  FILE* out = fopen(argv[5], "wb");
  if (!out) return 2;

  if (a.mode == "compact") {
    // weighted stores keep their (float) weights through compaction
    Job<float, algorithm::SSSP, true> job(a, 1);
    double t0 = now_s();
    insert_all(job, a);
    double secs = now_s() - t0;
    const uint64_t T = job.config->context_.tile_store_config.count_tiles_per_dimension;
    std::vector<uint64_t> tp(T * T + 1, 0);
    std::vector<uint8_t> cf(T * T, 0);
    std::vector<uint32_t> ed, wt;
    for (uint64_t x = 0; x < T; ++x)
      for (uint64_t y = 0; y < T; ++y) {
        auto* tm = job.ts->getTileManager(Coordinates{x, y});
        tp[x * T + y] = ed.size();
        cf[x * T + y] = tm->isCompactStorage() ? 1 : 0;
        // expand the CSR exactly as executeAlgoOnTile walks it (algorithm-executor.h:228-272)
        auto* targets = tm->getTargets();
        auto* weights = tm->getCSRWeights();
        uint32_t cur = 0;
        if (tm->isCompactStorage()) {
          local_vertex_id_t* counts = tm->getCounts();
          for (uint64_t s = 0; s < a.vpt; ++s)
            for (uint32_t k = 0; k < counts[s]; ++k, ++cur) {
              ed.push_back(((uint32_t)s << 16) | (*targets)[cur]);
              wt.push_back(a.weighted ? (uint32_t)(*weights)[cur] : 0u);
            }
        } else {
          for (const auto& src : *tm->getIdCounts())
            for (uint32_t k = 0; k < src.count; ++k, ++cur) {
              ed.push_back(((uint32_t)src.id << 16) | (*targets)[cur]);
              wt.push_back(a.weighted ? (uint32_t)(*weights)[cur] : 0u);
            }
        }
      }
    tp[T * T] = ed.size();
    uint64_t hdr[2] = {T * T, (uint64_t)ed.size()};
    write_or_die(out, hdr, sizeof(hdr));
    write_or_die(out, tp.data(), tp.size() * 8);
    write_or_die(out, cf.data(), cf.size());
    write_or_die(out, ed.data(), ed.size() * 4);
    write_or_die(out, wt.data(), wt.size() * 4);
    double res[1] = {secs};
    write_or_die(out, res, 8);
  } else if (a.mode == "bfs" || a.mode == "cc" || a.mode == "sssp" || a.mode == "prdelta") {
    bool conv = false;
    double secs = 0;
    uint64_t cnt = 0;
    std::vector<uint32_t> vals(a.n);
    if (a.mode == "bfs") {
      Job<uint32_t, algorithm::BFS, false> job(a, a.execs);
      insert_all(job, a);
      cnt = job.run(a, &conv, &secs);
      for (uint64_t v = 0; v < a.n; ++v) vals[v] = job.vs->vertices_.next[v];
    } else if (a.mode == "cc") {
      Job<uint32_t, algorithm::CC, false> job(a, a.execs);
      insert_all(job, a);
      cnt = job.run(a, &conv, &secs);
      for (uint64_t v = 0; v < a.n; ++v) vals[v] = job.vs->vertices_.next[v];
    } else if (a.mode == "sssp") {
      Job<float, algorithm::SSSP, true> job(a, a.execs);
      insert_all(job, a);
      cnt = job.run(a, &conv, &secs);
      for (uint64_t v = 0; v < a.n; ++v) {
        float d = job.vs->vertices_.next[v];
        vals[v] = (d >= FLT_MAX) ? 0xFFFFFFFFu : (uint32_t)d;
      }
    } else {
      // F4: the multi-executor reduce of PageRankDelta races; one executor
      Job<algorithm::PageRankDeltaVertexType_t, algorithm::PageRankDelta, false> job(a, 1);
      insert_all(job, a);
      cnt = job.run(a, &conv, &secs);
      for (uint64_t v = 0; v < a.n; ++v) memcpy(&vals[v], &job.vs->vertices_.next[v].rank, 4);
    }
    uint64_t hdr[3] = {cnt, (uint64_t)conv, a.n};
    write_or_die(out, hdr, sizeof(hdr));
    write_or_die(out, vals.data(), a.n * 4);
    write_or_die(out, &secs, 8);
  } else if (a.mode == "stream") {
    // CPU baseline: one job per program (as execute<> builds per job), every batch
    // inserted + compacted, then BFS / CC / SSSP run on the snapshot; times the runs.
    Job<uint32_t, algorithm::BFS, false> bfs(a, a.execs);
    Job<uint32_t, algorithm::CC, false> cc(a, a.execs);
    Job<float, algorithm::SSSP, true> sssp(a, a.execs);
    double run_s = 0, ins_s = 0;
    uint64_t edges = 0;
    uint64_t m2 = a.src.size();
    uint64_t nb = 0;
    for (uint64_t lo = 0; lo < m2; lo += a.batch, ++nb) {
      uint64_t hi = lo + a.batch < m2 ? lo + a.batch : m2;
      double t0 = now_s();
      bfs.insert(a, lo, hi);
      bfs.ts->doGlobalCompaction();
      ins_s += now_s() - t0;
      cc.insert(a, lo, hi);
      cc.ts->doGlobalCompaction();
      sssp.insert(a, lo, hi);
      sssp.ts->doGlobalCompaction();
      bool conv;
      double s;
      edges += bfs.run(a, &conv, &s);
      run_s += s;
      edges += cc.run(a, &conv, &s);
      run_s += s;
      edges += sssp.run(a, &conv, &s);
      run_s += s;
    }
    double res[4] = {(double)edges, run_s, ins_s, (double)nb};
    write_or_die(out, res, sizeof(res));
  } else if (a.mode == "istream") {
    // CPU baseline of the streaming workload: BFS / CC / SSSP as incremental reference
    // jobs (IncJob); per batch: the insert + compaction time of the three stores, the run
    // time of the three runs and their processed-edge counts (algorithm-executor.h:424-426).
    IncJob<uint32_t, algorithm::BFS, false> bfs(a, a.execs);
    IncJob<uint32_t, algorithm::CC, false> cc(a, a.execs);
    IncJob<float, algorithm::SSSP, true> sssp(a, a.execs);
    const uint64_t m2 = a.src.size();
    std::vector<double> rec;
    for (uint64_t lo = 0; lo < m2; lo += a.batch) {
      const uint64_t hi = lo + a.batch < m2 ? lo + a.batch : m2;
      double t0 = now_s();
      bfs.insert(a, lo, hi);
      bfs.base.ts->doGlobalCompaction();
      cc.insert(a, lo, hi);
      cc.base.ts->doGlobalCompaction();
      sssp.insert(a, lo, hi);
      sssp.base.ts->doGlobalCompaction();
      double t1 = now_s();
      bool conv = false, all = true;
      uint64_t edges = bfs.run(&conv);
      all = all && conv;
      edges += cc.run(&conv);
      all = all && conv;
      edges += sssp.run(&conv);
      all = all && conv;
      double t2 = now_s();
      rec.push_back((double)edges);
      rec.push_back(t1 - t0);
      rec.push_back(t2 - t1);
      rec.push_back(all ? 1.0 : 0.0);
    }
    uint64_t nb = rec.size() / 4;
    write_or_die(out, &nb, 8);
    write_or_die(out, rec.data(), rec.size() * 8);
    // final values, for parity checks of the incremental path
    std::vector<uint32_t> vals(3 * a.n);
    for (uint64_t v = 0; v < a.n; ++v) {
      vals[v] = bfs.base.vs->vertices_.next[v];
      vals[a.n + v] = cc.base.vs->vertices_.next[v];
      float d = sssp.base.vs->vertices_.next[v];
      vals[2 * a.n + v] = (d >= FLT_MAX) ? 0xFFFFFFFFu : (uint32_t)d;
    }
    write_or_die(out, vals.data(), vals.size() * 4);
  } else {
    fprintf(stderr, "unknown mode %s\n", a.mode.c_str());
    return 1;
  }
  fclose(out);
  return 0;
}
