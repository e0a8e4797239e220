// persist.cu — the reference's on-disk formats: the edge log and the results dumps.
//
// Edge log (EdgesWriter, src/include/tile-manager/edges-writer.h:114-185): every inserted
// batch is appended, in arrival order and with duplicates, as packed little-endian
// records edge_compact_t {u32 src; u32 tgt} or, for weighted stores,
// edge_compact_weighted_t {u32 src; u32 tgt; float weight}
// (src/include/util/datatypes.h:55-64). Reading a log back (EdgesWriter::readEdges,
// edges-writer.h:30-90) inserts its records in batches.
//
// Results (ResultsWriter::run, src/include/core/results-writer.h:46-81): the raw array of
// a job's VertexType values, vertex by vertex: uint32 (BFS, CC), float (SSSP and SSWP,
// FLT_MAX for "not reached" / the widest-path start), the 12-byte
// PageRankDeltaVertexType_t {float delta_sum; float rank; float delta}
// (examples/pagerank-delta.cc:30-33) and float (PageRank).
#include <cuda_runtime.h>
#include <float.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <string>
#include <vector>

#include "engine.h"

namespace cytom {

int pagerank_result(Ctx* c, Job* j, void* out, int where);
int pagerank_delta_out(Ctx* c, Job* j, float* rank, float* delta);

struct EdgeLog {
  FILE* f = nullptr;
  std::string path;
};

static EdgeLog* log_of(Ctx* c) { return reinterpret_cast<EdgeLog*>(c->edge_log); }

void edge_log_close(Ctx* c) {
  EdgeLog* l = log_of(c);
  if (!l) return;
  if (l->f) fclose(l->f);
  delete l;
  c->edge_log = nullptr;
}

// Appends one batch (host or device pointers) to the open log.
int edge_log_append(Ctx* c, const uint32_t* src, const uint32_t* tgt, const uint32_t* w, uint64_t count,
                    int where) {
  EdgeLog* l = log_of(c);
  if (!l || !l->f || count == 0) return CYTOM_OK;
  const bool weighted = c->wtype != CYTOM_UNWEIGHTED;
  std::vector<uint32_t> hs, ht, hw;
  if (where == CYTOM_PTR_DEVICE) {
    hs.resize(count);
    ht.resize(count);
    cudaError_t e = cudaMemcpyAsync(hs.data(), src, count * 4, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(ht.data(), tgt, count * 4, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess && weighted && w) {
      hw.resize(count);
      e = cudaMemcpyAsync(hw.data(), w, count * 4, cudaMemcpyDeviceToHost, c->stream);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_err(c, e, "edge log");
    src = hs.data();
    tgt = ht.data();
    w = hw.empty() ? nullptr : hw.data();
  }
  const size_t rec = weighted ? 12 : 8;
  std::vector<uint32_t> out(count * rec / 4);
  for (uint64_t i = 0; i < count; ++i) {
    uint32_t* r = out.data() + i * (rec / 4);
    r[0] = src[i];
    r[1] = tgt[i];
    if (weighted) {
      float fw = 0.f;
      if (w) {
        if (c->wtype == CYTOM_WEIGHT_F32) memcpy(&fw, &w[i], 4);
        else fw = (float)w[i];
      }
      memcpy(&r[2], &fw, 4);
    }
  }
  if (fwrite(out.data(), 1, out.size() * 4, l->f) != out.size() * 4)
    return set_err(c, CYTOM_ERR_IO, "edge log write to " + l->path);
  return CYTOM_OK;
}

}  // namespace cytom

using namespace cytom;

extern "C" {

int cytom_persist_edges(cytom_ctx* ctx, const char* path) {
  Ctx* c = (Ctx*)ctx;
  if (c) join_runs(c);
  if (!c) return CYTOM_ERR_INVAL;
  edge_log_close(c);
  if (!path) return CYTOM_OK;
  EdgeLog* l = new (std::nothrow) EdgeLog();
  if (!l) return CYTOM_ERR_OOM;
  l->path = path;
  l->f = fopen(path, "wb");
  if (!l->f) {
    delete l;
    return set_err(c, CYTOM_ERR_IO, std::string("cannot open ") + path);
  }
  c->edge_log = l;
  return CYTOM_OK;
}

int cytom_read_edges(cytom_ctx* ctx, const char* path, uint64_t batch, uint64_t* count) {
  Ctx* c = (Ctx*)ctx;
  if (!c || !path) return CYTOM_ERR_INVAL;
  FILE* f = fopen(path, "rb");
  if (!f) return set_err(c, CYTOM_ERR_IO, std::string("cannot open ") + path);
  const bool weighted = c->wtype != CYTOM_UNWEIGHTED;
  const size_t rec = weighted ? 12 : 8;
  if (batch == 0) batch = 1ULL << 20;
  std::vector<uint32_t> buf(batch * rec / 4), hs(batch), ht(batch), hw(weighted ? batch : 0);
  uint64_t total = 0;
  int rc = CYTOM_OK;
  while (true) {
    const size_t got = fread(buf.data(), 1, batch * rec, f);
    const uint64_t m = got / rec;
    if (m == 0) break;
    for (uint64_t i = 0; i < m; ++i) {
      const uint32_t* r = buf.data() + i * (rec / 4);
      hs[i] = r[0];
      ht[i] = r[1];
      if (weighted) {
        float fw;
        memcpy(&fw, &r[2], 4);
        if (c->wtype == CYTOM_WEIGHT_F32) memcpy(&hw[i], &fw, 4);
        else hw[i] = fw <= 0.f ? 0u : (fw >= 4294967040.f ? 0xFFFFFFFFu : (uint32_t)(fw + 0.5f));
      }
    }
    rc = cytom_insert_batch(ctx, hs.data(), ht.data(), weighted ? hw.data() : nullptr, m, CYTOM_PTR_HOST);
    if (rc) break;
    total += m;
    if (got < batch * rec) break;
  }
  fclose(f);
  if (count) *count = total;
  return rc;
}

int cytom_write_results(cytom_ctx* ctx, int job_id, const char* path) {
  Ctx* c = (Ctx*)ctx;
  if (c) join_runs(c);
  if (!c || !path || job_id < 0 || job_id >= (int)c->jobs.size() || !c->jobs[job_id]) return CYTOM_ERR_INVAL;
  Job* j = c->jobs[job_id];
  const uint64_t n = c->n;
  std::vector<uint32_t> words;
  int rc = CYTOM_OK;
  switch (j->algo) {
    case CYTOM_ALGO_BFS:
    case CYTOM_ALGO_CC:
      words.resize(n);
      rc = cytom_get_result(ctx, job_id, words.data(), CYTOM_PTR_HOST);
      break;
    case CYTOM_ALGO_SSSP:
    case CYTOM_ALGO_SSWP: {
      std::vector<uint32_t> v(n);
      rc = cytom_get_result(ctx, job_id, v.data(), CYTOM_PTR_HOST);
      words.resize(n);
      for (uint64_t i = 0; i < n; ++i) {
        const float f = v[i] == 0xFFFFFFFFu ? FLT_MAX : (float)v[i];
        memcpy(&words[i], &f, 4);
      }
      break;
    }
    case CYTOM_ALGO_PR_DELTA: {
      std::vector<float> rank(n), delta(n);
      rc = pagerank_delta_out(c, j, rank.data(), delta.data());
      words.resize(3 * n);
      const float alpha = (float)j->params.alpha;
      for (uint64_t i = 0; i < n; ++i) {
        // delta_sum: the in-edge sum that produced the last delta (delta = alpha * sum)
        const float ds = alpha != 0.f ? delta[i] / alpha : 0.f;
        memcpy(&words[3 * i], &ds, 4);
        memcpy(&words[3 * i + 1], &rank[i], 4);
        memcpy(&words[3 * i + 2], &delta[i], 4);
      }
      break;
    }
    default:
      words.resize(n);
      rc = pagerank_result(c, j, words.data(), CYTOM_PTR_HOST);
  }
  if (rc) return rc;
  FILE* f = fopen(path, "wb");
  if (!f) return set_err(c, CYTOM_ERR_IO, std::string("cannot open ") + path);
  const size_t bytes = words.size() * 4;
  const bool ok = fwrite(words.data(), 1, bytes, f) == bytes;
  fclose(f);
  return ok ? CYTOM_OK : set_err(c, CYTOM_ERR_IO, std::string("write to ") + path);
}

}  // extern "C"
