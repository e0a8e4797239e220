// harness.cc — a compiled C++ caller of libcytom_gpu.so. It includes the C++ binding of
// INTEGRATION.md as it stands (tests/test_gpu_c_caller.py extracts that code block into
// binding.inc) and supplies stand-ins for the two reference types the binding reads:
// Config (src/include/util/config.h: context_.max_count_vertices,
// tile_store_config.vertices_per_tile, enable_adaptive_scheduling,
// algorithm_iterations, algorithm_config.{algo_start_id, delta}) and Edge
// (schema.fbs: src(), tgt(), weight()).
//
// usage: harness <bfs|cc|sssp> <vertices> <vertices_per_tile> <batch> <edges.bin> <out.bin>
//   edges.bin: u64 count, then u32 src[count], u32 tgt[count], u32 w[count]
//   out.bin:   u32 result[vertices]
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

struct Config {
  struct {
    uint64_t max_count_vertices = 0;
    struct {
      uint64_t vertices_per_tile = 0;
    } tile_store_config;
    bool enable_adaptive_scheduling = true;
    uint32_t algorithm_iterations = 100;
    struct {
      uint64_t algo_start_id = 0;
      double delta = 0.01;
    } algorithm_config;
  } context_;
};

class Edge {
 public:
  Edge(uint64_t s, uint64_t t, float w) : s_(s), t_(t), w_(w) {}
  uint64_t src() const { return s_; }
  uint64_t tgt() const { return t_; }
  float weight() const { return w_; }

 private:
  uint64_t s_, t_;
  float w_;
};

#include "binding.inc"

int main(int argc, char** argv) {
  if (argc != 7) {
    fprintf(stderr, "usage: %s <bfs|cc|sssp> <vertices> <vpt> <batch> <edges.bin> <out.bin>\n", argv[0]);
    return 2;
  }
  const std::string algo = argv[1];
  Config cfg;
  cfg.context_.max_count_vertices = strtoull(argv[2], nullptr, 10);
  cfg.context_.tile_store_config.vertices_per_tile = strtoull(argv[3], nullptr, 10);
  cfg.context_.algorithm_iterations = 1000;
  const uint64_t batch = strtoull(argv[4], nullptr, 10);
  FILE* f = fopen(argv[5], "rb");
  if (!f) return 3;
  uint64_t m = 0;
  if (fread(&m, 8, 1, f) != 1) return 3;
  std::vector<uint32_t> s(m), t(m), w(m);
  if (fread(s.data(), 4, m, f) != m || fread(t.data(), 4, m, f) != m || fread(w.data(), 4, m, f) != m) return 3;
  fclose(f);
  std::vector<std::vector<Edge>> batches;
  for (uint64_t lo = 0; lo < m; lo += batch) {
    batches.emplace_back();
    for (uint64_t i = lo; i < m && i < lo + batch; ++i) batches.back().emplace_back(s[i], t[i], (float)w[i]);
  }
  std::vector<uint32_t> result;
  try {
    if (algo == "bfs") execute_gpu<CYTOM_ALGO_BFS>(cfg, batches, &result);
    else if (algo == "cc") execute_gpu<CYTOM_ALGO_CC>(cfg, batches, &result);
    else if (algo == "sssp") execute_gpu<CYTOM_ALGO_SSSP>(cfg, batches, &result);
    else return 2;
  } catch (const std::exception& e) {
    fprintf(stderr, "execute_gpu failed: %s\n", e.what());
    return 4;
  }
  FILE* o = fopen(argv[6], "wb");
  if (!o || fwrite(result.data(), 4, result.size(), o) != result.size()) return 5;
  fclose(o);
  return 0;
}
