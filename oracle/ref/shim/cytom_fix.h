// Force-included into every translation unit of the reference pin build.
#pragma once
#include <stdint.h>
#include <string.h>
// F1: the reference tests a 64-vertex bitmap block by widening ONE byte
// ("(uint64_t) bitmap[i]", tile-manager.h:414,438, examples/bfs.cc:147, cc.cc:145,
// pagerank-delta.cc:226); the recipe rewrites those sites to load all 8 bytes.
static inline uint64_t cytom_load64(const uint8_t* p) {
  uint64_t v;
  memcpy(&v, p, 8);
  return v;
}
#ifndef PAGE_SIZE
#define PAGE_SIZE 4096
#endif
namespace evolving_graphs {
// Stand-in for MetaTileStore, which only the TILE_DISTRIBUTOR scheduling path (not
// pinned) consults.
template <typename VertexType, class Algorithm, bool is_weighted>
class MetaTileStore {
 public:
  struct Manager {
    uint64_t edgesPerMetaTile(uint64_t) { return 0; }
  };
  Manager* getMetaTileManager(uint64_t) { return &manager_; }

 private:
  Manager manager_;
};
}
