// Stand-ins for the flatbuffers-generated message types of src/flatbuffer/schema.fbs
// (test infrastructure for the reference pin). Edge carries (src, tgt, weight) like the
// schema's struct; the messages are inert: the pinned paths never send any.
#pragma once
#include <stdint.h>
#include <algorithm>
#include <set>
#include <vector>
#include "flatbuffers/flatbuffers.h"

namespace evolving_graphs {
struct Edge {
  Edge() : s_(0), t_(0), w_(0.f) {}
  Edge(uint64_t s, uint64_t t, float w) : s_(s), t_(t), w_(w) {}
  uint64_t src() const { return s_; }
  uint64_t tgt() const { return t_; }
  float weight() const { return w_; }
  void mutate_src(uint64_t v) { s_ = v; }
  void mutate_tgt(uint64_t v) { t_ = v; }
  void mutate_weight(float v) { w_ = v; }

 private:
  uint64_t s_, t_;
  float w_;
};
struct TileDistributorMessage {
  bool shutdown() const { return true; }
  const flatbuffers::Vector<uint64_t>* tiles() const { return &v_; }
  flatbuffers::Vector<uint64_t> v_;
};
struct AlgorithmMessage {
  bool shutdown() const { return true; }
  uint64_t count_edges() const { return 0; }
};
struct PerfEventMessage {};
template <class B, class... A>
flatbuffers::Offset<TileDistributorMessage> CreateTileDistributorMessage(B&, A...) {
  return {};
}
template <class B, class... A>
flatbuffers::Offset<AlgorithmMessage> CreateAlgorithmMessage(B&, A...) {
  return {};
}
}  // namespace evolving_graphs
