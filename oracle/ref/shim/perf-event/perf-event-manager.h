// No-op perf-event manager (test infrastructure for the reference pin).
#pragma once
#include "ring-buffer/ring-buffer.h"
namespace evolving_graphs {
namespace perf_event {
class PerfEventManager {
 public:
  Ringbuffer getRingBuffer() { return Ringbuffer(); }
  template <class... A>
  void start(A&&...) {}
  void stop() {}
};
}  // namespace perf_event
}  // namespace evolving_graphs
