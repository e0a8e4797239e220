// No-op scoped perf event (test infrastructure for the reference pin).
#pragma once
#include "ring-buffer/ring-buffer.h"
namespace evolving_graphs {
namespace perf_event {
class PerfEventScoped {
 public:
  template <class... A>
  PerfEventScoped(A&&...) {}
};
}  // namespace perf_event
}  // namespace evolving_graphs
