// exec_pagerank.cu — PageRank-delta and normalised PageRank executors.
#include <cuda_runtime.h>
#include <stdint.h>

#include "engine.h"

namespace cytom {

int pagerank_alloc(Ctx* c, Job* j) {
  (void)j;
  return set_err(c, CYTOM_ERR_UNIMPLEMENTED, "PageRank executors are not built yet");
}
int pagerank_init(Ctx* c, Job* j) {
  (void)j;
  return set_err(c, CYTOM_ERR_UNIMPLEMENTED, "PageRank executors are not built yet");
}
int pagerank_seed(Ctx* c, Job* j, const uint32_t*, const uint32_t*, const uint32_t*, uint64_t) {
  (void)j;
  return set_err(c, CYTOM_ERR_UNIMPLEMENTED, "PageRank executors are not built yet");
}
int pagerank_run(Ctx* c, Job* j) {
  (void)j;
  return set_err(c, CYTOM_ERR_UNIMPLEMENTED, "PageRank executors are not built yet");
}
int pagerank_result(Ctx* c, Job* j, void*, int) {
  (void)j;
  return set_err(c, CYTOM_ERR_UNIMPLEMENTED, "PageRank executors are not built yet");
}

}  // namespace cytom
