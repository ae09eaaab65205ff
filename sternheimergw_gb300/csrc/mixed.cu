// Mixed-precision batched solve (complex64 Krylov, FP64 refinement).
#include "host.cuh"

namespace sgw {
sgw_status solve_mixed(sgw_operator*, const BatchDev&, int, double) {
  set_error("mixed precision is not available yet");
  return SGW_ERR_UNSUPPORTED;
}
}  // namespace sgw
