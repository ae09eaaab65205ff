// FP32 instantiations of the solver and operator kernels.
#include "launch.cuh"

namespace sgw {
template sgw_status run_msbicg<float>(sgw_operator*, const BatchDev&);
template sgw_status run_sgw<float>(sgw_operator*, const SgwArgs<float>&);
template sgw_status run_apply<float>(sgw_operator*, int, const cplx<float>*, long long, cplx<float>*, long long, zcd);
}  // namespace sgw
