// FP64 instantiations of the solver and operator kernels.
#include "launch.cuh"

namespace sgw {
template sgw_status run_msbicg<double>(sgw_operator*, const BatchDev&);
template sgw_status run_sgw<double>(sgw_operator*, const SgwArgs<double>&);
template sgw_status run_apply<double>(sgw_operator*, int, const cplx<double>*, long long, cplx<double>*, long long, zcd);
}  // namespace sgw

namespace sgw {
template sgw_status run_msbicg_in<double>(sgw_operator*, const BatchDev&, unsigned char*, size_t);
}  // namespace sgw
