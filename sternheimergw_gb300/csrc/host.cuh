// Host-side state of an operator handle and its workspaces.
#pragma once
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/sgw_capi.h"
#include "msbicg.cuh"
#include "sgwsolver.cuh"

namespace sgw {

void set_error(const std::string& msg);

#define SGW_CK(call)                                                                        \
  do {                                                                                      \
    cudaError_t e_ = (call);                                                                \
    if (e_ != cudaSuccess) {                                                                \
      ::sgw::set_error(std::string(#call) + " failed: " + cudaGetErrorString(e_));          \
      return SGW_ERR_CUDA;                                                                  \
    }                                                                                       \
  } while (0)

struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  sgw_status ensure(size_t want) {
    if (want <= bytes && p) return SGW_OK;
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
    if (want == 0) want = 16;
    cudaError_t e = cudaMalloc(&p, want);
    if (e != cudaSuccess) {
      p = nullptr;
      set_error(std::string("cudaMalloc(") + std::to_string(want) + ") failed: " + cudaGetErrorString(e));
      return e == cudaErrorMemoryAllocation ? SGW_ERR_NOMEM : SGW_ERR_CUDA;
    }
    bytes = want;
    return SGW_OK;
  }
  template <typename T> sgw_status upload(const T* host, size_t count) {
    sgw_status s = ensure(count * sizeof(T));
    if (s != SGW_OK) return s;
    if (count) SGW_CK(cudaMemcpy(p, host, count * sizeof(T), cudaMemcpyHostToDevice));
    return SGW_OK;
  }
  template <typename T> T* as() const { return reinterpret_cast<T*>(p); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
};

// Pruned-FFT launch shape of a plane-wave operator in one precision.
struct PwShape {
  int ng = 1;            // plane groups (stage FFT) or planes in flight (line FFT)
  bool lines = false;    // line-per-thread register FFT
  bool col_in_smem = true;
  size_t smem = 0;       // dynamic shared memory bytes
};

// A batch with every array already in device memory.
struct BatchDev {
  int nrhs, nshift, lmax, max_iter, history_iters;
  double threshold;
  const void* bb;
  long long ldb;
  const zcd* sigma;
  long long lds;
  void* xx;
  long long ldx, ldr;
  int* ierr;
  int* iters;
  const int* active;  // optional: 0 skips a right-hand side
  zcd* zeta;          // optional: per-shift residual factors at exit
  int gemm_tc = 0;     // FP32: basis product on the tensor cores (3xTF32)
};

struct Workspace {
  DevBuf vec, coef, col, counter;
};

// Kernel kinds timed with CUDA events on the operator's stream.
// Timed spans of the last call, by kind: the solve kernels (0-2), the caller-side
// kernels (3-5), the host-path copies of sgw_solve_batch (6 in, 7 out), the
// screened Coulomb and self-energy kernels (8, 9) and the FP32 residual update
// of the mixed rounds (10).
enum KernelKind {
  K_MSBICG_F64 = 0,
  K_MSBICG_F32 = 1,
  K_RESIDUAL_F64 = 2,
  K_RHS = 3,
  K_CHI = 4,
  K_VJP = 5,
  K_COPY_IN = 6,
  K_COPY_OUT = 7,
  K_SCREEN = 8,
  K_SIGMA = 9,
  K_RESIDUAL_F32 = 10,
  K_NUM = 11
};
constexpr int kMaxTimedLaunches = 64;

}  // namespace sgw

struct sgw_operator {
  int kind = 0;  // 0 dense, 1 plane-wave
  int n = 0, npwx = 0;
  int device = 0, num_sms = 0;
  size_t smem_optin = 0, smem_per_sm = 0;
  cudaStream_t stream = nullptr;
  // the caller's stream (sgw_operator_set_stream; cudaStreamLegacy by default):
  // every call makes `stream` wait for the work queued on it before its first launch
  cudaStream_t caller_stream = cudaStreamLegacy;
  cudaEvent_t ev_caller = nullptr;
  cudaStream_t copy_stream = nullptr;                 // host-path result copies overlapped with the solve
  cudaEvent_t ev_acc = nullptr, ev_copied = nullptr;  // its hand-offs (no timing)
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  // page-locked staging of the small per-call outputs of the host-memory form
  // (ierr, iters, residual estimates): copied to the caller's arrays after the
  // stream is synchronised (host_staging)
  void* h_small = nullptr;
  size_t h_small_bytes = 0;
  cudaEvent_t lev0 = nullptr, lev1 = nullptr;  // sgw_coulomb_rhs / sgw_chi timing
  double last_ms = 0.0;
  long long last_launches = 0;
  // per-kernel timing of the last solve: event pairs recorded around launches
  cudaEvent_t kev[2 * sgw::kMaxTimedLaunches] = {};
  int kev_kind[sgw::kMaxTimedLaunches] = {};
  int kev_used = 0;
  double kernel_ms[sgw::K_NUM] = {};
  long long kernel_launches[sgw::K_NUM] = {};
  double alpha_pv = 0.0;
  // tables
  unsigned long long xmask = 0;
  sgw::DevBuf nlkq, ymask, zmask, gcol, gi3, colpos, i1list, g2k64, g2k32, vrs64, vrs32, vkb64, vkb32, dvan64, dvan32, evq64, evq32,
      tw64, tw32, a64, a32;
  sgw::PwView<double> pw64{};
  sgw::PwView<float> pw32{};
  sgw::DenseView<double> dn64{};
  sgw::DenseView<float> dn32{};
  sgw::PwShape shape64, shape32;
  // workspaces and staging
  sgw::Workspace ws64, ws32;
  sgw::DevBuf st_bb, st_sigma, st_xx, st_ierr, st_iters, st_misc, st_misc2, st_misc3;
  sgw::DevBuf st_ref, st_ref2, st_resid;  // restart rounds and warm starts (sgw_solve_batch_ex)
  // right-hand-side build and chi accumulation
  sgw::DevBuf lt_psi, lt_box, lt_nlk, lt_evc, lt_dv, lt_bb, lt_flag, lt_part, lt_sidx, lt_xx, lt_chi;
  // screened Coulomb interaction and self-energy
  sgw::DevBuf lt_w, lt_wwork, lt_sig;
};

namespace sgw {
template <typename T> struct Ipt;
template <> struct Ipt<double> { static constexpr int v = 1; };
template <> struct Ipt<float> { static constexpr int v = 1; };

template <typename T> PwView<T>& pwview(sgw_operator* op);
template <> inline PwView<double>& pwview<double>(sgw_operator* op) { return op->pw64; }
template <> inline PwView<float>& pwview<float>(sgw_operator* op) { return op->pw32; }
template <typename T> DenseView<T>& dnview(sgw_operator* op);
template <> inline DenseView<double>& dnview<double>(sgw_operator* op) { return op->dn64; }
template <> inline DenseView<float>& dnview<float>(sgw_operator* op) { return op->dn32; }
template <typename T> PwShape& pwshape(sgw_operator* op);
template <> inline PwShape& pwshape<double>(sgw_operator* op) { return op->shape64; }
template <> inline PwShape& pwshape<float>(sgw_operator* op) { return op->shape32; }
template <typename T> Workspace& wsp(sgw_operator* op);
template <> inline Workspace& wsp<double>(sgw_operator* op) { return op->ws64; }
template <> inline Workspace& wsp<float>(sgw_operator* op) { return op->ws32; }

template <typename T>
inline long long col_elems(sgw_operator* op) {
  return op->kind == 1 ? (long long)pwview<T>(op).ncol * pwview<T>(op).ldz : 0;
}


// Event pair around one launch (no-op once the pool of pairs is used up).
inline int ktime_begin(sgw_operator* op, int kind) {
  if (op->kev_used >= kMaxTimedLaunches || !op->kev[0]) return -1;
  const int i = op->kev_used++;
  op->kev_kind[i] = kind;
  cudaEventRecord(op->kev[2 * i], op->stream);
  return i;
}
inline void ktime_end(sgw_operator* op, int i) {
  if (i >= 0) cudaEventRecord(op->kev[2 * i + 1], op->stream);
}

// Prologue of every entry point that queues device work on a handle: the
// handle's device becomes current for the call (the caller's current device is
// restored on exit), and the handle's stream waits for everything the caller
// has queued on its stream (sgw_operator_set_stream; the legacy default stream
// unless set) - so inputs written and outputs initialised by the caller just
// before the call are complete when the first kernel starts.  Every call
// synchronises the handle's stream before it returns.
class CallScope {
 public:
  explicit CallScope(sgw_operator* op);
  ~CallScope();
  sgw_status status() const { return st_; }

 private:
  int prev_ = -1, dev_ = -1;
  sgw_status st_ = SGW_OK;
};
// Sum the per-kernel event pairs of the last call into kernel_ms / kernel_launches
// (the handle's stream must be synchronised).
void collect_kernel_times(sgw_operator* op);
// A device int, read on the host after the work queued on op->stream, through
// the operator's page-locked staging (host_staging).
sgw_status read_count(sgw_operator* op, const int* dev, int* out);
// The operator's page-locked staging for small device-to-host results, at
// least `bytes` long.  Device-to-host copies into pageable memory were measured
// to slow later copies into registered buffers (such as sgw_host_alloc's) to
// 6-8 GB/s; small results therefore land here and are copied on the host.
sgw_status host_staging(sgw_operator* op, size_t bytes, void** out);
// `stream` waits for the work queued so far on `caller` (event `ev` is reused).
sgw_status order_after(cudaStream_t stream, cudaStream_t caller, cudaEvent_t ev);

template <typename T> sgw_status run_msbicg(sgw_operator* op, const BatchDev& b);
template <typename T> sgw_status run_sgw(sgw_operator* op, const SgwArgs<T>& a);
template <typename T>
sgw_status run_apply(sgw_operator* op, int m, const cplx<T>* x, long long ldi, cplx<T>* ax, long long ldo, zcd sigma);
// A device-to-host copy of the solutions (packed [nrhs][S][n], `bytes` long) that
// solve_mixed issues on op->copy_stream after each FP64 accumulation that may be
// the last one, waiting for it before a later accumulation writes x; it overlaps
// the closing FP64 residual.  `issued` is true when such a copy followed the last
// accumulation: the caller then makes op->stream wait on op->ev_copied before
// using the host data; otherwise the caller copies x itself (op->stream already
// waits for any earlier copy).
struct OutCopy {
  void* host = nullptr;
  size_t bytes = 0;
  bool issued = false;
};
// What a mixed solve leaves behind (device pointers into the handle's staging
// buffers, valid until the next call on the handle): residual factors Z with
// shifted residual = Z^sigma r for every (right-hand side, shift), the FP64 true
// residual r of the seed shift after the last accumulation, its norm and the
// right-hand-side norms.
struct RoundState {
  zcd* Z = nullptr;
  zcd* r64 = nullptr;
  double* scale = nullptr;
  double* bnorm = nullptr;
};
// norm_ref (optional, leading dimension norm_ld): the right-hand sides whose
// norms set the FP64 refinement target (refine_thr |norm_ref_r|) instead of
// b.bb's own - a warm start solves for a small correction whose accuracy is
// measured against the full right-hand side.
sgw_status solve_mixed(sgw_operator* op, const BatchDev& b, int refine_max, double refine_thr, OutCopy* out = nullptr,
                       RoundState* st = nullptr, const zcd* norm_ref = nullptr, long long norm_ld = 0);

// Host-side view of sgw_batch_options (defaults filled in); resid is a device
// array [nrhs][nshift] or null.
struct BatchOptions {
  int shift_refine = 0;  // 0 reference semantics, 1 + per-shift estimates, 2 + restart rounds
  double shift_tol = 1e-6;
  int rounds = 0;
  int round_iters = 6;
  int warm_start = 0;
  double* resid = nullptr;
};
sgw_status solve_batch_opts(sgw_operator* op, const BatchDev& b, int precision, int refine_max, double refine_thr,
                            const BatchOptions& o);
template <typename T>
sgw_status run_msbicg_in(sgw_operator* op, const BatchDev& b, unsigned char* region, size_t region_bytes);
}  // namespace sgw
