// sgw_solve_batch_noalloc: the batched FP64 multishift solve for callers that
// cannot allocate device memory while they solve.
//
// Some host programs fix their GPU memory before the solver runs: a Fortran
// code that reserves its device budget at start-up, a process whose GPU
// memory belongs to another framework's pool allocator (a cudaMalloc behind
// the pool's back would fragment it or fail against its cap), or a plug-in
// running under a hard per-process memory limit.  Such callers still own and
// pass the inputs and outputs (device pointers); everything the solver needs
// besides them comes from one fixed-size array in this library's device
// image, so the call itself allocates nothing.
//
// Limits and behaviour:
//   * the scratch array holds SGW_NOALLOC_SCRATCH_BYTES (32 MiB); every GPU that
//     loads the library keeps it until the process exits;
//   * a problem whose per-right-hand-side scratch does not fit is rejected with
//     SGW_ERR_UNSUPPORTED and a message saying so; smaller problems run with as
//     many concurrent right-hand sides and as long a history window as fit;
//   * every call uses the same array and leaves its contents behind; the call
//     clears what must start at zero (the work counter) and the kernel
//     initialises everything else it reads, but two calls whose work overlaps
//     on the GPU (other streams, other threads) race on the array;
//   * the call runs on the handle's device (made current for the call), and
//     the first call on a device looks the array's address up with
//     cudaGetSymbolAddress (once per device, with that device current).
#include <mutex>

#include "host.cuh"

namespace sgw {

static __device__ __align__(256) unsigned char g_noalloc_scratch[SGW_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
static void* g_scratch_addr[kMaxDevices] = {};
static std::mutex g_scratch_mutex;

// Host code cannot use g_noalloc_scratch directly: its host-side name is only a
// stand-in.  The device address comes from cudaGetSymbolAddress, per device.
static sgw_status scratch_address(unsigned char** out) {
  int dev = 0;
  SGW_CK(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) {
    set_error("device index out of range for the no-allocation scratch table");
    return SGW_ERR_UNSUPPORTED;
  }
  std::lock_guard<std::mutex> lock(g_scratch_mutex);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      set_error(std::string("cudaGetSymbolAddress(no-allocation scratch) failed: ") + cudaGetErrorString(e));
      return SGW_ERR_CUDA;
    }
    g_scratch_addr[dev] = p;
  }
  *out = static_cast<unsigned char*>(g_scratch_addr[dev]);
  return SGW_OK;
}

}  // namespace sgw

using namespace sgw;

extern "C" sgw_status sgw_solve_batch_noalloc(sgw_operator* op, const sgw_batch_desc* d) {
  if (!op || !d) {
    set_error("null argument");
    return SGW_ERR_ARG;
  }
  if (d->memory != 1) {
    set_error("sgw_solve_batch_noalloc needs device pointers (memory = 1)");
    return SGW_ERR_ARG;
  }
  if (d->precision != 0) {
    set_error("sgw_solve_batch_noalloc runs the FP64 solve only (precision = 0)");
    return SGW_ERR_ARG;
  }
  if (d->nrhs < 0 || d->num_shift < 1 || d->lmax < 1 || d->lmax > kMaxL - 1 || d->max_iter < 1) {
    set_error("invalid batch sizes (num_shift >= 1, 1 <= lmax <= 15, max_iter >= 1)");
    return SGW_ERR_ARG;
  }
  if (d->nrhs > 0 && (!d->bb || !d->sigma || !d->xx || !d->ierr)) {
    set_error("null batch array");
    return SGW_ERR_ARG;
  }
  if (d->ldb < op->n || d->lds < d->num_shift || d->ldx < op->n || d->ldr < d->ldx * (d->num_shift - 1) + op->n) {
    set_error("leading dimensions too small");
    return SGW_ERR_ARG;
  }
  if (d->nrhs == 0) return SGW_OK;
  // the handle's device is current from here on, so the symbol lookup and the
  // launch use that device's copy of the array
  CallScope cs(op);
  if (cs.status() != SGW_OK) return cs.status();
  unsigned char* region = nullptr;
  sgw_status s = scratch_address(&region);
  if (s != SGW_OK) return s;
  BatchDev b{d->nrhs, d->num_shift, d->lmax, d->max_iter, d->history_iters, d->threshold, d->bb, d->ldb,
             reinterpret_cast<const zcd*>(d->sigma), d->lds, d->xx, d->ldx, d->ldr, d->ierr, d->iters};
  op->last_launches = 0;
  op->kev_used = 0;
  SGW_CK(cudaEventRecord(op->ev0, op->stream));
  s = run_msbicg_in<double>(op, b, region, SGW_NOALLOC_SCRATCH_BYTES);
  if (s != SGW_OK) return s;
  SGW_CK(cudaEventRecord(op->ev1, op->stream));
  SGW_CK(cudaStreamSynchronize(op->stream));
  float ms = 0.f;
  SGW_CK(cudaEventElapsedTime(&ms, op->ev0, op->ev1));
  op->last_ms = ms;
  collect_kernel_times(op);
  return SGW_OK;
}
