// Uneven batches: many independent systems (each its own operator handle,
// G-sphere, FFT box, band/perturbation count and shift list) solved together.
//
// Every iteration stage is one persistent launch over the (system, rhs) items
// of all systems: the FP64 multishift solve (precision 0), or per mixed round
// the FP32 multishift solve and the FP64 seed residual (precision 1).  Items
// are ordered longest-first (estimated operator cost x shifts) and pulled from
// one atomic queue, so a CTA that finishes a small system takes the next item
// of any system; converged right-hand sides leave in place through the active
// masks.  The per-system solver arguments and operator views live in constant
// memory (one copy per launch, uploaded device-to-device inside the stream),
// so the solver reads them through the constant cache exactly as it reads a
// single system's kernel parameters.  Systems whose FFT lengths have no
// register line kernel use the shared-memory FFT variant: one launch per
// variant present.  The whole sequence has no host synchronisation, so it can
// be captured once as a CUDA graph and replayed.
//
// Per-system completion time: each item's CTA stamps %globaltimer into its
// system's slot (atomicMax) when it finishes; the run reports the largest
// stamp minus a stamp taken at the start of the sequence.
#include <algorithm>
#include <cmath>
#include <map>
#include <mutex>
#include <numeric>
#include <string>
#include <vector>

#include "host.cuh"
#include "launch.cuh"
#include "mxkern.cuh"

namespace sgw {
namespace {

struct MultiItem {
  int sys, rhs;
};

template <typename T, class ApplyT>
struct SolveEntry {
  SolverArgs<T> a;
  ApplyT A;
};

template <class ApplyT>
struct ResEntry {
  ApplyT A;
  int n;
  const zcd* bb;
  long long ldb;
  const zcd* sigma;
  long long lds;
  const zcd* x;
  long long ldr;
  zcd* r;
  long long ldrr;
  const int* active;
};

// FP32 seed-residual update of one system (mixed rounds after the first):
// r -= A(sigma_1) c, c = the round's increment of x_1 (see mx_residual_update)
template <class ApplyT>
struct ResUpdEntry {
  ApplyT A;
  int n;
  const zcd* sigma;
  long long lds;
  const zcf* c;  // [nrhs][ldrr]
  zcf* ac;       // A c: the round's seed rows of y32
  long long ldac;
  zcd* r;
  long long ldrr;
  const int* active;
};

constexpr size_t kConstBytes = 60 * 1024;
__constant__ __align__(16) unsigned char c_entries[kConstBytes];

__device__ __forceinline__ unsigned long long gtimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__global__ void stamp_kernel(unsigned long long* t) { *t = gtimer(); }

template <typename T, class ApplyT, int THREADS>
__global__ void __launch_bounds__(THREADS, CtasPerSm<T>::v)
    msbicg_multi_kernel(const MultiItem* items, int nitems, int* counter, cplx<T>* col_global, long long col_slot,
                        unsigned long long* sys_end) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ SeedShared ss;
  __shared__ int s_item;
  const SolveEntry<T, ApplyT>* E = reinterpret_cast<const SolveEntry<T, ApplyT>*>(c_entries);
  cplx<T>* sm = reinterpret_cast<cplx<T>*>(smem_raw);
  int cur = -1;
  while (true) {
    if (threadIdx.x == 0) s_item = atomicAdd(counter, 1);
    __syncthreads();
    const int it = s_item;
    __syncthreads();
    if (it >= nitems) break;
    const MultiItem m = items[it];
    const SolverArgs<T>& a = E[m.sys].a;
    const ApplyT& A = E[m.sys].A;
    if (a.active && !a.active[m.rhs]) continue;
    if (m.sys != cur) {
      A.setup(sm);
      cur = m.sys;
    }
    cplx<T>* col = A.col_in_smem ? sm + A.smem_small() : col_global + (size_t)blockIdx.x * col_slot;
    solve_one<T, ApplyT>(a, A, m.rhs, blockIdx.x, sm, col, ss);
    if (threadIdx.x == 0) atomicMax(sys_end + m.sys, gtimer());
  }
}

// r = b - A(sigma_1) x_1 in FP64 for the active right-hand sides of every system
template <class ApplyT, int THREADS>
__global__ void __launch_bounds__(THREADS, 1)
    residual_multi_kernel(const MultiItem* items, int nitems, int* counter, zcd* col_global, long long col_slot,
                          unsigned long long* sys_end) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int s_item;
  const ResEntry<ApplyT>* E = reinterpret_cast<const ResEntry<ApplyT>*>(c_entries);
  zcd* sm = reinterpret_cast<zcd*>(smem_raw);
  int cur = -1;
  while (true) {
    if (threadIdx.x == 0) s_item = atomicAdd(counter, 1);
    __syncthreads();
    const int it = s_item;
    __syncthreads();
    if (it >= nitems) break;
    const MultiItem m = items[it];
    const ResEntry<ApplyT>& e = E[m.sys];
    if (!e.active[m.rhs]) continue;
    if (m.sys != cur) {
      e.A.setup(sm);
      cur = m.sys;
    }
    zcd* col = e.A.col_in_smem ? sm + e.A.smem_small() : col_global + (size_t)blockIdx.x * col_slot;
    zcd* out = e.r + (size_t)m.rhs * e.ldrr;
    e.A.apply(e.x + (size_t)m.rhs * e.ldr, out, nullptr, e.sigma[(size_t)m.rhs * e.lds], sm, col);
    const zcd* b = e.bb + (size_t)m.rhs * e.ldb;
    for (int g = threadIdx.x; g < e.n; g += blockDim.x) out[g] = b[g] - out[g];
    __syncthreads();
    if (threadIdx.x == 0) atomicMax(sys_end + m.sys, gtimer());
  }
}

// r -= A(sigma_1) c in FP32 for the active right-hand sides of every system
template <class ApplyT, int THREADS>
__global__ void __launch_bounds__(THREADS, 1)
    residual_update_multi_kernel(const MultiItem* items, int nitems, int* counter, zcf* col_global,
                                 long long col_slot, unsigned long long* sys_end) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int s_item;
  const ResUpdEntry<ApplyT>* E = reinterpret_cast<const ResUpdEntry<ApplyT>*>(c_entries);
  zcf* sm = reinterpret_cast<zcf*>(smem_raw);
  int cur = -1;
  while (true) {
    if (threadIdx.x == 0) s_item = atomicAdd(counter, 1);
    __syncthreads();
    const int it = s_item;
    __syncthreads();
    if (it >= nitems) break;
    const MultiItem m = items[it];
    const ResUpdEntry<ApplyT>& e = E[m.sys];
    if (!e.active[m.rhs]) continue;
    if (m.sys != cur) {
      e.A.setup(sm);
      cur = m.sys;
    }
    zcf* col = e.A.col_in_smem ? sm + e.A.smem_small() : col_global + (size_t)blockIdx.x * col_slot;
    zcf* out = e.ac + (size_t)m.rhs * e.ldac;
    e.A.apply(e.c + (size_t)m.rhs * e.ldrr, out, nullptr, e.sigma[(size_t)m.rhs * e.lds], sm, col);
    zcd* rr = e.r + (size_t)m.rhs * e.ldrr;
    for (int g = threadIdx.x; g < e.n; g += blockDim.x) rr[g] = rr[g] - zcd{(double)out[g].re, (double)out[g].im};
    __syncthreads();
    if (threadIdx.x == 0) atomicMax(sys_end + m.sys, gtimer());
  }
}

// Floating-point work of one operator apply of a system (FFT lines actually
// needed, V_loc multiply, projectors): the cost model of the item order.
double apply_cost(const PwView<double>& v) {
  auto line = [](int m) { return m > 1 ? 5.0 * m * std::log2((double)m) : 0.0; };
  return 2.0 * (v.ncol * line(v.nr3) + (double)v.ni1 * v.nr3 * line(v.nr2) + (double)v.nr2 * v.nr3 * line(v.nr1)) +
         2.0 * v.nnr + 16.0 * v.npw * (v.nkb + v.nocc);
}

std::mutex g_const_mutex;  // c_entries is one per process: runs never overlap

}  // namespace

// Per-precision plan of one stage: the launch groups (one per operator
// variant) with their constant-memory images and item lists.
struct MultiGroup {
  bool lines = false;
  DevBuf entries;  // device copy of the constant-memory image
  DevBuf entries_tc;  // FP32 correction rounds: the same image with the tensor-core basis product
  size_t entry_bytes = 0;
  DevBuf items;
  int nitems = 0;
  size_t smem = 0;
};

}  // namespace sgw

struct sgw_multi {
  int nsys = 0;
  std::vector<sgw_operator*> ops;
  std::vector<sgw_batch_desc> d;
  sgw_multi_options opt{};
  cudaStream_t stream = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaEvent_t ev_caller = nullptr;  // orders the plan's stream after the caller's
  int num_sms = 0, nslots = 0;
  // solve stage (FP64 solve for precision 0, FP32 rounds for precision 1) and FP64 residual stage
  std::vector<sgw::MultiGroup> solve_groups, res_groups, upd_groups;
  sgw::DevBuf vec, coef, col, col64, counters, stamps;
  // mixed precision, per system: r64, r32, y32, Z, zeta, scale, bnorm, active, iters_round, nactive
  sgw::DevBuf mixed;
  struct MixedSys {
    zcd* r64;
    zcf* r32;
    zcf* y32;
    zcd* Z;
    zcd* zeta;
    double* scale;
    double* bnorm;
    int* active;
    int* iters_round;
    int* nactive;
    int* bad;
  };
  std::vector<MixedSys> ms;
  std::vector<int> npwx;
  long long launches = 0;
  int ncounters = 0;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t gexec = nullptr;
};

namespace sgw {
namespace {

sgw_status multi_error(const std::string& m) {
  set_error(m);
  return SGW_ERR_ARG;
}

// Number of vector slots one right-hand side of this system needs (as run_msbicg).
struct SlotNeed {
  int Kcap, P, mode;
  long long nvec;
  long long ncoef;
};

template <typename T>
SlotNeed slot_need(const sgw_operator* op, const sgw_batch_desc& d, int l, int max_iter) {
  const int Sm1 = d.num_shift - 1, Db = 2 * l + 2;
  SlotNeed s{};
  s.P = std::max(32, (Sm1 + 31) / 32 * 32);
  int Tw = d.history_iters;
  if (Tw <= 0) {
    const double per_iter = (double)Db * op->npwx * sizeof(cplx<T>);
    Tw = (int)std::max(1.0, std::min((double)max_iter, (32.0 * 1024 * 1024) / per_iter));
  }
  Tw = std::max(1, std::min(Tw, max_iter));
  s.mode = l > 8 ? 1 : 0;
  s.Kcap = (Sm1 > 0 && s.mode == 0) ? Db * Tw : 0;
  s.nvec = (2LL * l + 4) + (s.mode == 0 ? s.Kcap + (Sm1 > 0 ? Sm1 : 0) : (long long)Sm1 * (l + 2));
  s.ncoef = CoefLayout(l, s.P, s.Kcap).total;
  return s;
}

template <typename T, bool LINES>
using PwA = PwApply<T, Ipt<T>::v, LINES>;

template <typename T>
PwView<T> view_of(sgw_operator* op) {
  PwView<T> v = pwview<T>(op);
  v.alpha_pv = op->alpha_pv;
  return v;
}

// Build the launch groups of one solve stage (precision T) over all systems.
// mk(i) returns the SolverArgs<T> of system i with everything but the workspace.
template <typename T, class MK>
sgw_status build_solve_groups(sgw_multi* P, std::vector<MultiGroup>& groups, DevBuf& vec, DevBuf& coef, DevBuf& col,
                              MK&& mk) {
  const int ns = P->nsys;
  long long vec_stride = 0, coef_stride = 0, col_stride = 0;
  std::vector<SolverArgs<T>> args(ns);
  for (int i = 0; i < ns; ++i) {
    args[i] = mk(i);
    const SlotNeed need = slot_need<T>(P->ops[i], P->d[i], args[i].lmax, args[i].max_iter);
    args[i].Kcap = need.Kcap;
    args[i].P = need.P;
    args[i].mode = need.mode;
    vec_stride = std::max(vec_stride, need.nvec * P->ops[i]->npwx);
    coef_stride = std::max(coef_stride, need.ncoef);
    if (!pwshape<T>(P->ops[i]).col_in_smem) col_stride = std::max(col_stride, col_elems<T>(P->ops[i]));
  }
  sgw_status s;
  if ((s = vec.ensure(sizeof(cplx<T>) * (size_t)P->nslots * vec_stride)) != SGW_OK) return s;
  if ((s = coef.ensure(sizeof(zcd) * (size_t)P->nslots * coef_stride)) != SGW_OK) return s;
  if ((s = col.ensure(sizeof(cplx<T>) * (size_t)P->nslots * std::max<long long>(col_stride, 1))) != SGW_OK) return s;
  for (int i = 0; i < ns; ++i) {
    args[i].ws_vec = vec.as<cplx<T>>();
    args[i].vec_stride = vec_stride;
    args[i].ws_coef = coef.as<zcd>();
    args[i].ncoef_slot = coef_stride;
    args[i].col_global = col.as<cplx<T>>();
    args[i].col_slot = col_stride;
    args[i].counter = nullptr;
  }
  // items longest first: operator cost x (2l applies + shift work)
  std::vector<double> cost(ns);
  for (int i = 0; i < ns; ++i) {
    const PwView<double>& v = P->ops[i]->pw64;
    cost[i] = apply_cost(v) * 2 * P->d[i].lmax + 8.0 * v.npw * (2 * P->d[i].lmax + 2) * P->d[i].num_shift;
  }
  groups.clear();
  for (int variant = 0; variant < 2; ++variant) {
    const bool lines = variant == 0;
    std::vector<int> sys;
    for (int i = 0; i < ns; ++i)
      if (pwshape<T>(P->ops[i]).lines == lines) sys.push_back(i);
    if (sys.empty()) continue;
    MultiGroup g;
    g.lines = lines;
    std::vector<MultiItem> items;
    std::vector<int> order(sys);
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return cost[x] > cost[y]; });
    for (int i : order)
      for (int r = 0; r < P->d[i].nrhs; ++r) items.push_back(MultiItem{i, r});
    g.nitems = (int)items.size();
    if ((s = g.items.upload(items.data(), std::max<size_t>(items.size(), 1))) != SGW_OK) return s;
    // constant-memory image indexed by system number (systems of the other variant are left zero)
    auto build = [&](auto tag) -> sgw_status {
      using AT = decltype(tag);
      using E = SolveEntry<T, AT>;
      if (sizeof(E) * ns > kConstBytes) {
        set_error("too many systems for one launch: at most " + std::to_string(kConstBytes / sizeof(E)));
        return SGW_ERR_UNSUPPORTED;
      }
      std::vector<E> img(ns);
      std::memset(static_cast<void*>(img.data()), 0, sizeof(E) * ns);
      for (int i : sys) {
        const PwShape& sh = pwshape<T>(P->ops[i]);
        img[i].a = args[i];
        img[i].A = AT{view_of<T>(P->ops[i]), sh.col_in_smem, sh.ng};
        g.smem = std::max(g.smem, sh.smem);
      }
      g.entry_bytes = sizeof(E) * ns;
      sgw_status st = g.entries.upload(reinterpret_cast<unsigned char*>(img.data()), g.entry_bytes);
      if (st != SGW_OK || sizeof(T) == 8) return st;
      for (int i : sys) img[i].a.gemm_tc = 1;
      return g.entries_tc.upload(reinterpret_cast<unsigned char*>(img.data()), g.entry_bytes);
    };
    s = lines ? build(PwA<T, true>{}) : build(PwA<T, false>{});
    if (s != SGW_OK) return s;
    groups.push_back(std::move(g));
  }
  return SGW_OK;
}

// FP64 seed-residual groups (mixed precision)
sgw_status build_res_groups(sgw_multi* P) {
  const int ns = P->nsys;
  long long col_stride = 0;
  for (int i = 0; i < ns; ++i)
    if (!pwshape<double>(P->ops[i]).col_in_smem) col_stride = std::max(col_stride, col_elems<double>(P->ops[i]));
  sgw_status s;
  if ((s = P->col64.ensure(sizeof(zcd) * (size_t)P->nslots * std::max<long long>(col_stride, 1))) != SGW_OK) return s;
  P->res_groups.clear();
  for (int variant = 0; variant < 2; ++variant) {
    const bool lines = variant == 0;
    std::vector<int> sys;
    for (int i = 0; i < ns; ++i)
      if (pwshape<double>(P->ops[i]).lines == lines) sys.push_back(i);
    if (sys.empty()) continue;
    MultiGroup g;
    g.lines = lines;
    std::vector<MultiItem> items;
    for (int i : sys)
      for (int r = 0; r < P->d[i].nrhs; ++r) items.push_back(MultiItem{i, r});
    g.nitems = (int)items.size();
    if ((s = g.items.upload(items.data(), std::max<size_t>(items.size(), 1))) != SGW_OK) return s;
    auto build = [&](auto tag) -> sgw_status {
      using AT = decltype(tag);
      using E = ResEntry<AT>;
      if (sizeof(E) * ns > kConstBytes) {
        set_error("too many systems for one launch");
        return SGW_ERR_UNSUPPORTED;
      }
      std::vector<E> img(ns);
      std::memset(static_cast<void*>(img.data()), 0, sizeof(E) * ns);
      for (int i : sys) {
        const PwShape& sh = pwshape<double>(P->ops[i]);
        const sgw_batch_desc& d = P->d[i];
        img[i].A = AT{view_of<double>(P->ops[i]), sh.col_in_smem, sh.ng};
        img[i].n = P->ops[i]->n;
        img[i].bb = reinterpret_cast<const zcd*>(d.bb);
        img[i].ldb = d.ldb;
        img[i].sigma = reinterpret_cast<const zcd*>(d.sigma);
        img[i].lds = d.lds;
        img[i].x = reinterpret_cast<const zcd*>(d.xx);
        img[i].ldr = d.ldr;
        img[i].r = P->ms[i].r64;
        img[i].ldrr = P->ops[i]->npwx;
        img[i].active = P->ms[i].active;
        g.smem = std::max(g.smem, sh.smem);
      }
      g.entry_bytes = sizeof(E) * ns;
      return g.entries.upload(reinterpret_cast<unsigned char*>(img.data()), g.entry_bytes);
    };
    s = lines ? build(PwA<double, true>{}) : build(PwA<double, false>{});
    if (s != SGW_OK) return s;
    P->res_groups.push_back(std::move(g));
  }
  return SGW_OK;
}

// Launch one stage: every group of it (constant image, counter reset, persistent launch).
template <typename T>
sgw_status launch_solve_stage(sgw_multi* P, std::vector<MultiGroup>& groups, int& counter_idx, DevBuf& col,
                              bool tc = false) {
  for (MultiGroup& g : groups) {
    int* counter = P->counters.as<int>() + counter_idx++;
    SGW_CK(cudaMemsetAsync(counter, 0, sizeof(int), P->stream));
    SGW_CK(cudaMemcpyToSymbolAsync(c_entries, (tc ? g.entries_tc : g.entries).p, g.entry_bytes, 0,
                                   cudaMemcpyDeviceToDevice, P->stream));
    constexpr int NT = CtaThreads<T>::v;
    const int grid = std::max(1, std::min(P->num_sms * CtasPerSm<T>::v, g.nitems));
    unsigned long long* sys_end = P->stamps.as<unsigned long long>() + 1;
    long long col_slot = 0;
    for (int i = 0; i < P->nsys; ++i)
      if (!pwshape<T>(P->ops[i]).col_in_smem) col_slot = std::max(col_slot, col_elems<T>(P->ops[i]));
    if (g.lines) {
      auto k = msbicg_multi_kernel<T, PwA<T, true>, NT>;
      k<<<grid, NT, g.smem, P->stream>>>(g.items.as<MultiItem>(), g.nitems, counter, col.as<cplx<T>>(), col_slot,
                                          sys_end);
    } else {
      auto k = msbicg_multi_kernel<T, PwA<T, false>, NT>;
      k<<<grid, NT, g.smem, P->stream>>>(g.items.as<MultiItem>(), g.nitems, counter, col.as<cplx<T>>(), col_slot,
                                          sys_end);
    }
    SGW_CK(cudaGetLastError());
    P->launches += 1;
  }
  return SGW_OK;
}

sgw_status launch_res_stage(sgw_multi* P, int& counter_idx) {
  for (MultiGroup& g : P->res_groups) {
    int* counter = P->counters.as<int>() + counter_idx++;
    SGW_CK(cudaMemsetAsync(counter, 0, sizeof(int), P->stream));
    SGW_CK(cudaMemcpyToSymbolAsync(c_entries, g.entries.p, g.entry_bytes, 0, cudaMemcpyDeviceToDevice, P->stream));
    constexpr int NT = CtaThreads<double>::v;
    const int grid = std::max(1, std::min(P->num_sms, g.nitems));
    unsigned long long* sys_end = P->stamps.as<unsigned long long>() + 1;
    long long col_slot = 0;
    for (int i = 0; i < P->nsys; ++i)
      if (!pwshape<double>(P->ops[i]).col_in_smem) col_slot = std::max(col_slot, col_elems<double>(P->ops[i]));
    if (g.lines) {
      auto k = residual_multi_kernel<PwA<double, true>, NT>;
      k<<<grid, NT, g.smem, P->stream>>>(g.items.as<MultiItem>(), g.nitems, counter, P->col64.as<zcd>(), col_slot,
                                          sys_end);
    } else {
      auto k = residual_multi_kernel<PwA<double, false>, NT>;
      k<<<grid, NT, g.smem, P->stream>>>(g.items.as<MultiItem>(), g.nitems, counter, P->col64.as<zcd>(), col_slot,
                                          sys_end);
    }
    SGW_CK(cudaGetLastError());
    P->launches += 1;
  }
  return SGW_OK;
}

// FP32 seed-residual update groups (mixed rounds after the first)
sgw_status build_upd_groups(sgw_multi* P) {
  const int ns = P->nsys;
  sgw_status s;
  P->upd_groups.clear();
  for (int variant = 0; variant < 2; ++variant) {
    const bool lines = variant == 0;
    std::vector<int> sys;
    for (int i = 0; i < ns; ++i)
      if (pwshape<float>(P->ops[i]).lines == lines) sys.push_back(i);
    if (sys.empty()) continue;
    MultiGroup g;
    g.lines = lines;
    std::vector<MultiItem> items;
    for (int i : sys)
      for (int r = 0; r < P->d[i].nrhs; ++r) items.push_back(MultiItem{i, r});
    g.nitems = (int)items.size();
    if ((s = g.items.upload(items.data(), std::max<size_t>(items.size(), 1))) != SGW_OK) return s;
    auto build = [&](auto tag) -> sgw_status {
      using AT = decltype(tag);
      using E = ResUpdEntry<AT>;
      if (sizeof(E) * ns > kConstBytes) {
        set_error("too many systems for one launch");
        return SGW_ERR_UNSUPPORTED;
      }
      std::vector<E> img(ns);
      std::memset(static_cast<void*>(img.data()), 0, sizeof(E) * ns);
      for (int i : sys) {
        const PwShape& sh = pwshape<float>(P->ops[i]);
        const sgw_batch_desc& d = P->d[i];
        const long long npwx = P->ops[i]->npwx;
        img[i].A = AT{view_of<float>(P->ops[i]), sh.col_in_smem, sh.ng};
        img[i].n = P->ops[i]->n;
        img[i].sigma = reinterpret_cast<const zcd*>(d.sigma);
        img[i].lds = d.lds;
        img[i].c = P->ms[i].r32;
        img[i].ac = P->ms[i].y32;
        img[i].ldac = (long long)d.num_shift * npwx;
        img[i].r = P->ms[i].r64;
        img[i].ldrr = npwx;
        img[i].active = P->ms[i].active;
        g.smem = std::max(g.smem, sh.smem);
      }
      g.entry_bytes = sizeof(E) * ns;
      return g.entries.upload(reinterpret_cast<unsigned char*>(img.data()), g.entry_bytes);
    };
    s = lines ? build(PwA<float, true>{}) : build(PwA<float, false>{});
    if (s != SGW_OK) return s;
    P->upd_groups.push_back(std::move(g));
  }
  return SGW_OK;
}

sgw_status launch_upd_stage(sgw_multi* P, int& counter_idx) {
  for (MultiGroup& g : P->upd_groups) {
    int* counter = P->counters.as<int>() + counter_idx++;
    SGW_CK(cudaMemsetAsync(counter, 0, sizeof(int), P->stream));
    SGW_CK(cudaMemcpyToSymbolAsync(c_entries, g.entries.p, g.entry_bytes, 0, cudaMemcpyDeviceToDevice, P->stream));
    constexpr int NT = CtaThreads<float>::v;
    const int grid = std::max(1, std::min(P->num_sms, g.nitems));
    unsigned long long* sys_end = P->stamps.as<unsigned long long>() + 1;
    long long col_slot = 0;
    for (int i = 0; i < P->nsys; ++i)
      if (!pwshape<float>(P->ops[i]).col_in_smem) col_slot = std::max(col_slot, col_elems<float>(P->ops[i]));
    if (g.lines) {
      auto k = residual_update_multi_kernel<PwA<float, true>, NT>;
      k<<<grid, NT, g.smem, P->stream>>>(g.items.as<MultiItem>(), g.nitems, counter, P->col.as<zcf>(), col_slot,
                                          sys_end);
    } else {
      auto k = residual_update_multi_kernel<PwA<float, false>, NT>;
      k<<<grid, NT, g.smem, P->stream>>>(g.items.as<MultiItem>(), g.nitems, counter, P->col.as<zcf>(), col_slot,
                                          sys_end);
    }
    SGW_CK(cudaGetLastError());
    P->launches += 1;
  }
  return SGW_OK;
}

sgw_status set_upd_attrs(std::vector<MultiGroup>& groups) {
  constexpr int NT = CtaThreads<float>::v;
  for (MultiGroup& g : groups) {
    if (g.lines) {
      SGW_CK(cudaFuncSetAttribute(residual_update_multi_kernel<PwA<float, true>, NT>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, (int)g.smem));
    } else {
      SGW_CK(cudaFuncSetAttribute(residual_update_multi_kernel<PwA<float, false>, NT>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, (int)g.smem));
    }
  }
  return SGW_OK;
}

template <typename T>
sgw_status set_smem_attrs(std::vector<MultiGroup>& groups) {
  constexpr int NT = CtaThreads<T>::v;
  for (MultiGroup& g : groups) {
    if (g.lines) {
      SGW_CK(cudaFuncSetAttribute(msbicg_multi_kernel<T, PwA<T, true>, NT>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, (int)g.smem));
    } else {
      SGW_CK(cudaFuncSetAttribute(msbicg_multi_kernel<T, PwA<T, false>, NT>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, (int)g.smem));
    }
  }
  return SGW_OK;
}

sgw_status set_res_attrs(std::vector<MultiGroup>& groups) {
  constexpr int NT = CtaThreads<double>::v;
  for (MultiGroup& g : groups) {
    if (g.lines) {
      SGW_CK(cudaFuncSetAttribute(residual_multi_kernel<PwA<double, true>, NT>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, (int)g.smem));
    } else {
      SGW_CK(cudaFuncSetAttribute(residual_multi_kernel<PwA<double, false>, NT>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, (int)g.smem));
    }
  }
  return SGW_OK;
}

// The whole solve as stream work (no host synchronisation): graph-capturable.
sgw_status enqueue(sgw_multi* P) {
  P->launches = 0;
  int ci = 0;
  const int ns = P->nsys;
  SGW_CK(cudaMemsetAsync(P->stamps.p, 0, sizeof(unsigned long long) * (ns + 1), P->stream));
  stamp_kernel<<<1, 1, 0, P->stream>>>(P->stamps.as<unsigned long long>());
  P->launches += 1;
  if (P->opt.precision == 0) return launch_solve_stage<double>(P, P->solve_groups, ci, P->col);
  const int tb = 256;
  const int rounds = P->opt.refine_max > 0 ? P->opt.refine_max : 4;
  const double thr = P->opt.refine_threshold > 0.0 ? P->opt.refine_threshold : 1e-9;
  for (int i = 0; i < ns; ++i) {
    const sgw_batch_desc& d = P->d[i];
    const auto& m = P->ms[i];
    const int R = d.nrhs, S = d.num_shift, n = P->ops[i]->n, npwx = P->ops[i]->npwx;
    if (R == 0) continue;
    mx_init<<<(R * S + tb - 1) / tb, tb, 0, P->stream>>>(R, S, m.Z, m.active, d.iters, m.bad);
    mx_bnorm<<<R, tb, 0, P->stream>>>(R, n, reinterpret_cast<const zcd*>(d.bb), d.ldb, m.bnorm);
    SGW_CK(cudaMemcpy2DAsync(m.r64, sizeof(zcd) * npwx, d.bb, sizeof(zcd) * d.ldb, sizeof(zcd) * n, R,
                             cudaMemcpyDeviceToDevice, P->stream));
    P->launches += 2;
  }
  for (int round = 0; round <= rounds; ++round) {
    for (int i = 0; i < ns; ++i) {
      const sgw_batch_desc& d = P->d[i];
      const auto& m = P->ms[i];
      const int R = d.nrhs, n = P->ops[i]->n, npwx = P->ops[i]->npwx;
      if (R == 0) continue;
      mx_normalise<<<R, tb, 0, P->stream>>>(R, n, npwx, m.r64, npwx, m.r32, m.scale, round == 0 ? nullptr : m.bnorm,
                                            thr, m.active, m.nactive);
      P->launches += 1;
    }
    if (round == rounds) break;
    sgw_status s = launch_solve_stage<float>(P, P->solve_groups, ci, P->col, round > 0);
    if (s != SGW_OK) return s;
    for (int i = 0; i < ns; ++i) {
      const sgw_batch_desc& d = P->d[i];
      const auto& m = P->ms[i];
      const int R = d.nrhs, S = d.num_shift, n = P->ops[i]->n, npwx = P->ops[i]->npwx;
      if (R == 0) continue;
      mx_accumulate<<<R * S, tb, 0, P->stream>>>(R, S, n, npwx, m.y32, reinterpret_cast<zcd*>(d.xx), d.ldx, d.ldr,
                                                 m.Z, m.scale, m.active, round == 0, m.bad,
                                                 round > 0 ? m.r32 : nullptr);
      mx_update_z<<<(R * S + tb - 1) / tb, tb, 0, P->stream>>>(R, S, m.Z, m.zeta, m.active, d.iters, m.iters_round);
      P->launches += 2;
    }
    // round 0: FP64 b - A x; later rounds: r -= A c in FP32
    if ((s = round == 0 ? launch_res_stage(P, ci) : launch_upd_stage(P, ci)) != SGW_OK) return s;
  }
  for (int i = 0; i < ns; ++i) {
    const sgw_batch_desc& d = P->d[i];
    const int R = d.nrhs;
    if (R == 0) continue;
    mx_finish<<<(R + tb - 1) / tb, tb, 0, P->stream>>>(R, P->ms[i].active, P->ms[i].bad, d.ierr, 1);
    P->launches += 1;
  }
  SGW_CK(cudaGetLastError());
  return SGW_OK;
}

sgw_status multi_create(int nsys, sgw_operator* const* ops, const sgw_batch_desc* descs,
                        const sgw_multi_options* opt, sgw_multi** out) {
  if (out) *out = nullptr;
  if (nsys < 1 || !ops || !descs || !out) return multi_error("invalid multi-system arguments");
  sgw_multi_options o{};
  if (opt) o = *opt;
  if (o.precision != 0 && o.precision != 1) return multi_error("precision must be 0 (FP64) or 1 (mixed)");
  for (int i = 0; i < nsys; ++i) {
    const sgw_operator* op = ops[i];
    const sgw_batch_desc& d = descs[i];
    if (!op || op->kind != 1) return multi_error("every system needs a plane-wave operator");
    if (op->device != ops[0]->device) return multi_error("all operators must live on one device");
    if (d.memory != 1) return multi_error("multi-system batches take device pointers (memory = 1)");
    if (d.nrhs < 0 || d.num_shift < 1 || d.lmax < 1 || d.lmax > kMaxL - 1 || d.max_iter < 1)
      return multi_error("invalid batch sizes of system " + std::to_string(i));
    if (d.nrhs > 0 && (!d.bb || !d.sigma || !d.xx || !d.ierr || !d.iters))
      return multi_error("null batch array of system " + std::to_string(i) + " (iters is required)");
    if (d.ldb < op->n || d.lds < d.num_shift || d.ldx < op->n || d.ldr < d.ldx * (d.num_shift - 1) + op->n)
      return multi_error("leading dimensions too small in system " + std::to_string(i));
    if (op->shape64.ng < 1 || op->shape32.ng < 1) return multi_error("FFT box too large for shared memory");
  }
  sgw_multi* P = new sgw_multi();
  P->nsys = nsys;
  P->ops.assign(ops, ops + nsys);
  P->d.assign(descs, descs + nsys);
  P->opt = o;
  P->num_sms = ops[0]->num_sms;
  P->nslots = P->num_sms * std::max(CtasPerSm<float>::v, CtasPerSm<double>::v);
  auto fail = [&](sgw_status s) {
    sgw_multi_destroy(P);
    return s;
  };
  if (cudaStreamCreateWithFlags(&P->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&P->e0) != cudaSuccess || cudaEventCreate(&P->e1) != cudaSuccess ||
      cudaEventCreateWithFlags(&P->ev_caller, cudaEventDisableTiming) != cudaSuccess) {
    set_error("stream/event creation failed");
    return fail(SGW_ERR_CUDA);
  }
  sgw_status s;
  if ((s = P->stamps.ensure(sizeof(unsigned long long) * (nsys + 1))) != SGW_OK) return fail(s);
  const int rounds = o.refine_max > 0 ? o.refine_max : 4;
  P->ncounters = 4 * (rounds + 1) + 4;
  if ((s = P->counters.ensure(sizeof(int) * P->ncounters)) != SGW_OK) return fail(s);
  if (o.precision == 0) {
    s = build_solve_groups<double>(P, P->solve_groups, P->vec, P->coef, P->col, [&](int i) {
      const sgw_batch_desc& d = P->d[i];
      SolverArgs<double> a{};
      a.lmax = d.lmax;
      a.max_iter = d.max_iter;
      a.threshold = d.threshold;
      a.nshift = d.num_shift;
      a.nrhs = d.nrhs;
      a.npw = P->ops[i]->n;
      a.npwx = P->ops[i]->npwx;
      a.bb = reinterpret_cast<const zcd*>(d.bb);
      a.ldb = d.ldb;
      a.sigma = reinterpret_cast<const zcd*>(d.sigma);
      a.lds = d.lds;
      a.xx = reinterpret_cast<zcd*>(d.xx);
      a.ldx = d.ldx;
      a.ldr = d.ldr;
      a.ierr = d.ierr;
      a.iters = d.iters;
      return a;
    });
    if (s != SGW_OK) return fail(s);
    if ((s = set_smem_attrs<double>(P->solve_groups)) != SGW_OK) return fail(s);
  } else {
    // per-system mixed workspace, 256-byte aligned pieces
    auto al = [](size_t v) { return (v + 255) / 256 * 256; };
    std::vector<size_t> off(nsys + 1, 0);
    for (int i = 0; i < nsys; ++i) {
      const size_t R = P->d[i].nrhs, S = P->d[i].num_shift, npwx = P->ops[i]->npwx;
      off[i + 1] = off[i] + al(sizeof(zcd) * R * npwx) + al(sizeof(zcf) * R * npwx) + al(sizeof(zcf) * R * S * npwx) +
                   2 * al(sizeof(zcd) * R * S) + 2 * al(sizeof(double) * R) + 4 * al(sizeof(int) * R) + 256;
    }
    if ((s = P->mixed.ensure(std::max<size_t>(off[nsys], 256))) != SGW_OK) return fail(s);
    P->ms.resize(nsys);
    for (int i = 0; i < nsys; ++i) {
      const size_t R = P->d[i].nrhs, S = P->d[i].num_shift, npwx = P->ops[i]->npwx;
      unsigned char* p = reinterpret_cast<unsigned char*>(P->mixed.p) + off[i];
      auto take = [&](size_t bytes) {
        unsigned char* q = p;
        p += al(bytes);
        return q;
      };
      auto& m = P->ms[i];
      m.r64 = reinterpret_cast<zcd*>(take(sizeof(zcd) * R * npwx));
      m.r32 = reinterpret_cast<zcf*>(take(sizeof(zcf) * R * npwx));
      m.y32 = reinterpret_cast<zcf*>(take(sizeof(zcf) * R * S * npwx));
      m.Z = reinterpret_cast<zcd*>(take(sizeof(zcd) * R * S));
      m.zeta = reinterpret_cast<zcd*>(take(sizeof(zcd) * R * S));
      m.scale = reinterpret_cast<double*>(take(sizeof(double) * R));
      m.bnorm = reinterpret_cast<double*>(take(sizeof(double) * R));
      m.active = reinterpret_cast<int*>(take(sizeof(int) * R));
      m.iters_round = reinterpret_cast<int*>(take(sizeof(int) * R));
      m.nactive = reinterpret_cast<int*>(take(sizeof(int) * R));
      m.bad = reinterpret_cast<int*>(take(sizeof(int) * R));
    }
    s = build_solve_groups<float>(P, P->solve_groups, P->vec, P->coef, P->col, [&](int i) {
      const sgw_batch_desc& d = P->d[i];
      const auto& m = P->ms[i];
      const int npwx = P->ops[i]->npwx;
      SolverArgs<float> a{};
      a.lmax = std::min(d.lmax, kMixedMaxL);
      a.max_iter = d.max_iter;
      a.threshold = kRoundRelThreshold;
      a.nshift = d.num_shift;
      a.nrhs = d.nrhs;
      a.npw = P->ops[i]->n;
      a.npwx = npwx;
      a.bb = m.r32;
      a.ldb = npwx;
      a.sigma = reinterpret_cast<const zcd*>(d.sigma);
      a.lds = d.lds;
      a.xx = m.y32;
      a.ldx = npwx;
      a.ldr = (long long)d.num_shift * npwx;
      a.ierr = d.ierr;
      a.iters = m.iters_round;
      a.active = m.active;
      a.zeta = m.zeta;
      return a;
    });
    if (s != SGW_OK) return fail(s);
    if ((s = set_smem_attrs<float>(P->solve_groups)) != SGW_OK) return fail(s);
    if ((s = build_res_groups(P)) != SGW_OK) return fail(s);
    if ((s = set_res_attrs(P->res_groups)) != SGW_OK) return fail(s);
    if ((s = build_upd_groups(P)) != SGW_OK) return fail(s);
    if ((s = set_upd_attrs(P->upd_groups)) != SGW_OK) return fail(s);
  }
  if (o.use_graph) {
    std::lock_guard<std::mutex> lk(g_const_mutex);
    if (cudaStreamBeginCapture(P->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
      set_error("cudaStreamBeginCapture failed");
      return fail(SGW_ERR_CUDA);
    }
    s = enqueue(P);
    cudaGraph_t g = nullptr;
    const cudaError_t ec = cudaStreamEndCapture(P->stream, &g);
    if (s != SGW_OK) return fail(s);
    if (ec != cudaSuccess || !g) {
      set_error(std::string("stream capture failed: ") + cudaGetErrorString(ec));
      return fail(SGW_ERR_CUDA);
    }
    P->graph = g;
    if (cudaGraphInstantiate(&P->gexec, g, 0) != cudaSuccess) {
      set_error("cudaGraphInstantiate failed");
      return fail(SGW_ERR_CUDA);
    }
  }
  *out = P;
  return SGW_OK;
}

sgw_status multi_run(sgw_multi* P, double* total_ms, double* sys_ms) {
  if (!P) return multi_error("null plan");
  std::lock_guard<std::mutex> lk(g_const_mutex);
  // the plan's device and the caller's stream of its first system's handle
  CallScope cs(P->ops[0]);
  if (cs.status() != SGW_OK) return cs.status();
  sgw_status so = order_after(P->stream, P->ops[0]->caller_stream, P->ev_caller);
  if (so != SGW_OK) return so;
  SGW_CK(cudaEventRecord(P->e0, P->stream));
  if (P->gexec) {
    SGW_CK(cudaGraphLaunch(P->gexec, P->stream));
  } else {
    sgw_status s = enqueue(P);
    if (s != SGW_OK) return s;
  }
  SGW_CK(cudaEventRecord(P->e1, P->stream));
  std::vector<unsigned long long> st(P->nsys + 1);
  SGW_CK(cudaMemcpyAsync(st.data(), P->stamps.p, sizeof(unsigned long long) * (P->nsys + 1), cudaMemcpyDeviceToHost,
                         P->stream));
  SGW_CK(cudaStreamSynchronize(P->stream));
  float ms = 0.f;
  SGW_CK(cudaEventElapsedTime(&ms, P->e0, P->e1));
  if (total_ms) *total_ms = ms;
  if (sys_ms)
    for (int i = 0; i < P->nsys; ++i) sys_ms[i] = st[i + 1] > st[0] ? (double)(st[i + 1] - st[0]) * 1e-6 : 0.0;
  return SGW_OK;
}

// ---------------------------------------------------------------------------
// Autotuner: pick the FFT launch shape (register-line vs shared-memory FFT,
// planes in flight, column store in shared or global memory) of an operator
// by timing its apply kernel on a batch of vectors; results are cached per
// geometry for the process.
// ---------------------------------------------------------------------------
std::mutex g_tune_mutex;
std::map<std::string, PwShape> g_tune_cache;

template <typename T>
std::string tune_key(sgw_operator* op) {
  const PwView<T>& v = pwview<T>(op);
  return std::to_string(sizeof(T)) + ":" + std::to_string(v.nr1) + "x" + std::to_string(v.nr2) + "x" +
         std::to_string(v.nr3) + ":" + std::to_string(v.npw) + ":" + std::to_string(v.ncol) + ":" +
         std::to_string(v.ni1) + ":" + std::to_string(v.nkb) + ":" + std::to_string(v.nocc) + ":" +
         std::to_string(op->smem_optin);
}

template <typename T>
std::vector<PwShape> tune_candidates(sgw_operator* op) {
  const PwView<T>& v = pwview<T>(op);
  const size_t static_bytes = sizeof(SeedShared) + 64;
  const size_t per_cta = std::min(op->smem_optin, op->smem_per_sm / CtasPerSm<T>::v - 1024);
  const size_t budget = per_cta > static_bytes ? per_cta - static_bytes : 0;
  const size_t colb = (size_t)v.ncol * v.ldz * sizeof(cplx<T>);
  auto small = [&](int ng) { return (size_t)pw_smem_small(v, ng) * sizeof(cplx<T>); };
  std::vector<PwShape> c;
  const bool reg = fft_reg_supported<T>(v.nr1) && fft_reg_supported<T>(v.nr2) && fft_reg_supported<T>(v.nr3);
  for (int lines = reg ? 1 : 0; lines >= 0; --lines)
    for (int in_smem = 1; in_smem >= 0; --in_smem) {
      // line FFT: every plane count up to 32 (the counts that fill the i2 and
      // i1 passes' thread rounds evenly differ from box to box)
      std::vector<int> pfs;
      if (lines)
        for (int pf = 1; pf <= 32; ++pf) pfs.push_back(pf);
      else
        pfs = {1, 2, 4};
      for (int pf : pfs) {
        if (lines && pf > v.nr3) continue;
        const size_t need = small(pf) + (in_smem ? colb : 0);
        if (need > budget) continue;
        PwShape s;
        s.lines = lines;
        s.ng = pf;
        s.col_in_smem = in_smem;
        s.smem = need;
        c.push_back(s);
      }
    }
  return c;
}

template <typename T>
__global__ void tune_fill(cplx<T>* p, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    p[i] = cplx<T>{(T)(0.5 + 1e-3 * (double)(i % 97)), (T)(-0.25 + 1e-3 * (double)(i % 89))};
}

template <typename T>
sgw_status tune(sgw_operator* op, sgw_tune_result* res) {
  const std::string key = tune_key<T>(op);
  {
    std::lock_guard<std::mutex> lk(g_tune_mutex);
    auto it = g_tune_cache.find(key);
    if (it != g_tune_cache.end()) {
      pwshape<T>(op) = it->second;
      if (res) {
        res->lines = it->second.lines;
        res->col_in_smem = it->second.col_in_smem;
        res->planes = it->second.ng;
        res->us_per_apply = 0.0;
        res->candidates = 0;
        res->cached = 1;
      }
      return SGW_OK;
    }
  }
  const std::vector<PwShape> cand = tune_candidates<T>(op);
  if (cand.empty()) {
    set_error("no FFT launch shape fits in shared memory");
    return SGW_ERR_UNSUPPORTED;
  }
  const int m = 2 * op->num_sms * CtasPerSm<T>::v;
  const int npwx = op->npwx;
  DevBuf x, y;
  sgw_status s;
  if ((s = x.ensure(sizeof(cplx<T>) * (size_t)m * npwx)) != SGW_OK) return s;
  if ((s = y.ensure(sizeof(cplx<T>) * (size_t)m * npwx)) != SGW_OK) return s;
  tune_fill<T><<<op->num_sms, 256, 0, op->stream>>>(x.as<cplx<T>>(), (long long)m * npwx);
  SGW_CK(cudaGetLastError());
  const PwShape keep = pwshape<T>(op);
  double best = 1e30;
  PwShape best_s = keep;
  for (const PwShape& c : cand) {
    pwshape<T>(op) = c;
    float tmin = 1e30f;
    for (int rep = 0; rep < 4; ++rep) {
      SGW_CK(cudaEventRecord(op->lev0, op->stream));
      s = run_apply<T>(op, m, x.as<cplx<T>>(), npwx, y.as<cplx<T>>(), npwx, zcd{-0.3, 0.1});
      if (s != SGW_OK) {
        pwshape<T>(op) = keep;
        return s;
      }
      SGW_CK(cudaEventRecord(op->lev1, op->stream));
      SGW_CK(cudaEventSynchronize(op->lev1));
      float t = 0.f;
      SGW_CK(cudaEventElapsedTime(&t, op->lev0, op->lev1));
      if (rep > 0) tmin = std::min(tmin, t);
    }
    const double us = 1e3 * tmin * op->num_sms * CtasPerSm<T>::v / (double)m;  // one apply on one CTA
    if (us < best) {
      best = us;
      best_s = c;
    }
  }
  pwshape<T>(op) = best_s;
  {
    std::lock_guard<std::mutex> lk(g_tune_mutex);
    g_tune_cache[key] = best_s;
  }
  if (res) {
    res->lines = best_s.lines;
    res->col_in_smem = best_s.col_in_smem;
    res->planes = best_s.ng;
    res->us_per_apply = best;
    res->candidates = (int)cand.size();
    res->cached = 0;
  }
  return SGW_OK;
}

}  // namespace
}  // namespace sgw

extern "C" {

sgw_status sgw_multi_create(int32_t nsys, sgw_operator* const* ops, const sgw_batch_desc* descs,
                            const sgw_multi_options* opt, sgw_multi** plan) {
  try {
    sgw::CallScope cs(nsys > 0 && ops ? ops[0] : nullptr);
    if (cs.status() != SGW_OK) return cs.status();
    return sgw::multi_create(nsys, ops, descs, opt, plan);
  } catch (...) {
    sgw::set_error("host exception in sgw_multi_create");
    return SGW_ERR_NOMEM;
  }
}

sgw_status sgw_multi_run(sgw_multi* plan, double* total_ms, double* sys_ms) {
  try {
    return sgw::multi_run(plan, total_ms, sys_ms);
  } catch (...) {
    sgw::set_error("host exception in sgw_multi_run");
    return SGW_ERR_NOMEM;
  }
}

sgw_status sgw_multi_info(sgw_multi* plan, int64_t* launches_per_run, int32_t* stage_launch_groups,
                          int32_t* graph) {
  if (!plan) {
    sgw::set_error("null plan");
    return SGW_ERR_ARG;
  }
  if (launches_per_run) *launches_per_run = plan->launches;
  if (stage_launch_groups) *stage_launch_groups = (int32_t)plan->solve_groups.size();
  if (graph) *graph = plan->gexec ? 1 : 0;
  return SGW_OK;
}

sgw_status sgw_multi_destroy(sgw_multi* plan) {
  if (!plan) return SGW_OK;
  if (plan->stream) cudaStreamSynchronize(plan->stream);
  if (plan->gexec) cudaGraphExecDestroy(plan->gexec);
  if (plan->graph) cudaGraphDestroy(plan->graph);
  for (auto* gs : {&plan->solve_groups, &plan->res_groups, &plan->upd_groups})
    for (auto& g : *gs) {
      g.entries.release();
      g.entries_tc.release();
      g.items.release();
    }
  for (sgw::DevBuf* b : {&plan->vec, &plan->coef, &plan->col, &plan->col64, &plan->counters, &plan->stamps,
                         &plan->mixed})
    b->release();
  if (plan->e0) cudaEventDestroy(plan->e0);
  if (plan->e1) cudaEventDestroy(plan->e1);
  if (plan->ev_caller) cudaEventDestroy(plan->ev_caller);
  if (plan->stream) cudaStreamDestroy(plan->stream);
  delete plan;
  return SGW_OK;
}

sgw_status sgw_operator_autotune(sgw_operator* op, int32_t precision, sgw_tune_result* result) {
  try {
    if (!op || op->kind != 1) {
      sgw::set_error("sgw_operator_autotune needs a plane-wave operator");
      return SGW_ERR_ARG;
    }
    sgw::CallScope cs(op);
    if (cs.status() != SGW_OK) return cs.status();
    if (precision == 0) return sgw::tune<double>(op, result);
    if (precision == 1) return sgw::tune<float>(op, result);
    sgw::set_error("precision must be 0 (FP64 kernels) or 1 (FP32 kernels)");
    return SGW_ERR_ARG;
  } catch (...) {
    sgw::set_error("host exception in sgw_operator_autotune");
    return SGW_ERR_NOMEM;
  }
}

}  // extern "C"
