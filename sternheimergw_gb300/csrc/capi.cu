// C-ABI entry points of libsgw_gb300.so (declared in include/sgw_capi.h).
#include <sys/mman.h>
#include <unistd.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <unordered_map>
#include <utility>
#include <vector>

#include "host.cuh"
#include "fftreg.cuh"
#include "sgwsolver.cuh"

namespace sgw {

static thread_local std::string g_error;
void set_error(const std::string& msg) { g_error = msg; }

static sgw_status arg_error(const std::string& msg) {
  set_error(msg);
  return SGW_ERR_ARG;
}

// ---------------------------------------------------------------------------
// FFT plans and twiddles
// ---------------------------------------------------------------------------
static bool make_plan(int n, FftPlan& p) {
  if (n < 1 || n > kMaxFftLen) return false;
  p.n = n;
  p.nstage = 0;
  p.rmin = 8;
  int m = n;
  for (int r : {8, 5, 4, 3, 2}) {
    while (m % r == 0) {
      if (p.nstage >= kMaxStages) return false;
      p.radix[p.nstage++] = r;
      p.rmin = std::min(p.rmin, r);
      m /= r;
    }
  }
  if (n == 1) {
    p.radix[0] = 2;  // never used: a length-1 line is the identity
    p.nstage = 0;
    p.rmin = 1;
  }
  return m == 1;
}

template <typename T>
static void twiddles(int n, std::vector<cplx<T>>& out) {
  const long double pi = 3.14159265358979323846264338327950288L;
  for (int e = 0; e < n; ++e) {
    const long double ang = 2.0L * pi * (long double)e / (long double)n;
    out.push_back(cplx<T>{(T)cosl(ang), (T)sinl(ang)});
  }
}

// ---------------------------------------------------------------------------
// Launch-shape selection
// ---------------------------------------------------------------------------
template <typename T>
static PwShape choose_shape(const PwView<T>& v, size_t smem_optin, size_t smem_per_sm) {
  const size_t static_bytes = sizeof(SeedShared) + 64;
  const size_t per_cta = std::min(smem_optin, smem_per_sm / CtasPerSm<T>::v - 1024);
  const size_t budget = per_cta > static_bytes ? per_cta - static_bytes : 0;
  const size_t colb = (size_t)v.ncol * v.ldz * sizeof(cplx<T>);
  auto small = [&](int ng) { return (size_t)pw_smem_small(v, ng) * sizeof(cplx<T>); };
  PwShape s;
  if (fft_reg_supported<T>(v.nr1) && fft_reg_supported<T>(v.nr2) && fft_reg_supported<T>(v.nr3)) {
    // line FFT: as many planes in flight as shared memory holds (column store first)
    s.lines = true;
    for (bool in_smem : {true, false}) {
      int best = 0;
      for (int pf = 1; pf <= v.nr3; ++pf)
        if (small(pf) + (in_smem ? colb : 0) <= budget) best = pf;
      if (best >= (in_smem ? 2 : 1)) {
        s.ng = best;
        s.col_in_smem = in_smem;
        s.smem = small(best) + (in_smem ? colb : 0);
        return s;
      }
    }
    s.lines = false;
  }
  for (int ng : {4, 2, 1}) {
    if (small(ng) + colb <= budget) {
      s.ng = ng;
      s.col_in_smem = true;
      s.smem = small(ng) + colb;
      return s;
    }
  }
  for (int ng : {4, 2, 1}) {
    if (small(ng) <= budget) {
      s.ng = ng;
      s.col_in_smem = false;
      s.smem = small(ng);
      return s;
    }
  }
  s.ng = 0;
  return s;
}

// ---------------------------------------------------------------------------
// Operator construction
// ---------------------------------------------------------------------------
static sgw_status init_common(sgw_operator* op) {
  SGW_CK(cudaGetDevice(&op->device));
  cudaDeviceProp prop;
  SGW_CK(cudaGetDeviceProperties(&prop, op->device));
  op->num_sms = prop.multiProcessorCount;
  op->smem_optin = prop.sharedMemPerBlockOptin;
  op->smem_per_sm = prop.sharedMemPerMultiprocessor;
  SGW_CK(cudaStreamCreateWithFlags(&op->stream, cudaStreamNonBlocking));
  SGW_CK(cudaStreamCreateWithFlags(&op->copy_stream, cudaStreamNonBlocking));
  SGW_CK(cudaEventCreateWithFlags(&op->ev_acc, cudaEventDisableTiming));
  SGW_CK(cudaEventCreateWithFlags(&op->ev_copied, cudaEventDisableTiming));
  SGW_CK(cudaEventCreateWithFlags(&op->ev_caller, cudaEventDisableTiming));
  SGW_CK(cudaEventCreate(&op->ev0));
  SGW_CK(cudaEventCreate(&op->ev1));
  SGW_CK(cudaEventCreate(&op->lev0));
  SGW_CK(cudaEventCreate(&op->lev1));
  for (int i = 0; i < 2 * kMaxTimedLaunches; ++i) SGW_CK(cudaEventCreate(&op->kev[i]));
  return host_staging(op, (size_t)1 << 20, nullptr);
}

sgw_status host_staging(sgw_operator* op, size_t bytes, void** out) {
  if (bytes > op->h_small_bytes) {
    if (op->h_small) {
      SGW_CK(cudaStreamSynchronize(op->stream));
      cudaFreeHost(op->h_small);
      op->h_small = nullptr;
      op->h_small_bytes = 0;
    }
    SGW_CK(cudaHostAlloc(&op->h_small, bytes, cudaHostAllocDefault));
    op->h_small_bytes = bytes;
  }
  if (out) *out = op->h_small;
  return SGW_OK;
}

sgw_status read_count(sgw_operator* op, const int* dev, int* out) {
  void* hs = nullptr;
  const sgw_status s = host_staging(op, sizeof(int), &hs);
  if (s != SGW_OK) return s;
  SGW_CK(cudaMemcpyAsync(hs, dev, sizeof(int), cudaMemcpyDeviceToHost, op->stream));
  SGW_CK(cudaStreamSynchronize(op->stream));
  std::memcpy(out, hs, sizeof(int));
  return SGW_OK;
}

sgw_status order_after(cudaStream_t stream, cudaStream_t caller, cudaEvent_t ev) {
  if (!ev || caller == stream) return SGW_OK;
  SGW_CK(cudaEventRecord(ev, caller));
  SGW_CK(cudaStreamWaitEvent(stream, ev, 0));
  return SGW_OK;
}

CallScope::CallScope(sgw_operator* op) {
  if (!op) return;
  if (cudaGetDevice(&prev_) != cudaSuccess) prev_ = -1;
  if (prev_ != op->device) {
    const cudaError_t e = cudaSetDevice(op->device);
    if (e != cudaSuccess) {
      set_error(std::string("cudaSetDevice(handle's device) failed: ") + cudaGetErrorString(e));
      st_ = SGW_ERR_CUDA;
      return;
    }
    dev_ = op->device;
  }
  st_ = order_after(op->stream, op->caller_stream, op->ev_caller);
}

CallScope::~CallScope() {
  if (dev_ >= 0 && prev_ >= 0) cudaSetDevice(prev_);
}

// Sum the per-kernel event pairs of the finished solve (stream already synchronised).
void collect_kernel_times(sgw_operator* op) {
  // the kinds timed through the event pool; rhs/chi/vjp/screen/sigma keep their own
  for (int k : {K_MSBICG_F64, K_MSBICG_F32, K_RESIDUAL_F64, K_COPY_IN, K_COPY_OUT, K_RESIDUAL_F32}) {
    op->kernel_ms[k] = 0.0;
    op->kernel_launches[k] = 0;
  }
  for (int i = 0; i < op->kev_used; ++i) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, op->kev[2 * i], op->kev[2 * i + 1]) == cudaSuccess) {
      op->kernel_ms[op->kev_kind[i]] += ms;
      op->kernel_launches[op->kev_kind[i]] += 1;
    }
  }
  op->kev_used = 0;
}

template <typename T>
static sgw_status upload_pw(sgw_operator* op, const sgw_pw_operator_desc* d, const std::vector<int>& gcol_h,
                            const std::vector<int>& gi3_h, const std::vector<int>& colpos_h,
                            const std::vector<int>& i1_h, int ncol, int ldz, int pitch, const FftPlan& p1,
                            const FftPlan& p2, const FftPlan& p3, DevBuf& g2k, DevBuf& vrs, DevBuf& vkb, DevBuf& dvan,
                            DevBuf& evq, DevBuf& tw) {
  const int npw = d->npw, npwx = op->npwx;
  const size_t nnr = (size_t)d->nr1 * d->nr2 * d->nr3;
  std::vector<T> g2(npw), vr(nnr), dv(std::max(d->nkb, 1));
  for (int g = 0; g < npw; ++g) g2[g] = (T)d->g2kin[g];
  for (size_t r = 0; r < nnr; ++r) vr[r] = (T)d->vrs[r];
  for (int i = 0; i < d->nkb; ++i) dv[i] = (T)d->dvan[i];
  std::vector<cplx<T>> kb((size_t)std::max(d->nkb, 1) * npwx, cplx<T>{0, 0});
  for (int i = 0; i < d->nkb; ++i)
    for (int g = 0; g < npw; ++g) {
      const sgw_zcomplex z = d->vkb[(size_t)i * d->npwx + g];
      kb[(size_t)i * npwx + g] = cplx<T>{(T)z.re, (T)z.im};
    }
  std::vector<cplx<T>> ev((size_t)std::max(d->nbnd_occ, 1) * npwx, cplx<T>{0, 0});
  for (int v = 0; v < d->nbnd_occ; ++v)
    for (int g = 0; g < npw; ++g) {
      const sgw_zcomplex z = d->evq[(size_t)v * d->npwx + g];
      ev[(size_t)v * npwx + g] = cplx<T>{(T)z.re, (T)z.im};
    }
  std::vector<cplx<T>> twv;
  twiddles<T>(d->nr1, twv);
  twiddles<T>(d->nr2, twv);
  twiddles<T>(d->nr3, twv);
  sgw_status s;
  if ((s = g2k.upload(g2.data(), g2.size())) != SGW_OK) return s;
  if ((s = vrs.upload(vr.data(), vr.size())) != SGW_OK) return s;
  if ((s = vkb.upload(kb.data(), kb.size())) != SGW_OK) return s;
  if ((s = dvan.upload(dv.data(), dv.size())) != SGW_OK) return s;
  if ((s = evq.upload(ev.data(), ev.size())) != SGW_OK) return s;
  if ((s = tw.upload(twv.data(), twv.size())) != SGW_OK) return s;
  PwView<T>& v = pwview<T>(op);
  v.npw = npw;
  v.npwx = npwx;
  v.nr1 = d->nr1;
  v.nr2 = d->nr2;
  v.nr3 = d->nr3;
  v.nnr = (int)nnr;
  v.ncol = ncol;
  v.ni1 = (int)i1_h.size();
  v.ldz = ldz;
  v.pitch = pitch;
  v.g_col = op->gcol.as<int>();
  v.g_i3 = op->gi3.as<int>();
  v.col_pos = op->colpos.as<int>();
  v.i1_list = op->i1list.as<int>();
  v.ymask = op->ymask.as<unsigned long long>();
  v.xmask = op->xmask;
  v.zmask = op->zmask.as<unsigned long long>();
  v.g2kin = g2k.as<T>();
  v.vrs = vrs.as<T>();
  v.nkb = d->nkb;
  v.vkb = vkb.as<cplx<T>>();
  v.dvan = dvan.as<T>();
  v.nocc = d->nbnd_occ;
  v.evq = evq.as<cplx<T>>();
  v.alpha_pv = d->alpha_pv;
  v.p1 = p1;
  v.p2 = p2;
  v.p3 = p3;
  v.tw = tw.as<cplx<T>>();
  pwshape<T>(op) = choose_shape(v, op->smem_optin, op->smem_per_sm);
  return SGW_OK;
}

static sgw_status create_pw(const sgw_pw_operator_desc* d, sgw_operator** out) {
  if (out) *out = nullptr;
  if (!d || !out) return arg_error("null argument");
  if (d->npw < 1 || d->npwx < d->npw || d->nr1 < 1 || d->nr2 < 1 || d->nr3 < 1 || !d->nl || !d->g2kin || !d->vrs)
    return arg_error("invalid plane-wave operator description");
  if (d->nkb < 0 || (d->nkb > 0 && (!d->vkb || !d->dvan)) || d->nbnd_occ < 0 || (d->nbnd_occ > 0 && !d->evq))
    return arg_error("invalid projector description");
  FftPlan p1, p2, p3;
  if (!make_plan(d->nr1, p1) || !make_plan(d->nr2, p2) || !make_plan(d->nr3, p3))
    return arg_error("FFT dimensions must be 2,3,5-smooth and at most 64");
  const long long nnr = (long long)d->nr1 * d->nr2 * d->nr3;
  // sphere -> columns of the box
  std::map<std::pair<int, int>, int> colmap;  // (i2, i1) -> column
  std::vector<int> gcol(d->npw), gi3(d->npw);
  std::vector<std::pair<int, int>> cols;
  for (int g = 0; g < d->npw; ++g) {
    const long long b = d->nl[g];
    if (b < 0 || b >= nnr) return arg_error("nl index outside the FFT box");
    const int i1 = (int)(b % d->nr1), i2 = (int)((b / d->nr1) % d->nr2), i3 = (int)(b / ((long long)d->nr1 * d->nr2));
    auto key = std::make_pair(i2, i1);
    auto it = colmap.find(key);
    if (it == colmap.end()) it = colmap.emplace(key, 0).first;
    gi3[g] = i3;
    (void)it;
  }
  int c = 0;
  for (auto& kv : colmap) {
    kv.second = c++;
    cols.push_back(kv.first);
  }
  for (int g = 0; g < d->npw; ++g) {
    const long long b = d->nl[g];
    const int i1 = (int)(b % d->nr1), i2 = (int)((b / d->nr1) % d->nr2);
    gcol[g] = colmap[std::make_pair(i2, i1)];
  }
  // each box point may hold one sphere point only
  {
    std::vector<long long> seen(d->nl, d->nl + d->npw);
    std::sort(seen.begin(), seen.end());
    if (std::adjacent_find(seen.begin(), seen.end()) != seen.end()) return arg_error("duplicate nl index");
  }
  const int ncol = (int)cols.size();
  const int ldz = d->nr3 | 1;
  const int pitch = d->nr1 | 1;
  std::vector<int> colpos(ncol);
  std::vector<int> i1v;
  for (int k = 0; k < ncol; ++k) {
    colpos[k] = cols[k].second + pitch * cols[k].first;
    i1v.push_back(cols[k].second);
  }
  std::sort(i1v.begin(), i1v.end());
  i1v.erase(std::unique(i1v.begin(), i1v.end()), i1v.end());

  sgw_operator* op = new sgw_operator();
  op->kind = 1;
  op->n = d->npw;
  op->npwx = (d->npw + 31) / 32 * 32;
  op->alpha_pv = d->alpha_pv;
  sgw_status s = init_common(op);
  if (s == SGW_OK) {
    std::vector<int> nl(d->nl, d->nl + d->npw);
    s = op->nlkq.upload(nl.data(), nl.size());
  }
  if (s == SGW_OK) s = op->gcol.upload(gcol.data(), gcol.size());
  if (s == SGW_OK) s = op->gi3.upload(gi3.data(), gi3.size());
  if (s == SGW_OK) s = op->colpos.upload(colpos.data(), colpos.size());
  if (s == SGW_OK) s = op->i1list.upload(i1v.data(), i1v.size());
  if (s == SGW_OK) {
    // column masks of the register-line apply: i2 positions per listed i1, and the listed i1
    std::vector<unsigned long long> ym(i1v.size(), 0ull);
    op->xmask = 0ull;
    for (size_t l = 0; l < i1v.size(); ++l) op->xmask |= 1ull << i1v[l];
    for (int k = 0; k < ncol; ++k) {
      const size_t l = std::lower_bound(i1v.begin(), i1v.end(), cols[k].second) - i1v.begin();
      ym[l] |= 1ull << cols[k].first;
    }
    s = op->ymask.upload(ym.data(), ym.size());
  }
  if (s == SGW_OK) {
    std::vector<unsigned long long> zm(ncol, 0ull);
    for (int g = 0; g < d->npw; ++g) zm[gcol[g]] |= 1ull << gi3[g];
    s = op->zmask.upload(zm.data(), zm.size());
  }
  if (s == SGW_OK)
    s = upload_pw<double>(op, d, gcol, gi3, colpos, i1v, ncol, ldz, pitch, p1, p2, p3, op->g2k64, op->vrs64,
                          op->vkb64, op->dvan64, op->evq64, op->tw64);
  if (s == SGW_OK)
    s = upload_pw<float>(op, d, gcol, gi3, colpos, i1v, ncol, ldz, pitch, p1, p2, p3, op->g2k32, op->vrs32,
                         op->vkb32, op->dvan32, op->evq32, op->tw32);
  if (s == SGW_OK && (op->shape64.ng == 0 || op->shape32.ng == 0)) {
    set_error("FFT plane does not fit in shared memory");
    s = SGW_ERR_UNSUPPORTED;
  }
  if (s != SGW_OK) {
    sgw_operator_destroy(op);
    return s;
  }
  *out = op;
  return SGW_OK;
}

static sgw_status create_dense(int n, const sgw_zcomplex* a, long long lda, sgw_operator** out) {
  if (out) *out = nullptr;
  if (!a || !out || n < 1 || lda < n) return arg_error("invalid dense operator");
  sgw_operator* op = new sgw_operator();
  op->kind = 0;
  op->n = n;
  op->npwx = (n + 31) / 32 * 32;
  sgw_status s = init_common(op);
  std::vector<zcd> h64((size_t)n * n);
  std::vector<zcf> h32((size_t)n * n);
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) {
      const sgw_zcomplex z = a[(size_t)j * lda + i];
      h64[(size_t)j * n + i] = zcd{z.re, z.im};
      h32[(size_t)j * n + i] = zcf{(float)z.re, (float)z.im};
    }
  if (s == SGW_OK) s = op->a64.upload(h64.data(), h64.size());
  if (s == SGW_OK) s = op->a32.upload(h32.data(), h32.size());
  if (s != SGW_OK) {
    sgw_operator_destroy(op);
    return s;
  }
  op->dn64 = DenseView<double>{n, op->npwx, op->a64.as<zcd>()};
  op->dn32 = DenseView<float>{n, op->npwx, op->a32.as<zcf>()};
  *out = op;
  return SGW_OK;
}

// ---------------------------------------------------------------------------
// Batched multishift BiCGStab(l) (device pointers)
// ---------------------------------------------------------------------------
static sgw_status check_batch(sgw_operator* op, const sgw_batch_desc* d) {
  if (!op || !d) return arg_error("null argument");
  if (d->nrhs < 0 || d->num_shift < 1 || d->lmax < 1 || d->lmax > kMaxL - 1 || d->max_iter < 1)
    return arg_error("invalid batch sizes (num_shift >= 1, 1 <= lmax <= 15, max_iter >= 1)");
  if (d->nrhs > 0 && (!d->bb || !d->sigma || !d->xx || !d->ierr)) return arg_error("null batch array");
  if (d->ldb < op->n || d->lds < d->num_shift || d->ldx < op->n || d->ldr < d->ldx * (d->num_shift - 1) + op->n)
    return arg_error("leading dimensions too small");
  if (d->precision != 0 && d->precision != 1) return arg_error("precision must be 0 (FP64) or 1 (mixed)");
  if (d->memory != 0 && d->memory != 1) return arg_error("memory must be 0 (host) or 1 (device)");
  return SGW_OK;
}

static sgw_status solve_batch_device(sgw_operator* op, const BatchDev& b, int precision, int refine_max,
                                     double refine_thr, OutCopy* out = nullptr) {
  if (b.nrhs == 0) return SGW_OK;
  if (precision == 0) return run_msbicg<double>(op, b);
  return solve_mixed(op, b, refine_max, refine_thr, out);
}

static sgw_status to_options(const sgw_batch_options* o, BatchOptions& bo) {
  if (!o) return SGW_OK;
  if (o->shift_refine < 0 || o->shift_refine > 2) return arg_error("shift_refine must be 0, 1 or 2");
  if (o->warm_start != 0 && o->warm_start != 1) return arg_error("warm_start must be 0 or 1");
  if (o->shift_threshold < 0.0 || o->shift_rounds < 0 || o->round_iters < 0)
    return arg_error("negative refinement option");
  bo.shift_refine = o->shift_refine;
  bo.shift_tol = o->shift_threshold > 0.0 ? o->shift_threshold : 1e-6;
  bo.rounds = o->shift_rounds > 0 ? o->shift_rounds : 3;
  bo.round_iters = o->round_iters > 0 ? o->round_iters : 6;
  bo.warm_start = o->warm_start;
  return SGW_OK;
}

static sgw_status solve_batch(sgw_operator* op, const sgw_batch_desc* d, const sgw_batch_options* opt = nullptr) {
  sgw_status s = check_batch(op, d);
  if (s != SGW_OK) return s;
  BatchOptions bo;
  if ((s = to_options(opt, bo)) != SGW_OK) return s;
  const bool extended = opt && (bo.shift_refine > 0 || bo.warm_start);
  double* resid_user = opt && bo.shift_refine > 0 ? opt->shift_resid : nullptr;
  op->last_launches = 0;
  op->kev_used = 0;
  if (d->nrhs == 0) {
    op->last_ms = 0.0;
    return SGW_OK;
  }
  BatchDev b{d->nrhs, d->num_shift, d->lmax, d->max_iter, d->history_iters, d->threshold, nullptr, 0, nullptr, 0,
             nullptr, 0, 0, nullptr, nullptr};
  const int n = op->n, S = d->num_shift, R = d->nrhs;
  std::vector<int> iters_h;
  if (d->memory == 1) {
    b.bb = d->bb;
    b.ldb = d->ldb;
    b.sigma = reinterpret_cast<const zcd*>(d->sigma);
    b.lds = d->lds;
    b.xx = d->xx;
    b.ldx = d->ldx;
    b.ldr = d->ldr;
    b.ierr = d->ierr;
    if ((s = op->st_iters.ensure(sizeof(int) * std::max(R, 1))) != SGW_OK) return s;
    b.iters = d->iters ? d->iters : op->st_iters.as<int>();
    SGW_CK(cudaEventRecord(op->ev0, op->stream));
    if (extended) {
      bo.resid = resid_user;
      s = solve_batch_opts(op, b, d->precision, d->refine_max, d->refine_threshold, bo);
    } else {
      s = solve_batch_device(op, b, d->precision, d->refine_max, d->refine_threshold);
    }
    if (s != SGW_OK) return s;
    SGW_CK(cudaEventRecord(op->ev1, op->stream));
    SGW_CK(cudaStreamSynchronize(op->stream));
  } else {
    // stage host arrays (packed) on the device, copies inside the timed call
    if ((s = op->st_bb.ensure(sizeof(zcd) * (size_t)R * n)) != SGW_OK) return s;
    if ((s = op->st_sigma.ensure(sizeof(zcd) * (size_t)R * S)) != SGW_OK) return s;
    if ((s = op->st_xx.ensure(sizeof(zcd) * (size_t)R * S * n)) != SGW_OK) return s;
    if ((s = op->st_ierr.ensure(sizeof(int) * R)) != SGW_OK) return s;
    if ((s = op->st_iters.ensure(sizeof(int) * R)) != SGW_OK) return s;
    SGW_CK(cudaEventRecord(op->ev0, op->stream));
    const int tin = ktime_begin(op, K_COPY_IN);
    SGW_CK(cudaMemcpy2DAsync(op->st_bb.p, sizeof(zcd) * n, d->bb, sizeof(zcd) * d->ldb, sizeof(zcd) * n, R,
                             cudaMemcpyHostToDevice, op->stream));
    SGW_CK(cudaMemcpy2DAsync(op->st_sigma.p, sizeof(zcd) * S, d->sigma, sizeof(zcd) * d->lds, sizeof(zcd) * S, R,
                             cudaMemcpyHostToDevice, op->stream));
    ktime_end(op, tin);
    b.bb = op->st_bb.p;
    b.ldb = n;
    b.sigma = op->st_sigma.as<zcd>();
    b.lds = S;
    b.xx = op->st_xx.p;
    b.ldx = n;
    b.ldr = (long long)S * n;
    b.ierr = op->st_ierr.as<int>();
    b.iters = op->st_iters.as<int>();
    // a packed host array takes one linear copy; in mixed precision it is issued
    // on the copy stream after each accumulation and overlaps the closing residual
    const bool packed = d->ldx == n && d->ldr == (long long)S * n;
    OutCopy oc;
    oc.host = d->xx;
    oc.bytes = sizeof(zcd) * (size_t)R * S * n;
    if (extended) {
      if (bo.warm_start) {  // the starting guess comes in with the other inputs
        if (packed) {
          SGW_CK(cudaMemcpyAsync(op->st_xx.p, d->xx, oc.bytes, cudaMemcpyHostToDevice, op->stream));
        } else {
          for (int r = 0; r < R; ++r)
            SGW_CK(cudaMemcpy2DAsync(op->st_xx.as<zcd>() + (size_t)r * S * n, sizeof(zcd) * n,
                                     reinterpret_cast<const zcd*>(d->xx) + (size_t)r * d->ldr, sizeof(zcd) * d->ldx,
                                     sizeof(zcd) * n, S, cudaMemcpyHostToDevice, op->stream));
        }
      }
      if (resid_user && (s = op->st_resid.ensure(sizeof(double) * (size_t)R * S)) != SGW_OK) return s;
      bo.resid = resid_user ? op->st_resid.as<double>() : nullptr;
      s = solve_batch_opts(op, b, d->precision, d->refine_max, d->refine_threshold, bo);
      if (s == SGW_OK && resid_user) {  // through the page-locked staging, after ierr and iters
        void* hs = nullptr;
        if ((s = host_staging(op, 2 * sizeof(int) * (size_t)R + sizeof(double) * (size_t)R * S, &hs)) != SGW_OK)
          return s;
        SGW_CK(cudaMemcpyAsync(static_cast<char*>(hs) + 2 * sizeof(int) * (size_t)R, op->st_resid.p,
                               sizeof(double) * (size_t)R * S, cudaMemcpyDeviceToHost, op->stream));
      }
    } else {
      s = solve_batch_device(op, b, d->precision, d->refine_max, d->refine_threshold, packed ? &oc : nullptr);
    }
    if (s != SGW_OK) {
      cudaStreamSynchronize(op->copy_stream);  // no copy into the caller's array outlives the call
      return s;
    }
    // kind 7 times what the copies add after the solve (the part not overlapped)
    const int tout = ktime_begin(op, K_COPY_OUT);
    if (oc.issued) {
      SGW_CK(cudaStreamWaitEvent(op->stream, op->ev_copied, 0));
    } else if (packed) {
      SGW_CK(cudaMemcpyAsync(d->xx, op->st_xx.p, oc.bytes, cudaMemcpyDeviceToHost, op->stream));
    } else if (d->ldr == (long long)S * d->ldx) {  // one copy: every (rhs, shift) row at a uniform host pitch
      SGW_CK(cudaMemcpy2DAsync(d->xx, sizeof(zcd) * d->ldx, op->st_xx.p, sizeof(zcd) * n, sizeof(zcd) * n,
                               (size_t)R * S, cudaMemcpyDeviceToHost, op->stream));
    } else {
      for (int r = 0; r < R; ++r)
        SGW_CK(cudaMemcpy2DAsync(reinterpret_cast<zcd*>(d->xx) + (size_t)r * d->ldr, sizeof(zcd) * d->ldx,
                                 op->st_xx.as<zcd>() + (size_t)r * S * n, sizeof(zcd) * n, sizeof(zcd) * n, S,
                                 cudaMemcpyDeviceToHost, op->stream));
    }
    // ierr and iters through the page-locked staging (they may be pageable arrays)
    void* hs = nullptr;
    const size_t resid_bytes = (extended && resid_user) ? sizeof(double) * (size_t)R * S : 0;
    if ((s = host_staging(op, 2 * sizeof(int) * (size_t)R + resid_bytes, &hs)) != SGW_OK) return s;
    int* hs_ierr = static_cast<int*>(hs);
    SGW_CK(cudaMemcpyAsync(hs_ierr, op->st_ierr.p, sizeof(int) * R, cudaMemcpyDeviceToHost, op->stream));
    if (d->iters)
      SGW_CK(cudaMemcpyAsync(hs_ierr + R, op->st_iters.p, sizeof(int) * R, cudaMemcpyDeviceToHost, op->stream));
    ktime_end(op, tout);
    SGW_CK(cudaEventRecord(op->ev1, op->stream));
    SGW_CK(cudaStreamSynchronize(op->stream));
    std::memcpy(d->ierr, hs_ierr, sizeof(int) * R);
    if (d->iters) std::memcpy(d->iters, hs_ierr + R, sizeof(int) * R);
    if (resid_bytes) std::memcpy(resid_user, hs_ierr + 2 * R, resid_bytes);
  }
  float ms = 0.f;
  SGW_CK(cudaEventElapsedTime(&ms, op->ev0, op->ev1));
  op->last_ms = ms;
  collect_kernel_times(op);
  return SGW_OK;
}

// ---------------------------------------------------------------------------
// Single right-hand side: bicgstab / linear_solver / select_solver
// ---------------------------------------------------------------------------
static sgw_status single_bicgstab(sgw_operator* op, int lmax, double thr, int max_iter, const sgw_zcomplex* bb, int n,
                                  const sgw_zcomplex* sigma, int S, sgw_zcomplex* xx, long long ldx, int* ierr) {
  if (!op || !bb || !sigma || !xx || !ierr) return arg_error("null argument");
  if (n != op->n) return arg_error("right-hand side and operator sizes differ");
  if (S < 1 || ldx < n) return arg_error("we need one solution vector per shift for the result");
  sgw_batch_desc d{};
  d.nrhs = 1;
  d.num_shift = S;
  d.lmax = lmax;
  d.max_iter = max_iter;
  d.threshold = thr;
  d.precision = 0;
  d.memory = 0;
  d.bb = bb;
  d.ldb = n;
  d.sigma = sigma;
  d.lds = S;
  d.xx = xx;
  d.ldx = ldx;
  d.ldr = ldx * (S - 1) + n;
  d.ierr = ierr;
  d.iters = nullptr;
  return solve_batch(op, &d);
}

static sgw_status single_sgw(sgw_operator* op, double thr, int max_iter, const sgw_zcomplex* bb, int n,
                             const sgw_zcomplex* sigma, int S, sgw_zcomplex* xx, long long ldx, int* ierr) {
  if (!op || !bb || !sigma || !xx || !ierr) return arg_error("null argument");
  if (n != op->n) return arg_error("right-hand side and operator sizes differ");
  if (S < 1 || ldx < n) return arg_error("invalid shifts or leading dimension");
  op->last_launches = 0;
  const int npwx = op->npwx;
  const int kcap = std::min(std::min(max_iter, n), 4096) + 1;
  sgw_status s;
  DevBuf& w = op->ws64.vec;
  if ((s = w.ensure(sizeof(zcd) * ((size_t)2 * kcap + 2) * npwx)) != SGW_OK) return s;
  if ((s = op->st_bb.ensure(sizeof(zcd) * npwx)) != SGW_OK) return s;
  if ((s = op->st_sigma.ensure(sizeof(zcd) * S)) != SGW_OK) return s;
  if ((s = op->st_xx.ensure(sizeof(zcd) * (size_t)S * n)) != SGW_OK) return s;
  if ((s = op->st_ierr.ensure(sizeof(int))) != SGW_OK) return s;
  const long long colsz = col_elems<double>(op);
  if (op->kind == 1 && !op->shape64.col_in_smem)
    if ((s = op->ws64.col.ensure(sizeof(zcd) * colsz)) != SGW_OK) return s;
  SGW_CK(cudaEventRecord(op->ev0, op->stream));
  SGW_CK(cudaMemcpyAsync(op->st_bb.p, bb, sizeof(zcd) * n, cudaMemcpyHostToDevice, op->stream));
  SGW_CK(cudaMemcpyAsync(op->st_sigma.p, sigma, sizeof(zcd) * S, cudaMemcpyHostToDevice, op->stream));
  SgwArgs<double> a{};
  a.threshold = thr;
  a.max_iter = max_iter;
  a.nshift = S;
  a.npw = n;
  a.npwx = npwx;
  a.kcap = kcap;
  a.bb = op->st_bb.as<zcd>();
  a.sigma = op->st_sigma.as<zcd>();
  a.xx = op->st_xx.as<zcd>();
  a.ldx = n;
  a.ierr = op->st_ierr.as<int>();
  a.vv = w.as<zcd>();
  a.ww = a.vv + (size_t)kcap * npwx;
  a.res = a.ww + (size_t)kcap * npwx;
  a.newv = a.res + npwx;
  a.col_global = op->ws64.col.as<zcd>();
  s = run_sgw<double>(op, a);
  if (s != SGW_OK) return s;
  SGW_CK(cudaMemcpy2DAsync(xx, sizeof(zcd) * ldx, op->st_xx.p, sizeof(zcd) * n, sizeof(zcd) * n, S,
                           cudaMemcpyDeviceToHost, op->stream));
  SGW_CK(cudaMemcpyAsync(ierr, op->st_ierr.p, sizeof(int), cudaMemcpyDeviceToHost, op->stream));
  SGW_CK(cudaEventRecord(op->ev1, op->stream));
  SGW_CK(cudaStreamSynchronize(op->stream));
  float ms = 0.f;
  SGW_CK(cudaEventElapsedTime(&ms, op->ev0, op->ev1));
  op->last_ms = ms;
  return SGW_OK;
}

static sgw_status apply_host(sgw_operator* op, sgw_zcomplex sigma, int m, const sgw_zcomplex* x, long long ldi,
                             sgw_zcomplex* ax, long long ldo) {
  if (!op || (m > 0 && (!x || !ax)) || m < 0 || ldi < op->n || ldo < op->n) return arg_error("invalid apply arguments");
  if (m == 0) return SGW_OK;
  const int n = op->n, npwx = op->npwx;
  sgw_status s;
  if ((s = op->st_misc.ensure(sizeof(zcd) * (size_t)m * npwx)) != SGW_OK) return s;
  if ((s = op->st_misc2.ensure(sizeof(zcd) * (size_t)m * npwx)) != SGW_OK) return s;
  SGW_CK(cudaMemsetAsync(op->st_misc.p, 0, sizeof(zcd) * (size_t)m * npwx, op->stream));
  SGW_CK(cudaMemcpy2DAsync(op->st_misc.p, sizeof(zcd) * npwx, x, sizeof(zcd) * ldi, sizeof(zcd) * n, m,
                           cudaMemcpyHostToDevice, op->stream));
  s = run_apply<double>(op, m, op->st_misc.as<zcd>(), npwx, op->st_misc2.as<zcd>(), npwx, zcd{sigma.re, sigma.im});
  if (s != SGW_OK) return s;
  SGW_CK(cudaMemcpy2DAsync(ax, sizeof(zcd) * ldo, op->st_misc2.p, sizeof(zcd) * npwx, sizeof(zcd) * n, m,
                           cudaMemcpyDeviceToHost, op->stream));
  SGW_CK(cudaStreamSynchronize(op->stream));
  return SGW_OK;
}

__global__ void widen_kernel(const zcf* in, zcd* out, long long count) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count; i += (long long)gridDim.x * blockDim.x)
    out[i] = zcd{(double)in[i].re, (double)in[i].im};
}
__global__ void narrow_kernel(const zcd* in, zcf* out, long long count) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count; i += (long long)gridDim.x * blockDim.x)
    out[i] = zcf{(float)in[i].re, (float)in[i].im};
}

// A(sigma) x with the FP64 (precision 0) or FP32 (precision 1) operator kernels;
// host (memory 0) or device (memory 1) complex128 vectors.  The FP32 form
// narrows x on the device, applies the mixed-precision solve's operator and
// widens the result.
static sgw_status apply_ex(sgw_operator* op, int precision, int memory, sgw_zcomplex sigma, int m,
                           const sgw_zcomplex* x, long long ldi, sgw_zcomplex* ax, long long ldo) {
  if (!op || (m > 0 && (!x || !ax)) || m < 0 || ldi < op->n || ldo < op->n) return arg_error("invalid apply arguments");
  if (precision != 0 && precision != 1) return arg_error("precision must be 0 (FP64) or 1 (FP32)");
  if (memory != 0 && memory != 1) return arg_error("memory must be 0 (host) or 1 (device)");
  if (m == 0) return SGW_OK;
  const int n = op->n, npwx = op->npwx;
  const long long cnt = (long long)m * npwx;
  const cudaMemcpyKind in_kind = memory ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  const cudaMemcpyKind out_kind = memory ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
  sgw_status s;
  if ((s = op->st_misc.ensure(sizeof(zcd) * (size_t)cnt)) != SGW_OK) return s;
  if ((s = op->st_misc2.ensure(sizeof(zcd) * (size_t)cnt)) != SGW_OK) return s;
  SGW_CK(cudaMemsetAsync(op->st_misc.p, 0, sizeof(zcd) * (size_t)cnt, op->stream));
  SGW_CK(cudaMemcpy2DAsync(op->st_misc.p, sizeof(zcd) * npwx, x, sizeof(zcd) * ldi, sizeof(zcd) * n, m, in_kind,
                           op->stream));
  const zcd sg{sigma.re, sigma.im};
  const int grid = (int)std::min<long long>((cnt + 255) / 256, (long long)op->num_sms * 8);
  if (precision == 0) {
    s = run_apply<double>(op, m, op->st_misc.as<zcd>(), npwx, op->st_misc2.as<zcd>(), npwx, sg);
    if (s != SGW_OK) return s;
  } else {
    if ((s = op->st_misc3.ensure(2 * sizeof(zcf) * (size_t)cnt)) != SGW_OK) return s;
    zcf* x32 = op->st_misc3.as<zcf>();
    zcf* y32 = x32 + cnt;
    narrow_kernel<<<grid, 256, 0, op->stream>>>(op->st_misc.as<zcd>(), x32, cnt);
    s = run_apply<float>(op, m, x32, npwx, y32, npwx, sg);
    if (s != SGW_OK) return s;
    widen_kernel<<<grid, 256, 0, op->stream>>>(y32, op->st_misc2.as<zcd>(), cnt);
    SGW_CK(cudaGetLastError());
  }
  SGW_CK(cudaMemcpy2DAsync(ax, sizeof(zcd) * ldo, op->st_misc2.p, sizeof(zcd) * npwx, sizeof(zcd) * n, m, out_kind,
                           op->stream));
  SGW_CK(cudaStreamSynchronize(op->stream));
  return SGW_OK;
}

// ---------------------------------------------------------------------------
// Page-locked host buffers
// ---------------------------------------------------------------------------
static std::mutex g_host_mu;
static std::unordered_map<void*, size_t> g_host_bufs;  // start -> mapped length

static sgw_status host_alloc(size_t bytes, void** ptr) {
  if (!ptr) return arg_error("null pointer argument");
  *ptr = nullptr;
  if (bytes == 0) return SGW_OK;
  if (bytes > ((size_t)1 << 62)) return arg_error("sgw_host_alloc: size out of range");
  const size_t page = (size_t)sysconf(_SC_PAGESIZE);
  const size_t len = (bytes + page - 1) / page * page;
  void* raw = mmap(nullptr, len, PROT_READ | PROT_WRITE, MAP_PRIVATE | MAP_ANONYMOUS, -1, 0);
  if (raw == MAP_FAILED) {
    set_error("mmap of " + std::to_string(len) + " bytes failed");
    return SGW_ERR_NOMEM;
  }
  char* p = static_cast<char*>(raw);
  // Base pages, populated with a non-zero pattern, pinned, then zeroed.  On
  // the GB300 hosts measured, 4.6 GB buffers on transparent huge pages, and
  // buffers populated with zeros before cudaHostRegister, copied at 3-36 GB/s
  // out once large solves had run (cudaHostAlloc memory at 6-18 GB/s); this
  // form copied at 193 GB/s out and 211 GB/s in at every checkpoint.
  madvise(p, len, MADV_NOHUGEPAGE);
  std::memset(p, 0x5a, len);
  const cudaError_t e = cudaHostRegister(p, len, cudaHostRegisterPortable);
  if (e != cudaSuccess) {
    munmap(p, len);
    set_error(std::string("cudaHostRegister failed: ") + cudaGetErrorString(e));
    return SGW_ERR_CUDA;
  }
  std::memset(p, 0, len);
  {
    std::lock_guard<std::mutex> g(g_host_mu);
    g_host_bufs[p] = len;
  }
  *ptr = p;
  return SGW_OK;
}

static sgw_status host_free(void* ptr) {
  if (!ptr) return SGW_OK;
  size_t len = 0;
  {
    std::lock_guard<std::mutex> g(g_host_mu);
    auto it = g_host_bufs.find(ptr);
    if (it == g_host_bufs.end()) return arg_error("sgw_host_free: pointer not from sgw_host_alloc");
    len = it->second;
    g_host_bufs.erase(it);
  }
  const cudaError_t e = cudaHostUnregister(ptr);
  munmap(ptr, len);
  if (e != cudaSuccess) {
    set_error(std::string("cudaHostUnregister failed: ") + cudaGetErrorString(e));
    return SGW_ERR_CUDA;
  }
  return SGW_OK;
}

}  // namespace sgw

// ---------------------------------------------------------------------------
// extern "C"
// ---------------------------------------------------------------------------
using namespace sgw;

extern "C" {

sgw_status sgw_operator_create_pw(const sgw_pw_operator_desc* desc, sgw_operator** op) {
  try {
    return create_pw(desc, op);
  } catch (...) {
    set_error("host exception in sgw_operator_create_pw");
    return SGW_ERR_NOMEM;
  }
}

sgw_status sgw_operator_create_dense(int32_t n, const sgw_zcomplex* a, int64_t lda, sgw_operator** op) {
  try {
    return create_dense(n, a, lda, op);
  } catch (...) {
    set_error("host exception in sgw_operator_create_dense");
    return SGW_ERR_NOMEM;
  }
}

sgw_status sgw_operator_destroy(sgw_operator* op) {
  if (!op) return SGW_OK;
  if (op->stream) cudaStreamSynchronize(op->stream);
  if (op->copy_stream) cudaStreamSynchronize(op->copy_stream);
  DevBuf* bufs[] = {&op->ymask, &op->zmask, &op->gcol, &op->gi3, &op->colpos, &op->i1list, &op->g2k64, &op->g2k32, &op->vrs64, &op->vrs32,
                    &op->vkb64, &op->vkb32, &op->dvan64, &op->dvan32, &op->evq64, &op->evq32, &op->tw64, &op->tw32,
                    &op->a64, &op->a32, &op->ws64.vec, &op->ws64.coef, &op->ws64.col, &op->ws64.counter,
                    &op->ws32.vec, &op->ws32.coef, &op->ws32.col, &op->ws32.counter, &op->st_bb, &op->st_sigma,
                    &op->st_xx, &op->st_ierr, &op->st_iters, &op->st_misc, &op->st_misc2, &op->st_misc3,
                    &op->st_ref, &op->st_ref2, &op->st_resid, &op->nlkq, &op->lt_psi, &op->lt_box, &op->lt_nlk, &op->lt_evc, &op->lt_dv, &op->lt_bb,
                    &op->lt_flag, &op->lt_part, &op->lt_sidx, &op->lt_xx, &op->lt_chi, &op->lt_w,
                    &op->lt_wwork, &op->lt_sig};
  for (DevBuf* b : bufs) b->release();
  for (int i = 0; i < 2 * kMaxTimedLaunches; ++i)
    if (op->kev[i]) cudaEventDestroy(op->kev[i]);
  if (op->ev0) cudaEventDestroy(op->ev0);
  if (op->ev1) cudaEventDestroy(op->ev1);
  if (op->lev0) cudaEventDestroy(op->lev0);
  if (op->lev1) cudaEventDestroy(op->lev1);
  if (op->ev_acc) cudaEventDestroy(op->ev_acc);
  if (op->ev_copied) cudaEventDestroy(op->ev_copied);
  if (op->ev_caller) cudaEventDestroy(op->ev_caller);
  if (op->copy_stream) cudaStreamDestroy(op->copy_stream);
  if (op->stream) cudaStreamDestroy(op->stream);
  if (op->h_small) cudaFreeHost(op->h_small);
  delete op;
  return SGW_OK;
}

sgw_status sgw_operator_trim(sgw_operator* op) {
  if (!op) return arg_error("null operator");
  if (op->stream) SGW_CK(cudaStreamSynchronize(op->stream));
  DevBuf* bufs[] = {&op->ws64.vec, &op->ws64.coef, &op->ws64.col, &op->ws64.counter, &op->ws32.vec, &op->ws32.coef,
                    &op->ws32.col, &op->ws32.counter, &op->st_bb, &op->st_sigma, &op->st_xx, &op->st_ierr,
                    &op->st_iters, &op->st_misc, &op->st_misc2, &op->st_misc3, &op->st_ref, &op->st_ref2,
                    &op->st_resid, &op->lt_psi, &op->lt_box,
                    &op->lt_nlk, &op->lt_evc, &op->lt_dv, &op->lt_bb, &op->lt_flag, &op->lt_part, &op->lt_sidx,
                    &op->lt_xx, &op->lt_chi, &op->lt_w, &op->lt_wwork, &op->lt_sig};
  for (DevBuf* b : bufs) b->release();
  return SGW_OK;
}

sgw_status sgw_operator_set_stream(sgw_operator* op, void* stream) {
  if (!op) return arg_error("null operator");
  op->caller_stream = stream ? static_cast<cudaStream_t>(stream) : cudaStreamLegacy;
  return SGW_OK;
}

sgw_status sgw_operator_set_alpha_pv(sgw_operator* op, double alpha_pv) {
  if (!op) return arg_error("null operator");
  op->alpha_pv = alpha_pv;
  return SGW_OK;
}

sgw_status sgw_operator_apply(sgw_operator* op, sgw_zcomplex sigma, int32_t m, const sgw_zcomplex* x, int64_t ldx_in,
                              sgw_zcomplex* ax, int64_t ldx_out) {
  try {
    CallScope cs(op);
    if (cs.status() != SGW_OK) return cs.status();
    return apply_host(op, sigma, m, x, ldx_in, ax, ldx_out);
  } catch (...) {
    set_error("host exception in sgw_operator_apply");
    return SGW_ERR_NOMEM;
  }
}

sgw_status sgw_operator_apply_ex(sgw_operator* op, int32_t precision, int32_t memory, sgw_zcomplex sigma, int32_t m,
                                 const sgw_zcomplex* x, int64_t ldx_in, sgw_zcomplex* ax, int64_t ldx_out) {
  try {
    CallScope cs(op);
    if (cs.status() != SGW_OK) return cs.status();
    return apply_ex(op, precision, memory, sigma, m, x, ldx_in, ax, ldx_out);
  } catch (...) {
    set_error("host exception in sgw_operator_apply_ex");
    return SGW_ERR_NOMEM;
  }
}

sgw_status sgw_bicgstab(sgw_operator* op, int32_t lmax, double threshold, int32_t max_iter, const sgw_zcomplex* bb,
                        int32_t n, const sgw_zcomplex* sigma, int32_t num_shift, sgw_zcomplex* xx, int64_t ldx,
                        int32_t* ierr) {
  try {
    CallScope cs(op);
    if (cs.status() != SGW_OK) return cs.status();
    sgw_status s = single_bicgstab(op, lmax, threshold, max_iter, bb, n, sigma, num_shift, xx, ldx, ierr);
    return s == SGW_OK ? (sgw_status)*ierr : s;
  } catch (...) {
    set_error("host exception in sgw_bicgstab");
    return SGW_ERR_NOMEM;
  }
}

sgw_status sgw_linear_solver(sgw_operator* op, double threshold, int32_t max_iter, const sgw_zcomplex* bb, int32_t n,
                             const sgw_zcomplex* sigma, int32_t num_shift, sgw_zcomplex* xx, int64_t ldx,
                             int32_t* ierr) {
  try {
    CallScope cs(op);
    if (cs.status() != SGW_OK) return cs.status();
    sgw_status s = single_sgw(op, threshold, max_iter, bb, n, sigma, num_shift, xx, ldx, ierr);
    return s == SGW_OK ? (sgw_status)*ierr : s;
  } catch (...) {
    set_error("host exception in sgw_linear_solver");
    return SGW_ERR_NOMEM;
  }
}

// select_solver.f90:67-161: try the solvers in priority order until ierr == 0.
sgw_status sgw_select_solver(sgw_operator* op, const sgw_solver_config* cfg, const sgw_zcomplex* bb, int32_t n,
                             const sgw_zcomplex* sigma, int32_t num_shift, sgw_zcomplex* xx, int64_t ldx,
                             int32_t* ierr) {
  if (!cfg || !ierr) return arg_error("null argument");
  if (cfg->num_priority < 1 || cfg->num_priority > 8)
    return arg_error("priority of the solvers not specified");  // select_solver.f90:116-118
  *ierr = 1;
  for (int k = 0; k < cfg->num_priority; ++k) {
    sgw_status s = SGW_OK;
    switch (cfg->priority[k]) {
      case SGW_BICGSTAB_MULTI:
        s = sgw_bicgstab(op, cfg->bicg_lmax, cfg->threshold, cfg->max_iter, bb, n, sigma, num_shift, xx, ldx, ierr);
        break;
      case SGW_BICGSTAB_NO_MULTI:
        // the reference solves the full shift list once per shift (select_solver.f90:144-146)
        for (int r = 0; r < num_shift; ++r) {
          s = sgw_bicgstab(op, cfg->bicg_lmax, cfg->threshold, cfg->max_iter, bb, n, sigma, num_shift, xx, ldx, ierr);
          if (s < 0) break;
        }
        break;
      case SGW_SGW_LINEAR_SOLVER:
        s = sgw_linear_solver(op, cfg->threshold, cfg->max_iter, bb, n, sigma, num_shift, xx, ldx, ierr);
        break;
      default:
        break;
    }
    if (s < 0) return s;
    if (*ierr == 0) break;
  }
  return (sgw_status)*ierr;
}

sgw_status sgw_solve_batch(sgw_operator* op, const sgw_batch_desc* desc) {
  try {
    CallScope cs(op);
    if (cs.status() != SGW_OK) return cs.status();
    return solve_batch(op, desc);
  } catch (...) {
    set_error("host exception in sgw_solve_batch");
    return SGW_ERR_NOMEM;
  }
}

sgw_status sgw_solve_batch_ex(sgw_operator* op, const sgw_batch_desc* desc, const sgw_batch_options* opt) {
  try {
    CallScope cs(op);
    if (cs.status() != SGW_OK) return cs.status();
    return solve_batch(op, desc, opt);
  } catch (...) {
    set_error("host exception in sgw_solve_batch_ex");
    return SGW_ERR_NOMEM;
  }
}

sgw_status sgw_last_timing(sgw_operator* op, double* ms, int64_t* launches) {
  if (!op) return arg_error("null operator");
  if (ms) *ms = op->last_ms;
  if (launches) *launches = op->last_launches;
  return SGW_OK;
}

sgw_status sgw_kernel_timing(sgw_operator* op, int32_t kernel, double* ms, int64_t* launches) {
  if (!op || kernel < 0 || kernel >= K_NUM) return arg_error("invalid kernel timing query");
  if (ms) *ms = op->kernel_ms[kernel];
  if (launches) *launches = op->kernel_launches[kernel];
  return SGW_OK;
}

sgw_status sgw_host_alloc(size_t bytes, void** ptr) {
  try {
    return host_alloc(bytes, ptr);
  } catch (...) {
    set_error("host exception in sgw_host_alloc");
    return SGW_ERR_NOMEM;
  }
}

sgw_status sgw_host_free(void* ptr) { return host_free(ptr); }

const char* sgw_last_error(void) { return g_error.c_str(); }

const char* sgw_version(void) { return "sgw_gb300 0.1 (sm_103a)"; }

}  // extern "C"

