// C-ABI of the caller-side kernels around the solve: the Coulomb right-hand
// sides (dvqpsi_us + orthogonalize, rhs.cuh) and the density response with
// the +-omega average (chi.cuh).
#include <algorithm>
#include <cstdint>
#include <string>
#include <vector>

#include "chi.cuh"
#include "host.cuh"
#include "rhs.cuh"
#include "vjp.cuh"

namespace sgw {

static sgw_status lt_arg_error(const std::string& msg) {
  set_error(msg);
  return SGW_ERR_ARG;
}

static sgw_status coulomb_rhs(sgw_operator* op, const sgw_rhs_desc* d) {
  if (!op || !d) return lt_arg_error("null argument");
  if (op->kind != 1) return lt_arg_error("sgw_coulomb_rhs needs a plane-wave operator");
  const PwView<double>& v = op->pw64;
  const int nocc = v.nocc, npw = v.npw;
  const long long nnr = v.nnr;
  if (d->npert < 0 || d->npw_k < 0 || d->memory < 0 || d->memory > 1) return lt_arg_error("invalid rhs description");
  if (d->npert == 0 || nocc == 0) return SGW_OK;
  if (!d->nl_k || !d->evc || !d->dvbare || !d->bb) return lt_arg_error("null rhs array");
  if (d->ldk < d->npw_k || d->lddv < nnr || d->ldb < npw) return lt_arg_error("leading dimensions too small");
  const int nslot = std::min(d->npert * nocc, op->num_sms);
  sgw_status s;
  if ((s = op->lt_psi.ensure(sizeof(zcd) * nocc * nnr)) != SGW_OK) return s;
  if ((s = op->lt_box.ensure(sizeof(zcd) * nslot * nnr)) != SGW_OK) return s;
  if ((s = op->lt_flag.ensure(sizeof(int))) != SGW_OK) return s;
  RhsArgs a{};
  a.npert = d->npert;
  a.nocc = nocc;
  a.npw_k = d->npw_k;
  a.npw = npw;
  a.npwx = v.npwx;
  a.nr1 = v.nr1;
  a.nr2 = v.nr2;
  a.nr3 = v.nr3;
  a.nl = op->nlkq.as<int>();
  a.evq = v.evq;
  a.psi_r = op->lt_psi.as<zcd>();
  a.box = op->lt_box.as<zcd>();
  a.bad_index = op->lt_flag.as<int>();
  a.p1 = v.p1;
  a.p2 = v.p2;
  a.p3 = v.p3;
  a.tw = v.tw;
  SGW_CK(cudaMemsetAsync(a.bad_index, 0, sizeof(int), op->stream));
  if (d->memory == 0) {
    for (int g = 0; g < d->npw_k; ++g)
      if (d->nl_k[g] < 0 || d->nl_k[g] >= nnr) return lt_arg_error("nl_k index outside the FFT box");
    if ((s = op->lt_nlk.ensure(sizeof(int) * std::max(d->npw_k, 1))) != SGW_OK) return s;
    if ((s = op->lt_evc.ensure(sizeof(zcd) * (size_t)nocc * std::max(d->npw_k, 1))) != SGW_OK) return s;
    if ((s = op->lt_dv.ensure(sizeof(zcd) * (size_t)d->npert * nnr)) != SGW_OK) return s;
    if ((s = op->lt_bb.ensure(sizeof(zcd) * (size_t)d->npert * nocc * npw)) != SGW_OK) return s;
    SGW_CK(cudaEventRecord(op->lev0, op->stream));
    SGW_CK(cudaMemcpyAsync(op->lt_nlk.p, d->nl_k, sizeof(int) * d->npw_k, cudaMemcpyHostToDevice, op->stream));
    SGW_CK(cudaMemcpy2DAsync(op->lt_evc.p, sizeof(zcd) * d->npw_k, d->evc, sizeof(zcd) * d->ldk,
                             sizeof(zcd) * d->npw_k, nocc, cudaMemcpyHostToDevice, op->stream));
    SGW_CK(cudaMemcpy2DAsync(op->lt_dv.p, sizeof(zcd) * nnr, d->dvbare, sizeof(zcd) * d->lddv, sizeof(zcd) * nnr,
                             d->npert, cudaMemcpyHostToDevice, op->stream));
    a.nl_k = op->lt_nlk.as<int>();
    a.evc = op->lt_evc.as<zcd>();
    a.ldk = d->npw_k;
    a.dv = op->lt_dv.as<zcd>();
    a.lddv = nnr;
    a.bb = op->lt_bb.as<zcd>();
    a.ldb = npw;
  } else {
    SGW_CK(cudaEventRecord(op->lev0, op->stream));
    a.nl_k = d->nl_k;
    a.evc = reinterpret_cast<const zcd*>(d->evc);
    a.ldk = d->ldk;
    a.dv = reinterpret_cast<const zcd*>(d->dvbare);
    a.lddv = d->lddv;
    a.bb = reinterpret_cast<zcd*>(d->bb);
    a.ldb = d->ldb;
  }
  const size_t tw_bytes = sizeof(zcd) * (v.nr1 + v.nr2 + v.nr3);
  rhs_psi_kernel<<<nocc, 256, tw_bytes, op->stream>>>(a);
  SGW_CK(cudaGetLastError());
  rhs_kernel<<<nslot, 256, tw_bytes + sizeof(zcd) * nocc, op->stream>>>(a);
  SGW_CK(cudaGetLastError());
  if (d->memory == 0)
    SGW_CK(cudaMemcpy2DAsync(d->bb, sizeof(zcd) * d->ldb, a.bb, sizeof(zcd) * npw, sizeof(zcd) * npw,
                             (size_t)d->npert * nocc, cudaMemcpyDeviceToHost, op->stream));
  SGW_CK(cudaEventRecord(op->lev1, op->stream));
  int bad = 0;
  {
    const sgw_status sc = read_count(op, a.bad_index, &bad);
    if (sc != SGW_OK) return sc;
  }
  float ms = 0.f;
  SGW_CK(cudaEventElapsedTime(&ms, op->lev0, op->lev1));
  op->kernel_ms[K_RHS] = ms;
  op->kernel_launches[K_RHS] = 2;
  if (bad) return lt_arg_error("nl_k index outside the FFT box");
  return SGW_OK;
}

static sgw_status chi(sgw_operator* op, const sgw_chi_desc* d) {
  if (!op || !d) return lt_arg_error("null argument");
  if (d->npert_b < 0 || d->npert_x < 0 || d->nbnd < 0 || d->npw < 1 || d->nfreq < 0 || d->memory < 0 ||
      d->memory > 1)
    return lt_arg_error("invalid chi description");
  const int P = d->npert_b, Q = d->npert_x, F = d->nfreq;
  if (P == 0 || Q == 0 || F == 0) return SGW_OK;
  if (!d->bb || !d->xx || !d->chi || !d->shift_plus || !d->shift_minus) return lt_arg_error("null chi array");
  if (d->ldb < d->npw || d->ldx < d->npw || d->ldc < P) return lt_arg_error("leading dimensions too small");
  int smax = 0;
  for (int f = 0; f < F; ++f) {
    if (d->shift_plus[f] < 0) return lt_arg_error("shift_plus must be >= 0");
    smax = std::max(smax, std::max(d->shift_plus[f], d->shift_minus[f]));
  }
  if (d->ldr < d->ldx * smax + d->npw) return lt_arg_error("ldr too small for the shifts named");
  // K split: enough CTAs to fill every SM a few times over
  const int tiles = ((P + kChiTile - 1) / kChiTile) * ((Q + kChiTile - 1) / kChiTile) * F;
  const long long chunks = (long long)d->nbnd * ((d->npw + kChiKc - 1) / kChiKc);
  int ksplit = std::max(1, (4 * op->num_sms + tiles - 1) / tiles);
  ksplit = (int)std::min<long long>(ksplit, std::max<long long>(chunks, 1));
  const size_t nout = (size_t)F * P * Q;
  sgw_status s;
  if ((s = op->lt_part.ensure(sizeof(zcd) * ksplit * nout)) != SGW_OK) return s;
  if ((s = op->lt_sidx.ensure(sizeof(int) * 2 * F)) != SGW_OK) return s;
  std::vector<int> sidx(2 * F);
  std::copy(d->shift_plus, d->shift_plus + F, sidx.begin());
  for (int f = 0; f < F; ++f) sidx[F + f] = d->shift_minus[f] < 0 ? -1 : d->shift_minus[f];
  ChiArgs a{};
  a.npert_b = P;
  a.npert_x = Q;
  a.nbnd = d->nbnd;
  a.npw = d->npw;
  a.nfreq = F;
  a.ksplit = ksplit;
  a.weight = d->weight;
  a.part = op->lt_part.as<zcd>();
  a.s_plus = op->lt_sidx.as<int>();
  a.s_minus = op->lt_sidx.as<int>() + F;
  zcd* chi_out;
  SGW_CK(cudaEventRecord(op->lev0, op->stream));
  SGW_CK(cudaMemcpyAsync(op->lt_sidx.p, sidx.data(), sizeof(int) * 2 * F, cudaMemcpyHostToDevice, op->stream));
  if (d->memory == 0) {
    const int S = smax + 1;
    if ((s = op->lt_bb.ensure(sizeof(zcd) * (size_t)P * d->nbnd * d->npw)) != SGW_OK) return s;
    if ((s = op->lt_xx.ensure(sizeof(zcd) * (size_t)Q * d->nbnd * S * d->npw)) != SGW_OK) return s;
    if ((s = op->lt_chi.ensure(sizeof(zcd) * (size_t)Q * F * P)) != SGW_OK) return s;
    SGW_CK(cudaMemcpy2DAsync(op->lt_bb.p, sizeof(zcd) * d->npw, d->bb, sizeof(zcd) * d->ldb, sizeof(zcd) * d->npw,
                             (size_t)P * d->nbnd, cudaMemcpyHostToDevice, op->stream));
    for (long long r = 0; r < (long long)Q * d->nbnd; ++r)
      SGW_CK(cudaMemcpy2DAsync(op->lt_xx.as<zcd>() + (size_t)r * S * d->npw, sizeof(zcd) * d->npw,
                               reinterpret_cast<const zcd*>(d->xx) + (size_t)r * d->ldr, sizeof(zcd) * d->ldx,
                               sizeof(zcd) * d->npw, S, cudaMemcpyHostToDevice, op->stream));
    a.bb = op->lt_bb.as<zcd>();
    a.ldb = d->npw;
    a.xx = op->lt_xx.as<zcd>();
    a.ldx = d->npw;
    a.ldr = (long long)S * d->npw;
    chi_out = op->lt_chi.as<zcd>();
  } else {
    a.bb = reinterpret_cast<const zcd*>(d->bb);
    a.ldb = d->ldb;
    a.xx = reinterpret_cast<const zcd*>(d->xx);
    a.ldx = d->ldx;
    a.ldr = d->ldr;
    chi_out = reinterpret_cast<zcd*>(d->chi);
  }
  chi_kernel<<<tiles * ksplit, 256, 0, op->stream>>>(a);
  SGW_CK(cudaGetLastError());
  const long long ldc = d->memory == 0 ? P : d->ldc;
  const int rblocks = (int)std::min<size_t>((nout + 255) / 256, (size_t)op->num_sms * 8);
  chi_reduce_kernel<<<rblocks, 256, 0, op->stream>>>(a.part, ksplit, F, Q, P, chi_out, ldc);
  SGW_CK(cudaGetLastError());
  if (d->memory == 0)
    SGW_CK(cudaMemcpy2DAsync(d->chi, sizeof(zcd) * d->ldc, chi_out, sizeof(zcd) * P, sizeof(zcd) * P, (size_t)Q * F,
                             cudaMemcpyDeviceToHost, op->stream));
  SGW_CK(cudaEventRecord(op->lev1, op->stream));
  SGW_CK(cudaStreamSynchronize(op->stream));
  float ms = 0.f;
  SGW_CK(cudaEventElapsedTime(&ms, op->lev0, op->lev1));
  op->kernel_ms[K_CHI] = ms;
  op->kernel_launches[K_CHI] = 2;
  return SGW_OK;
}

// Green's function right-hand sides -delta_{G, ig} and shifts -omega for every listed G' point.
__global__ void green_rhs_kernel(int nrhs, int n, const int* ig_of_rhs, zcd* bb, const zcd* omega, int S, zcd* sigma) {
  const long long tot = (long long)nrhs * n;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < tot; e += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(e / n), g = (int)(e - (long long)r * n);
    bb[e] = zcd{g == ig_of_rhs[r] - 1 ? -1.0 : 0.0, 0.0};
  }
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < (long long)nrhs * S;
       e += (long long)gridDim.x * blockDim.x)
    sigma[e] = -omega[e % S];
}

// green[(f * num_gp + igp) * ldg + i] = x[rhs(igp)][f][map[i] - 1] where 0 < map[i] < n, else 0
__global__ void green_gather_kernel(int num_gp, int num_g_corr, int S, int n, const int* rhs_of_gp, const int* map,
                                    const zcd* x, zcd* green, long long ldg) {
  const long long tot = (long long)S * num_gp * num_g_corr;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < tot; e += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(e % num_g_corr);
    const long long fg = e / num_g_corr;
    const int igp = (int)(fg % num_gp), f = (int)(fg / num_gp);
    const int r = rhs_of_gp[igp], m = map[i];
    zcd v = {0.0, 0.0};
    if (r >= 0 && m > 0 && m < n) v = x[((size_t)r * S + f) * n + (m - 1)];
    green[((size_t)f * num_gp + igp) * ldg + i] = v;
  }
}

static sgw_status green_function(sgw_operator* op, const sgw_green_desc* d) {
  if (!op || !d) return lt_arg_error("null argument");
  if (op->kind != 1) return lt_arg_error("sgw_green_function needs a plane-wave operator");
  if (d->num_gp < 0 || d->num_g_corr < 0 || d->num_freq < 1 || d->lmax < 1 || d->lmax > kMaxL - 1 ||
      d->max_iter < 1 || (d->precision != 0 && d->precision != 1) || d->memory < 0 || d->memory > 1)
    return lt_arg_error("invalid Green's function description");
  if (!d->ierr || (d->num_gp > 0 && (!d->ig_of_gp || !d->green)) || (d->num_g_corr > 0 && !d->map) || !d->omega)
    return lt_arg_error("null Green's function array");
  if (d->ldg < d->num_g_corr) return lt_arg_error("ldg too small");
  const int n = op->n, S = d->num_freq, G = d->num_gp, M = d->num_g_corr;
  // the G' list decides the right-hand sides: read it on the host
  std::vector<int> ig(G);
  if (G > 0) {
    if (d->memory == 1)
      SGW_CK(cudaMemcpy(ig.data(), d->ig_of_gp, sizeof(int) * G, cudaMemcpyDeviceToHost));
    else
      std::copy(d->ig_of_gp, d->ig_of_gp + G, ig.begin());
  }
  std::vector<int> rhs_of_gp(G, -1), ig_of_rhs;
  for (int p = 0; p < G; ++p) {
    if (ig[p] < 0 || ig[p] > n) return lt_arg_error("ig_of_gp outside 0..npw");
    if (ig[p] != 0) {
      rhs_of_gp[p] = (int)ig_of_rhs.size();
      ig_of_rhs.push_back(ig[p]);
    }
  }
  const int R = (int)ig_of_rhs.size();
  sgw_status s;
  DevBuf& bbuf = op->lt_bb;   // bb [R][n], then sigma [R][S], the int tables, omega
  DevBuf& xbuf = op->lt_xx;   // x [R][S][n]
  DevBuf& gbuf = op->lt_chi;  // green staging (host memory mode)
  const size_t bb_b = sizeof(zcd) * (size_t)std::max(R, 1) * n;
  const size_t sg_b = sizeof(zcd) * (size_t)std::max(R, 1) * S;
  const size_t tab_b = sizeof(int) * ((size_t)std::max(R, 1) + G + std::max(M, 1)) + sizeof(zcd) * S + 256;
  if ((s = bbuf.ensure(bb_b + sg_b + tab_b)) != SGW_OK) return s;
  if ((s = xbuf.ensure(sizeof(zcd) * (size_t)std::max(R, 1) * S * n)) != SGW_OK) return s;
  if ((s = op->st_ierr.ensure(sizeof(int) * std::max(R, 1))) != SGW_OK) return s;
  if ((s = op->st_iters.ensure(sizeof(int) * std::max(R, 1))) != SGW_OK) return s;
  unsigned char* base = reinterpret_cast<unsigned char*>(bbuf.p);
  zcd* bb = reinterpret_cast<zcd*>(base);
  zcd* sigma = reinterpret_cast<zcd*>(base + bb_b);
  int* t_ig = reinterpret_cast<int*>(base + bb_b + sg_b);
  int* t_rhs = t_ig + std::max(R, 1);
  int* t_map = t_rhs + G;
  zcd* t_om = reinterpret_cast<zcd*>(reinterpret_cast<unsigned char*>(t_map + std::max(M, 1)) +
                                     (16 - (reinterpret_cast<uintptr_t>(t_map + std::max(M, 1)) & 15)) % 16);
  const double keep_alpha = op->alpha_pv;
  op->alpha_pv = 0.0;  // green_operator (green.f90:283)
  struct Restore {
    sgw_operator* o;
    double a;
    ~Restore() { o->alpha_pv = a; }
  } restore{op, keep_alpha};
  SGW_CK(cudaEventRecord(op->lev0, op->stream));
  if (R > 0) SGW_CK(cudaMemcpyAsync(t_ig, ig_of_rhs.data(), sizeof(int) * R, cudaMemcpyHostToDevice, op->stream));
  if (G > 0) SGW_CK(cudaMemcpyAsync(t_rhs, rhs_of_gp.data(), sizeof(int) * G, cudaMemcpyHostToDevice, op->stream));
  const cudaMemcpyKind in_kind = d->memory == 1 ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  if (M > 0) SGW_CK(cudaMemcpyAsync(t_map, d->map, sizeof(int) * M, in_kind, op->stream));
  SGW_CK(cudaMemcpyAsync(t_om, d->omega, sizeof(zcd) * S, in_kind, op->stream));
  int worst = 0;
  if (R > 0) {
    const int grid = std::min(op->num_sms * 8, (int)std::max<long long>(1, ((long long)R * n + 255) / 256));
    green_rhs_kernel<<<grid, 256, 0, op->stream>>>(R, n, t_ig, bb, t_om, S, sigma);
    SGW_CK(cudaGetLastError());
    BatchDev b{R, S, d->lmax, d->max_iter, 0, d->threshold, bb, n, sigma, S, xbuf.p, n, (long long)S * n,
               op->st_ierr.as<int>(), op->st_iters.as<int>()};
    s = d->precision == 0 ? run_msbicg<double>(op, b) : solve_mixed(op, b, 0, 0.0);
    if (s != SGW_OK) return s;
    std::vector<int> ierr_h(R);
    SGW_CK(cudaMemcpyAsync(ierr_h.data(), op->st_ierr.p, sizeof(int) * R, cudaMemcpyDeviceToHost, op->stream));
    SGW_CK(cudaStreamSynchronize(op->stream));
    for (int v : ierr_h) worst = std::max(worst, v);
  }
  if (G > 0 && M > 0) {
    zcd* gout;
    long long ldg = d->ldg;
    if (d->memory == 1) {
      gout = reinterpret_cast<zcd*>(d->green);
    } else {
      if ((s = gbuf.ensure(sizeof(zcd) * (size_t)S * G * M)) != SGW_OK) return s;
      gout = gbuf.as<zcd>();
      ldg = M;
    }
    const long long tot = (long long)S * G * M;
    green_gather_kernel<<<(int)std::min<long long>((tot + 255) / 256, op->num_sms * 16), 256, 0, op->stream>>>(
        G, M, S, n, t_rhs, t_map, xbuf.as<zcd>(), gout, ldg);
    SGW_CK(cudaGetLastError());
    if (d->memory == 0)
      SGW_CK(cudaMemcpy2DAsync(d->green, sizeof(zcd) * d->ldg, gout, sizeof(zcd) * M, sizeof(zcd) * M,
                               (size_t)S * G, cudaMemcpyDeviceToHost, op->stream));
  }
  SGW_CK(cudaEventRecord(op->lev1, op->stream));
  SGW_CK(cudaStreamSynchronize(op->stream));
  if (d->memory == 1)
    SGW_CK(cudaMemcpy(d->ierr, &worst, sizeof(int), cudaMemcpyHostToDevice));
  else
    *d->ierr = worst;
  return SGW_OK;
}

// lambda_rs = A(sigma_rs)^-H g_rs = (H + conj(sigma_rs) + alpha_pv P_v)^-1 g_rs: every (rhs, shift)
// pair is its own single-shift system of the batched solver.
__global__ void adjoint_pack_kernel(const zcd* sigma, long long lds, int nrhs, int nshift, zcd* out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nrhs * nshift; i += gridDim.x * blockDim.x) {
    const int r = i / nshift, s = i - r * nshift;
    out[i] = conj(sigma[(size_t)r * lds + s]);
  }
}

static sgw_status solve_adjoint(sgw_operator* op, const sgw_adjoint_desc* d) {
  if (!op || !d) return lt_arg_error("null argument");
  const int R = d->nrhs, S = d->num_shift, n = op->n;
  if (R < 0 || S < 1 || d->lmax < 1 || d->lmax > kMaxL - 1 || d->max_iter < 1 || d->memory < 0 || d->memory > 1 ||
      d->precision < 0 || d->precision > 1)
    return lt_arg_error("invalid adjoint description");
  if (R == 0) return SGW_OK;
  if (!d->sigma || !d->gbar || !d->lam || !d->ierr) return lt_arg_error("null adjoint array");
  if (d->lds < S || d->ldx < n || d->ldr != (long long)S * d->ldx)
    return lt_arg_error("adjoint layout must be packed per right-hand side: ldr = num_shift * ldx, ldx >= n");
  const long long M = (long long)R * S;
  if (M > 0x7fffffffLL) return lt_arg_error("too many adjoint systems");
  const int ck = d->checkpoint_iters > 0 ? d->checkpoint_iters : 8;
  BatchDev b{(int)M, 1, d->lmax, d->max_iter, std::max(1, (ck + 2 * d->lmax - 1) / (2 * d->lmax)), d->threshold,
             nullptr, d->ldx, nullptr, 1, nullptr, d->ldx, d->ldx, nullptr, nullptr};
  sgw_status s;
  if ((s = op->lt_sidx.ensure(sizeof(zcd) * M)) != SGW_OK) return s;
  if ((s = op->st_iters.ensure(sizeof(int) * M)) != SGW_OK) return s;
  zcd* sig = op->lt_sidx.as<zcd>();
  op->last_launches = 0;
  op->kev_used = 0;
  if (d->memory == 1) {
    SGW_CK(cudaEventRecord(op->ev0, op->stream));
    adjoint_pack_kernel<<<std::max(1, std::min<int>((int)((M + 255) / 256), op->num_sms * 4)), 256, 0, op->stream>>>(
        reinterpret_cast<const zcd*>(d->sigma), d->lds, R, S, sig);
    SGW_CK(cudaGetLastError());
    b.bb = d->gbar;
    b.xx = d->lam;
    b.ierr = d->ierr;
  } else {
    std::vector<zcd> sh(M);
    for (int r = 0; r < R; ++r)
      for (int k = 0; k < S; ++k) {
        const sgw_zcomplex z = d->sigma[(size_t)r * d->lds + k];
        sh[(size_t)r * S + k] = zcd{z.re, -z.im};
      }
    if ((s = op->st_bb.ensure(sizeof(zcd) * M * n)) != SGW_OK) return s;
    if ((s = op->st_xx.ensure(sizeof(zcd) * M * n)) != SGW_OK) return s;
    if ((s = op->st_ierr.ensure(sizeof(int) * M)) != SGW_OK) return s;
    SGW_CK(cudaEventRecord(op->ev0, op->stream));
    SGW_CK(cudaMemcpyAsync(sig, sh.data(), sizeof(zcd) * M, cudaMemcpyHostToDevice, op->stream));
    SGW_CK(cudaMemcpy2DAsync(op->st_bb.p, sizeof(zcd) * n, d->gbar, sizeof(zcd) * d->ldx, sizeof(zcd) * n, M,
                             cudaMemcpyHostToDevice, op->stream));
    b.bb = op->st_bb.p;
    b.ldb = n;
    b.xx = op->st_xx.p;
    b.ldx = n;
    b.ldr = n;
    b.ierr = op->st_ierr.as<int>();
  }
  b.sigma = sig;
  b.iters = op->st_iters.as<int>();
  s = d->precision == 0 ? run_msbicg<double>(op, b) : solve_mixed(op, b, 0, 0.0);
  if (s != SGW_OK) return s;
  if (d->memory == 0) {
    SGW_CK(cudaMemcpy2DAsync(d->lam, sizeof(zcd) * d->ldx, op->st_xx.p, sizeof(zcd) * n, sizeof(zcd) * n, M,
                             cudaMemcpyDeviceToHost, op->stream));
    SGW_CK(cudaMemcpyAsync(d->ierr, op->st_ierr.p, sizeof(int) * M, cudaMemcpyDeviceToHost, op->stream));
  }
  SGW_CK(cudaEventRecord(op->ev1, op->stream));
  SGW_CK(cudaStreamSynchronize(op->stream));
  float ms = 0.f;
  SGW_CK(cudaEventElapsedTime(&ms, op->ev0, op->ev1));
  op->last_ms = ms;
  return SGW_OK;
}

static sgw_status vjp(sgw_operator* op, const sgw_vjp_desc* d) {
  if (!op || !d) return lt_arg_error("null argument");
  if (op->kind != 1) return lt_arg_error("sgw_vjp needs a plane-wave operator");
  const PwView<double>& v = op->pw64;
  const int nocc = v.nocc, npw = v.npw, P = d->npert, S = d->num_shift;
  const int nnr = v.nnr;
  if (P < 0 || S < 1 || d->npw_k < 0 || d->memory < 0 || d->memory > 1) return lt_arg_error("invalid vjp description");
  if (P == 0 || nocc == 0) return SGW_OK;
  if (!d->xx || !d->lam || (!d->grad_vloc && !d->grad_dvbare)) return lt_arg_error("null vjp array");
  if (d->grad_dvbare && (!d->nl_k || !d->evc || d->ldk < d->npw_k || d->ldg < nnr))
    return lt_arg_error("the Delta V gradient needs nl_k, evc (ldk >= npw_k) and ldg >= nnr");
  if (d->ldx < npw || d->ldr < d->ldx * (S - 1) + npw) return lt_arg_error("leading dimensions too small");
  const long long R = (long long)P * nocc;
  const int nslot_v = (int)std::min<long long>(R * S, op->num_sms);
  const int nslot_p = std::min(P, op->num_sms);
  const int nslot = std::max(nslot_v, nslot_p);
  sgw_status s;
  if ((s = op->lt_box.ensure(sizeof(zcd) * 2 * (size_t)nslot * nnr)) != SGW_OK) return s;
  if ((s = op->lt_part.ensure(sizeof(double) * (size_t)nslot_v * nnr)) != SGW_OK) return s;
  if ((s = op->lt_chi.ensure(sizeof(zcd) * (size_t)nslot_p * v.npwx)) != SGW_OK) return s;
  if ((s = op->lt_psi.ensure(sizeof(zcd) * (size_t)nocc * nnr)) != SGW_OK) return s;
  if ((s = op->lt_flag.ensure(sizeof(int))) != SGW_OK) return s;
  VjpArgs a{};
  a.nr1 = v.nr1;
  a.nr2 = v.nr2;
  a.nr3 = v.nr3;
  a.p1 = v.p1;
  a.p2 = v.p2;
  a.p3 = v.p3;
  a.tw = v.tw;
  a.npw = npw;
  a.npwx = v.npwx;
  a.nocc = nocc;
  a.npert = P;
  a.nshift = S;
  a.nl = op->nlkq.as<int>();
  a.evq = v.evq;
  a.psi_r = op->lt_psi.as<zcd>();
  a.box = op->lt_box.as<zcd>();
  a.sphere = op->lt_chi.as<zcd>();
  a.part_v = op->lt_part.as<double>();
  a.ldg = nnr;
  RhsArgs ra{};
  ra.nocc = nocc;
  ra.npw_k = d->npw_k;
  ra.nr1 = v.nr1;
  ra.nr2 = v.nr2;
  ra.nr3 = v.nr3;
  ra.p1 = v.p1;
  ra.p2 = v.p2;
  ra.p3 = v.p3;
  ra.tw = v.tw;
  ra.psi_r = op->lt_psi.as<zcd>();
  ra.bad_index = op->lt_flag.as<int>();
  double* gv = nullptr;
  zcd* gd = nullptr;
  SGW_CK(cudaMemsetAsync(ra.bad_index, 0, sizeof(int), op->stream));
  SGW_CK(cudaEventRecord(op->lev0, op->stream));
  if (d->memory == 0) {
    if (d->grad_dvbare)
      for (int g = 0; g < d->npw_k; ++g)
        if (d->nl_k[g] < 0 || d->nl_k[g] >= nnr) return lt_arg_error("nl_k index outside the FFT box");
    const size_t M = (size_t)R * S;
    if ((s = op->st_xx.ensure(sizeof(zcd) * M * npw)) != SGW_OK) return s;
    if ((s = op->st_bb.ensure(sizeof(zcd) * M * npw)) != SGW_OK) return s;
    for (long long r = 0; r < R; ++r) {
      SGW_CK(cudaMemcpy2DAsync(op->st_xx.as<zcd>() + (size_t)r * S * npw, sizeof(zcd) * npw,
                               reinterpret_cast<const zcd*>(d->xx) + (size_t)r * d->ldr, sizeof(zcd) * d->ldx,
                               sizeof(zcd) * npw, S, cudaMemcpyHostToDevice, op->stream));
      SGW_CK(cudaMemcpy2DAsync(op->st_bb.as<zcd>() + (size_t)r * S * npw, sizeof(zcd) * npw,
                               reinterpret_cast<const zcd*>(d->lam) + (size_t)r * d->ldr, sizeof(zcd) * d->ldx,
                               sizeof(zcd) * npw, S, cudaMemcpyHostToDevice, op->stream));
    }
    a.xx = op->st_xx.as<zcd>();
    a.lam = op->st_bb.as<zcd>();
    a.ldx = npw;
    a.ldr = (long long)S * npw;
    if (d->grad_dvbare) {
      if ((s = op->lt_nlk.ensure(sizeof(int) * std::max(d->npw_k, 1))) != SGW_OK) return s;
      if ((s = op->lt_evc.ensure(sizeof(zcd) * (size_t)nocc * std::max(d->npw_k, 1))) != SGW_OK) return s;
      SGW_CK(cudaMemcpyAsync(op->lt_nlk.p, d->nl_k, sizeof(int) * d->npw_k, cudaMemcpyHostToDevice, op->stream));
      SGW_CK(cudaMemcpy2DAsync(op->lt_evc.p, sizeof(zcd) * d->npw_k, d->evc, sizeof(zcd) * d->ldk,
                               sizeof(zcd) * d->npw_k, nocc, cudaMemcpyHostToDevice, op->stream));
      ra.nl_k = op->lt_nlk.as<int>();
      ra.evc = op->lt_evc.as<zcd>();
      ra.ldk = d->npw_k;
    }
    if ((s = op->lt_dv.ensure(sizeof(zcd) * ((size_t)P * nnr + nnr))) != SGW_OK) return s;
    gd = op->lt_dv.as<zcd>();
    gv = reinterpret_cast<double*>(gd + (size_t)P * nnr);
  } else {
    a.xx = reinterpret_cast<const zcd*>(d->xx);
    a.lam = reinterpret_cast<const zcd*>(d->lam);
    a.ldx = d->ldx;
    a.ldr = d->ldr;
    ra.nl_k = d->nl_k;
    ra.evc = reinterpret_cast<const zcd*>(d->evc);
    ra.ldk = d->ldk;
    gd = reinterpret_cast<zcd*>(d->grad_dvbare);
    gv = d->grad_vloc;
    a.ldg = d->ldg;
  }
  const size_t tw_bytes = sizeof(zcd) * (v.nr1 + v.nr2 + v.nr3);
  int launches = 0;
  if (d->grad_vloc) {
    vjp_vloc_kernel<<<nslot_v, 256, tw_bytes, op->stream>>>(a);
    SGW_CK(cudaGetLastError());
    vjp_vloc_reduce<<<std::max(1, std::min((nnr + 255) / 256, op->num_sms * 4)), 256, 0, op->stream>>>(
        a.part_v, nslot_v, nnr, gv);
    SGW_CK(cudaGetLastError());
    launches += 2;
  }
  if (d->grad_dvbare) {
    rhs_psi_kernel<<<nocc, 256, tw_bytes, op->stream>>>(ra);
    SGW_CK(cudaGetLastError());
    a.grad_dv = gd;
    vjp_dv_kernel<<<nslot_p, 256, tw_bytes + sizeof(zcd) * nocc, op->stream>>>(a);
    SGW_CK(cudaGetLastError());
    launches += 2;
  }
  if (d->memory == 0) {
    if (d->grad_vloc)
      SGW_CK(cudaMemcpyAsync(d->grad_vloc, gv, sizeof(double) * nnr, cudaMemcpyDeviceToHost, op->stream));
    if (d->grad_dvbare)
      SGW_CK(cudaMemcpy2DAsync(d->grad_dvbare, sizeof(zcd) * d->ldg, gd, sizeof(zcd) * nnr, sizeof(zcd) * nnr, P,
                               cudaMemcpyDeviceToHost, op->stream));
  }
  SGW_CK(cudaEventRecord(op->lev1, op->stream));
  int bad = 0;
  {
    const sgw_status sc = read_count(op, ra.bad_index, &bad);
    if (sc != SGW_OK) return sc;
  }
  float ms = 0.f;
  SGW_CK(cudaEventElapsedTime(&ms, op->lev0, op->lev1));
  op->kernel_ms[K_VJP] = ms;
  op->kernel_launches[K_VJP] = launches;
  if (bad) return lt_arg_error("nl_k index outside the FFT box");
  return SGW_OK;
}

template <typename T>
static sgw_status upload_vloc(sgw_operator* op, const double* vrs, long long nnr, DevBuf& dst) {
  std::vector<T> h(nnr);
  for (long long i = 0; i < nnr; ++i) h[i] = (T)vrs[i];
  SGW_CK(cudaStreamSynchronize(op->stream));
  SGW_CK(cudaMemcpy(dst.p, h.data(), sizeof(T) * nnr, cudaMemcpyHostToDevice));
  return SGW_OK;
}

static sgw_status set_vloc(sgw_operator* op, const double* vrs, long long nnr) {
  if (!op || !vrs) return lt_arg_error("null argument");
  if (op->kind != 1) return lt_arg_error("sgw_operator_set_vloc needs a plane-wave operator");
  if (nnr != op->pw64.nnr) return lt_arg_error("V_loc size differs from the FFT box");
  sgw_status s = upload_vloc<double>(op, vrs, nnr, op->vrs64);
  if (s == SGW_OK) s = upload_vloc<float>(op, vrs, nnr, op->vrs32);
  return s;
}

}  // namespace sgw

extern "C" {

sgw_status sgw_solve_adjoint(sgw_operator* op, const sgw_adjoint_desc* desc) {
  try {
    sgw::CallScope cs(op);
    if (cs.status() != SGW_OK) return cs.status();
    return sgw::solve_adjoint(op, desc);
  } catch (...) {
    sgw::set_error("host exception in sgw_solve_adjoint");
    return SGW_ERR_NOMEM;
  }
}

sgw_status sgw_vjp(sgw_operator* op, const sgw_vjp_desc* desc) {
  try {
    sgw::CallScope cs(op);
    if (cs.status() != SGW_OK) return cs.status();
    return sgw::vjp(op, desc);
  } catch (...) {
    sgw::set_error("host exception in sgw_vjp");
    return SGW_ERR_NOMEM;
  }
}

sgw_status sgw_green_function(sgw_operator* op, const sgw_green_desc* desc) {
  try {
    sgw::CallScope cs(op);
    if (cs.status() != SGW_OK) return cs.status();
    return sgw::green_function(op, desc);
  } catch (...) {
    sgw::set_error("host exception in sgw_green_function");
    return SGW_ERR_NOMEM;
  }
}

sgw_status sgw_operator_set_vloc(sgw_operator* op, const double* vrs, int64_t nnr) {
  try {
    sgw::CallScope cs(op);
    if (cs.status() != SGW_OK) return cs.status();
    return sgw::set_vloc(op, vrs, nnr);
  } catch (...) {
    sgw::set_error("host exception in sgw_operator_set_vloc");
    return SGW_ERR_NOMEM;
  }
}


sgw_status sgw_coulomb_rhs(sgw_operator* op, const sgw_rhs_desc* desc) {
  try {
    sgw::CallScope cs(op);
    if (cs.status() != SGW_OK) return cs.status();
    return sgw::coulomb_rhs(op, desc);
  } catch (...) {
    sgw::set_error("host exception in sgw_coulomb_rhs");
    return SGW_ERR_NOMEM;
  }
}

sgw_status sgw_chi(sgw_operator* op, const sgw_chi_desc* desc) {
  try {
    sgw::CallScope cs(op);
    if (cs.status() != SGW_OK) return cs.status();
    return sgw::chi(op, desc);
  } catch (...) {
    sgw::set_error("host exception in sgw_chi");
    return SGW_ERR_NOMEM;
  }
}

}  // extern "C"
