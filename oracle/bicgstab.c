/*
 * TEST INFRASTRUCTURE ONLY (the oracle): CPU restatement of the reference's
 * linear solvers.  Each routine cites the reference file:line it follows.
 *
 * Conventions kept from the reference because the results depend on them:
 *   - unconjugated dot products (ZDOTU) in the BiCG and MR parts
 *     (bicgstab.f90:595,615,790,797,799);
 *   - inverse phi/theta storage (bicgstab.f90:30-32);
 *   - the delayed alpha_old update (bicgstab.f90:666-670) and delayed r_0
 *     update (bicgstab.f90:915-925);
 *   - only the seed residual is tested for convergence, absolute 2-norm
 *     (bicgstab.f90:237,245,278-301).
 */
#include "sgw_oracle.h"

#include <complex.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef double complex zc;

static zc* zalloc(size_t n) { return (zc*)calloc(n ? n : 1, sizeof(zc)); }

/* ZDOTU */
static zc dotu(int n, const zc* x, const zc* y) {
  zc s = 0;
  for (int i = 0; i < n; ++i) s += x[i] * y[i];
  return s;
}
/* ZDOTC */
static zc dotc(int n, const zc* x, const zc* y) {
  zc s = 0;
  for (int i = 0; i < n; ++i) s += conj(x[i]) * y[i];
  return s;
}
/* ZAXPY y += a x */
static void axpy(int n, zc a, const zc* x, zc* y) {
  for (int i = 0; i < n; ++i) y[i] += a * x[i];
}
/* ZSCAL x *= a */
static void scal(int n, zc a, zc* x) {
  for (int i = 0; i < n; ++i) x[i] = a * x[i];
}

/* norm.f90:73-107 (ZLANGE 'F' of a 1 x n matrix): scaled sum of squares. */
double oracle_norm(int n, const double* xr) {
  const zc* x = (const zc*)xr;
  double scale = 0.0, ssq = 1.0;
  for (int i = 0; i < n; ++i) {
    double parts[2] = {creal(x[i]), cimag(x[i])};
    for (int k = 0; k < 2; ++k) {
      double a = fabs(parts[k]);
      if (a != 0.0) {
        if (scale < a) {
          ssq = 1.0 + ssq * (scale / a) * (scale / a);
          scale = a;
        } else {
          ssq += (a / scale) * (a / scale);
        }
      }
    }
  }
  return scale * sqrt(ssq);
}

/* ---------------------------------------------------------------------------
 * Shifted BiCGStab(l), bicgstab.f90.
 * ------------------------------------------------------------------------- */

typedef struct seed_t {
  zc *uu, *rr, *xx, *tr0;
  zc sigma, rho, rho_old, alpha, alpha_old, beta, omega;
  zc *gamma, *gamma_p, *gamma_pp; /* 1-based, length lmax+1 */
} seed_t;

typedef struct shift_t {
  zc *uu, *xx;
  zc sigma, inv_phi_old, inv_phi, inv_phi_new, inv_theta, alpha, beta;
  zc *mu, *gamma, *gamma_p, *gamma_pp;
} shift_t;

#define U(sys, i) ((sys)->uu + (size_t)(i) * n)
#define R(sys, i) ((sys)->rr + (size_t)(i) * n)
/* mu_ij triangle (bicgstab.f90:409-483): row j in 0..l-1, col i in 0..j */
#define MUIDX(j, i) ((j) * ((j) + 1) / 2 + (i))
/* tau triangle (bicgstab.f90:764,782-790): row j in 1..l, col i in 1..j-1 */
#define TAUIDX(j, i) ((j) * ((j) + 1) / 2 + (i))

/* init_seed, bicgstab.f90:304-350 */
static void init_seed(int lmax, int n, const zc* bb, zc sigma, seed_t* s) {
  s->uu = zalloc((size_t)n * (lmax + 1));
  s->rr = zalloc((size_t)n * (lmax + 1));
  s->xx = zalloc(n);
  s->tr0 = zalloc(n);
  s->gamma = zalloc(lmax + 1);
  s->gamma_p = zalloc(lmax + 1);
  s->gamma_pp = zalloc(lmax + 1);
  memcpy(s->rr, bb, sizeof(zc) * n);
  memcpy(s->tr0, bb, sizeof(zc) * n);
  s->sigma = sigma;
  s->rho_old = 1.0;
  s->alpha_old = 1.0;
  s->alpha = 0.0;
  s->omega = 1.0;
}

/* init_shift, bicgstab.f90:370-490 */
static void init_shift(int lmax, int n, int nshift, const zc* sigma, shift_t* sh) {
  int mu_size = lmax * (lmax + 1) / 2;
  double* binomial = (double*)calloc(mu_size ? mu_size : 1, sizeof(double));
  zc* sigma_pow = zalloc(lmax);
  for (int jj = 0; jj < lmax; ++jj)
    for (int ii = 0; ii <= jj; ++ii) {
      int ij = MUIDX(jj, ii);
      binomial[ij] = (ii == 0) ? 1.0 : (binomial[ij - 1] * (jj - ii + 1)) / ii;
    }
  for (int is = 0; is < nshift - 1; ++is) {
    shift_t* a = sh + is;
    a->uu = zalloc((size_t)n * (lmax + 1));
    a->xx = zalloc(n);
    a->gamma = zalloc(lmax + 1);
    a->gamma_p = zalloc(lmax + 1);
    a->gamma_pp = zalloc(lmax + 1);
    a->mu = zalloc(mu_size);
    a->inv_phi_old = 1.0;
    a->inv_phi = 1.0;
    a->inv_theta = 1.0;
    a->sigma = sigma[is + 1] - sigma[0];
    sigma_pow[0] = 1.0;
    for (int ii = 1; ii < lmax; ++ii) sigma_pow[ii] = a->sigma * sigma_pow[ii - 1];
    for (int jj = 0; jj < lmax; ++jj)
      for (int ii = 0; ii <= jj; ++ii) a->mu[MUIDX(jj, ii)] = binomial[MUIDX(jj, ii)] * sigma_pow[jj - ii];
  }
  free(binomial);
  free(sigma_pow);
}

static void destroy_seed(seed_t* s) {
  free(s->uu); free(s->rr); free(s->xx); free(s->tr0);
  free(s->gamma); free(s->gamma_p); free(s->gamma_pp);
}
static void destroy_shift(int nshift, shift_t* sh) {
  for (int is = 0; is < nshift - 1; ++is) {
    free(sh[is].uu); free(sh[is].xx); free(sh[is].mu);
    free(sh[is].gamma); free(sh[is].gamma_p); free(sh[is].gamma_pp);
  }
}

/* bicg_part, bicgstab.f90:520-702 (Frommer's algorithm 3) */
static void bicg_part(int lmax, int n, oracle_apply_fn aa, void* ctx, seed_t* s, int nsh, shift_t* sh,
                      int64_t* applies) {
  const zc one = 1.0;
  s->rho_old = -s->omega * s->rho_old; /* L3 */
  for (int jj = 0; jj < lmax; ++jj) {
    s->rho = dotu(n, R(s, jj), s->tr0); /* L6 */
    s->beta = s->alpha * s->rho / s->rho_old;
    s->rho_old = s->rho;
    for (int ii = 0; ii <= jj; ++ii) { /* L8 */
      scal(n, -s->beta, U(s, ii));
      axpy(n, one, R(s, ii), U(s, ii));
    }
    aa(ctx, (const double*)&s->sigma, (const double*)U(s, jj), (double*)U(s, jj + 1), n); /* L10 */
    ++*applies;
    s->alpha = s->rho / dotu(n, U(s, jj + 1), s->tr0); /* L11 */
    for (int is = 0; is < nsh; ++is) {
      shift_t* a = sh + is;
      /* L13 */
      a->inv_phi_new = a->inv_phi / (one + s->alpha * a->sigma +
                                     s->alpha * s->beta / s->alpha_old * (a->inv_phi / a->inv_phi_old - one));
      zc ratio = a->inv_phi / a->inv_phi_old;
      a->beta = ratio * ratio * s->beta;
      a->alpha = (a->inv_phi_new / a->inv_phi) * s->alpha;
      zc factor = a->inv_theta * a->inv_phi;
      for (int ii = 0; ii <= jj; ++ii) { /* L15 */
        scal(n, -a->beta, U(a, ii));
        axpy(n, factor, R(s, ii), U(a, ii));
      }
      axpy(n, a->alpha, U(a, 0), a->xx); /* L17 */
      a->inv_phi_old = a->inv_phi;       /* L18 */
      a->inv_phi = a->inv_phi_new;
      memcpy(U(a, jj + 1), R(s, jj), sizeof(zc) * n); /* L19 */
      scal(n, factor, U(a, jj + 1));
    }
    s->alpha_old = s->alpha; /* L18 (delayed) */
    for (int ii = 0; ii <= jj; ++ii) axpy(n, -s->alpha, U(s, ii + 1), R(s, ii)); /* L22 */
    aa(ctx, (const double*)&s->sigma, (const double*)R(s, jj), (double*)R(s, jj + 1), n); /* L24 */
    ++*applies;
    axpy(n, s->alpha, U(s, 0), s->xx); /* L25 */
    for (int is = 0; is < nsh; ++is) { /* L26 */
      shift_t* a = sh + is;
      zc factor = -a->inv_theta * a->inv_phi;
      axpy(n, factor, R(s, jj), U(a, jj + 1));
      scal(n, 1.0 / a->alpha, U(a, jj + 1));
      axpy(n, -a->sigma, U(a, jj), U(a, jj + 1));
    }
  }
}

/* horner_scheme, bicgstab.f90:941-999 (Frommer's algorithm 5), 1-based arrays */
static void horner(int lmax, const zc* g, zc sigma, zc* gs, zc* psi) {
  gs[lmax] = -g[lmax];
  for (int jj = lmax - 1; jj >= 1; --jj) gs[jj] = -sigma * gs[jj + 1] - g[jj];
  *psi = -sigma * gs[1] + 1.0;
  for (int ii = 1; ii <= lmax - 1; ++ii)
    for (int jj = lmax - 1; jj >= ii; --jj) gs[jj] = -sigma * gs[jj + 1] + gs[jj];
  for (int jj = 1; jj <= lmax; ++jj) gs[jj] = -gs[jj] / *psi;
}

/* mr_part, bicgstab.f90:708-931 (Frommer's algorithm 4) */
static void mr_part(int lmax, int n, seed_t* s, int nsh, shift_t* sh) {
  zc* nu = zalloc(lmax + 1);
  zc* tau = zalloc((size_t)(lmax + 1) * (lmax + 2) / 2 + 1);
  for (int jj = 1; jj <= lmax; ++jj) { /* L1-L5 */
    for (int ii = 1; ii <= jj - 1; ++ii) {
      tau[TAUIDX(jj, ii)] = dotu(n, R(s, jj), R(s, ii)) / nu[ii];
      axpy(n, -tau[TAUIDX(jj, ii)], R(s, ii), R(s, jj));
    }
    nu[jj] = dotu(n, R(s, jj), R(s, jj));
    s->gamma_p[jj] = dotu(n, R(s, 0), R(s, jj)) / nu[jj];
  }
  s->gamma[lmax] = s->gamma_p[lmax]; /* L7 */
  s->omega = s->gamma[lmax];
  for (int jj = lmax - 1; jj >= 1; --jj) { /* L8-L9 */
    s->gamma[jj] = s->gamma_p[jj];
    for (int ii = jj + 1; ii <= lmax; ++ii) s->gamma[jj] = s->gamma[jj] - tau[TAUIDX(ii, jj)] * s->gamma[ii];
  }
  for (int jj = 1; jj <= lmax - 1; ++jj) { /* L11-L12 */
    s->gamma_pp[jj] = s->gamma[jj + 1];
    for (int ii = jj + 1; ii <= lmax - 1; ++ii)
      s->gamma_pp[jj] = s->gamma_pp[jj] + tau[TAUIDX(ii, jj)] * s->gamma[ii + 1];
  }
  axpy(n, s->gamma[1], R(s, 0), s->xx);         /* L14 */
  axpy(n, -s->gamma[lmax], U(s, lmax), U(s, 0));
  for (int jj = 1; jj <= lmax - 1; ++jj) {       /* L15-L17 */
    axpy(n, -s->gamma[jj], U(s, jj), U(s, 0));
    axpy(n, s->gamma_pp[jj], R(s, jj), s->xx);
  }
  for (int is = 0; is < nsh; ++is) {
    shift_t* a = sh + is;
    zc psi;
    horner(lmax, s->gamma, a->sigma, a->gamma, &psi); /* L20 */
    zc inv_xi = a->inv_theta * a->inv_phi;            /* L21 */
    a->inv_theta = a->inv_theta / psi;
    for (int jj = 1; jj <= lmax; ++jj) { /* L22-L23 */
      a->gamma_p[jj] = 0;
      for (int ii = jj; ii <= lmax; ++ii) a->gamma_p[jj] = a->gamma_p[jj] + a->mu[MUIDX(ii - 1, jj - 1)] * a->gamma[ii];
    }
    for (int jj = 1; jj <= lmax - 1; ++jj) { /* L25-L26 */
      a->gamma_pp[jj] = a->gamma_p[jj + 1];
      for (int ii = jj + 1; ii <= lmax - 1; ++ii)
        a->gamma_pp[jj] = a->gamma_pp[jj] + tau[TAUIDX(ii, jj)] * a->gamma_p[ii + 1];
    }
    axpy(n, a->gamma_p[1] * inv_xi, R(s, 0), a->xx); /* L28 */
    axpy(n, -s->gamma[lmax], U(a, lmax), U(a, 0));  /* corrected u_l^sigma, :891-894 */
    for (int jj = 1; jj <= lmax - 1; ++jj) {         /* L29-L31 */
      axpy(n, -s->gamma[jj], U(a, jj), U(a, 0));
      axpy(n, a->gamma_pp[jj] * inv_xi, R(s, jj), a->xx);
    }
    scal(n, 1.0 / psi, U(a, 0)); /* L34 */
  }
  for (int jj = 1; jj <= lmax; ++jj) axpy(n, -s->gamma_p[jj], R(s, jj), R(s, 0)); /* delayed L32 */
  free(nu);
  free(tau);
}

/* bicgstab, bicgstab.f90:154-275 */
int oracle_bicgstab(const oracle_bicgstab_cfg* cfg, oracle_apply_fn aa, void* ctx, int n,
                    const double* bbr, int nshift, const double* sigmar, double* xxr,
                    int* iters, int64_t* applies) {
  const zc* bb = (const zc*)bbr;
  const zc* sigma = (const zc*)sigmar;
  zc* xx = (zc*)xxr;
  int lmax = cfg->lmax;
  int ierr = 0;
  int64_t napply = 0;
  seed_t seed;
  shift_t* sh = (shift_t*)calloc(nshift > 1 ? nshift - 1 : 1, sizeof(shift_t));
  init_seed(lmax, n, bb, sigma[0], &seed);
  init_shift(lmax, n, nshift, sigma, sh);
  int iter;
  for (iter = 1; iter <= cfg->max_iter; ++iter) {
    bicg_part(lmax, n, aa, ctx, &seed, nshift - 1, sh, &napply);
    if (oracle_norm(n, (const double*)seed.rr) < cfg->threshold) break;
    mr_part(lmax, n, &seed, nshift - 1, sh);
    if (oracle_norm(n, (const double*)seed.rr) < cfg->threshold) break;
  }
  if (iter > cfg->max_iter) ierr = 1;
  memcpy(xx, seed.xx, sizeof(zc) * n);
  for (int is = 1; is < nshift; ++is) memcpy(xx + (size_t)is * n, sh[is - 1].xx, sizeof(zc) * n);
  for (size_t i = 0; i < (size_t)n * nshift; ++i)
    if (isnan(creal(xx[i])) || isnan(cimag(xx[i]))) { ierr = 2; break; }
  destroy_seed(&seed);
  destroy_shift(nshift, sh);
  free(sh);
  if (iters) *iters = iter > cfg->max_iter ? cfg->max_iter : iter;
  if (applies) *applies = napply;
  return ierr;
}

/* ---------------------------------------------------------------------------
 * SternheimerGW subspace solver, linear_solver.f90, and gram_schmidt.f90.
 * ------------------------------------------------------------------------- */

/* gram_schmidt.f90:35-134; `first` is 1-based. */
void oracle_gram_schmidt(int first, int n, int nbasis, double* basisr, double* vectorr) {
  zc* basis = (zc*)basisr;
  zc* vector = (zc*)vectorr;
  for (int ib = first - 1; ib < nbasis; ++ib)
    for (int jb = 0; jb < first - 1; ++jb) {
      zc nrm = dotc(n, basis + (size_t)jb * n, basis + (size_t)ib * n);
      axpy(n, -nrm, basis + (size_t)jb * n, basis + (size_t)ib * n);
      if (vector) axpy(n, -nrm, vector + (size_t)jb * n, vector + (size_t)ib * n);
    }
  for (int ib = first - 1; ib < nbasis; ++ib) {
    zc nrm = 1.0 / oracle_norm(n, (const double*)(basis + (size_t)ib * n));
    scal(n, nrm, basis + (size_t)ib * n);
    if (vector) scal(n, nrm, vector + (size_t)ib * n);
    for (int jb = ib + 1; jb < nbasis; ++jb) {
      nrm = dotc(n, basis + (size_t)ib * n, basis + (size_t)jb * n);
      axpy(n, -nrm, basis + (size_t)ib * n, basis + (size_t)jb * n);
      if (vector) axpy(n, -nrm, vector + (size_t)ib * n, vector + (size_t)jb * n);
    }
  }
}

/* DNRM2 of 2n reals */
static double dnrm2z(int n, const zc* x) { return oracle_norm(n, (const double*)x); }

/* linear_solver.f90:82-194 with _threshold :200-215, _orthogonal_subspace
 * :272-300, _residual :312-383, _expand_subspace :391-440, _obtain_result
 * :453-503.  The subspace arrays are grown by reallocation as in the
 * reference (MOVE_ALLOC). */
int oracle_linear_solver(double threshold, int max_iter, oracle_apply_fn aa, void* ctx, int n,
                         const double* bbr, int nshift, const double* sigmar, double* xxr) {
  const zc* bb = (const zc*)bbr;
  const zc* sigma = (const zc*)sigmar;
  zc* xx = (zc*)xxr;
  int ierr = 0;
  double abs_threshold = threshold * oracle_norm(n, bbr);
  zc sub_sigma = 0;
  int nbasis = 0, cap = 16;
  zc* vv = zalloc((size_t)n * cap);
  zc* ww = zalloc((size_t)n * cap);
  zc* residual = zalloc(n);
  zc* newv = zalloc(n);
  for (int is = 0; is < nshift; ++is) {
    /* _orthogonal_subspace */
    zc diff = sigma[is] - sub_sigma;
    axpy(n * nbasis, diff, vv, ww);
    if (nbasis > 0) oracle_gram_schmidt(1, n, nbasis, (double*)ww, (double*)vv);
    sub_sigma = sigma[is];
    int conv = 0;
    for (int iter = 1; iter <= max_iter; ++iter) {
      /* _residual */
      memcpy(residual, bb, sizeof(zc) * n);
      for (int ib = 0; ib < nbasis; ++ib) {
        zc ov = dotc(n, ww + (size_t)ib * n, bb);
        for (int i = 0; i < n; ++i) residual[i] = residual[i] - ov * ww[(size_t)ib * n + i];
      }
      double nrm = dnrm2z(n, residual);
      conv = nrm < abs_threshold;
      ierr = (!conv && nbasis == n) ? 3 : 0;
      if (conv || ierr != 0) break;
      aa(ctx, (const double*)&sigma[is], (const double*)residual, (double*)newv, n);
      /* _expand_subspace */
      if (nbasis + 1 > cap) {
        cap *= 2;
        vv = (zc*)realloc(vv, sizeof(zc) * (size_t)n * cap);
        ww = (zc*)realloc(ww, sizeof(zc) * (size_t)n * cap);
      }
      memcpy(ww + (size_t)nbasis * n, newv, sizeof(zc) * n);
      memcpy(vv + (size_t)nbasis * n, residual, sizeof(zc) * n);
      ++nbasis;
      oracle_gram_schmidt(nbasis, n, nbasis, (double*)ww, (double*)vv);
    }
    if (!conv) {
      /* a complete basis (ierr 3, :376-378) also ends here as "did not converge" (:176-180) */
      ierr = 1;
      break;
    }
    /* _obtain_result */
    zc* x = xx + (size_t)is * n;
    for (int i = 0; i < n; ++i) x[i] = 0;
    for (int ib = 0; ib < nbasis; ++ib) {
      zc ov = dotc(n, ww + (size_t)ib * n, bb);
      axpy(n, ov, vv + (size_t)ib * n, x);
    }
    int bad = 0;
    for (int i = 0; i < n; ++i)
      if (isnan(creal(x[i])) || isnan(cimag(x[i]))) bad = 1;
    if (bad) { ierr = 2; break; }
  }
  free(vv); free(ww); free(residual); free(newv);
  return ierr;
}

/* select_solver.f90:67-161 */
int oracle_select_solver(const int* priority, int npriority, int max_iter, double threshold,
                         int bicg_lmax, oracle_apply_fn aa, void* ctx, int n, const double* bb,
                         int nshift, const double* sigma, double* xx) {
  int ierr = 1;
  oracle_bicgstab_cfg cfg = {bicg_lmax, threshold, max_iter};
  for (int is = 0; is < npriority; ++is) {
    switch (priority[is]) {
      case 1:
        ierr = oracle_bicgstab(&cfg, aa, ctx, n, bb, nshift, sigma, xx, NULL, NULL);
        break;
      case 2: /* the reference solves the full shift list once per shift (:144-146) */
        for (int k = 0; k < nshift; ++k) ierr = oracle_bicgstab(&cfg, aa, ctx, n, bb, nshift, sigma, xx, NULL, NULL);
        break;
      case 3:
        ierr = oracle_linear_solver(threshold, max_iter, aa, ctx, n, bb, nshift, sigma, xx);
        break;
      default:
        break;
    }
    if (ierr == 0) break;
  }
  return ierr;
}

void oracle_bicgstab_many(const oracle_bicgstab_cfg* cfg, int kind, void* op, int n, int nrhs,
                          const double* bb, int nshift, const double* sigma, double* xx,
                          int* ierr, int* iters, int nthreads) {
  oracle_apply_fn fn = kind == 0 ? oracle_dense_apply : oracle_pw_apply;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1)
#endif
  for (int r = 0; r < nrhs; ++r) {
    int it = 0;
    ierr[r] = oracle_bicgstab(cfg, fn, op, n, bb + (size_t)2 * n * r, nshift, sigma + (size_t)2 * nshift * r,
                              xx + (size_t)2 * n * nshift * r, &it, NULL);
    if (iters) iters[r] = it;
  }
  (void)nthreads;
}

/* m independent applies ax_i = A(sigma_i) x_i (test infrastructure: true
 * residuals of many solutions at once), OpenMP over the vectors. */
void oracle_apply_many(int kind, void* op, int n, int m, const double* sigma, const double* x, double* ax,
                       int nthreads) {
  oracle_apply_fn fn = kind == 0 ? oracle_dense_apply : oracle_pw_apply;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1)
#endif
  for (int i = 0; i < m; ++i)
    fn(op, sigma + (size_t)2 * i, x + (size_t)2 * n * i, ax + (size_t)2 * n * i, n);
  (void)nthreads;
}
