/*
 * TEST INFRASTRUCTURE ONLY (the oracle): the shifted operator
 *   A(sigma) psi = (H + sigma S + alpha_pv P_v) psi      (linear_op.f90:46-144)
 * for a norm-conserving collinear insulator (S = 1), with H restated from the
 * Quantum ESPRESSO h_psi semantics the reference calls at linear_op.f90:116:
 *   H psi(G) = |k+G|^2 psi(G)                                     (kinetic, Ry)
 *            + fwfft[ V_loc(r) * invfft[psi scattered on the box] ](G)
 *            + sum_i beta_i(G) D_i <beta_i|psi>                   (Kleinman-Bylander)
 * and P_v psi = psi_occ (psi_occ^dagger psi)            (projector_psi, :147-206).
 *
 * The FFT is a plain mixed-radix Cooley-Tukey written here (no FFTW in the
 * image).  Sign convention of QE's FFTXlib: invfft (G->r) uses exp(+i G.r)
 * and no scaling; fwfft (r->G) uses exp(-i G.r) and scales by 1/(nr1 nr2 nr3).
 */
#include "sgw_oracle.h"

#include <complex.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

typedef double complex zc;

/* Dense operator: linear_problem_apply (linear_problem.f90:100-113). */
void oracle_dense_apply(void* ctx, const double* sigmar, const double* xr, double* axr, int n) {
  const oracle_dense_op* op = (const oracle_dense_op*)ctx;
  const zc* a = (const zc*)op->a;
  const zc* x = (const zc*)xr;
  zc* ax = (zc*)axr;
  zc sigma = *(const zc*)sigmar;
  for (int i = 0; i < n; ++i) ax[i] = 0;
  for (int j = 0; j < n; ++j) {
    zc xj = x[j];
    const zc* col = a + (size_t)j * n;
    for (int i = 0; i < n; ++i) ax[i] += col[i] * xj;
  }
  for (int i = 0; i < n; ++i) ax[i] += sigma * x[i];
}

/* ---- 1-D mixed-radix DFT of a contiguous line (in place, recursive) ------ */

static int smallest_factor(int n) {
  for (int p = 2; p * p <= n; ++p)
    if (n % p == 0) return p;
  return n;
}

/* out[k] = sum_j in[j*istride] w^(j k), w = exp(sign 2 pi i / n); tw[j] = w^j.
 * twn is the length of the table (the full line length N); this level uses
 * w_n = w_N^(N/n). */
static void dft_rec(const zc* in, int istride, zc* out, int n, const zc* tw, int twn, zc* tmp) {
  if (n == 1) {
    out[0] = in[0];
    return;
  }
  int p = smallest_factor(n);
  int m = n / p;
  for (int q = 0; q < p; ++q) dft_rec(in + (size_t)q * istride, istride * p, out + (size_t)q * m, m, tw, twn, tmp);
  int step = twn / n; /* w_n^e = tw[e * step] */
  for (int k = 0; k < m; ++k) {
    for (int q = 0; q < p; ++q) tmp[q] = out[(size_t)q * m + k];
    for (int s = 0; s < p; ++s) {
      zc acc = 0;
      int kk = k + m * s;
      for (int q = 0; q < p; ++q) {
        int e = (int)(((long)q * kk) % n);
        acc += tmp[q] * tw[(size_t)e * step];
      }
      out[k + (size_t)m * s] = acc;
    }
  }
}

static void fft_line(zc* line, int n, int stride, const zc* tw, zc* buf, zc* buf2, zc* tmp) {
  for (int i = 0; i < n; ++i) buf[i] = line[(size_t)i * stride];
  dft_rec(buf, 1, buf2, n, tw, n, tmp);
  for (int i = 0; i < n; ++i) line[(size_t)i * stride] = buf2[i];
}

static zc* twiddles(int n, int sign) {
  zc* tw = (zc*)malloc(sizeof(zc) * (size_t)n);
  for (int j = 0; j < n; ++j) {
    long double ang = (long double)sign * 2.0L * 3.14159265358979323846264338327950288L * (long double)j / (long double)n;
    tw[j] = (double)cosl(ang) + I * (double)sinl(ang);
  }
  return tw;
}

void oracle_fft3d(double* boxr, int nr1, int nr2, int nr3, int sign) {
  zc* box = (zc*)boxr;
  int nmax = nr1 > nr2 ? nr1 : nr2;
  nmax = nmax > nr3 ? nmax : nr3;
  zc* buf = (zc*)malloc(sizeof(zc) * nmax);
  zc* buf2 = (zc*)malloc(sizeof(zc) * nmax);
  zc* tmp = (zc*)malloc(sizeof(zc) * nmax);
  zc* tw1 = twiddles(nr1, sign);
  zc* tw2 = twiddles(nr2, sign);
  zc* tw3 = twiddles(nr3, sign);
  for (int i3 = 0; i3 < nr3; ++i3)
    for (int i2 = 0; i2 < nr2; ++i2) fft_line(box + (size_t)nr1 * (i2 + (size_t)nr2 * i3), nr1, 1, tw1, buf, buf2, tmp);
  for (int i3 = 0; i3 < nr3; ++i3)
    for (int i1 = 0; i1 < nr1; ++i1) fft_line(box + i1 + (size_t)nr1 * nr2 * i3, nr2, nr1, tw2, buf, buf2, tmp);
  for (int i2 = 0; i2 < nr2; ++i2)
    for (int i1 = 0; i1 < nr1; ++i1) fft_line(box + i1 + (size_t)nr1 * i2, nr3, nr1 * nr2, tw3, buf, buf2, tmp);
  if (sign < 0) {
    double scale = 1.0 / ((double)nr1 * nr2 * nr3);
    for (size_t i = 0; i < (size_t)nr1 * nr2 * nr3; ++i) box[i] *= scale;
  }
  free(buf); free(buf2); free(tmp); free(tw1); free(tw2); free(tw3);
}

/* H psi for m vectors (QE h_psi semantics, see file header). */
void oracle_pw_hpsi(const oracle_pw_op* op, int m, const double* psir, double* hpsir) {
  const zc* psi = (const zc*)psir;
  zc* hpsi = (zc*)hpsir;
  const zc* vkb = (const zc*)op->vkb;
  int n = op->npw;
  size_t nnr = (size_t)op->nr1 * op->nr2 * op->nr3;
  zc* box = (zc*)malloc(sizeof(zc) * nnr);
  zc* bec = (zc*)malloc(sizeof(zc) * (op->nkb > 0 ? op->nkb : 1));
  for (int ib = 0; ib < m; ++ib) {
    const zc* p = psi + (size_t)ib * n;
    zc* h = hpsi + (size_t)ib * n;
    /* kinetic */
    for (int ig = 0; ig < n; ++ig) h[ig] = op->g2kin[ig] * p[ig];
    /* local potential: scatter, invfft, multiply, fwfft, gather */
    memset(box, 0, sizeof(zc) * nnr);
    for (int ig = 0; ig < n; ++ig) box[op->nl[ig]] = p[ig];
    oracle_fft3d((double*)box, op->nr1, op->nr2, op->nr3, +1);
    for (size_t ir = 0; ir < nnr; ++ir) box[ir] *= op->vrs[ir];
    oracle_fft3d((double*)box, op->nr1, op->nr2, op->nr3, -1);
    for (int ig = 0; ig < n; ++ig) h[ig] += box[op->nl[ig]];
    /* nonlocal: becp = beta^dagger psi, then H += beta D becp */
    for (int k = 0; k < op->nkb; ++k) {
      zc s = 0;
      const zc* b = vkb + (size_t)k * n;
      for (int ig = 0; ig < n; ++ig) s += conj(b[ig]) * p[ig];
      bec[k] = op->dvan[k] * s;
    }
    for (int k = 0; k < op->nkb; ++k) {
      const zc* b = vkb + (size_t)k * n;
      for (int ig = 0; ig < n; ++ig) h[ig] += b[ig] * bec[k];
    }
  }
  free(box);
  free(bec);
}

/* linear_op.f90:46-144 for one vector: (H + sigma + alpha_pv P_v) x */
void oracle_pw_apply(void* ctx, const double* sigmar, const double* xr, double* axr, int n) {
  const oracle_pw_op* op = (const oracle_pw_op*)ctx;
  const zc* x = (const zc*)xr;
  zc* ax = (zc*)axr;
  zc sigma = *(const zc*)sigmar;
  oracle_pw_hpsi(op, 1, xr, axr);
  for (int i = 0; i < n; ++i) ax[i] += sigma * x[i];
  if (fabs(op->alpha_pv) > 1e-14) { /* eps14, linear_op.f90:131 */
    const zc* evq = (const zc*)op->evq;
    for (int v = 0; v < op->nocc; ++v) {
      const zc* e = evq + (size_t)v * n;
      zc proj = 0;
      for (int i = 0; i < n; ++i) proj += conj(e[i]) * x[i];
      proj *= op->alpha_pv;
      for (int i = 0; i < n; ++i) ax[i] += e[i] * proj;
    }
  }
}
