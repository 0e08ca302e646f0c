/*
 * ss_oracle.c -- CPU oracle for the two-electron ZV-MC path (TEST INFRASTRUCTURE).
 *
 * A plain-C restatement of the reference's FP64 algorithms, used only as the
 * checker of the CUDA path (tests/, the smoke check) and as the CPU baseline
 * of bench.py.  Each function cites the reference file:line it follows.
 * Built with -ffp-contract=off so no fused multiply-adds change the rounding
 * of the reference's expressions.
 *
 * Parity status: parity unpinned.  The reference has no tests or golden outputs
 * and cannot be compiled here (Fortran, no compiler), so nothing of the
 * reference's own pins this restatement; it is checked instead against
 * analytic known-answer tests (closed forms, quadrature; tests/test_oracle_kat.py).
 *
 * Known, documented deviations from the reference's arithmetic:
 *  - fact(n) (src/fact.F90:1-27) returns exp(logfact(n)) on the first call
 *    for a new n and the memoised product afterwards; the oracle always uses
 *    the memoised product memo(i) = memo(i-1)*i (the steady state).
 */
#include "ss_oracle.h"

#include <math.h>
#include <time.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define MAXD 160 /* polynomial scratch; the reference uses 0:511 (max_dim) */
static const double THRESH = 1.e-15;
static const double PI_5_2 = 34.9868366552; /* 12-digit constant, src/general_primitive_integral.F90:25 */

/* ------------------------------------------------------------------ */
/* factorials (src/fact.F90:1-34, src/logfact.F90:1-29)                */
/* ------------------------------------------------------------------ */
static double g_fact[101];
static double g_logfact[101];
static double g_binom[16][16];
static int g_init = 0;

static void init_tables(void) {
  if (g_init) return;
  g_fact[0] = 1.0;
  g_fact[1] = 1.0;
  for (int i = 2; i <= 100; i++) g_fact[i] = g_fact[i - 1] * (double)i;
  g_logfact[0] = 0.0;
  g_logfact[1] = 0.0;
  for (int i = 2; i <= 100; i++) g_logfact[i] = g_logfact[i - 1] + log((double)i);
  /* binom_func memo (src/binom_func.F90:14-21) */
  for (int k = 0; k <= 15; k++)
    for (int l = 0; l <= 15; l++) {
      double lf_kl = (k - l) < 2 ? 0.0 : g_logfact[k - l];
      g_binom[k][l] = exp(g_logfact[k] - g_logfact[l] - lf_kl);
    }
  g_init = 1;
}

static double fact(int n) { return n < 2 ? 1.0 : g_fact[n]; }
static double fact_inv(int n) { return 1.0 / fact(n); }

static double logfact(int n) {
  if (n < 2) return 0.0;
  if (n <= 100) return g_logfact[n];
  double v = g_logfact[100];
  for (int i = 101; i <= n; i++) v += log((double)i);
  return v;
}

static double binom_func(int i, int j) {
  if (i <= 15 && j <= 15 && i >= 0 && j >= 0) return g_binom[i][j];
  return exp(logfact(i) - logfact(j) - logfact(i - j));
}

/* ------------------------------------------------------------------ */
/* polynomial helpers                                                  */
/* ------------------------------------------------------------------ */
/* D(t) += B(t)*C(t) ; nd = highest nonzero index (src/multiply_poly.F90:1-40) */
static void multiply_poly(const double *b, int nb, const double *c, int nc, double *d, int *nd) {
  if (nb < 0 || nc < 0) return;
  int ndtmp = nb + nc;
  for (int ic = 0; ic <= nc; ic++) d[ic] = d[ic] + c[ic] * b[0];
  for (int ib = 1; ib <= nb; ib++) {
    d[ib] = d[ib] + c[0] * b[ib];
    for (int ic = 1; ic <= nc; ic++) d[ib + ic] = d[ib + ic] + c[ic] * b[ib];
  }
  int k;
  for (k = ndtmp; k >= 0; k--)
    if (d[k] != 0.0) break;
  *nd = k;
}

/* D(t) += cst*B(t) (src/add_poly_multiply.F90:1-28) */
static void add_poly_multiply(const double *b, int nb, double cst, double *d, int *nd) {
  *nd = (*nd > nb) ? *nd : nb;
  if (*nd != -1) {
    for (int ib = 0; ib <= nb; ib++) d[ib] = d[ib] + cst * b[ib];
    while (d[*nd] == 0.0) {
      (*nd)--;
      if (*nd < 0) break;
    }
  }
}

/* (x - x_A)^a expanded around x_P (src/give_explicit_poly_and_gaussian.F90:86-220) */
static void recentered_poly(double *P, double x_A, double x_P, int a) {
  double pw[MAXD];
  if (a < 0) return;
  pw[0] = 1.0;
  pw[1] = x_P - x_A;
  switch (a) {
    case 0: P[0] = pw[0]; return;
    case 1: P[0] = pw[1]; P[1] = pw[0]; return;
    case 2:
      pw[2] = pw[1] * pw[1];
      P[0] = pw[2]; P[1] = 2.0 * pw[1]; P[2] = pw[0];
      return;
    case 3:
      pw[2] = pw[1] * pw[1]; pw[3] = pw[2] * pw[1];
      P[0] = pw[3]; P[1] = 3.0 * pw[2]; P[2] = 3.0 * pw[1]; P[3] = pw[0];
      return;
    case 4:
      pw[2] = pw[1] * pw[1]; pw[3] = pw[2] * pw[1]; pw[4] = pw[2] * pw[2];
      P[0] = pw[4]; P[1] = 4.0 * pw[3]; P[2] = 6.0 * pw[2]; P[3] = 4.0 * pw[1]; P[4] = pw[0];
      return;
    default: break;
  }
  for (int i = 2; i <= a; i++) pw[i] = pw[i - 1] * pw[1];
  if (a <= 8) {
    /* cases 5..8: exact integer binomials times powers */
    static const double bin[9][9] = {
        {1}, {1, 1}, {1, 2, 1}, {1, 3, 3, 1}, {1, 4, 6, 4, 1}, {1, 5, 10, 10, 5, 1},
        {1, 6, 15, 20, 15, 6, 1}, {1, 7, 21, 35, 35, 21, 7, 1}, {1, 8, 28, 56, 70, 56, 28, 8, 1}};
    P[0] = pw[a];
    for (int i = 1; i <= a; i++) P[i] = bin[a][i] * pw[a - i];
    return;
  }
  P[0] = pw[a];
  for (int i = 1; i <= a; i++) P[i] = binom_func(a, a - i) * pw[a - i];
}

/* 3D Gaussian product (src/gaussian_product.F90:1-33); returns 0 if exponent > 40 */
static void gaussian_product(double a, const double *xa, double b, const double *xb, double *k,
                             double *p, double *xp) {
  *p = a + b;
  double p_inv = 1.0 / (a + b);
  double ab = a * b;
  double xab0 = xa[0] - xb[0], xab1 = xa[1] - xb[1], xab2 = xa[2] - xb[2];
  ab = ab * p_inv;
  double kk = ab * (xab0 * xab0 + xab1 * xab1 + xab2 * xab2);
  if (kk > 40.0) {
    *k = 0.0;
    xp[0] = xp[1] = xp[2] = 0.0; /* left unset by the reference; never used */
    return;
  }
  *k = exp(-kk);
  xp[0] = (a * xa[0] + b * xb[0]) * p_inv;
  xp[1] = (a * xa[1] + b * xb[1]) * p_inv;
  xp[2] = (a * xa[2] + b * xb[2]) * p_inv;
}

/* (src/give_explicit_poly_and_gaussian.F90:1-84); P_new[axis*MAXD + i] */
static void give_explicit_poly_and_gaussian(double *P_new, double *P_center, double *p,
                                            double *fact_k, int *iorder, double alpha, double beta,
                                            const int *a, const int *b, const double *A,
                                            const double *B) {
  iorder[0] = iorder[1] = iorder[2] = 0;
  P_new[0] = P_new[MAXD] = P_new[2 * MAXD] = 0.0;
  gaussian_product(alpha, A, beta, B, fact_k, p, P_center);
  if (*fact_k < THRESH) {
    *fact_k = 0.0;
    return;
  }
  for (int ax = 0; ax < 3; ax++) {
    double Pa[MAXD], Pb[MAXD];
    recentered_poly(Pa, A[ax], P_center[ax], a[ax]);
    recentered_poly(Pb, B[ax], P_center[ax], b[ax]);
    iorder[ax] = a[ax] + b[ax];
    double *Pn = P_new + ax * MAXD;
    for (int i = 0; i <= iorder[ax]; i++) Pn[i] = 0.0;
    int n_new = 0;
    multiply_poly(Pa, a[ax], Pb, b[ax], Pn, &n_new);
  }
}

/* ------------------------------------------------------------------ */
/* Rys-like polynomial recursions in t (src/I_x1_pol_mult*.F90, I_x2_pol_mult.F90) */
/* ------------------------------------------------------------------ */
typedef struct {
  double B10[3], B01[3], B00[3], C00[3], D00[3];
} rec_coef;

static void I_x2_pol_mult(int c, const rec_coef *R, double *d, int *nd, int dim);
static void I_x1_pol_mult_a1(int c, const rec_coef *R, double *d, int *nd, int n_pt_in);
static void I_x1_pol_mult_a2(int c, const rec_coef *R, double *d, int *nd, int n_pt_in);
static void I_x1_pol_mult_recurs(int a, int c, const rec_coef *R, double *d, int *nd, int n_pt_in);

/* (src/I_x2_pol_mult.F90:1-84) */
static void I_x2_pol_mult(int c, const rec_coef *R, double *d, int *nd, int dim) {
  double X[MAXD], Y[MAXD];
  int nx, ny;
  if (c == 0) {
    *nd = 0;
    d[0] = 1.0;
    return;
  }
  if (c < 0) {
    *nd = -1;
    return;
  }
  if (c == 1) {
    *nd = 2;
    d[0] = R->D00[0]; d[1] = R->D00[1]; d[2] = R->D00[2];
    return;
  }
  if (c == 2) {
    *nd = 2;
    d[0] = R->B01[0]; d[1] = R->B01[1]; d[2] = R->B01[2];
    ny = 2;
    Y[0] = R->D00[0]; Y[1] = R->D00[1]; Y[2] = R->D00[2];
    multiply_poly(Y, ny, R->D00, 2, d, nd);
    return;
  }
  for (int ix = 0; ix <= c + c; ix++) X[ix] = 0.0;
  nx = 0;
  I_x2_pol_mult(c - 2, R, X, &nx, dim);
  for (int ix = 0; ix <= nx; ix++) X[ix] = X[ix] * (double)(c - 1);
  multiply_poly(X, nx, R->B01, 2, d, nd);
  ny = 0;
  for (int ix = 0; ix <= c + c; ix++) Y[ix] = 0.0;
  I_x2_pol_mult(c - 1, R, Y, &ny, dim);
  multiply_poly(Y, ny, R->D00, 2, d, nd);
}

/* (src/I_x1_pol_mult_a1.F90:1-59) */
static void I_x1_pol_mult_a1(int c, const rec_coef *R, double *d, int *nd, int n_pt_in) {
  double X[MAXD], Y[MAXD];
  int nx, ny;
  if (c < 0 || *nd < 0) {
    *nd = -1;
    return;
  }
  nx = *nd;
  for (int ix = 0; ix <= n_pt_in; ix++) X[ix] = 0.0;
  I_x2_pol_mult(c - 1, R, X, &nx, n_pt_in);
  if (c > 1)
    for (int ix = 0; ix <= nx; ix++) X[ix] = X[ix] * (double)c;
  multiply_poly(X, nx, R->B00, 2, d, nd);
  ny = 0;
  for (int ix = 0; ix <= n_pt_in; ix++) Y[ix] = 0.0;
  I_x2_pol_mult(c, R, Y, &ny, n_pt_in);
  multiply_poly(Y, ny, R->C00, 2, d, nd);
}

/* (src/I_x1_pol_mult_a2.F90:1-61) */
static void I_x1_pol_mult_a2(int c, const rec_coef *R, double *d, int *nd, int n_pt_in) {
  double X[MAXD], Y[MAXD];
  int nx, ny;
  for (int ix = 0; ix <= n_pt_in; ix++) X[ix] = 0.0;
  nx = 0;
  I_x2_pol_mult(c, R, X, &nx, n_pt_in);
  multiply_poly(X, nx, R->B10, 2, d, nd);
  nx = *nd;
  for (int ix = 0; ix <= n_pt_in; ix++) X[ix] = 0.0;
  I_x1_pol_mult_a1(c - 1, R, X, &nx, n_pt_in);
  if (c > 1)
    for (int ix = 0; ix <= nx; ix++) X[ix] = X[ix] * (double)c;
  multiply_poly(X, nx, R->B00, 2, d, nd);
  ny = 0;
  for (int ix = 0; ix <= n_pt_in; ix++) Y[ix] = 0.0;
  I_x1_pol_mult_a1(c, R, Y, &ny, n_pt_in);
  multiply_poly(Y, ny, R->C00, 2, d, nd);
}

/* (src/I_x1_pol_mult_recurs.F90:1-80) */
static void I_x1_pol_mult_recurs(int a, int c, const rec_coef *R, double *d, int *nd, int n_pt_in) {
  double X[MAXD], Y[MAXD];
  int nx, ny;
  for (int ix = 0; ix <= n_pt_in; ix++) X[ix] = 0.0;
  nx = 0;
  if (a == 3)
    I_x1_pol_mult_a1(c, R, X, &nx, n_pt_in);
  else if (a == 4)
    I_x1_pol_mult_a2(c, R, X, &nx, n_pt_in);
  else
    I_x1_pol_mult_recurs(a - 2, c, R, X, &nx, n_pt_in);
  for (int ix = 0; ix <= nx; ix++) X[ix] = X[ix] * (double)(a - 1);
  multiply_poly(X, nx, R->B10, 2, d, nd);
  nx = *nd;
  for (int ix = 0; ix <= n_pt_in; ix++) X[ix] = 0.0;
  if (c > 0) {
    if (a == 3)
      I_x1_pol_mult_a2(c - 1, R, X, &nx, n_pt_in);
    else
      I_x1_pol_mult_recurs(a - 1, c - 1, R, X, &nx, n_pt_in);
    if (c > 1)
      for (int ix = 0; ix <= nx; ix++) X[ix] = X[ix] * (double)c;
    multiply_poly(X, nx, R->B00, 2, d, nd);
  }
  ny = 0;
  for (int ix = 0; ix <= n_pt_in; ix++) Y[ix] = 0.0;
  if (a == 3)
    I_x1_pol_mult_a2(c, R, Y, &ny, n_pt_in);
  else
    I_x1_pol_mult_recurs(a - 1, c, R, Y, &ny, n_pt_in);
  multiply_poly(Y, ny, R->C00, 2, d, nd);
}

/* (src/I_x1_pol_mult.F90:1-47) */
static void I_x1_pol_mult(int a, int c, const rec_coef *R, double *d, int *nd, int n_pt_in) {
  if (c >= 0 && *nd >= 0) {
    if (a == 1)
      I_x1_pol_mult_a1(c, R, d, nd, n_pt_in);
    else if (a == 2)
      I_x1_pol_mult_a2(c, R, d, nd, n_pt_in);
    else if (a > 2)
      I_x1_pol_mult_recurs(a, c, R, d, nd, n_pt_in);
    else {
      if (c == 0) {
        *nd = 0;
        d[0] = 1.0;
        return;
      }
      I_x2_pol_mult(c, R, d, nd, n_pt_in);
    }
  } else {
    *nd = -1;
  }
}

/* (src/give_polynom_mult_center_x.F90:1-74) */
static void give_polynom_mult_center_x(double P_center, double Q_center, int a_x, int d_x, double p,
                                       double q, int n_pt_in, double pq_inv, double pq_inv_2,
                                       double p10_1, double p01_1, double p10_2, double p01_2,
                                       double *d, int *n_pt_out) {
  rec_coef R;
  R.B10[0] = p10_1; R.B10[1] = 0.0; R.B10[2] = -p10_2;
  R.B01[0] = p01_1; R.B01[1] = 0.0; R.B01[2] = -p01_2;
  R.B00[0] = 0.0; R.B00[1] = 0.0; R.B00[2] = pq_inv;
  for (int i = 0; i <= n_pt_in; i++) d[i] = 0.0;
  int n_pt1 = n_pt_in;
  R.C00[0] = 0.0; R.C00[1] = 0.0; R.C00[2] = -q * (P_center - Q_center) * pq_inv_2;
  R.D00[0] = 0.0; R.D00[1] = 0.0; R.D00[2] = -p * (Q_center - P_center) * pq_inv_2;
  I_x1_pol_mult(a_x, d_x, &R, d, &n_pt1, n_pt_in);
  *n_pt_out = n_pt1;
  if (n_pt1 < 0) {
    *n_pt_out = -1;
    for (int i = 0; i <= n_pt_in; i++) d[i] = 0.0;
  }
}

/* ------------------------------------------------------------------ */
/* Boys-type integrals                                                 */
/* ------------------------------------------------------------------ */
/* Taylor series of F_n for rho < 1 (src/rint1.F90:1-59); NaN if not converged */
static double rint1(int n, double rho) {
  const double eps = 1.e-15;
  double r, rho_tmp = 1.0, diff = 0.0;
  if (n < 50) {
    r = 1.0 / (double)(n + n + 1);
    for (int k = 1; k <= 20; k++) {
      rho_tmp = -rho_tmp * rho;
      diff = rho_tmp * fact_inv(k) * (1.0 / (double)(2 * (k + n) + 1));
      r = r + diff;
      if (fabs(diff) > eps) continue;
      return r;
    }
  } else {
    r = 1.0 / (double)(n + n + 1);
    for (int k = 1; k <= 20; k++) {
      rho_tmp = -rho_tmp * rho;
      diff = rho_tmp * fact_inv(k) / (double)(2 * (k + n) + 1);
      r = r + diff;
      if (fabs(diff) > eps) continue;
      return r;
    }
  }
  return NAN; /* the reference stops the program here (src/rint1.F90:56-58) */
}

/* (src/hermite.F90:1-24) */
static double hermite(int n, double x) {
  double h0 = 1.0, h1, h2 = 0.0;
  if (n == 0) return h0;
  h1 = x + x;
  if (n == 1) return h1;
  for (int k = 1; k <= n - 1; k++) {
    h2 = (x + x) * h1 - (double)(k + k) * h0;
    h0 = h1;
    h1 = h2;
  }
  return h2;
}

static double powi(double x, int k) { /* x**k, binary exponentiation */
  double r = 1.0, b = x;
  while (k > 0) {
    if (k & 1) r *= b;
    b *= b;
    k >>= 1;
  }
  return r;
}

/* (src/rint_large_n.F90:1-29) */
static double rint_large_n(int n, double rho) {
  double u = sqrt(rho), accu = 0.0, eps = 1.0;
  int k = 0;
  while (eps > 1.e-15 && k < 200) {
    double t1 = 1.0;
    for (int l = 0; l <= k; l++) t1 = t1 * ((double)(n + n + l) + 1.0);
    double t2 = 0.0;
    for (int l = 0; l <= k; l++) t2 = t2 + ((l & 1) ? -1.0 : 1.0) / (fact(l + 1) * fact(k - l));
    double alpha_k = t2 * fact(k + 1) * fact(k) * ((k & 1) ? -1.0 : 1.0);
    alpha_k = alpha_k / t1;
    double rajout = ((k & 1) ? -1.0 : 1.0) * powi(u, k) * hermite(k, u) * alpha_k / fact(k);
    accu = accu + rajout;
    eps = fabs(rajout) / accu;
    k = k + 1;
  }
  return exp(-rho) * accu;
}

double orc_rint_sum(int n_pt_out, double rho, const double *d1) {
  init_tables();
  const double sqpi = sqrt(M_PI);
  double r;
  if (rho < 1.0) {
    if (rho == 0.0) {
      r = d1[0];
    } else {
      double u_inv = 1.0 / sqrt(rho);
      double u = rho * u_inv;
      r = 0.5 * u_inv * sqpi * erf(u) * d1[0];
    }
    for (int i = 2; i <= n_pt_out; i += 2) r = r + d1[i] * rint1(i >> 1, rho);
  } else {
    double v = (rho > 80.0) ? 0.0 : exp(-rho);
    double u_inv = 1.0 / sqrt(rho);
    double u = rho * u_inv;
    double two_rho_inv = 0.5 * u_inv * u_inv;
    double val0 = 0.5 * u_inv * sqpi * erf(u);
    r = val0 * d1[0];
    double rint_tmp = (val0 - v) * two_rho_inv;
    double di = 3.0;
    int top = n_pt_out < 40 ? n_pt_out : 40;
    for (int i = 2; i <= top; i += 2) {
      r = r + d1[i] * rint_tmp;
      rint_tmp = (rint_tmp * di - v) * two_rho_inv;
      di = di + 2.0;
    }
    for (int i = 42; i <= n_pt_out; i += 2) r = r + d1[i] * rint_large_n(i >> 1, rho);
  }
  return r;
}

/* (src/rint.F90:1-63) */
double orc_rint(int n, double rho) {
  init_tables();
  const double sqpi = sqrt(M_PI);
  if (n == 0) {
    if (rho == 0.0) return 1.0;
    double u_inv = 1.0 / sqrt(rho);
    double u = rho * u_inv;
    return 0.5 * u_inv * sqpi * erf(u);
  }
  if (rho < 1.0) return rint1(n, rho);
  if (n <= 20) {
    double u_inv = 1.0 / sqrt(rho);
    double v = (rho > 80.0) ? 0.0 : exp(-rho);
    double u = rho * u_inv;
    double two_rho_inv = 0.5 * u_inv * u_inv;
    double val0 = 0.5 * u_inv * sqpi * erf(u);
    double r = (val0 - v) * two_rho_inv;
    for (int k = 2; k <= n; k++) r = (r * (double)(k + k - 1) - v) * two_rho_inv;
    return r;
  }
  return rint_large_n(n, rho);
}

/* ------------------------------------------------------------------ */
/* primitive ERI                                                       */
/* ------------------------------------------------------------------ */
/* (src/general_primitive_integral.F90:9-194) */
static double general_primitive_integral(const double *P_new, const double *P_center, double fact_p,
                                         double p, double p_inv, const int *iorder_p,
                                         const double *Q_new, const double *Q_center, double fact_q,
                                         double q, double q_inv, const int *iorder_q) {
  double Ix_pol[MAXD], Iy_pol[MAXD], Iz_pol[MAXD], dx[MAXD], d_poly[MAXD], d1[MAXD];
  int n_Ix, n_Iy, n_Iz, nx;
  double pq = p_inv * 0.5 * q_inv;
  double pq_inv = 0.5 / (p + q);
  double p10_1 = q * pq;
  double p01_1 = p * pq;
  double pq_inv_2 = pq_inv + pq_inv;
  double p10_2 = pq_inv_2 * p10_1 * q;
  double p01_2 = pq_inv_2 * p01_1 * p;
  int iorder;

  /* Ix: note the x-axis skips |P| < thresh, y and z process |P| > thresh */
  iorder = iorder_p[0] + iorder_q[0] + iorder_p[0] + iorder_q[0];
  for (int ix = 0; ix <= iorder; ix++) Ix_pol[ix] = 0.0;
  n_Ix = 0;
  for (int ix = 0; ix <= iorder_p[0]; ix++) {
    if (fabs(P_new[ix]) < THRESH) continue;
    double a = P_new[ix];
    for (int jx = 0; jx <= iorder_q[0]; jx++) {
      double d = a * Q_new[jx];
      if (fabs(d) < THRESH) continue;
      give_polynom_mult_center_x(P_center[0], Q_center[0], ix, jx, p, q, iorder, pq_inv, pq_inv_2,
                                 p10_1, p01_1, p10_2, p01_2, dx, &nx);
      add_poly_multiply(dx, nx, d, Ix_pol, &n_Ix);
    }
  }
  if (n_Ix == -1) return 0.0;

  iorder = iorder_p[1] + iorder_q[1] + iorder_p[1] + iorder_q[1];
  for (int ix = 0; ix <= iorder; ix++) Iy_pol[ix] = 0.0;
  n_Iy = 0;
  for (int iy = 0; iy <= iorder_p[1]; iy++) {
    if (fabs(P_new[MAXD + iy]) > THRESH) {
      double b = P_new[MAXD + iy];
      for (int jy = 0; jy <= iorder_q[1]; jy++) {
        double e = b * Q_new[MAXD + jy];
        if (fabs(e) < THRESH) continue;
        give_polynom_mult_center_x(P_center[1], Q_center[1], iy, jy, p, q, iorder, pq_inv,
                                   pq_inv_2, p10_1, p01_1, p10_2, p01_2, dx, &nx);
        add_poly_multiply(dx, nx, e, Iy_pol, &n_Iy);
      }
    }
  }
  if (n_Iy == -1) return 0.0;

  iorder = iorder_p[2] + iorder_q[2] + iorder_p[2] + iorder_q[2];
  for (int ix = 0; ix <= iorder; ix++) Iz_pol[ix] = 0.0;
  n_Iz = 0;
  for (int iz = 0; iz <= iorder_p[2]; iz++) {
    if (fabs(P_new[2 * MAXD + iz]) > THRESH) {
      double c = P_new[2 * MAXD + iz];
      for (int jz = 0; jz <= iorder_q[2]; jz++) {
        double f = c * Q_new[2 * MAXD + jz];
        if (fabs(f) < THRESH) continue;
        give_polynom_mult_center_x(P_center[2], Q_center[2], iz, jz, p, q, iorder, pq_inv,
                                   pq_inv_2, p10_1, p01_1, p10_2, p01_2, dx, &nx);
        add_poly_multiply(dx, nx, f, Iz_pol, &n_Iz);
      }
    }
  }
  if (n_Iz == -1) return 0.0;

  double rho = p * q * pq_inv_2;
  double dist = (P_center[0] - Q_center[0]) * (P_center[0] - Q_center[0]) +
                (P_center[1] - Q_center[1]) * (P_center[1] - Q_center[1]) +
                (P_center[2] - Q_center[2]) * (P_center[2] - Q_center[2]);
  double cst = dist * rho;

  int n_pt_tmp = n_Ix + n_Iy;
  for (int i = 0; i <= n_pt_tmp; i++) d_poly[i] = 0.0;
  multiply_poly(Ix_pol, n_Ix, Iy_pol, n_Iy, d_poly, &n_pt_tmp);
  if (n_pt_tmp == -1) return 0.0;
  int n_pt_out = n_pt_tmp + n_Iz;
  for (int i = 0; i <= n_pt_out; i++) d1[i] = 0.0;
  multiply_poly(d_poly, n_pt_tmp, Iz_pol, n_Iz, d1, &n_pt_out);

  double accu = 0.0;
  accu = accu + orc_rint_sum(n_pt_out, cst, d1);
  return fact_p * fact_q * accu * PI_5_2 * p_inv * q_inv / sqrt(p + q);
}

/* (src/bielec_integral.F90:1-55) */
double orc_bielec_integral(double alpha, double beta, double delta, double gama, const double *A,
                           const double *B, const double *C, const double *D, const int *pA,
                           const int *pB, const int *pC, const int *pD) {
  init_tables();
  double P_new[3 * MAXD], Q_new[3 * MAXD], P_center[3], Q_center[3], pp, qq, fact_p, fact_q;
  int iorder_p[3], iorder_q[3];
  give_explicit_poly_and_gaussian(P_new, P_center, &pp, &fact_p, iorder_p, alpha, beta, pA, pB, A, B);
  double p_inv = 1.0 / pp;
  give_explicit_poly_and_gaussian(Q_new, Q_center, &qq, &fact_q, iorder_q, delta, gama, pC, pD, C, D);
  double q_inv = 1.0 / qq;
  return general_primitive_integral(P_new, P_center, fact_p, pp, p_inv, iorder_p, Q_new, Q_center,
                                    fact_q, qq, q_inv, iorder_q);
}

/* ------------------------------------------------------------------ */
/* contracted ERI of the fits                                          */
/* ------------------------------------------------------------------ */
#define CG(b, m, i, t) ((b)->c_gauss[(m) + (int64_t)(b)->ld * ((i) + (int64_t)(b)->n * (t))])
#define GG(b, m, i) ((b)->g_gauss[(m) + (int64_t)(b)->ld * (i)])

/* cartesian components of one fitted function (src/gauss_ijkl.F90:68-123) */
static int components(const orc_basis *b, int io, int n_c[4][3], int *coef_t) {
  const int *np = b->npower + 3 * io;
  int it = b->i_type[io];
  if (it == 1) {
    for (int l = 0; l < 3; l++) n_c[0][l] = np[l];
    coef_t[0] = 0;
    return 1;
  }
  if (it == 2) {
    for (int ii = 0; ii < 3; ii++) {
      for (int l = 0; l < 3; l++) n_c[ii][l] = np[l] + (l == ii ? 2 : 0);
      coef_t[ii] = 1;
    }
    return 3;
  }
  /* i_type 3: r^0 and r^2 parts */
  for (int ii = 0; ii < 4; ii++) {
    for (int l = 0; l < 3; l++) n_c[ii][l] = np[l] + (l == ii - 1 ? 2 : 0);
    coef_t[ii] = ii == 0 ? 0 : 1;
  }
  return 4;
}

/* 0: sequential FP64 accumulation as the reference (src/gauss_ijkl.F90:125-152);
 * 1: same terms accumulated in long double (the exactly-summed value the parity tests use,
 *    since the reference's own sequential sum over ~1e7 terms carries ~1e-12 rounding). */
static int g_sum_mode = 0;
void orc_set_sum_mode(int mode) { g_sum_mode = mode; }

double orc_gauss_ijkl(const orc_basis *b, int i, int k, int j, int l) {
  init_tables();
  int orb[4] = {i, k, j, l};
  int nc[4], n_c[4][4][3], ct[4][4];
  for (int kk = 0; kk < 4; kk++) nc[kk] = components(b, orb[kk], n_c[kk], ct[kk]);
  const double *A = b->center + 3 * i, *B = b->center + 3 * k, *C = b->center + 3 * j,
               *D = b->center + 3 * l;
  double rint = 0.0;
  long double rint_ext = 0.0L;
  for (int i1 = 0; i1 < b->n_gauss[i]; i1++)
    for (int i2 = 0; i2 < b->n_gauss[k]; i2++)
      for (int i3 = 0; i3 < b->n_gauss[j]; i3++)
        for (int i4 = 0; i4 < b->n_gauss[l]; i4++)
          for (int ii1 = 0; ii1 < nc[0]; ii1++)
            for (int ii2 = 0; ii2 < nc[1]; ii2++)
              for (int ii3 = 0; ii3 < nc[2]; ii3++)
                for (int ii4 = 0; ii4 < nc[3]; ii4++) {
                  double d1 = CG(b, i1, i, ct[0][ii1]);
                  double d2 = CG(b, i2, k, ct[1][ii2]);
                  double d3 = CG(b, i3, j, ct[2][ii3]);
                  double d4 = CG(b, i4, l, ct[3][ii4]);
                  double term = d1 * d2 * d3 * d4 *
                                orc_bielec_integral(GG(b, i1, i), GG(b, i2, k), GG(b, i3, j),
                                                    GG(b, i4, l), A, B, C, D, n_c[0][ii1],
                                                    n_c[1][ii2], n_c[2][ii3], n_c[3][ii4]);
                  rint = rint + term;
                  rint_ext += (long double)term;
                }
  return g_sum_mode ? (double)rint_ext : rint;
}

static int nc_of(const orc_basis *b, int io) {
  int t = b->i_type[io];
  return t == 1 ? 1 : (t == 2 ? 3 : 4);
}

double orc_count_primitive_quartets(const orc_basis *b, int64_t nint, const int32_t *is,
                                    const int32_t *js, const int32_t *ks, const int32_t *ls) {
  double tot = 0.0;
  for (int64_t q = 0; q < nint; q++) {
    int o[4] = {is[q] - 1, ks[q] - 1, js[q] - 1, ls[q] - 1};
    double c = 1.0;
    for (int t = 0; t < 4; t++) c *= (double)(b->n_gauss[o[t]] * nc_of(b, o[t]));
    tot += c;
  }
  return tot;
}

void orc_precond(const orc_basis *b, double *precond, int nthreads) {
  int n = b->n;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
#pragma omp parallel for schedule(dynamic, 1) collapse(2)
  for (int k = 0; k < n; k++)
    for (int i = 0; i < n; i++) precond[i + n * k] = orc_gauss_ijkl(b, i, k, i, k);
}

int64_t orc_gauss_eri(const orc_basis *b, int64_t nint, const int32_t *is, const int32_t *js,
                      const int32_t *ks, const int32_t *ls, const double *precond, double *out,
                      int nthreads) {
  const double seuil = 1.e-15;
  int n = b->n;
  int64_t nzero = 0;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : nzero)
  for (int64_t q = 0; q < nint; q++) {
    int i = is[q] - 1, k = ks[q] - 1, j = js[q] - 1, l = ls[q] - 1;
    double pik = precond[i + n * k], pjl = precond[j + n * l];
    if (fabs(pik * pjl) < seuil * seuil) nzero++;
    if (i == j && k == l)
      out[q] = pik;
    else if (fabs(pik * pjl) >= seuil * seuil)
      out[q] = orc_gauss_ijkl(b, i, k, j, l);
    else
      out[q] = 0.0;
  }
  return nzero;
}

/* gauss_ijkl of every listed quartet, no Schwarz screening and no diagonal shortcut (the
 * entries of the Schwarz diagonal a subset of quartets needs, src/two_e_slater.F90:230-236) */
void orc_gauss_list(const orc_basis *b, int64_t nint, const int32_t *is, const int32_t *js,
                    const int32_t *ks, const int32_t *ls, double *out, int nthreads) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t q = 0; q < nint; q++) out[q] = orc_gauss_ijkl(b, is[q] - 1, ks[q] - 1, js[q] - 1, ls[q] - 1);
}

/* the same, with the seconds each quartet took on the thread that computed it (seconds may be
 * NULL); quartets are handed out one at a time, so a sample of quartets from several classes
 * runs on all threads at once and each quartet's time is its own single-thread cost */
void orc_gauss_list_timed(const orc_basis *b, int64_t nint, const int32_t *is, const int32_t *js,
                          const int32_t *ks, const int32_t *ls, double *out, double *seconds, int nthreads) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t q = 0; q < nint; q++) {
    struct timespec t0, t1;
    clock_gettime(CLOCK_MONOTONIC, &t0);
    out[q] = orc_gauss_ijkl(b, is[q] - 1, ks[q] - 1, js[q] - 1, ls[q] - 1);
    clock_gettime(CLOCK_MONOTONIC, &t1);
    if (seconds) seconds[q] = (double)(t1.tv_sec - t0.tv_sec) + 1e-9 * (double)(t1.tv_nsec - t0.tv_nsec);
  }
}

/* ------------------------------------------------------------------ */
/* walker transform (src/dierfc.F90:3-68)                              */
/* ------------------------------------------------------------------ */
double orc_dierfc(double y) {
  const double qa = 9.16461398268964e-01, qb = 2.31729200323405e-01, qc = 4.88826640273108e-01,
               qd = 1.24610454613712e-01, q0 = 4.99999303439796e-01, q1 = 1.16065025341614e-01,
               q2 = 1.50689047360223e-01, q3 = 2.69999308670029e-01, q4 = -7.28846765585675e-02;
  const double pa = 3.97886080735226000e+00, pb = 1.20782237635245222e-01,
               p0 = 2.44044510593190935e-01, p1 = 4.34397492331430115e-01,
               p2 = 6.86265948274097816e-01, p3 = 9.56464974744799006e-01,
               p4 = 1.16374581931560831e+00, p5 = 1.21448730779995237e+00,
               p6 = 1.05375024970847138e+00, p7 = 7.13657635868730364e-01,
               p8 = 3.16847638520135944e-01, p9 = 1.47297938331485121e-02,
               p10 = -1.05872177941595488e-01, p11 = -7.43424357241784861e-02,
               p12 = 2.20995927012179067e-03, p13 = 3.46494207789099922e-02,
               p14 = 1.42961988697898018e-02, p15 = -1.18598117047771104e-02,
               p16 = -1.12749169332504870e-02, p17 = 3.39721910367775861e-03,
               p18 = 6.85649426074558612e-03, p19 = -7.71708358954120939e-04,
               p20 = -3.51287146129100025e-03, p21 = 1.05739299623423047e-04,
               p22 = 1.12648096188977922e-03;
  double z = y, w, u, s, t, x;
  if (y > 1.0) z = 2.0 - y;
  w = qa - log(z);
  u = sqrt(w);
  s = (qc + log(u)) / w;
  t = 1.0 / (u + qb);
  x = u * (1 - s * (0.5 + s * qd)) - ((((q4 * t + q3) * t + q2) * t + q1) * t + q0) * t;
  t = pa / (pa + x);
  u = t - 0.5;
  s = (((((((((p22 * u + p21) * u + p20) * u + p19) * u + p18) * u + p17) * u + p16) * u + p15) *
            u + p14) * u + p13) * u + p12;
  s = ((((((((((((s * u + p11) * u + p10) * u + p9) * u + p8) * u + p7) * u + p6) * u + p5) * u +
             p4) * u + p3) * u + p2) * u + p1) * u + p0) * t -
      z * exp(x * x - pb);
  x = x + s * (1.0 + x * s);
  if (y > 1.0) x = -x;
  return x;
}

/* ------------------------------------------------------------------ */
/* pair densities (src/compute_densities.F90:1-95, u_orb.F90, u_gauss.F90) */
/* ------------------------------------------------------------------ */
static double u_orb(const orc_basis *b, int i, double r) {
  /* c_contract = 1 (src/read_basis.F90:35), single contraction (src/u_orb.F90:8-27) */
  double g = b->g_slater[i];
  switch (b->n_sto[i]) {
    case 0: return 1.0 * exp(-g * r);
    case 1: return 1.0 * r * exp(-g * r);
    case 2: { double r2 = r * r; return 1.0 * r2 * exp(-g * r); }
    case 3: { double r2 = r * r; return 1.0 * r2 * r * exp(-g * r); }
    case 4: { double r2 = r * r; return 1.0 * r2 * r2 * exp(-g * r); }
    default: return 1.0 * pow(r, b->n_sto[i]) * exp(-g * r);
  }
}

static double u_gauss(const orc_basis *b, int i, double r) {
  double r2 = r * r, u = 0.0;
  for (int m = 0; m < b->n_gauss[i]; m++)
    u = u + (CG(b, m, i, 0) + CG(b, m, i, 1) * r2) * exp(-GG(b, m, i) * r2);
  return u;
}

/* one electron's pair densities at point u (src/compute_densities.F90:17-53) */
static void pair_density_at(const orc_basis *b, int i, int k, const double *u, double *rS,
                            double *rG) {
  const double *ci = b->center + 3 * i, *ck = b->center + 3 * k;
  const int *pi = b->npower + 3 * i, *pk = b->npower + 3 * k;
  double dx = u[0] - ci[0], dy = u[1] - ci[1], dz = u[2] - ci[2];
  double poly_i = 1.0;
  for (int t = 0; t < pi[0]; t++) poly_i = poly_i * dx;
  for (int t = 0; t < pi[1]; t++) poly_i = poly_i * dy;
  for (int t = 0; t < pi[2]; t++) poly_i = poly_i * dz;
  double r_i = sqrt(dx * dx + dy * dy + dz * dz);
  dx = u[0] - ck[0]; dy = u[1] - ck[1]; dz = u[2] - ck[2];
  double poly_k = 1.0;
  for (int t = 0; t < pk[0]; t++) poly_k = poly_k * dx;
  for (int t = 0; t < pk[1]; t++) poly_k = poly_k * dy;
  for (int t = 0; t < pk[2]; t++) poly_k = poly_k * dz;
  double r_k = sqrt(dx * dx + dy * dy + dz * dz);
  double poly_ik = poly_i * poly_k;
  *rS = poly_ik * u_orb(b, i, r_i) * u_orb(b, k, r_k);
  *rG = poly_ik * u_gauss(b, i, r_i) * u_gauss(b, k, r_k);
}

void orc_pair_densities(const orc_basis *b, int npairs, const int *ip, const int *kp, int64_t S,
                        const double *u, double *rhoS, double *rhoG) {
#pragma omp parallel for schedule(static)
  for (int p = 0; p < npairs; p++)
    for (int64_t s = 0; s < S; s++)
      pair_density_at(b, ip[p], kp[p], u + 3 * s, rhoS + (int64_t)p * S + s, rhoG + (int64_t)p * S + s);
}

/* ------------------------------------------------------------------ */
/* faithful ZV-MC (src/two_e_slater.F90:339-496)                       */
/* ------------------------------------------------------------------ */
#define NW 40         /* walkers per chunk, src/common_data.F90:4 */
#define SUPER (NW * 64) /* walkers whose densities are held at once */

int orc_zvmc_faithful(const orc_basis *b, int64_t nint, const int32_t *is, const int32_t *js,
                      const int32_t *ks, const int32_t *ls, double a_zv, const double *r1,
                      const double *r2, int nblocks, int64_t npts, int mode, double *mean,
                      double *err, double *xb, int nthreads) {
  init_tables();
  if (npts % NW != 0) return -1; /* src/two_e_slater.F90:148 */
  int n = b->n;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
  /* pair table: pair index for (i,k), i >= k, that is used (src/two_e_slater.F90:373-382) */
  int *pidx = (int *)malloc(sizeof(int) * n * n);
  for (int t = 0; t < n * n; t++) pidx[t] = -1;
  int np = 0;
  for (int64_t q = 0; q < nint; q++) {
    int i = is[q] - 1, k = ks[q] - 1, j = js[q] - 1, l = ls[q] - 1;
    if (pidx[i + n * k] < 0) pidx[i + n * k] = np++;
    if (pidx[j + n * l] < 0) pidx[j + n * l] = np++;
  }
  int *pi_ = (int *)malloc(sizeof(int) * np), *pk_ = (int *)malloc(sizeof(int) * np);
  for (int k = 0; k < n; k++)
    for (int i = 0; i < n; i++)
      if (pidx[i + n * k] >= 0) { pi_[pidx[i + n * k]] = i; pk_[pidx[i + n * k]] = k; }
  /* G_center and ZV factors (src/two_e_slater.F90:339-348, :406) */
  double *G = (double *)malloc(sizeof(double) * 3 * np);
  double *fzv = (double *)malloc(sizeof(double) * np);  /* 0.5 a / (g_i+g_k) */
  double *fjac = (double *)malloc(sizeof(double) * np); /* a / (g_i+g_k) */
  for (int p = 0; p < np; p++) {
    int i = pi_[p], k = pk_[p];
    double gi = b->g_slater[i], gk = b->g_slater[k];
    for (int l = 0; l < 3; l++)
      G[3 * p + l] = (gi * b->center[l + 3 * i] + gk * b->center[l + 3 * k]) / (gi + gk);
    fzv[p] = 0.5 * a_zv / (gi + gk);
    fjac[p] = a_zv / (gi + gk);
  }
  /* per super-chunk buffers: [p][s] */
  size_t ps = (size_t)np * SUPER;
  double *ut1 = (double *)malloc(sizeof(double) * 3 * ps), *ut2 = (double *)malloc(sizeof(double) * 3 * ps);
  double *rh1 = (double *)malloc(sizeof(double) * ps), *rh2 = (double *)malloc(sizeof(double) * ps);
  double *rg1 = (double *)malloc(sizeof(double) * ps), *rg2 = (double *)malloc(sizeof(double) * ps);
  double *j1 = (double *)malloc(sizeof(double) * ps), *j2 = (double *)malloc(sizeof(double) * ps);
  double *pi0 = (double *)malloc(sizeof(double) * SUPER);
  double *eS = (double *)malloc(sizeof(double) * nint), *eG = (double *)malloc(sizeof(double) * nint);
  double *acc = (double *)calloc(nint, sizeof(double)), *acc2 = (double *)calloc(nint, sizeof(double));
  const double fpi0 = 1.0 / ((2.0 * M_PI) * (2.0 * M_PI) * (2.0 * M_PI));

  for (int blk = 0; blk < nblocks; blk++) {
    for (int64_t q = 0; q < nint; q++) eS[q] = eG[q] = 0.0;
    for (int64_t s0 = 0; s0 < npts; s0 += SUPER) {
      int ns = (int)((npts - s0) < SUPER ? (npts - s0) : SUPER);
      const double *R1 = r1 + 3 * ((int64_t)blk * npts + s0);
      const double *R2 = r2 + 3 * ((int64_t)blk * npts + s0);
      /* pi_0 (src/compute_jacobian_and_pi0.F90:12-18) */
      for (int s = 0; s < ns; s++) {
        double m1 = R1[3 * s] * R1[3 * s] + R1[3 * s + 1] * R1[3 * s + 1] + R1[3 * s + 2] * R1[3 * s + 2];
        double m2 = R2[3 * s] * R2[3 * s] + R2[3 * s + 1] * R2[3 * s + 1] + R2[3 * s + 2] * R2[3 * s + 2];
        pi0[s] = exp(-0.5 * (m1 + m2)) * fpi0;
      }
#pragma omp parallel for schedule(dynamic, 1)
      for (int p = 0; p < np; p++) {
        int i = pi_[p], k = pk_[p];
        for (int s = 0; s < ns; s++) {
          const double *a1 = R1 + 3 * s, *a2 = R2 + 3 * s;
          double r1m = sqrt(a1[0] * a1[0] + a1[1] * a1[1] + a1[2] * a1[2]);
          double r2m = sqrt(a2[0] * a2[0] + a2[1] * a2[1] + a2[2] * a2[2]);
          double u1[3], u2[3];
          for (int l = 0; l < 3; l++) {
            u1[l] = fzv[p] * a1[l] * r1m + G[3 * p + l]; /* src/two_e_slater.F90:410 */
            u2[l] = fzv[p] * a2[l] * r2m + G[3 * p + l];
            ut1[(size_t)p * 3 * SUPER + 3 * s + l] = u1[l];
            ut2[(size_t)p * 3 * SUPER + 3 * s + l] = u2[l];
          }
          pair_density_at(b, i, k, u1, &rh1[(size_t)p * SUPER + s], &rg1[(size_t)p * SUPER + s]);
          pair_density_at(b, i, k, u2, &rh2[(size_t)p * SUPER + s], &rg2[(size_t)p * SUPER + s]);
          /* src/compute_jacobian_and_pi0.F90:22-30 */
          double f1 = fjac[p] * r1m, f2 = fjac[p] * r2m;
          j1[(size_t)p * SUPER + s] = 0.25 * fabs(f1 * f1 * f1);
          j2[(size_t)p * SUPER + s] = 0.25 * fabs(f2 * f2 * f2);
        }
      }
      /* accumulation (src/two_e_slater.F90:424-453), chunks of NW walkers */
#pragma omp parallel for schedule(static)
      for (int64_t q = 0; q < nint; q++) {
        int i = is[q] - 1, k = ks[q] - 1, j = js[q] - 1, l = ls[q] - 1;
        int pik = pidx[i + n * k], pjl = pidx[j + n * l];
        const double *U1 = ut1 + (size_t)pik * 3 * SUPER, *U2 = ut2 + (size_t)pjl * 3 * SUPER;
        const double *RS1 = rh1 + (size_t)pik * SUPER, *RS2 = rh2 + (size_t)pjl * SUPER;
        const double *RG1 = rg1 + (size_t)pik * SUPER, *RG2 = rg2 + (size_t)pjl * SUPER;
        const double *J1 = j1 + (size_t)pik * SUPER, *J2 = j2 + (size_t)pjl * SUPER;
        double es = eS[q], eg = eG[q];
        for (int c0 = 0; c0 < ns; c0 += NW) {
          double sw = 0.0, swg = 0.0;
          for (int kw = c0; kw < c0 + NW; kw++) {
            double dx0 = U1[3 * kw] - U2[3 * kw];
            double dx1 = U1[3 * kw + 1] - U2[3 * kw + 1];
            double dx2 = U1[3 * kw + 2] - U2[3 * kw + 2];
            double r12_2 = dx0 * dx0 + dx1 * dx1 + dx2 * dx2;
            double rjacob = J1[kw] * J2[kw];
            double factor, r12_inv;
            if (mode == 0) {
              factor = (double)((float)rjacob / (float)pi0[kw]);
              r12_inv = (double)(1.0f / sqrtf((float)r12_2));
            } else {
              factor = rjacob / pi0[kw];
              r12_inv = 1.0 / sqrt(r12_2);
            }
            double weight = factor * RS1[kw] * RS2[kw];
            double weight_G = factor * RG1[kw] * RG2[kw];
            sw = sw + weight * r12_inv;
            swg = swg + weight_G * r12_inv;
          }
          es = es + sw;
          eg = eg + swg;
        }
        eS[q] = es;
        eG[q] = eg;
      }
    }
    /* block moments (src/two_e_slater.F90:463-481) */
    double factor = 1.0 / (double)npts;
    for (int64_t q = 0; q < nint; q++) {
      double x = eS[q] * factor - eG[q] * factor;
      if (xb) xb[(int64_t)blk * nint + q] = x;
      acc[q] = acc[q] + x;
      acc2[q] = acc2[q] + x * x;
    }
  }
  /* src/two_e_slater.F90:488-492 */
  for (int64_t q = 0; q < nint; q++) {
    double m = acc[q] / nblocks, m2 = acc2[q] / nblocks;
    mean[q] = m;
    err[q] = sqrt(fabs(m2 - m * m)) / sqrt((double)nblocks);
  }
  free(pidx); free(pi_); free(pk_); free(G); free(fzv); free(fjac);
  free(ut1); free(ut2); free(rh1); free(rh2); free(rg1); free(rg2); free(j1); free(j2);
  free(pi0); free(eS); free(eG); free(acc); free(acc2);
  return 0;
}

/* ------------------------------------------------------------------ */
/* shared-walker estimator in FP64                                     */
/* ------------------------------------------------------------------ */
int orc_zvmc_shared(const orc_basis *b, int64_t nint, const int32_t *is, const int32_t *js,
                    const int32_t *ks, const int32_t *ls, const double *u1, const double *u2,
                    const double *w, int nblocks, int64_t npts, int symmetrize, double *mean,
                    double *err, double *xb, int nthreads) {
  init_tables();
  int n = b->n;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
  int *pidx = (int *)malloc(sizeof(int) * n * n);
  for (int t = 0; t < n * n; t++) pidx[t] = -1;
  int np = 0;
  for (int64_t q = 0; q < nint; q++) {
    int i = is[q] - 1, k = ks[q] - 1, j = js[q] - 1, l = ls[q] - 1;
    if (pidx[i + n * k] < 0) pidx[i + n * k] = np++;
    if (pidx[j + n * l] < 0) pidx[j + n * l] = np++;
  }
  int *pi_ = (int *)malloc(sizeof(int) * np), *pk_ = (int *)malloc(sizeof(int) * np);
  for (int k = 0; k < n; k++)
    for (int i = 0; i < n; i++)
      if (pidx[i + n * k] >= 0) { pi_[pidx[i + n * k]] = i; pk_[pidx[i + n * k]] = k; }
  const int CH = 4096;
  size_t ps = (size_t)np * CH;
  double *s1 = (double *)malloc(sizeof(double) * ps), *g1 = (double *)malloc(sizeof(double) * ps);
  double *s2 = (double *)malloc(sizeof(double) * ps), *g2 = (double *)malloc(sizeof(double) * ps);
  double *e = (double *)malloc(sizeof(double) * nint);
  double *acc = (double *)calloc(nint, sizeof(double)), *acc2 = (double *)calloc(nint, sizeof(double));
  for (int blk = 0; blk < nblocks; blk++) {
    for (int64_t q = 0; q < nint; q++) e[q] = 0.0;
    for (int64_t s0 = 0; s0 < npts; s0 += CH) {
      int ns = (int)((npts - s0) < CH ? (npts - s0) : CH);
      int64_t base = (int64_t)blk * npts + s0;
#pragma omp parallel for schedule(dynamic, 1)
      for (int p = 0; p < np; p++)
        for (int s = 0; s < ns; s++) {
          pair_density_at(b, pi_[p], pk_[p], u1 + 3 * (base + s), &s1[(size_t)p * CH + s], &g1[(size_t)p * CH + s]);
          pair_density_at(b, pi_[p], pk_[p], u2 + 3 * (base + s), &s2[(size_t)p * CH + s], &g2[(size_t)p * CH + s]);
        }
#pragma omp parallel for schedule(static)
      for (int64_t q = 0; q < nint; q++) {
        int i = is[q] - 1, k = ks[q] - 1, j = js[q] - 1, l = ls[q] - 1;
        size_t a = (size_t)pidx[i + n * k] * CH, c = (size_t)pidx[j + n * l] * CH;
        double t = 0.0;
        for (int s = 0; s < ns; s++) {
          double x = (s1[a + s] * s2[c + s] - g1[a + s] * g2[c + s]);
          if (symmetrize) x = 0.5 * (x + (s1[c + s] * s2[a + s] - g1[c + s] * g2[a + s]));
          t += x * w[base + s];
        }
        e[q] += t;
      }
    }
    for (int64_t q = 0; q < nint; q++) {
      double x = e[q] / (double)npts;
      if (xb) xb[(int64_t)blk * nint + q] = x;
      acc[q] += x;
      acc2[q] += x * x;
    }
  }
  for (int64_t q = 0; q < nint; q++) {
    double m = acc[q] / nblocks, m2 = acc2[q] / nblocks;
    mean[q] = m;
    err[q] = nblocks > 1 ? sqrt(fabs(m2 - m * m) / (double)(nblocks - 1)) : 0.0;
  }
  free(pidx); free(pi_); free(pk_); free(s1); free(g1); free(s2); free(g2); free(e); free(acc); free(acc2);
  return 0;
}

/* ======================================================================================
 * One-electron integrals of the Gaussian fits (src/one_e_slater.F90:81-89 and one_elect.F90)
 * ====================================================================================== */

/* src/doublefact.F90:1-14 (1 for n <= 2) */
static double doublefact(int n) {
  if (n <= 2) return 1.0;
  double d = 1.0;
  for (int i = n; i >= 1; i -= 2) d = d * (double)i;
  return d;
}

/* src/binom.F90 (i >= 0 branch) */
static double binom_i(int i, int j) { return fact(i) / (fact(j) * fact(i - j)); }

/* src/one_electron_I.F90:1-29 */
static double one_electron_I(int na, double ra, int nb, double rb, double gam, double rp) {
  double rint = 0.0;
  for (int kx = 0; kx <= na; kx++)
    for (int lx = 0; lx <= nb; lx++) {
      int kbig = na + nb - kx - lx;
      if (kbig % 2 == 1) continue;
      kbig = kbig / 2;
      double f3 = doublefact(2 * kbig - 1);
      double f2 = powi(1.0 / (2.0 * gam), kbig);
      rint = rint + f2 * f3 * binom_i(na, kx) * binom_i(nb, lx) * powi(rp - ra, kx) * powi(rp - rb, lx);
    }
  return sqrt(M_PI / gam) * rint;
}

/* src/one_electron_sij.F90:19-54 */
static double one_electron_Sij(const int *na, const double *ra, double gamA, const int *nb, const double *rb,
                               double gamB) {
  double gamtot = gamA + gamB;
  double rmu = gamA * gamB / gamtot;
  double rp[3];
  for (int l = 0; l < 3; l++) rp[l] = (gamA * ra[l] + gamB * rb[l]) / gamtot;
  double x = ra[0] - rb[0], y = ra[1] - rb[1], z = ra[2] - rb[2];
  double AmB = x * x + y * y + z * z;
  double arg = rmu * AmB;
  if (arg > -log(1.e-15)) return 0.0;
  double s = 1.0;
  for (int l = 0; l < 3; l++) s = s * one_electron_I(na[l], ra[l], nb[l], rb[l], gamtot, rp[l]);
  return exp(-arg) * s;
}

/* src/one_electron_Kij.F90:1-46 */
static double one_electron_Kij(const int *na, const double *ra, double gamA, const int *nb, const double *rb,
                               double gamB) {
  int na2[3];
  double sab = one_electron_Sij(na, ra, gamA, nb, rb, gamB);
  double term1 = gamA * (3.0 + 2.0 * (na[0] + na[1] + na[2])) * sab;
  double sab_2 = 0.0;
  for (int l = 0; l < 3; l++) {
    for (int li = 0; li < 3; li++) na2[li] = na[li] + (li == l ? 2 : 0);
    sab_2 = sab_2 + one_electron_Sij(na2, ra, gamA, nb, rb, gamB);
  }
  double term2 = -2.0 * gamA * gamA * sab_2;
  double sab_12 = 0.0;
  for (int l = 0; l < 3; l++) {
    for (int li = 0; li < 3; li++) na2[li] = (li == l && na[li] >= 2) ? na[li] - 2 : na[li];
    sab_12 = sab_12 + na[l] * (na[l] - 1) * one_electron_Sij(na2, ra, gamA, nb, rb, gamB);
  }
  double term3 = -0.5 * sab_12;
  return term1 + term2 + term3;
}

#define NAI_DIM 512

/* src/multiply_poly_2.F90:1-31: d += b * c, degree nd tracked */
static void multiply_poly_2(const double *b, int nb, const double *c, int nc, double *d, int *nd) {
  if (nc == -1 || nb == -1) return;
  int ndtmp = nb + nc;
  for (int ib = 0; ib <= nb; ib++) {
    if (b[ib] == 0.0) continue;
    for (int ic = 0; ic <= nc; ic++) d[ib + ic] = d[ib + ic] + c[ic] * b[ib];
  }
  ndtmp = ndtmp > *nd ? ndtmp : *nd;
  for (; ndtmp >= 0; ndtmp--)
    if (d[ndtmp] != 0.0) break;
  *nd = ndtmp;
}

static void I_x2_pol_mult_mono_elec(int c, const double *R1x, const double *R1xp, const double *R2x, double *d,
                                    int *nd);

/* src/I_x1_pol_mult_mono_elec.F90 (recursive, as the reference) */
static void I_x1_pol_mult_mono_elec(int a, int c, const double *R1x, const double *R1xp, const double *R2x,
                                    double *d, int *nd) {
  double X[NAI_DIM + 1], Y[NAI_DIM + 1];
  int nx, ny;
  if (a == 0 && c == 0) {
    *nd = 0;
    d[0] = 1.0;
    return;
  } else if (c < 0 || *nd < 0) {
    *nd = -1;
    return;
  } else if (a == 0 && c != 0) {
    I_x2_pol_mult_mono_elec(c, R1x, R1xp, R2x, d, nd);
  } else if (a == 1) {
    nx = *nd;
    for (int ix = 0; ix <= NAI_DIM; ix++) X[ix] = Y[ix] = 0.0;
    I_x2_pol_mult_mono_elec(c - 1, R1x, R1xp, R2x, X, &nx);
    for (int ix = 0; ix <= nx; ix++) X[ix] = X[ix] * c;
    multiply_poly_2(X, nx, R2x, 2, d, nd);
    ny = 0;
    I_x2_pol_mult_mono_elec(c, R1x, R1xp, R2x, Y, &ny);
    multiply_poly_2(Y, ny, R1x, 2, d, nd);
  } else {
    for (int ix = 0; ix <= NAI_DIM; ix++) X[ix] = Y[ix] = 0.0;
    nx = 0;
    I_x1_pol_mult_mono_elec(a - 2, c, R1x, R1xp, R2x, X, &nx);
    for (int ix = 0; ix <= nx; ix++) X[ix] = X[ix] * (a - 1);
    multiply_poly_2(X, nx, R2x, 2, d, nd);
    nx = *nd;
    for (int ix = 0; ix <= NAI_DIM; ix++) X[ix] = 0.0;
    I_x1_pol_mult_mono_elec(a - 1, c - 1, R1x, R1xp, R2x, X, &nx);
    for (int ix = 0; ix <= nx; ix++) X[ix] = X[ix] * c;
    multiply_poly_2(X, nx, R2x, 2, d, nd);
    ny = 0;
    I_x1_pol_mult_mono_elec(a - 1, c, R1x, R1xp, R2x, Y, &ny);
    multiply_poly_2(Y, ny, R1x, 2, d, nd);
  }
}

/* src/I_x2_pol_mult_mono_elec.F90 */
static void I_x2_pol_mult_mono_elec(int c, const double *R1x, const double *R1xp, const double *R2x, double *d,
                                    int *nd) {
  double X[NAI_DIM + 1], Y[NAI_DIM + 1];
  int nx, ny;
  if (c == 0) {
    *nd = 0;
    d[0] = 1.0;
    return;
  } else if (*nd < 0 || c < 0) {
    *nd = -1;
    return;
  }
  for (int ix = 0; ix <= NAI_DIM; ix++) X[ix] = Y[ix] = 0.0;
  nx = 0;
  I_x1_pol_mult_mono_elec(0, c - 2, R1x, R1xp, R2x, X, &nx);
  for (int ix = 0; ix <= nx; ix++) X[ix] = X[ix] * (c - 1);
  multiply_poly_2(X, nx, R2x, 2, d, nd);
  ny = 0;
  for (int ix = 0; ix <= NAI_DIM; ix++) Y[ix] = 0.0;
  I_x1_pol_mult_mono_elec(0, c - 1, R1x, R1xp, R2x, Y, &ny);
  if (ny >= 0) multiply_poly_2(Y, ny, R1xp, 2, d, nd);
}

/* src/give_polynom_mult_center_mono_elec.F90: d = Ix * Iy * Iz (polynomial in t) */
static void give_polynom_mult_center_mono_elec(const double *A, const double *B, double alpha, double beta,
                                               const int *pA, const int *pB, const double *C, double *d,
                                               int *n_pt_out) {
  double d1[NAI_DIM + 1], d2[NAI_DIM + 1], d3[NAI_DIM + 1];
  double p = alpha + beta, p_inv = 1.0 / p, p_inv_2 = 0.5 / p, P[3];
  for (int i = 0; i < 3; i++) P[i] = (alpha * A[i] + beta * B[i]) * p_inv;
  double R2x[3] = {p_inv_2, 0.0, -p_inv_2};
  for (int i = 0; i <= NAI_DIM; i++) d[i] = d1[i] = d2[i] = d3[i] = 0.0;
  double *dd[3] = {d1, d2, d3};
  int npt[3];
  for (int ax = 0; ax < 3; ax++) {
    double R1x[3] = {P[ax] - A[ax], 0.0, -(P[ax] - C[ax])};
    double R1xp[3] = {P[ax] - B[ax], 0.0, -(P[ax] - C[ax])};
    npt[ax] = NAI_DIM;
    I_x1_pol_mult_mono_elec(pA[ax], pB[ax], R1x, R1xp, R2x, dd[ax], &npt[ax]);
    if (npt[ax] < 0) {
      *n_pt_out = -1;
      for (int i = 0; i <= NAI_DIM; i++) d[i] = 0.0;
      return;
    }
  }
  int n_pt_tmp = 0;
  multiply_poly_2(d1, npt[0], d2, npt[1], d, &n_pt_tmp);
  for (int i = 0; i <= n_pt_tmp; i++) d1[i] = 0.0;
  int nout = 0;
  multiply_poly_2(d, n_pt_tmp, d3, npt[2], d1, &nout);
  for (int i = 0; i <= nout; i++) d[i] = d1[i];
  *n_pt_out = nout;
}

/* src/NAI_pol_mult.F90:1-60 */
static double NAI_pol_mult(const double *A, const double *B, const int *pA, const int *pB, double alpha,
                           double beta, const double *C) {
  double two_pi = 2.0 * acos(-1.0);
  double p = alpha + beta, p_inv = 1.0 / p, rho = alpha * beta * p_inv, dist = 0.0, dist_integral = 0.0, P[3];
  for (int i = 0; i < 3; i++) {
    P[i] = (alpha * A[i] + beta * B[i]) * p_inv;
    dist = dist + (A[i] - B[i]) * (A[i] - B[i]);
    dist_integral = dist_integral + (P[i] - C[i]) * (P[i] - C[i]);
  }
  double const_factor = dist * rho;
  double cst = p * dist_integral;
  double factor = exp(-const_factor);
  double coeff = two_pi * factor * p_inv;
  int n_pt = 2 * ((pA[0] + pB[0]) + (pA[1] + pB[1]) + (pA[2] + pB[2]));
  if (n_pt == 0) return coeff * orc_rint(0, cst);
  double d[NAI_DIM + 1];
  int n_pt_out;
  give_polynom_mult_center_mono_elec(A, B, alpha, beta, pA, pB, C, d, &n_pt_out);
  if (n_pt_out < 0) return 0.0;
  double accu = 0.0;
  for (int i = 0; i <= n_pt_out; i += 2) {
    if (fabs(d[i]) < 1.e-9) continue;
    accu = accu + d[i] * orc_rint(i / 2, cst);
  }
  return accu * coeff;
}

/* src/one_elect.F90:1-105 for all (i,k); S, V, K column-major n x n (X[i + n*k]);
 * nuclei: xyz[3*kn], charge[kn] (src/one_electron_Vij.F90) */
void orc_one_elect(const orc_basis *b, int nat, const double *xyz, const double *charge, double *S, double *V,
                   double *K) {
  init_tables();
  const int n = b->n;
  for (int i = 0; i < n; i++)
    for (int k = 0; k < n; k++) {
      int orb[2] = {i, k};
      int nc[2], n_c[2][4][3], ct[2][4];
      for (int kk = 0; kk < 2; kk++) nc[kk] = components(b, orb[kk], n_c[kk], ct[kk]);
      const double *A = b->center + 3 * i, *B = b->center + 3 * k;
      double s = 0.0, v = 0.0, kin = 0.0;
      for (int i1 = 0; i1 < b->n_gauss[i]; i1++)
        for (int i2 = 0; i2 < b->n_gauss[k]; i2++)
          for (int ii1 = 0; ii1 < nc[0]; ii1++)
            for (int ii2 = 0; ii2 < nc[1]; ii2++) {
              double dd = CG(b, i1, i, ct[0][ii1]) * CG(b, i2, k, ct[1][ii2]);
              double ga = GG(b, i1, i), gb = GG(b, i2, k);
              s = s + dd * one_electron_Sij(n_c[0][ii1], A, ga, n_c[1][ii2], B, gb);
              double ac = 0.0;
              for (int kn = 0; kn < nat; kn++)
                ac = ac - charge[kn] * NAI_pol_mult(A, B, n_c[0][ii1], n_c[1][ii2], ga, gb, xyz + 3 * kn);
              v = v + dd * ac;
              kin = kin + dd * one_electron_Kij(n_c[0][ii1], A, ga, n_c[1][ii2], B, gb);
            }
      S[i + (int64_t)n * k] = s;
      V[i + (int64_t)n * k] = v;
      K[i + (int64_t)n * k] = kin;
    }
}

/* =====================================================================================
 * Exact one-centre Slater ERIs: the do_exact_monocenter path (src/two_e_slater.F90:318-369)
 * through compute_int_slater (src/compute_int_slater.F90:1-85), ijkl_slater_xnynzn
 * (src/ijkl_slater_xnynzn.F90:1-158), ijkl_slater (src/ijkl_slater.F90:49-103), bigF
 * (src/bigF.F90:1-34), smallg (src/smallg.F90:1-12), compute_lmin_lmax
 * (src/compute_lmin_lmax.F90:1-25), norm_sto (src/norm_sto.F90:1-10).  The Gaunt coefficient
 * (src/gaunt.F90, a third-party routine) is restated from its published definition: the
 * Racah formula of the Wigner 3j symbol.
 * ===================================================================================== */

/* Wigner 3j symbol (j1 j2 j3; m1 m2 m3), Racah's single-sum formula */
static double wigner3j(int j1, int j2, int j3, int m1, int m2, int m3) {
  if (m1 + m2 + m3 != 0) return 0.0;
  if (j3 < abs(j1 - j2) || j3 > j1 + j2) return 0.0;
  if (abs(m1) > j1 || abs(m2) > j2 || abs(m3) > j3) return 0.0;
  const double delta = fact(j1 + j2 - j3) * fact(j1 - j2 + j3) * fact(-j1 + j2 + j3) / fact(j1 + j2 + j3 + 1);
  const double pre = sqrt(delta * fact(j1 + m1) * fact(j1 - m1) * fact(j2 + m2) * fact(j2 - m2) * fact(j3 + m3) *
                          fact(j3 - m3));
  int kmin = 0, kmax = j1 + j2 - j3;
  if (j2 - j3 - m1 > kmin) kmin = j2 - j3 - m1;
  if (j1 - j3 + m2 > kmin) kmin = j1 - j3 + m2;
  if (j1 - m1 < kmax) kmax = j1 - m1;
  if (j2 + m2 < kmax) kmax = j2 + m2;
  double s = 0.0;
  for (int k = kmin; k <= kmax; k++) {
    const double t = 1.0 / (fact(k) * fact(j1 + j2 - j3 - k) * fact(j1 - m1 - k) * fact(j2 + m2 - k) *
                            fact(j3 - j2 + m1 + k) * fact(j3 - j1 - m2 + k));
    s += (k & 1) ? -t : t;
  }
  return (((j1 - j2 - m3) % 2 + 2) % 2 ? -1.0 : 1.0) * pre * s;
}

/* gaunt(l1,l2,l3,m1,m2,m3) = int dOmega Y*_{l1 m1} Y_{l2 m2} Y_{l3 m3}, m1 = m2 + m3
 * (src/gaunt.F90:1-9, the calling convention of the reference) */
static double gaunt(int l1, int l2, int l3, int m1, int m2, int m3) {
  if (m1 - m2 - m3 != 0) return 0.0;
  if ((l1 + l2 + l3) & 1) return 0.0;
  const double c = sqrt((2.0 * l1 + 1.0) * (2.0 * l2 + 1.0) * (2.0 * l3 + 1.0) / (4.0 * acos(-1.0)));
  return ((m1 % 2 + 2) % 2 ? -1.0 : 1.0) * c * wigner3j(l1, l2, l3, 0, 0, 0) * wigner3j(l1, l2, l3, -m1, m2, m3);
}

/* (src/norm_sto.F90:1-10) */
static double norm_sto(double gam, int n) {
  const double g = 2.0 * gam;
  return sqrt(powi(g, 2 * n + 1) / fact(n + n));
}

/* (src/smallg.F90:1-12) */
static double smallg(int n, int m, double g, double gp, int l) {
  double s = 0.0;
  for (int i = 0; i <= n + l; i++)
    s = s + fact(n + l) * fact(n + m - 1 - i) / fact(n + l - i) / powi(g, i + 1) / powi(gp, n + m - i);
  return s;
}

/* (src/bigF.F90:20-34) */
static double bigF(int n12, double g12, int n34, double g34, int l) {
  const int l12 = -l, l34 = l + 1;
  const double g = g12 + g34;
  const double first = fact(n34 + l34 - 1) / powi(g34, n34 + l34) * fact(n12 + l12 - 1) / powi(g12, n12 + l12);
  return first + smallg(n34, n12, g34, g, l12 - 1) - smallg(n34, n12, g34, g, l34 - 1);
}

/* (src/compute_lmin_lmax.F90:1-25) */
static void compute_lmin_lmax(int l1, int l2, int l3, int l4, int m1, int m2, int m3, int m4, int *lmin, int *lmax) {
  *lmax = l1 + l2 < l3 + l4 ? l1 + l2 : l3 + l4;
  const int mx12 = abs(l1 - l2) > abs(m1 - m2) ? abs(l1 - l2) : abs(m1 - m2);
  const int l12min = ((*lmax + mx12) % 2 == 0) ? mx12 : mx12 + 1;
  const int mx34 = abs(l3 - l4) > abs(m3 - m4) ? abs(l3 - l4) : abs(m3 - m4);
  const int l34min = ((*lmax + mx34) % 2 == 0) ? mx34 : mx34 + 1;
  *lmin = l12min > l34min ? l12min : l34min;
}

/* (src/ijkl_slater.F90:49-103) */
static double ijkl_slater(const int *nslat, const int *lslat, const int *mslat, const double *gamma) {
  const int l1 = lslat[0], l2 = lslat[1], l3 = lslat[2], l4 = lslat[3];
  if ((l1 + l2 + l3 + l4) % 2 == 1) return 0.0;
  const int m1 = mslat[0], m2 = mslat[1], m3 = mslat[2], m4 = mslat[3];
  if (m2 - m1 != m3 - m4) return 0.0;
  const int m = m2 - m1;
  const double pi = acos(-1.0);
  double norm = 1.0;
  for (int i = 0; i < 4; i++) norm = norm * norm_sto(gamma[i], nslat[i]);
  int lmin, lmax;
  compute_lmin_lmax(l1, l2, l3, l4, m1, m2, m3, m4, &lmin, &lmax);
  const int n12 = nslat[0] + nslat[1], n34 = nslat[2] + nslat[3];
  const double g12 = gamma[0] + gamma[1], g34 = gamma[2] + gamma[3];
  double s = 0.0;
  for (int l = lmin; l <= lmax; l += 2)
    s = s + gaunt(l2, l, l1, m2, m, m1) * gaunt(l3, l, l4, m3, m, m4) * bigF(n12, g12, n34, g34, l) / (2.0 * l + 1.0);
  return 4.0 * pi * s * norm;
}

/* complex coefficients of x^nx y^ny z^nz / r^(nx+ny+nz) over Y_l^m, nx+ny+nz <= 2
 * (src/ijkl_slater_xnynzn.F90:59-124) */
static void xyz_ylm_coef(double re[3][3][3][3][5], double im[3][3][3][3][5]) {
  memset(re, 0, sizeof(double) * 3 * 3 * 3 * 3 * 5);
  memset(im, 0, sizeof(double) * 3 * 3 * 3 * 3 * 5);
  const double pi = acos(-1.0);
  const double r4 = sqrt(4.0 * pi), r43 = sqrt(4.0 * pi / 3.0), r15 = sqrt(pi / 15.0), s2 = sqrt(2.0),
               s3 = sqrt(3.0);
#define C(nx, ny, nz, l, m) [nx][ny][nz][l][(m) + 2]
  re C(0, 0, 0, 0, 0) = r4;
  re C(1, 0, 0, 1, -1) = r43 / s2;
  re C(1, 0, 0, 1, 1) = -r43 / s2;
  im C(0, 1, 0, 1, -1) = r43 / s2;
  im C(0, 1, 0, 1, 1) = r43 / s2;
  re C(0, 0, 1, 1, 0) = r43;
  im C(1, 1, 0, 2, -2) = r15 * s2;
  im C(1, 1, 0, 2, 2) = -r15 * s2;
  im C(0, 1, 1, 2, -1) = r15 * s2;
  im C(0, 1, 1, 2, 1) = r15 * s2;
  re C(1, 0, 1, 2, -1) = r15 * s2;
  re C(1, 0, 1, 2, 1) = -r15 * s2;
  re C(2, 0, 0, 0, 0) = r4 / 3.0;
  re C(2, 0, 0, 2, -2) = r15 * s2;
  re C(2, 0, 0, 2, 2) = r15 * s2;
  re C(2, 0, 0, 2, 0) = -r15 * 2.0 / s3;
  re C(0, 2, 0, 0, 0) = r4 / 3.0;
  re C(0, 2, 0, 2, -2) = -r15 * s2;
  re C(0, 2, 0, 2, 2) = -r15 * s2;
  re C(0, 2, 0, 2, 0) = -r15 * 2.0 / s3;
  re C(0, 0, 2, 0, 0) = r4 / 3.0;
  re C(0, 0, 2, 2, 0) = r15 * 4.0 / s3;
#undef C
}

/* (src/ijkl_slater_xnynzn.F90:1-158); returns -1 for a function with nx+ny+nz > 2 (the
 * reference stops there) */
int orc_ijkl_slater_xnynzn(const int *nix, const int *niy, const int *niz, const int *power, const double *gamma,
                           double *out) {
  static double cre[3][3][3][3][5], cim[3][3][3][3][5];
  static int have = 0;
  if (!g_init) init_tables();
  for (int k = 0; k < 4; k++)
    if (nix[k] + niy[k] + niz[k] > 2) return -1;
  if (!have) {
#ifdef _OPENMP
#pragma omp critical(orc_xyz_ylm)
#endif
    {
      if (!have) {
        xyz_ylm_coef(cre, cim);
        have = 1;
      }
    }
  }
  int nslat[4], lmax[4];
  for (int k = 0; k < 4; k++) {
    nslat[k] = 1 + nix[k] + niy[k] + niz[k] + power[k];
    lmax[k] = nix[k] + niy[k] + niz[k];
  }
  double rre = 0.0, rim = 0.0;
  for (int l1 = 0; l1 <= lmax[0]; l1++)
    for (int m1 = -l1; m1 <= l1; m1++)
      for (int l2 = 0; l2 <= lmax[1]; l2++)
        for (int m2 = -l2; m2 <= l2; m2++)
          for (int l3 = 0; l3 <= lmax[2]; l3++)
            for (int m3 = -l3; m3 <= l3; m3++)
              for (int l4 = 0; l4 <= lmax[3]; l4++)
                for (int m4 = -l4; m4 <= l4; m4++) {
                  const int ls[4] = {l1, l2, l3, l4};
                  const int ms[4] = {-m1, m2, -m3, m4};
                  const int lm[4][2] = {{l1, m1}, {l2, m2}, {l3, m3}, {l4, m4}};
                  double cr = 1.0, ci = 0.0;
                  for (int t = 0; t < 4; t++) {
                    const double ar = cre[nix[t]][niy[t]][niz[t]][lm[t][0]][lm[t][1] + 2];
                    const double ai = cim[nix[t]][niy[t]][niz[t]][lm[t][0]][lm[t][1] + 2];
                    const double nr = cr * ar - ci * ai, ni = cr * ai + ci * ar;
                    cr = nr;
                    ci = ni;
                  }
                  if (sqrt(cr * cr + ci * ci) > 1.e-20) {
                    const double v = (((m1 + m3) % 2 + 2) % 2 ? -1.0 : 1.0) * ijkl_slater(nslat, ls, ms, gamma);
                    rre = rre + cr * v;
                    rim = rim + ci * v;
                  }
                }
  double norm = 1.0;
  for (int k = 0; k < 4; k++) norm = norm * norm_sto(gamma[k], nslat[k]);
  *out = rre / norm;
  return 0;
}

/* One-centre quartets of the list (all four functions on one centre, src/two_e_slater.F90:
 * 318-327) get compute_int_slater(i,k,j,l) (src/compute_int_slater.F90); mask[q] = 1 for
 * them, 0 (and out[q] untouched) for the others.  Returns the number of one-centre quartets,
 * or -1 if one of them has a function with nx+ny+nz > 2. */
int64_t orc_monocenter(const orc_basis *b, int64_t nint, const int32_t *is, const int32_t *js, const int32_t *ks,
                       const int32_t *ls, double *out, int32_t *mask) {
  int64_t count = 0;
  int bad = 0;
  for (int64_t q = 0; q < nint; q++) {
    const int f[4] = {is[q] - 1, ks[q] - 1, js[q] - 1, ls[q] - 1}; /* (i, k, j, l) */
    int same = 1;
    for (int t = 1; t < 4; t++)
      for (int a = 0; a < 3; a++)
        if (b->center[3 * f[t] + a] != b->center[3 * f[0] + a]) same = 0;
    mask[q] = same;
    if (!same) continue;
    int nx[4], ny[4], nz[4], pw[4];
    double gam[4];
    for (int t = 0; t < 4; t++) {
      nx[t] = b->npower[3 * f[t]];
      ny[t] = b->npower[3 * f[t] + 1];
      nz[t] = b->npower[3 * f[t] + 2];
      pw[t] = b->n_sto[f[t]];
      gam[t] = b->g_slater[f[t]];
    }
    if (orc_ijkl_slater_xnynzn(nx, ny, nz, pw, gam, &out[q])) bad = 1;
    count++;
  }
  return bad ? -1 : count;
}
