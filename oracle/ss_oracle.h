/*
 * ss_oracle.h -- CPU oracle for the two-electron ZV-MC path (TEST INFRASTRUCTURE).
 *
 * This library is the checker, never the product: only tests/, the smoke
 * check and bench.py's CPU-baseline leg may load it.  It restates the
 * reference's algorithms (scemama/slater_stoch, Fortran) in plain C:
 *   - analytic ERIs of the Gaussian fits  (src/gauss_ijkl.F90 and callees)
 *   - Boys-type integrals                 (src/rint_sum.F90, rint1.F90, rint_large_n.F90)
 *   - Schwarz-screened analytic sweep      (src/two_e_slater.F90:219-284)
 *   - faithful ZV-MC estimator             (src/two_e_slater.F90:339-496)
 *   - walker transform                     (src/draw_configuration.F90, src/dierfc.F90)
 *   - shared-walker estimator in FP64 (the exact arithmetic the split-BF16
 *     GEMM path approximates; no reference counterpart, see shared_* below)
 *
 * Parity status: parity unpinned.  The reference ships no tests and no
 * expected outputs and cannot be compiled in this environment (Fortran), so no
 * output of the reference pins the oracle; it is checked against analytic
 * known-answer tests instead (closed-form s-Gaussian ERIs, Boys function
 * against quadrature, the STO 1s self-repulsion 5*pi^2/(8 zeta^5), closed-form
 * one-centre Slater integrals and one-electron integrals).
 *
 * Array layouts follow the reference's Fortran column-major arrays with
 * 0-based indices: center(3,n) -> center[l + 3*i]; npower(3,n) likewise;
 * c_gauss(ld,n,2) -> c_gauss[m + ld*(i + n*t)]; g_gauss(ld,n) -> g_gauss[m + ld*i].
 * Quartet indices is/js/ks/ls are 1-based as in src/build_mapping_ijkl.F90.
 */
#ifndef SS_ORACLE_H
#define SS_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  int n;                   /* nbasis */
  int ld;                  /* leading dimension of c_gauss / g_gauss */
  const double *center;    /* [3*n] bohr */
  const int *npower;       /* [3*n] */
  const int *n_sto;        /* [n] r^n_STO exp(-zeta r) */
  const int *i_type;       /* [n] 1: c exp(-g r^2); 2: c r^2 exp(-g r^2) */
  const int *n_gauss;      /* [n] */
  const double *c_gauss;   /* [ld*n*2] */
  const double *g_gauss;   /* [ld*n] */
  const double *g_slater;  /* [n] zeta */
} orc_basis;

/* Boys-type sum  sum_i d1(2i) F_i(rho)   (src/rint_sum.F90:1-68) */
double orc_rint_sum(int n_pt_out, double rho, const double *d1);
/* single F_n(rho) as the reference's rint() (src/rint.F90:1-63) */
double orc_rint(int n, double rho);

/* one primitive ERI (src/bielec_integral.F90:1-55) */
double orc_bielec_integral(double alpha, double beta, double delta, double gama,
                           const double *A, const double *B, const double *C, const double *D,
                           const int *pA, const int *pB, const int *pC, const int *pD);

/* accumulation of gauss_ijkl: 0 = sequential FP64 as the reference, 1 = long double */
void orc_set_sum_mode(int mode);

/* (ik|jl) of the Gaussian fits; 0-based function indices (src/gauss_ijkl.F90:51-154) */
double orc_gauss_ijkl(const orc_basis *b, int i, int k, int j, int l);

/* Schwarz diagonal precond[i + n*k] = (ik|ik)  (src/two_e_slater.F90:230-236) */
void orc_precond(const orc_basis *b, double *precond, int nthreads);

/* analytic sweep over quartets with the reference's screening
 * (src/two_e_slater.F90:264-279); returns number of Schwarz-removed quartets */
int64_t orc_gauss_eri(const orc_basis *b, int64_t nint, const int32_t *is, const int32_t *js,
                      const int32_t *ks, const int32_t *ls, const double *precond,
                      double *out, int nthreads);
void orc_gauss_list(const orc_basis *b, int64_t nint, const int32_t *is, const int32_t *js,
                    const int32_t *ks, const int32_t *ls, double *out, int nthreads);
void orc_gauss_list_timed(const orc_basis *b, int64_t nint, const int32_t *is, const int32_t *js,
                          const int32_t *ks, const int32_t *ls, double *out, double *seconds, int nthreads);

/* primitive-quartet count of the sweep (sum over quartets of prod n_gauss*nc) */
double orc_count_primitive_quartets(const orc_basis *b, int64_t nint, const int32_t *is,
                                    const int32_t *js, const int32_t *ks, const int32_t *ls);

/* inverse erfc (src/dierfc.F90:3-68) */
double orc_dierfc(double y);

/* Faithful ZV-MC estimator on caller-supplied walkers.
 * r1, r2: [3*S] walker-major (r[3*s + l]); S = nblocks * npts.
 * mode 0 = "ref32" (src/two_e_slater.F90:442,446 single-precision casts),
 * mode 1 = "fp64"  (the double-precision lines 443,447).
 * Outputs per quartet: mean (src/two_e_slater.F90:488-492), err (block sigma),
 * and optionally block values xb[b*nint + q] (may be NULL). */
int orc_zvmc_faithful(const orc_basis *b, int64_t nint, const int32_t *is, const int32_t *js,
                      const int32_t *ks, const int32_t *ls, double a_zv,
                      const double *r1, const double *r2, int nblocks, int64_t npts, int mode,
                      double *mean, double *err, double *xb, int nthreads);

/* Shared-walker estimator in FP64 (no reference counterpart; the exact sum the
 * split-BF16 GEMM approximates).  u1, u2: [3*S] sample points; w: [S] weights
 * 1/(|u1-u2| pi(u1) pi(u2)).  Block b covers samples [b*npts, (b+1)*npts).
 * x_b(ik|jl) = (1/npts) sum_s (rhoS_ik(u1) rhoS_jl(u2) - rhoG_ik(u1) rhoG_jl(u2)) w_s,
 * symmetrised with the (jl|ik) electron swap when symmetrize != 0. */
int orc_zvmc_shared(const orc_basis *b, int64_t nint, const int32_t *is, const int32_t *js,
                    const int32_t *ks, const int32_t *ls, const double *u1, const double *u2,
                    const double *w, int nblocks, int64_t npts, int symmetrize,
                    double *mean, double *err, double *xb, int nthreads);

/* pair densities at points (src/compute_densities.F90:17-91), used by tests:
 * rhoS[p*S + s], rhoG[p*S + s] for pairs (ip[p], kp[p]) (0-based) at points u[3*s+l] */
void orc_pair_densities(const orc_basis *b, int npairs, const int *ip, const int *kp,
                        int64_t S, const double *u, double *rhoS, double *rhoG);

/* One-electron integrals of the Gaussian fits for every (i,k) (src/one_elect.F90, with
 * one_electron_sij.F90, one_electron_Kij.F90, one_electron_Vij.F90, NAI_pol_mult.F90):
 * overlap S, nuclear attraction V (nuclei xyz[3*nat] bohr, charge[nat]) and kinetic K,
 * column-major n x n (X[i + n*k]). */
/* Exact one-centre Slater ERI of x^nix y^niy z^niz r^power e^(-gamma r) functions in the
 * order (1 2 | 3 4) (src/ijkl_slater_xnynzn.F90); -1 if a function has nix+niy+niz > 2. */
int orc_ijkl_slater_xnynzn(const int *nix, const int *niy, const int *niz, const int *power,
                           const double *gamma, double *out);

/* Exact values of the one-centre quartets of the list (src/two_e_slater.F90:318-369); mask[q]
 * = 1 for them.  Returns their number, -1 if one has a function beyond d. */
int64_t orc_monocenter(const orc_basis *b, int64_t nint, const int32_t *is, const int32_t *js,
                       const int32_t *ks, const int32_t *ls, double *out, int32_t *mask);

void orc_one_elect(const orc_basis *b, int nat, const double *xyz, const double *charge, double *S, double *V,
                   double *K);

#ifdef __cplusplus
}
#endif
#endif
