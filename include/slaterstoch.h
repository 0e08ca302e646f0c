/*
 * slaterstoch.h -- C ABI of libslaterstoch.so, the GB300 (sm_103a) implementation of the
 * two-electron path of scemama/slater_stoch: analytic ERIs of each STO's Gaussian fit,
 * the zero-variance Monte Carlo (ZV-MC) STO-minus-fit correction, and the PSD cleanup.
 *
 * Conventions (match the reference's Fortran data so a driver can pass its arrays as is):
 *  - arrays are column-major Fortran arrays: center(3,n), npower(3,n), c_gauss(ld,n,2),
 *    g_gauss(ld,n); quartet indices is/js/ks/ls are 1-based and (is,ks) is electron 1,
 *    (js,ls) electron 2, i.e. the value is (ik|jl) = <ij|kl> (src/build_mapping_ijkl.F90:24-43);
 *  - host arrays are caller-owned and read/written before the call returns;
 *  - every call returns 0 (SS_OK) or a negative SS_ERR_* code and never exits the process
 *    (the reference's `stop` statements become error codes); ss_last_error() gives a message;
 *  - one ss_ctx per host thread; a context owns all device memory it allocates.
 */
#ifndef SLATERSTOCH_H
#define SLATERSTOCH_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SS_OK 0
#define SS_ERR_ARG (-1)        /* invalid argument (sizes, indices, npts not a multiple of 40) */
#define SS_ERR_STATE (-2)      /* call out of order (e.g. no basis set) */
#define SS_ERR_CUDA (-3)       /* a CUDA runtime call failed */
#define SS_ERR_NOMEM (-4)      /* device allocation failed or exceeds the context's HBM budget */
#define SS_ERR_UNSUPPORTED (-5) /* input outside the kernels' limits (angular momentum, i_type 3) */
#define SS_ERR_TIMEOUT (-6)    /* a bounded device wait gave up */
#define SS_ERR_NUMERIC (-7)    /* non-finite result detected (e.g. Taylor series did not converge) */

#define SS_EST_FAITHFUL 0      /* per-pair ZV map, src/two_e_slater.F90:401-454 */
#define SS_EST_SHARED 1        /* one walker set for all pairs (tensor-core contraction) */
#define SS_JOB_MC_ONLY 256     /* or'ed into a job's estimator: the job returns the MC correction
                                  (mean) and its error bar instead of the merged ERIs */

#define SS_PREC_FP64 0         /* FP64 arithmetic (src/two_e_slater.F90:443,447 variant) */
#define SS_PREC_REF32 1        /* the reference's FP32 casts of weight and 1/r12 (:442,:446) */
#define SS_PREC_SPLIT_BF16 2   /* shared estimator: BF16 hi+lo, 3 products, FP32 accumulate */

#define SS_LAYOUT_REF_N2 0     /* svd_clean's n^2 x n^2 <ij|kl> matrix (src/svd_clean.F90:97-130) */
#define SS_LAYOUT_PACKED_PAIR 1 /* packed Coulomb metric M[(ik),(jl)] = (ik|jl) */

typedef struct ss_ctx ss_ctx;

/* Create a context on CUDA device `device`; hbm_budget bytes caps its device allocations
 * (0 = no cap).  Returns NULL on failure (see ss_last_error()). */
ss_ctx* ss_create(int device, size_t hbm_budget);
void ss_destroy(ss_ctx* ctx);
const char* ss_strerror(int code);
const char* ss_last_error(void);
/* number of kernels this context has launched (diagnostics) */
int64_t ss_launch_count(const ss_ctx* ctx);

/* Replaces the basis arrays of module common_data (src/common_data.F90:37-52) as built by
 * build_gaussian_expansion_of_orbitals (src/build_gaussian_expansion_of_orbitals.F90:1-473).
 * center(3,n) bohr; npower(3,n); n_sto(n); i_type(n) in {1,2}; n_gauss(n) <= ld;
 * c_gauss(ld,n,2); g_gauss(ld,n); g_slater(n) = zeta. */
int ss_basis_set(ss_ctx* ctx, int nbasis, const double* center, const int* npower,
                 const int* n_sto, const int* i_type, const int* n_gauss, const double* c_gauss,
                 int ld, const double* g_gauss, const double* g_slater);

/* No counterpart in the reference (it runs one system per process).  Declares that the basis set
 * by ss_basis_set holds nsys independent systems, system s being functions first[s] ..
 * first[s+1]-1 (1-based; first[0] = 1, first[nsys] = nbasis + 1): primitive pairs of functions
 * of two systems are never formed, so a quartet list that concatenates the systems' own quartets
 * is evaluated by ss_gauss_eri with one launch per kernel class for all of them.  The ZV-MC
 * entry points need a single system (SS_ERR_STATE otherwise): run each system's MC as its own
 * job (SS_JOB_MC_ONLY).  ss_basis_set resets the context to one system. */
int ss_basis_systems(ss_ctx* ctx, int nsys, const int* first);

/* Replaces is/js/ks/ls of common_data built by build_mapping_ijkl (src/build_mapping_ijkl.F90). */
int ss_quartets_set(ss_ctx* ctx, int64_t nint, const int32_t* is, const int32_t* js,
                    const int32_t* ks, const int32_t* ls);

/* Schwarz diagonal precond(i,k) = (ik|ik), n x n column-major, i >= k filled and mirrored
 * (replaces src/two_e_slater.F90:230-239). */
int ss_precond(ss_ctx* ctx, double* precond);

/* Analytic (ik|jl) of the Gaussian fits for every quartet, with the reference's Schwarz
 * screening and diagonal reuse (replaces the gauss_ijkl loop, src/two_e_slater.F90:264-284,
 * and gauss_ijkl itself, src/gauss_ijkl.F90:51).  out may be NULL (result kept on device);
 * n_removed (may be NULL) receives the Schwarz-removed count (:253-262). */
int ss_gauss_eri(ss_ctx* ctx, double* out, int64_t* n_removed);

/* ZV-MC correction <ij|kl>_STO - <ij|kl>_fit (replaces src/two_e_slater.F90:386-496).
 * Walkers come from a counter-based Philox4x32-10 stream keyed by `seed`.
 * estimator: SS_EST_FAITHFUL (precision FP64 or REF32) or SS_EST_SHARED (FP64 or SPLIT_BF16).
 * nblocks blocks of samples_per_block samples (faithful: a multiple of 40, src/two_e_slater.F90:148).
 * sigma_target > 0 stops after the first block boundary where max sigma <= target (needs >= 2
 * blocks done).  mean/sigma: nint each (may be NULL; kept on device). */
int ss_zvmc(ss_ctx* ctx, double a_zv, uint64_t seed, int64_t samples_per_block, int nblocks,
            int estimator, int precision, double sigma_target, double* mean, double* sigma);

/* Faithful estimator on caller-supplied walkers (the parity hook): r1, r2 are (3,S) walker-major
 * standard normals, S = nblocks*npts, as drawn by draw_configuration (src/draw_configuration.F90). */
int ss_zvmc_walkers(ss_ctx* ctx, double a_zv, const double* r1, const double* r2, int64_t npts,
                    int nblocks, int precision, double* mean, double* sigma);

/* The walkers the faithful estimator draws for (seed, first sample, S): r1, r2 (3,S). */
int ss_draw_walkers(ss_ctx* ctx, uint64_t seed, int64_t first, int64_t S, double* r1, double* r2);

/* Shared-walker estimator: the sample points u1, u2 (3,S) and weights w (S) it draws for
 * (seed, first sample), so a checker can recompute the estimator in FP64. */
int ss_shared_samples(ss_ctx* ctx, double a_zv, uint64_t seed, int64_t first, int64_t S,
                      double* u1, double* u2, double* w);

/* Final ERIs = analytic + MC mean (src/two_e_slater.F90:558-564); out nint. */
int ss_combine(ss_ctx* ctx, double* out);

/* The whole two-electron job of the reference driver on the resident basis and quartets
 * (src/two_e_slater.F90:219-564: Schwarz diagonal, analytic ERIs, ZV-MC blocks, merge),
 * recomputed from scratch.  Results stay on the device; fetch them with ss_combine /
 * ss_gauss_eri / the mean/sigma of a later ss_zvmc call.  eri/sigma (nint, may be NULL)
 * receive the merged integrals and their MC error. */
int ss_two_e_job(ss_ctx* ctx, double a_zv, uint64_t seed, int64_t samples_per_block, int nblocks,
                 int estimator, int precision, double sigma_target, double* eri, double* sigma);

/* Nuclei for the one-electron nuclear attraction: xyz (3,nat) bohr, charge (nat), as the
 * reference's centers_nuclei / charge (src/read_geometry.F90, src/common_data.F90). */
int ss_nuclei_set(ss_ctx* ctx, int nat, const double* xyz, const double* charge);

/* One-electron integrals of the Gaussian fits of the resident basis (the reference's
 * one_e_slater loop, src/one_e_slater.F90:81-89 over src/one_elect.F90): overlap S, nuclear
 * attraction V and kinetic K, each n x n column-major (S(i,k) = S[i + n*k]); any may be NULL. */
int ss_one_e(ss_ctx* ctx, double* S, double* V, double* K);

/* The reference's bielec_ao text output (src/two_e_slater.F90:603-613,
 * '(4(I5,X),2D22.15)' i,j,k,l, ERI, MC error): ss_write_bielec_ao writes the context's merged
 * ERIs and MC errors of the last job, streamed from the device in chunks;
 * ss_write_bielec_ao_arrays writes caller arrays (sigma may be NULL: written as 0). */
int ss_write_bielec_ao(ss_ctx* ctx, const char* path);
int ss_write_bielec_ao_arrays(const char* path, int64_t nint, const int32_t* is, const int32_t* js,
                              const int32_t* ks, const int32_t* ls, const double* eri, const double* sigma);
/* One matrix of ss_one_e (n x n column-major, [i,k]) in one_e_slater's text format
 * (src/one_e_slater.F90:125-135: '(2(I5,X),D22.15)' i,k,M(i,k), i outer): the files
 * overlap_ao_ex, nuclear_ao_ex and kinetic_ao_ex of the reference. */
int ss_write_one_e_matrix(const char* path, int n, const double* m);

/* Asynchronous job API (the reference runs one job per process and has none; these queue the
 * job of ss_two_e_job for a serving caller).  ss_job_submit copies the context's basis and
 * quartets and returns at once; the job runs on a worker thread with a private worker context
 * on the same device, so several jobs overlap on the GPU and later calls on ctx do not affect
 * them.  Worker contexts are kept by ctx and reused by later jobs (their device buffers only
 * grow).  A job with sigma_target > 0 stops at the first block boundary (after two blocks)
 * where its largest error bar is at or below the target.  ss_job_poll sets *done = 1 once the
 * job finished; ss_job_result waits for it, copies its eri and sigma (nint each, may be NULL)
 * and forgets the job, returning the job's status code.  ss_destroy waits for unfinished jobs,
 * drops their results and releases the worker contexts. */
int ss_job_submit(ss_ctx* ctx, double a_zv, uint64_t seed, int64_t samples_per_block, int nblocks,
                  int estimator, int precision, double sigma_target, int64_t* job_id);
/* The same for a job whose inputs are passed directly (ss_basis_set's and ss_quartets_set's
 * arrays and meanings): a serving caller submits each request's system without touching the
 * context's own basis.  The arrays are copied before the call returns; errors in them are
 * reported by the job (ss_job_result). */
int ss_job_submit_inputs(ss_ctx* ctx, int nbasis, const double* center, const int* npower,
                         const int* n_sto, const int* i_type, const int* n_gauss,
                         const double* c_gauss, int ld, const double* g_gauss,
                         const double* g_slater, int64_t nint, const int32_t* is,
                         const int32_t* js, const int32_t* ks, const int32_t* ls, double a_zv,
                         uint64_t seed, int64_t samples_per_block, int nblocks, int estimator,
                         int precision, double sigma_target, int64_t* job_id);
int ss_job_poll(ss_ctx* ctx, int64_t job_id, int* done);
/* Of a finished job (before ss_job_result): seconds it waited for admission, seconds it ran,
 * MC blocks it used and its largest error bar (any pointer may be NULL); SS_ERR_STATE while
 * it runs. */
int ss_job_info(ss_ctx* ctx, int64_t job_id, double* wait_s, double* run_s, int* blocks,
                double* max_sigma);
int ss_job_result(ss_ctx* ctx, int64_t job_id, double* eri, double* sigma);

/* Admission of the asynchronous jobs of this context: a job starts in submission order once
 * fewer than max_running jobs run (0 = no limit) and its ERI-buffer footprint,
 * ss_job_footprint(nint), fits in what the running jobs leave of eri_budget_bytes (0 = no
 * limit); a job starts regardless when no other job runs.  ss_job_submit refuses a job whose
 * footprint alone exceeds the budget (SS_ERR_NOMEM). */
int ss_job_limits(ss_ctx* ctx, size_t eri_budget_bytes, int max_running);
/* running / queued jobs now, the most that ran at once and their largest summed footprint */
int ss_job_stats(ss_ctx* ctx, int* running, int* queued, int* peak_running, size_t* peak_bytes);
/* device bytes per job that grow with its quartet count (96 per quartet) */
size_t ss_job_footprint(int64_t nint);

/* Drop cached device results (Schwarz diagonal, analytic ERIs, MC sums); inputs stay. */
int ss_invalidate(ss_ctx* ctx);

/* Exact one-centre Slater ERIs (the do_exact_monocenter path, src/two_e_slater.F90:318-369,
 * through compute_int_slater, src/compute_int_slater.F90): for every quartet of the list whose
 * four functions share one centre (identical coordinates), out[q] = the exact ERI of the STOs
 * themselves (src/ijkl_slater_xnynzn.F90) and mask[q] = 1; other quartets get 0 and 0.
 * out/mask (nint) may be NULL; n_mono receives the number of one-centre quartets.
 * SS_ERR_UNSUPPORTED if a one-centre quartet has a function beyond d (nx+ny+nz > 2), where the
 * reference stops. */
int ss_monocenter(ss_ctx* ctx, double* out, int32_t* mask, int64_t* n_mono);

/* No counterpart in the reference (it evaluates every primitive quartet in FP64).  Thresholds of
 * the analytic stage, relative to a quartet's Schwarz bound sqrt((ik|ik)(jl|jl)): a primitive
 * quartet whose Schwarz bound S_P S_Q is below screen_eps times it is skipped, one below
 * fp32_eps times it is evaluated in FP32, the rest in FP64.  Defaults 1e-18 and 1e-11;
 * fp32_eps <= screen_eps (e.g. 0) evaluates every kept primitive quartet in FP64.  Limits:
 * 0 <= screen_eps <= 1e-18, 0 <= fp32_eps <= 1e-10 (else SS_ERR_ARG).  A change invalidates the
 * analytic ERIs held by the context; jobs submitted afterwards use the new values. */
int ss_set_eri_tiers(ss_ctx* ctx, double screen_eps, double fp32_eps);

/* enable != 0: ss_combine, ss_two_e_job and the jobs give the one-centre quartets their exact
 * value with MC mean and error bar 0 (src/two_e_slater.F90:465-494, 558-562). */
int ss_set_exact_monocenter(ss_ctx* ctx, int enable);

/* Largest MC error of the last ZV-MC run, and the number of blocks it used. */
double ss_mc_max_sigma(const ss_ctx* ctx);
int ss_mc_blocks_done(const ss_ctx* ctx);

/* The context's CUDA stream (cudaStream_t, created with the device's greatest stream priority).
 * Every call's work is ordered on it: the internal side streams (the analytic ERI classes, and in
 * ss_two_e_job the whole analytic stage running beside the MC, at the lowest priority) fork from
 * it and join back into it before the call returns. */
void* ss_stream(ss_ctx* ctx);

/* The shared estimator's tensor-core contraction on caller data (no reference counterpart;
 * it replaces the quartet loop of src/two_e_slater.F90:424-453 for the shared estimator):
 * C(P,P) = A_hi B_hi^T + A_hi B_lo^T + A_lo B_hi^T with A*, B* (P,K) row-major BF16 bit
 * patterns, K a positive multiple of 64, C row-major FP32, FP32 accumulation per K slice of
 * ksplit (0 = automatic) summed in FP64. */
int ss_split_bf16_gemm(ss_ctx* ctx, int P, int64_t K, const uint16_t* a_hi, const uint16_t* a_lo,
                       const uint16_t* b_hi, const uint16_t* b_lo, int ksplit, float* c);

/* No counterpart in the reference.  The same contraction for callers that cannot allocate
 * device memory (their device memory belongs to their own pool, or cudaMalloc is not allowed
 * where they run): it allocates nothing and needs no ss_ctx.  All pointers are DEVICE pointers
 * owned by the caller (A*, B* (P,K) BF16 bits, C (P,P) FP32); stream is a cudaStream_t (NULL =
 * default stream).  The call waits for the stream (cudaStreamSynchronize) to read back the
 * error flag of the bounded device waits, so it returns after the stream has finished the work.
 * The K-slice partials go to a fixed 16 MiB device array inside the library, so P <= 2048
 * (larger P is rejected with SS_ERR_ARG) and ksplit is reduced to fit.  The first call on a
 * device looks up that array's device address (cudaGetSymbolAddress) and keeps it; make that
 * first call before any stream capture.  A device reset (cudaDeviceReset) after that first call
 * is not supported: the kept address would be stale.  All calls share the array: calls that
 * overlap on the GPU (other threads, other streams) race and must be serialised. */
int ss_split_bf16_gemm_noalloc(void* stream, int P, int64_t K, const uint16_t* a_hi,
                               const uint16_t* a_lo, const uint16_t* b_hi, const uint16_t* b_lo,
                               int ksplit, float* c);

/* PSD cleanup by randomized SVD deflation (replaces svd_clean, src/svd_clean.F90:1-426).
 * moy (nint) in/out; rank, q as in src/two_e_slater.F90:565-567 (oversample added to rank);
 * seed drives the Gaussian test matrices.  n_removed receives the removed negative components. */
int ss_psd_clean(ss_ctx* ctx, double* moy, int layout, int rank, int oversample, int q,
                 uint64_t seed, int* n_removed);

/* Exact removal of the negative eigencomponents of the ERI matrix in `layout` (replaces the
 * nbasis < 200 path of davidson_clean, src/davidson_clean.F90:30-116): full FP64
 * eigen-decomposition on the device, W -= sum_{lambda<0} lambda v v^T, canonical entries read
 * back into moy.  Matrix dimension <= 1024.  n_removed receives the removed count. */
int ss_psd_project(ss_ctx* ctx, double* moy, int layout, int* n_removed);

/* Lowest m eigenpairs of the ERI matrix in `layout` by Davidson with FP64 Rayleigh-Ritz
 * (follows src/davidson.F90:1-158).  evals (m), evecs (N x m column-major) may be NULL. */
int ss_davidson(ss_ctx* ctx, const double* moy, int layout, int m, double tol, int max_iter,
                double* evals, double* evecs);

/* Matrix-free removal of the negative eigencomponents (replaces the nbasis >= 200 path of
 * davidson_clean, src/davidson_clean.F90:120-323): the ERI matrix in `layout` is applied from
 * the unique quartet values only (never formed); block Davidson for the lowest `block` Ritz
 * pairs (<= 128; 0 = min(nbasis, 128), the reference's mmax) in a basis of at most block x max_blocks
 * vectors (0 = nbasis, the reference's NMAX; capped at the matrix dimension and 1024); each
 * search ends when the Ritz pairs up to index block/2 and all negative ones have residual
 * norm < tol (or the basis spans the whole space); its negative pairs are deflated,
 * moy -= E u(ii) u(jj), until a search finds none.
 * moy (nint) in/out; n_removed receives the deflated count.  max_iter bounds the Davidson
 * iterations over all searches. */
int ss_davidson_clean(ss_ctx* ctx, double* moy, int layout, int block, int max_blocks, double tol,
                      int max_iter, int* n_removed);

#ifdef __cplusplus
}
#endif
#endif
