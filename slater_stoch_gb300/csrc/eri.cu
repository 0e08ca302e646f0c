// eri.cu -- analytic FP64 ERIs of the STO Gaussian fits on sm_103a.
//
// Replaces gauss_ijkl (src/gauss_ijkl.F90:51-154) and its callees
// bielec_integral / give_explicit_poly_and_gaussian / general_primitive_integral /
// give_polynom_mult_center_x / I_x1_pol_mult* / I_x2_pol_mult / rint_sum.
//
// Design (GB300 FP64 is ~1/64 of the FP32 rate, so FP64 instruction count is the roofline):
//  * primitive pairs are precomputed once per function pair (Gaussian product, K_AB screening
//    of src/gaussian_product.F90:25-28 and src/give_explicit_poly_and_gaussian.F90:46-49; a
//    screened pair contributes exactly 0 in the reference and is simply not stored);
//  * one CTA per (function quartet, slice of bra primitive pairs); the ket primitive pairs of
//    the quartet are staged in shared memory and read as broadcasts;
//  * per primitive quartet the Boys values F_n(T) and the recursion coefficients are computed
//    once and shared by all cartesian components of the r^2-type fits (the reference recomputes
//    them for each of the up to 81 component combinations);
//  * the recursive polynomial routines I_x1_pol_mult / I_x2_pol_mult become a bottom-up table
//    I(a,c)(u), u = t^2, per axis, with the same per-coefficient operation order:
//      I(0,c) = (c-1) B01 I(0,c-2) + D00 I(0,c-1)
//      I(a,c) = (a-1) B10 I(a-2,c) + c B00 I(a-1,c-1) + C00 I(a-1,c)
//  * the thresholds of general_primitive_integral (|P_new| and |P_new Q_new| vs 1e-15,
//    src/general_primitive_integral.F90:71,75,96,100,122,126) are applied at the same places;
//  * partial sums go to a scratch buffer [quartet][slice] reduced in a fixed order, so results
//    are run-to-run deterministic.
#include <math.h>

#include "ss_common.cuh"


namespace ss {

constexpr double THRESH = 1.e-15;

// Functions i and k on the same centre with the same fit (exponents, coefficients, fit type)
// give bit-identical primitive-pair records for (m1, m2) and (m2, m1): the same Gaussian
// product (a A + b A = b A + a A), centre offsets and coefficient product, and the polynomial
// (x - A)^(a_i + a_k) does not depend on which exponent goes with which function.  This holds
// for i = k and for the cartesian components of one shell (px/py/pz, the six d's).
__device__ bool fold_pair(const BasisDev& B, int i, int k) {
  if (i == k) return true;
  const int ng = B.n_gauss[i];
  if (ng != B.n_gauss[k] || B.i_type[i] != B.i_type[k]) return false;
  for (int ax = 0; ax < 3; ax++)
    if (B.center[3 * i + ax] != B.center[3 * k + ax]) return false;
  const int64_t t = B.i_type[i] == 2 ? 1 : 0;
  for (int m = 0; m < ng; m++) {
    if (B.g_gauss[m + (int64_t)B.ld * i] != B.g_gauss[m + (int64_t)B.ld * k]) return false;
    if (B.c_gauss[m + (int64_t)B.ld * (i + B.n * t)] != B.c_gauss[m + (int64_t)B.ld * (k + B.n * t)]) return false;
  }
  return true;
}

__global__ void prim_pair_count(BasisDev B, int npairs, int* __restrict__ cnt) {
  int pidx = blockIdx.x;
  if (pidx >= npairs) return;
  int i = (int)((sqrt(8.0 * pidx + 1.0) - 1.0) * 0.5);
  while ((int64_t)i * (i + 1) / 2 > pidx) i--;
  while ((int64_t)(i + 1) * (i + 2) / 2 <= pidx) i++;
  int k = pidx - i * (i + 1) / 2;
  __shared__ int s_c;
  if (threadIdx.x == 0) s_c = 0;
  __syncthreads();
  const int ngi = B.n_gauss[i], ngk = B.n_gauss[k];
  const double* A = B.center + 3 * i;
  const double* Bc = B.center + 3 * k;
  const bool fold = fold_pair(B, i, k);
  const bool other_system = B.sys && B.sys[i] != B.sys[k];
  int local = 0;
  for (int t = threadIdx.x; t < (other_system ? 0 : ngi * ngk); t += blockDim.x) {
    int m1 = t / ngk, m2 = t % ngk;
    if (fold && m2 < m1) continue;  // folded into (m2, m1), see prim_pair_fill
    double a = B.g_gauss[m1 + (int64_t)B.ld * i], b = B.g_gauss[m2 + (int64_t)B.ld * k];
    double p_inv = 1.0 / (a + b);
    double ab = a * b;
    double x0 = A[0] - Bc[0], x1 = A[1] - Bc[1], x2 = A[2] - Bc[2];
    ab = ab * p_inv;
    double kk = ab * (x0 * x0 + x1 * x1 + x2 * x2);
    if (kk > 40.0) continue;
    if (exp(-kk) < THRESH) continue;
    local++;
  }
  atomicAdd(&s_c, local);
  __syncthreads();
  if (threadIdx.x == 0) cnt[pidx] = s_c;
}

__global__ void prim_pair_fill(BasisDev B, int npairs, const int64_t* __restrict__ off,
                               PrimPair* __restrict__ out) {
  int pidx = blockIdx.x;
  if (pidx >= npairs) return;
  int i = (int)((sqrt(8.0 * pidx + 1.0) - 1.0) * 0.5);
  while ((int64_t)i * (i + 1) / 2 > pidx) i--;
  while ((int64_t)(i + 1) * (i + 2) / 2 <= pidx) i++;
  int k = pidx - i * (i + 1) / 2;
  const int ngi = B.n_gauss[i], ngk = B.n_gauss[k];
  const double* A = B.center + 3 * i;
  const double* Bc = B.center + 3 * k;
  const int ti = B.i_type[i] == 2 ? 1 : 0, tk = B.i_type[k] == 2 ? 1 : 0;
  // sequential compaction in (m1, m2) order by thread 0 (ng <= 30: at most 900 entries).
  // For a folded pair (fold_pair) only m1 <= m2 is kept, with the coefficient doubled for
  // m1 < m2 (exact), which halves the primitive pairs of those function pairs.
  if (threadIdx.x != 0) return;
  if (B.sys && B.sys[i] != B.sys[k]) return;  // functions of two systems: no pairs
  const bool fold = fold_pair(B, i, k);
  int64_t o = off[pidx];
  for (int m1 = 0; m1 < ngi; m1++)
    for (int m2 = (fold ? m1 : 0); m2 < ngk; m2++) {
      double a = B.g_gauss[m1 + (int64_t)B.ld * i], b = B.g_gauss[m2 + (int64_t)B.ld * k];
      // src/gaussian_product.F90:17-32
      double p = a + b;
      double p_inv = 1.0 / (a + b);
      double ab = a * b;
      double x0 = A[0] - Bc[0], x1 = A[1] - Bc[1], x2 = A[2] - Bc[2];
      ab = ab * p_inv;
      double kk = ab * (x0 * x0 + x1 * x1 + x2 * x2);
      if (kk > 40.0) continue;
      double K = exp(-kk);
      if (K < THRESH) continue;  // src/give_explicit_poly_and_gaussian.F90:46-49
      PrimPair r;
      r.p = p;
      r.p_inv = 1.0 / p;  // bielec_integral's p_inv = 1.d0/pp (src/bielec_integral.F90:45)
      r.fact = K;
#pragma unroll
      for (int ax = 0; ax < 3; ax++) {
        r.P[ax] = (a * A[ax] + b * Bc[ax]) * p_inv;
        r.PA[ax] = r.P[ax] - A[ax];
        r.PB[ax] = r.P[ax] - Bc[ax];
      }
      r.coef = B.c_gauss[m1 + (int64_t)B.ld * (i + (int64_t)B.n * ti)] *
               B.c_gauss[m2 + (int64_t)B.ld * (k + (int64_t)B.n * tk)];
      if (fold && m1 != m2) r.coef = 2.0 * r.coef;
      r.pad[0] = 0.0;                    // Schwarz factor, set by the ERI kernel's self mode
      r.pad[1] = (double)(m1 * ngk + m2);  // position in the reference's (m1, m2) loop
      r.pad[2] = (r.fact * r.coef) * r.p_inv;  // w: the pair's factor of the quartet prefactor
      out[o++] = r;
    }
}

// partial sums -> ERIs; diagonal reuse and Schwarz screening (src/two_e_slater.F90:264-279)
__global__ void eri_finalize(int64_t nint, const int32_t* __restrict__ is, const int32_t* __restrict__ js,
                             const int32_t* __restrict__ ks, const int32_t* __restrict__ ls,
                             const int64_t* __restrict__ slot, const double* __restrict__ partial,
                             const double* __restrict__ pre, int n, double* __restrict__ out) {
  int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (q >= nint) return;
  int i = is[q] - 1, k = ks[q] - 1, j = js[q] - 1, l = ls[q] - 1;
  int64_t s = slot[q];
  double v;
  if (i == j && k == l) {
    v = pre[i + (int64_t)n * k];
  } else if (s < 0) {
    v = 0.0;
  } else {
    v = 0.0;
    const int64_t o = slot_offset(s);
    const int sp = slot_split(s);
    for (int t = 0; t < sp; t++) v = v + partial[o + t];
  }
  out[q] = v;
}

// Launch helpers ------------------------------------------------------------------------
cudaError_t eri_init_constants() { return cudaSuccess; }  // tables are compile-time

// ket pairs per shared-memory tile and the dynamic shared memory it needs
void eri_tile(int LK, bool t2, int max_cnt, int* ktile, size_t* smem) {
  // per ket pair: the record and its polynomials (ket degree bound LK) in FP64, and their FP32
  // copies
  const size_t per = eri_ket_bytes(LK, t2);
  // Small ket tiles: with ~53 KB of static tables and scans, 60 KB tiles let two CTAs share an
  // SM (8 warps) and leave unified L1 to the local arrays of the classes with r^2-type fits.  On
  // the 26-function H2O basis 168 KB (one CTA per SM) -> 60 KB tiles took the analytic stage from
  // 2.71 to 2.53 s.
  // (smaller tiles for the spilling LK = L >= 3 instances, to leave L1 to their local arrays,
  // were slower: 32 KB -> 1.458 s, 16 KB -> 1.473 s for the analytic stage, against 1.446 s)
  const size_t budget = (size_t)ERI_SMEM_MAX;
  int kt = (int)(budget / per);
  kt = kt < max_cnt ? kt : max_cnt;
  kt = kt < 1 ? 1 : kt;
  *ktile = kt;
  *smem = per * kt;
}

cudaError_t launch_eri_L0c0(dim3, int, size_t, cudaStream_t, const BasisDev&, const PrimPair*, const int64_t*, const int*, const int64_t*, int, const int32_t*, const int32_t*, const int32_t*, const int32_t*, const double*, double, double, double*, double*, const PrimPairF*);
cudaError_t launch_eri_L1c0(dim3, int, size_t, cudaStream_t, const BasisDev&, const PrimPair*, const int64_t*, const int*, const int64_t*, int, const int32_t*, const int32_t*, const int32_t*, const int32_t*, const double*, double, double, double*, double*, const PrimPairF*);
cudaError_t launch_eri_L2c0(dim3, int, size_t, cudaStream_t, const BasisDev&, const PrimPair*, const int64_t*, const int*, const int64_t*, int, const int32_t*, const int32_t*, const int32_t*, const int32_t*, const double*, double, double, double*, double*, const PrimPairF*);
cudaError_t launch_eri_L3c0(dim3, int, size_t, cudaStream_t, const BasisDev&, const PrimPair*, const int64_t*, const int*, const int64_t*, int, const int32_t*, const int32_t*, const int32_t*, const int32_t*, const double*, double, double, double*, double*, const PrimPairF*);
cudaError_t launch_eri_L4c0(dim3, int, size_t, cudaStream_t, const BasisDev&, const PrimPair*, const int64_t*, const int*, const int64_t*, int, const int32_t*, const int32_t*, const int32_t*, const int32_t*, const double*, double, double, double*, double*, const PrimPairF*);
cudaError_t launch_eri_L2c1(dim3, int, size_t, cudaStream_t, const BasisDev&, const PrimPair*, const int64_t*, const int*, const int64_t*, int, const int32_t*, const int32_t*, const int32_t*, const int32_t*, const double*, double, double, double*, double*, const PrimPairF*);
cudaError_t launch_eri_L3c1(dim3, int, size_t, cudaStream_t, const BasisDev&, const PrimPair*, const int64_t*, const int*, const int64_t*, int, const int32_t*, const int32_t*, const int32_t*, const int32_t*, const double*, double, double, double*, double*, const PrimPairF*);
cudaError_t launch_eri_L4c1(dim3, int, size_t, cudaStream_t, const BasisDev&, const PrimPair*, const int64_t*, const int*, const int64_t*, int, const int32_t*, const int32_t*, const int32_t*, const int32_t*, const double*, double, double, double*, double*, const PrimPairF*);
cudaError_t launch_eri_L2c2(dim3, int, size_t, cudaStream_t, const BasisDev&, const PrimPair*, const int64_t*, const int*, const int64_t*, int, const int32_t*, const int32_t*, const int32_t*, const int32_t*, const double*, double, double, double*, double*, const PrimPairF*);
cudaError_t launch_eri_L3c2(dim3, int, size_t, cudaStream_t, const BasisDev&, const PrimPair*, const int64_t*, const int*, const int64_t*, int, const int32_t*, const int32_t*, const int32_t*, const int32_t*, const double*, double, double, double*, double*, const PrimPairF*);
cudaError_t launch_eri_L4c2(dim3, int, size_t, cudaStream_t, const BasisDev&, const PrimPair*, const int64_t*, const int*, const int64_t*, int, const int32_t*, const int32_t*, const int32_t*, const int32_t*, const double*, double, double, double*, double*, const PrimPairF*);
cudaError_t launch_eri_L4c3(dim3, int, size_t, cudaStream_t, const BasisDev&, const PrimPair*, const int64_t*, const int*, const int64_t*, int, const int32_t*, const int32_t*, const int32_t*, const int32_t*, const double*, double, double, double*, double*, const PrimPairF*);
cudaError_t launch_eri_L4c4(dim3, int, size_t, cudaStream_t, const BasisDev&, const PrimPair*, const int64_t*, const int*, const int64_t*, int, const int32_t*, const int32_t*, const int32_t*, const int32_t*, const double*, double, double, double*, double*, const PrimPairF*);
cudaError_t launch_eri_L1c0k0(dim3, int, size_t, cudaStream_t, const BasisDev&, const PrimPair*, const int64_t*, const int*, const int64_t*, int, const int32_t*, const int32_t*, const int32_t*, const int32_t*, const double*, double, double, double*, double*, const PrimPairF*);
cudaError_t launch_eri_L2c0k0(dim3, int, size_t, cudaStream_t, const BasisDev&, const PrimPair*, const int64_t*, const int*, const int64_t*, int, const int32_t*, const int32_t*, const int32_t*, const int32_t*, const double*, double, double, double*, double*, const PrimPairF*);
cudaError_t launch_eri_L2c1k0(dim3, int, size_t, cudaStream_t, const BasisDev&, const PrimPair*, const int64_t*, const int*, const int64_t*, int, const int32_t*, const int32_t*, const int32_t*, const int32_t*, const double*, double, double, double*, double*, const PrimPairF*);
cudaError_t launch_eri_L3c0k0(dim3, int, size_t, cudaStream_t, const BasisDev&, const PrimPair*, const int64_t*, const int*, const int64_t*, int, const int32_t*, const int32_t*, const int32_t*, const int32_t*, const double*, double, double, double*, double*, const PrimPairF*);
cudaError_t launch_eri_L3c1k0(dim3, int, size_t, cudaStream_t, const BasisDev&, const PrimPair*, const int64_t*, const int*, const int64_t*, int, const int32_t*, const int32_t*, const int32_t*, const int32_t*, const double*, double, double, double*, double*, const PrimPairF*);
cudaError_t launch_eri_L2c0k1(dim3, int, size_t, cudaStream_t, const BasisDev&, const PrimPair*, const int64_t*, const int*, const int64_t*, int, const int32_t*, const int32_t*, const int32_t*, const int32_t*, const double*, double, double, double*, double*, const PrimPairF*);
cudaError_t launch_eri_L2c1k1(dim3, int, size_t, cudaStream_t, const BasisDev&, const PrimPair*, const int64_t*, const int*, const int64_t*, int, const int32_t*, const int32_t*, const int32_t*, const int32_t*, const double*, double, double, double*, double*, const PrimPairF*);
cudaError_t launch_eri_L3c0k1(dim3, int, size_t, cudaStream_t, const BasisDev&, const PrimPair*, const int64_t*, const int*, const int64_t*, int, const int32_t*, const int32_t*, const int32_t*, const int32_t*, const double*, double, double, double*, double*, const PrimPairF*);
cudaError_t launch_eri_L3c1k1(dim3, int, size_t, cudaStream_t, const BasisDev&, const PrimPair*, const int64_t*, const int*, const int64_t*, int, const int32_t*, const int32_t*, const int32_t*, const int32_t*, const double*, double, double, double*, double*, const PrimPairF*);
cudaError_t launch_eri_L3c2k1(dim3, int, size_t, cudaStream_t, const BasisDev&, const PrimPair*, const int64_t*, const int*, const int64_t*, int, const int32_t*, const int32_t*, const int32_t*, const int32_t*, const double*, double, double, double*, double*, const PrimPairF*);
cudaError_t launch_eri_L4c0k1(dim3, int, size_t, cudaStream_t, const BasisDev&, const PrimPair*, const int64_t*, const int*, const int64_t*, int, const int32_t*, const int32_t*, const int32_t*, const int32_t*, const double*, double, double, double*, double*, const PrimPairF*);
cudaError_t launch_eri_L4c1k1(dim3, int, size_t, cudaStream_t, const BasisDev&, const PrimPair*, const int64_t*, const int*, const int64_t*, int, const int32_t*, const int32_t*, const int32_t*, const int32_t*, const double*, double, double, double*, double*, const PrimPairF*);
cudaError_t launch_eri_L4c2k1(dim3, int, size_t, cudaStream_t, const BasisDev&, const PrimPair*, const int64_t*, const int*, const int64_t*, int, const int32_t*, const int32_t*, const int32_t*, const int32_t*, const double*, double, double, double*, double*, const PrimPairF*);
cudaError_t launch_eri_L3c0k2(dim3, int, size_t, cudaStream_t, const BasisDev&, const PrimPair*, const int64_t*, const int*, const int64_t*, int, const int32_t*, const int32_t*, const int32_t*, const int32_t*, const double*, double, double, double*, double*, const PrimPairF*);
cudaError_t launch_eri_L3c1k2(dim3, int, size_t, cudaStream_t, const BasisDev&, const PrimPair*, const int64_t*, const int*, const int64_t*, int, const int32_t*, const int32_t*, const int32_t*, const int32_t*, const double*, double, double, double*, double*, const PrimPairF*);
cudaError_t launch_eri_L3c2k2(dim3, int, size_t, cudaStream_t, const BasisDev&, const PrimPair*, const int64_t*, const int*, const int64_t*, int, const int32_t*, const int32_t*, const int32_t*, const int32_t*, const double*, double, double, double*, double*, const PrimPairF*);
cudaError_t launch_eri_L4c0k2(dim3, int, size_t, cudaStream_t, const BasisDev&, const PrimPair*, const int64_t*, const int*, const int64_t*, int, const int32_t*, const int32_t*, const int32_t*, const int32_t*, const double*, double, double, double*, double*, const PrimPairF*);
cudaError_t launch_eri_L4c1k2(dim3, int, size_t, cudaStream_t, const BasisDev&, const PrimPair*, const int64_t*, const int*, const int64_t*, int, const int32_t*, const int32_t*, const int32_t*, const int32_t*, const double*, double, double, double*, double*, const PrimPairF*);
cudaError_t launch_eri_L4c2k2(dim3, int, size_t, cudaStream_t, const BasisDev&, const PrimPair*, const int64_t*, const int*, const int64_t*, int, const int32_t*, const int32_t*, const int32_t*, const int32_t*, const double*, double, double, double*, double*, const PrimPairF*);
cudaError_t launch_eri_L4c3k2(dim3, int, size_t, cudaStream_t, const BasisDev&, const PrimPair*, const int64_t*, const int*, const int64_t*, int, const int32_t*, const int32_t*, const int32_t*, const int32_t*, const double*, double, double, double*, double*, const PrimPairF*);

// Kernel instance for class (L, tc) and ket bound LK.  tc: number of r^2-type fits among the
// four functions (0..4).  A quartet with r^2-type fits has L >= 2, and one with three or four has
// L = 4; an instance with a larger L serves any smaller one (degrees are runtime).  LK < L: the
// light-ket instances of ss_light_ket (a ket with L <= 1 holds no r^2-type fit, one with L = 2 at
// most one; a bra with L <= 3 at most one, with L = 4 at most two).
cudaError_t launch_eri_class(int L, int LK, int tc, dim3 grid, int ktile, size_t smem, cudaStream_t st,
                             const BasisDev& B, const PrimPair* pp, const int64_t* off, const int* cnt,
                             const int64_t* work, int split, const int32_t* is, const int32_t* js,
                             const int32_t* ks, const int32_t* ls, const double* pre, double eps,
                             double eps32, double* partial, double* self_out, const PrimPairF* ppf) {
  if (LK < L) {
#define SS_KV(LL, TT, KK)                                                                                       \
  if (L == LL && tc == TT && LK == KK)                                                                          \
    return launch_eri_L##LL##c##TT##k##KK(grid, ktile, smem, st, B, pp, off, cnt, work, split, is, js, ks, ls, \
                                          pre, eps, eps32, partial, self_out, ppf);
    SS_KV(1, 0, 0) SS_KV(2, 0, 0) SS_KV(2, 1, 0) SS_KV(3, 0, 0) SS_KV(3, 1, 0)
    SS_KV(2, 0, 1) SS_KV(2, 1, 1)
    SS_KV(3, 0, 1) SS_KV(3, 1, 1) SS_KV(3, 2, 1) SS_KV(4, 0, 1) SS_KV(4, 1, 1) SS_KV(4, 2, 1)
    SS_KV(3, 0, 2) SS_KV(3, 1, 2) SS_KV(3, 2, 2) SS_KV(4, 0, 2) SS_KV(4, 1, 2) SS_KV(4, 2, 2) SS_KV(4, 3, 2)
#undef SS_KV
    return cudaErrorInvalidValue;
  }
  if (tc == 0) {
    if (L == 0) return launch_eri_L0c0(grid, ktile, smem, st, B, pp, off, cnt, work, split, is, js, ks, ls, pre, eps, eps32, partial, self_out, ppf);
    if (L == 1) return launch_eri_L1c0(grid, ktile, smem, st, B, pp, off, cnt, work, split, is, js, ks, ls, pre, eps, eps32, partial, self_out, ppf);
    if (L == 2) return launch_eri_L2c0(grid, ktile, smem, st, B, pp, off, cnt, work, split, is, js, ks, ls, pre, eps, eps32, partial, self_out, ppf);
    if (L == 3) return launch_eri_L3c0(grid, ktile, smem, st, B, pp, off, cnt, work, split, is, js, ks, ls, pre, eps, eps32, partial, self_out, ppf);
    if (L == 4) return launch_eri_L4c0(grid, ktile, smem, st, B, pp, off, cnt, work, split, is, js, ks, ls, pre, eps, eps32, partial, self_out, ppf);
  } else if (tc == 1) {
    if (L <= 2) return launch_eri_L2c1(grid, ktile, smem, st, B, pp, off, cnt, work, split, is, js, ks, ls, pre, eps, eps32, partial, self_out, ppf);
    if (L == 3) return launch_eri_L3c1(grid, ktile, smem, st, B, pp, off, cnt, work, split, is, js, ks, ls, pre, eps, eps32, partial, self_out, ppf);
    if (L == 4) return launch_eri_L4c1(grid, ktile, smem, st, B, pp, off, cnt, work, split, is, js, ks, ls, pre, eps, eps32, partial, self_out, ppf);
  } else if (tc == 2) {
    if (L <= 2) return launch_eri_L2c2(grid, ktile, smem, st, B, pp, off, cnt, work, split, is, js, ks, ls, pre, eps, eps32, partial, self_out, ppf);
    if (L == 3) return launch_eri_L3c2(grid, ktile, smem, st, B, pp, off, cnt, work, split, is, js, ks, ls, pre, eps, eps32, partial, self_out, ppf);
    if (L == 4) return launch_eri_L4c2(grid, ktile, smem, st, B, pp, off, cnt, work, split, is, js, ks, ls, pre, eps, eps32, partial, self_out, ppf);
  } else if (tc == 3) {
    if (L <= 4) return launch_eri_L4c3(grid, ktile, smem, st, B, pp, off, cnt, work, split, is, js, ks, ls, pre, eps, eps32, partial, self_out, ppf);
  } else if (tc == 4) {
    if (L <= 4) return launch_eri_L4c4(grid, ktile, smem, st, B, pp, off, cnt, work, split, is, js, ks, ls, pre, eps, eps32, partial, self_out, ppf);
  }
  return cudaErrorInvalidValue;
}

// Sort the primitive pairs of every function pair by decreasing Schwarz factor (pad[0]), ties
// by the reference's loop position (pad[1]), so the order is a function of the values alone.
// One CTA per function pair, bitonic sort of up to 1024 keys in shared memory; out = sorted copy.
__global__ void __launch_bounds__(512) prim_pair_sort(const PrimPair* __restrict__ in, const int64_t* __restrict__ off,
                                                      const int* __restrict__ cnt, PrimPair* __restrict__ out) {
  __shared__ double s_key[1024], s_pos[1024];
  __shared__ int s_idx[1024];
  const int pidx = blockIdx.x;
  const int m = cnt[pidx];
  const PrimPair* src = in + off[pidx];
  PrimPair* dst = out + off[pidx];
  for (int t = threadIdx.x; t < 1024; t += blockDim.x) {
    s_key[t] = t < m ? src[t].pad[0] : -1.0;  // padding sorts last
    s_pos[t] = t < m ? src[t].pad[1] : 1.0e300;
    s_idx[t] = t;
  }
  __syncthreads();
  // "a before b": larger key first, then smaller reference position
  for (int k = 2; k <= 1024; k <<= 1)
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int t = threadIdx.x; t < 1024; t += blockDim.x) {
        const int u = t ^ j;
        if (u > t) {
          const bool up = (t & k) == 0;
          const bool t_first = s_key[t] > s_key[u] || (s_key[t] == s_key[u] && s_pos[t] < s_pos[u]);
          if (up != t_first) {
            const double kk = s_key[t], pp2 = s_pos[t];
            const int ii = s_idx[t];
            s_key[t] = s_key[u]; s_pos[t] = s_pos[u]; s_idx[t] = s_idx[u];
            s_key[u] = kk; s_pos[u] = pp2; s_idx[u] = ii;
          }
        }
      }
      __syncthreads();
    }
  for (int t = threadIdx.x; t < m; t += blockDim.x) dst[t] = src[s_idx[t]];
}

// FP32 copies of the (sorted) primitive pairs, fc = w = K_AB c p_inv
__global__ void prim_pair_to_f32(int64_t npp, const PrimPair* __restrict__ in, PrimPairF* __restrict__ out) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= npp) return;
  const PrimPair a = in[t];
  PrimPairF f;
  f.p = (float)a.p;
  f.p_inv = (float)a.p_inv;
  f.fc = (float)a.pad[2];
#pragma unroll
  for (int ax = 0; ax < 3; ax++) {
    f.P[ax] = (float)a.P[ax];
    f.PA[ax] = (float)a.PA[ax];
    f.PB[ax] = (float)a.PB[ax];
  }
  f.pad[0] = f.pad[1] = 0.f;
  out[t] = f;
}

}  // namespace ss
