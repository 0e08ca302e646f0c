// eri_kernel.cuh -- templates of the analytic ERI kernel (instantiated per class in eri_k*.cu).
#pragma once
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

#include "boys.cuh"
#include "ss_common.cuh"

// The per-primitive-quartet arithmetic below is plain IEEE arithmetic with explicit fma, so it
// also compiles as host C++ (the host build of the tests checks it against the oracle); the
// kernel itself is device-only.
#ifdef __CUDACC__
#define SS_DFI __device__ __forceinline__
#else
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#define SS_DFI inline
using std::fma;
using std::max;
using std::min;
inline double rsqrt(double x) { return 1.0 / std::sqrt(x); }
inline float rsqrt(float x) { return 1.0f / std::sqrt(x); }
#endif

namespace ss {

constexpr double THRESH = 1.e-15;
constexpr double PI_5_2 = 34.9868366552;  // src/general_primitive_integral.F90:25

// (x - x_A)^a around x_P: coefficients of (x-x_P)^i, pw1 = x_P - x_A
// (src/give_explicit_poly_and_gaussian.F90:86-220, cases 0..4; the powers and the exact
// integer binomials of each case)
template <int L, typename Real>
SS_DFI void recentered(Real pw1, int a, Real (&P)[L + 1]) {
#pragma unroll
  for (int t = 0; t <= L; t++) P[t] = Real(0);
  if (a == 0) {
    P[0] = Real(1);
  } else if (a == 1) {
    P[0] = pw1;
    if (L >= 1) P[1 % (L + 1)] = Real(1);
  } else if (a == 2) {
    const Real p2 = pw1 * pw1;
    P[0] = p2;
    if (L >= 2) { P[1 % (L + 1)] = Real(2) * pw1; P[2 % (L + 1)] = Real(1); }
  } else if (a == 3) {
    const Real p2 = pw1 * pw1, p3 = p2 * pw1;
    P[0] = p3;
    if (L >= 3) { P[1 % (L + 1)] = Real(3) * p2; P[2 % (L + 1)] = Real(3) * pw1; P[3 % (L + 1)] = Real(1); }
  } else {  // a == 4
    const Real p2 = pw1 * pw1, p3 = p2 * pw1, p4 = p2 * p2;
    P[0] = p4;
    if (L >= 4) {
      P[1 % (L + 1)] = Real(4) * p3; P[2 % (L + 1)] = Real(6) * p2; P[3 % (L + 1)] = Real(4) * pw1;
      P[4 % (L + 1)] = Real(1);
    }
  }
}

// P_new = recentered(A,a) * recentered(B,b) in multiply_poly's order (src/multiply_poly.F90:22-31)
template <int L, typename Real>
SS_DFI void pair_poly(Real pa, int a, Real pb, int b, Real* Pn) {
  Real Pa[L + 1], Pb[L + 1];
  recentered<L, Real>(pa, a, Pa);
  recentered<L, Real>(pb, b, Pb);
#pragma unroll
  for (int t = 0; t <= L; t++) Pn[t] = Real(0);
#pragma unroll
  for (int ib = 0; ib <= L; ib++)
#pragma unroll
    for (int ic = 0; ic <= L; ic++)
      if (ib + ic <= L && ib <= a && ic <= b) Pn[ib + ic] = Pn[ib + ic] + Pb[ic] * Pa[ib];
}

template <typename Real>
struct RecCoefT {
  Real p10_1, p10_2, p01_1, p01_2, pq_inv;
};

// Bottom-up table I(a,c)[m] (coefficients of u = t^2) for a <= amax <= L, c <= cmax <= LK,
// the terms of I_x1_pol_mult / I_x2_pol_mult in their order, each as one fused multiply-add with
// the integer factor folded into the recursion coefficient ((a-1) B10 is formed once per
// primitive quartet, not per entry):
//   I(0,c) = (c-1) B01 I(0,c-2) + D00 I(0,c-1);  I(a,c) = (a-1) B10 I(a-2,c) + c B00 I(a-1,c-1) + C00 I(a-1,c)
template <int L, int LK, typename Real>
SS_DFI void rys_table(const RecCoefT<Real>& R, Real Cc, Real Dd, int amax, int cmax,
                                          Real (&I)[L + 1][LK + 1][L + LK + 1]) {
#pragma unroll
  for (int c = 0; c <= LK; c++) {
    if (c > cmax) break;
#pragma unroll
    for (int m = 0; m <= LK; m++) {
      if (m > c) break;
      Real v = Real(0);
      if (c == 0) {
        v = Real(1);
      } else {
        if (c >= 2) {
          if (m >= 1 && m - 1 <= c - 2) v = fma(-R.p01_2 * (Real)(c - 1), I[0][c - 2][m - 1], v);
          if (m <= c - 2) v = fma(R.p01_1 * (Real)(c - 1), I[0][c - 2][m], v);
        }
        if (m >= 1) v = fma(Dd, I[0][c - 1][m - 1], v);
      }
      I[0][c][m] = v;
    }
  }
#pragma unroll
  for (int a = 1; a <= L; a++) {
    if (a > amax) break;
#pragma unroll
    for (int c = 0; c <= LK; c++) {
      if (c > cmax) break;
#pragma unroll
      for (int m = 0; m <= L + LK; m++) {
        if (m > a + c) break;
        Real v = Real(0);
        if (a >= 2) {
          const Real s = (Real)(a - 1);
          if (m >= 1 && m - 1 <= a - 2 + c) v = fma(-R.p10_2 * s, I[a - 2][c][m - 1], v);
          if (m <= a - 2 + c) v = fma(R.p10_1 * s, I[a - 2][c][m], v);
        }
        if (c >= 1 && m >= 1 && m - 1 <= a - 1 + c - 1) v = fma(R.pq_inv * (Real)c, I[a - 1][c - 1][m - 1], v);
        if (m >= 1) v = fma(Cc, I[a - 1][c][m - 1], v);
        I[a][c][m] = v;
      }
    }
  }
}

// The same table when bra and ket share one centre (all four functions on one atom): C00 and
// D00 vanish, so only the B10/B01/B00 terms remain and every entry with a + c odd is zero.
template <int L, int LK, typename Real>
SS_DFI void rys_table_1c(const RecCoefT<Real>& R, int amax, int cmax,
                                             Real (&I)[L + 1][LK + 1][L + LK + 1]) {
#pragma unroll
  for (int c = 0; c <= LK; c++) {
    if (c > cmax) break;
#pragma unroll
    for (int m = 0; m <= LK; m++) {
      if (m > c) break;
      Real v = Real(0);
      if (c == 0) {
        v = Real(1);
      } else if (!(c & 1) && c >= 2) {
        if (m >= 1 && m - 1 <= c - 2) v = fma(-R.p01_2 * (Real)(c - 1), I[0][c - 2][m - 1], v);
        if (m <= c - 2) v = fma(R.p01_1 * (Real)(c - 1), I[0][c - 2][m], v);
      }
      I[0][c][m] = v;
    }
  }
#pragma unroll
  for (int a = 1; a <= L; a++) {
    if (a > amax) break;
#pragma unroll
    for (int c = 0; c <= LK; c++) {
      if (c > cmax) break;
#pragma unroll
      for (int m = 0; m <= L + LK; m++) {
        if (m > a + c) break;
        Real v = Real(0);
        if (!((a + c) & 1)) {
          if (a >= 2) {
            const Real s = (Real)(a - 1);
            if (m >= 1 && m - 1 <= a - 2 + c) v = fma(-R.p10_2 * s, I[a - 2][c][m - 1], v);
            if (m <= a - 2 + c) v = fma(R.p10_1 * s, I[a - 2][c][m], v);
          }
          if (c >= 1 && m >= 1 && m - 1 <= a - 1 + c - 1) v = fma(R.pq_inv * (Real)c, I[a - 1][c - 1][m - 1], v);
        }
        I[a][c][m] = v;
      }
    }
  }
}

// |x| < t and |x| > t on the bit patterns (integer pipe; x finite, t > 0)
SS_DFI int32_t fbits_of(float x) {
#ifdef __CUDA_ARCH__
  return __float_as_int(x);
#else
  int32_t v;
  memcpy(&v, &x, sizeof v);
  return v;
#endif
}
SS_DFI bool abs_lt(double x, double t) { return (bits_of(x) & 0x7FFFFFFFFFFFFFFFLL) < bits_of(t); }
SS_DFI bool abs_gt(double x, double t) { return (bits_of(x) & 0x7FFFFFFFFFFFFFFFLL) > bits_of(t); }
SS_DFI bool abs_lt(float x, float t) { return (fbits_of(x) & 0x7FFFFFFF) < fbits_of(t); }
SS_DFI bool abs_gt(float x, float t) { return (fbits_of(x) & 0x7FFFFFFF) > fbits_of(t); }

// Ix = sum_{ix,jx} (Pn[ix] Qn[jx]) I(ix,jx) with the thresholds of general_primitive_integral
// (x axis: skip |P| < thresh; y, z: keep |P| > thresh; skip |P Q| < thresh).
template <int L, int LK, typename Real>
SS_DFI void axis_poly(const Real* Pn, int degP, const Real* Qn, int degQ,
                                          const Real (&I)[L + 1][LK + 1][L + LK + 1], bool x_axis,
                                          Real* out) {
#pragma unroll
  for (int m = 0; m <= L + LK; m++) out[m] = Real(0);
#pragma unroll
  for (int ix = 0; ix <= L; ix++) {
    if (ix > degP) break;
    const Real a = Pn[ix];
    if (x_axis ? abs_lt(a, (Real)THRESH) : !abs_gt(a, (Real)THRESH)) continue;
#pragma unroll
    for (int jx = 0; jx <= LK; jx++) {
      if (jx > degQ) break;
      const Real d = a * Qn[jx];
      if (abs_lt(d, (Real)THRESH)) continue;
#pragma unroll
      for (int m = 0; m <= L + LK; m++)
        if (m <= ix + jx) out[m] = fma(d, I[ix][jx][m], out[m]);
    }
  }
}

// CTA-uniform description of one function quartet (ik|jl): cartesian powers, which functions
// are r^2-type fits, the Boys order and the per-axis maximal degrees of bra and ket.
struct QuartetShape {
  int np[4][3];
  int t2[4];
  int nf;
  int amax[3], cmax[3];
  int nt, tf[4];  // number and positions (0..3 = i, k, j, l) of the r^2-type fits
  int onec;       // all four functions on one centre
};

template <bool T2>
SS_DFI QuartetShape quartet_shape(const BasisDev& B, int fi, int fk, int fj, int fl) {
  QuartetShape S;
  const int fn[4] = {fi, fk, fj, fl};
  S.nf = 0;
#pragma unroll
  for (int f = 0; f < 4; f++) {
    S.t2[f] = T2 ? (B.i_type[fn[f]] == 2) : 0;
#pragma unroll
    for (int ax = 0; ax < 3; ax++) {
      S.np[f][ax] = B.npower[3 * fn[f] + ax];
      S.nf += S.np[f][ax];
    }
    S.nf += 2 * S.t2[f];
  }
#pragma unroll
  for (int ax = 0; ax < 3; ax++) {
    S.amax[ax] = S.np[0][ax] + S.np[1][ax] + 2 * (S.t2[0] + S.t2[1]);
    S.cmax[ax] = S.np[2][ax] + S.np[3][ax] + 2 * (S.t2[2] + S.t2[3]);
  }
  S.nt = 0;
#pragma unroll
  for (int f = 0; f < 4; f++) {
    S.tf[f] = 0;
    if (S.t2[f]) S.tf[S.nt++] = f;
  }
  S.onec = 1;
#pragma unroll
  for (int f = 1; f < 4; f++)
#pragma unroll
    for (int ax = 0; ax < 3; ax++)
      if (B.center[3 * fn[f] + ax] != B.center[3 * fn[0] + ax]) S.onec = 0;
  return S;
}

// Which functions of the quartet take the +2 of their r^2 fit on one axis, for a subset s of
// the r^2-type functions (bit b of s = function tf[b]): bra option ob (bit0 = i, bit1 = k), ket
// option oc (bit0 = j, bit1 = l), as used by pair_polys.
SS_DFI void subset_options(const QuartetShape& S, int s, int& ob, int& oc) {
  int plus[4] = {0, 0, 0, 0};
#pragma unroll
  for (int b = 0; b < 4; b++)
    if (b < S.nt && ((s >> b) & 1)) plus[S.tf[b]] = 1;
  ob = plus[0] | (plus[1] << 1);
  oc = plus[2] | (plus[3] << 1);
}

// recentred pair polynomials of a primitive pair, per (axis, option); side 0 = bra (functions
// i, k), side 1 = ket (functions j, l).  Layout [ax][o][L+1].
template <int L, bool T2, typename Real, typename Rec>
SS_DFI void pair_polys(const QuartetShape& S, int side, const Rec& P, Real* out) {
  constexpr int NO = T2 ? 4 : 1;
  const int f0 = 2 * side, f1 = 2 * side + 1;
#pragma unroll
  for (int ax = 0; ax < 3; ax++)
#pragma unroll
    for (int o = 0; o < NO; o++) {
      if ((o & 1) && !S.t2[f0]) continue;
      if ((o & 2) && !S.t2[f1]) continue;
      pair_poly<L, Real>(P.PA[ax], S.np[f0][ax] + 2 * (o & 1), P.PB[ax], S.np[f1][ax] + (o & 2),
                         out + (ax * NO + o) * (L + 1));
    }
}

SS_DFI PairView<double> view64(const PrimPair& A) {
  return PairView<double>{A.p, A.p_inv, 0.5 * A.p_inv, {A.P[0], A.P[1], A.P[2]}, A.pad[2]};
}

SS_DFI PairView<float> view32(const PrimPairF& A) {
  return PairView<float>{A.p, A.p_inv, 0.5f * A.p_inv, {A.P[0], A.P[1], A.P[2]}, A.fc};
}

// One primitive quartet (src/general_primitive_integral.F90, summed over the cartesian
// components of the r^2-type fits), times the coefficient product of src/gauss_ijkl.F90:137 and
// divided by 2 pi^{5/2}: returns w_P w_Q / sqrt(p+q) * sum_n d1[n] F_n.  Pn, Qn: pair_polys of
// the bra and ket pairs.
// TC: the number of r^2-type fits among the four functions (0..4; with any, the subset recursion
// over the axes below).  L bounds the per-axis degree of the bra pair, LK that of the ket pair
// (Pn: [ax][o][L+1], Qn: [ax][o][LK+1]); the total degree is at most 3 (L + LK).
template <int L, int TC, typename Real, int LK = L>
SS_DFI Real prim_quartet(const QuartetShape& S, const PairView<Real>& P, const Real* Pn,
                                             const PairView<Real>& Q, const Real* Qn, const Real* s_boys) {
  constexpr bool T2 = TC > 0;
  constexpr int NO = T2 ? 4 : 1;
  constexpr int LT = L + LK;                       // per-axis degree bound of the quartet
  constexpr int NF = (3 * LT < 16) ? 3 * LT : 16;
  const Real p = P.p, qq = Q.p;
  // src/general_primitive_integral.F90:54-60, 142-146, with q/(p+q) and p/(p+q) formed once
  // (the same quantities, reassociated: they give p10_2, p01_2, rho and each axis's C00, D00)
  const Real pq = P.hp * Q.p_inv;    // p_inv q_inv / 2
  const Real rs_pq = rsqrt(p + qq);  // 1/sqrt(p+q): gives 1/(p+q) and the prefactor's root
  const Real pq_inv = Real(0.5) * (rs_pq * rs_pq);
  RecCoefT<Real> R;
  R.p10_1 = qq * pq;
  R.p01_1 = p * pq;
  const Real pq_inv_2 = pq_inv + pq_inv;
  const Real fq = qq * pq_inv_2, fp = p * pq_inv_2;  // q/(p+q), p/(p+q)
  R.p10_2 = R.p10_1 * fq;
  R.p01_2 = R.p01_1 * fp;
  R.pq_inv = pq_inv;
  const Real rho = p * fq;
  const Real dP[3] = {P.P[0] - Q.P[0], P.P[1] - Q.P[1], P.P[2] - Q.P[2]};
  const Real T = (dP[0] * dP[0] + dP[1] * dP[1] + dP[2] * dP[2]) * rho;
  Real F[NF + 1];
  if constexpr (sizeof(Real) == 8)
    boys_tab<NF>(T, S.nf, F, s_boys);
  else
    boys32<NF>(T, S.nf, F, s_boys);
  const int nf = S.nf;

  Real accu;
  if (!T2) {
    Real A[3][LT + 1];
    int deg[3];
#pragma unroll
    for (int ax = 0; ax < 3; ax++) {
      deg[ax] = S.amax[ax] + S.cmax[ax];
      if (deg[ax] == 0) {
        A[ax][0] = Real(1);
#pragma unroll
        for (int m = 1; m <= LT; m++) A[ax][m] = Real(0);
        continue;
      }
      Real I[L + 1][LK + 1][LT + 1];
      const Real Cc = -fq * dP[ax];  // src/give_polynom_mult_center_x.F90:58
      const Real Dd = fp * dP[ax];   // :62
      if (S.onec) rys_table_1c<L, LK>(R, S.amax[ax], S.cmax[ax], I);
      else rys_table<L, LK>(R, Cc, Dd, S.amax[ax], S.cmax[ax], I);
      axis_poly<L, LK>(Pn + ax * (L + 1), S.amax[ax], Qn + ax * (LK + 1), S.cmax[ax], I, ax == 0, A[ax]);
    }
    // d1 = (Ix Iy) Iz, then sum_n d1[n] F_n (src/general_primitive_integral.F90:148-173).  An
    // axis of degree 0 has the polynomial 1, and a product with it is a copy (fma(1, x, 0) = x
    // exactly), taken without the multiply-adds: quartet-uniform branches
    Real dp[2 * LT + 1];
    if (deg[0] == 0 || deg[1] == 0) {
      const bool x1 = deg[0] == 0;
#pragma unroll
      for (int t = 0; t <= 2 * LT; t++) dp[t] = t <= LT ? (x1 ? A[1][t % (LT + 1)] : A[0][t % (LT + 1)]) : Real(0);
    } else {
#pragma unroll
      for (int t = 0; t <= 2 * LT; t++) dp[t] = Real(0);
#pragma unroll
      for (int a = 0; a <= LT; a++) {
        if (a > deg[0]) break;
#pragma unroll
        for (int c = 0; c <= LT; c++) {
          if (c > deg[1]) break;
          dp[a + c] = fma(A[1][c], A[0][a], dp[a + c]);
        }
      }
    }
    Real d1[NF + 1];
    if (deg[2] == 0) {
#pragma unroll
      for (int t = 0; t <= NF; t++) d1[t] = t <= 2 * LT ? dp[t % (2 * LT + 1)] : Real(0);
    } else {
#pragma unroll
      for (int t = 0; t <= NF; t++) d1[t] = Real(0);
#pragma unroll
      for (int a = 0; a <= 2 * LT; a++) {
        if (a > deg[0] + deg[1] || a > NF) break;
#pragma unroll
        for (int c = 0; c <= LT; c++) {
          if (c > deg[2] || a + c > NF) break;
          d1[a + c] = fma(A[2][c], dp[a], d1[a + c]);
        }
      }
    }
    accu = d1[0] * F[0];
#pragma unroll
    for (int n = 1; n <= NF; n++)
      if (n <= nf) accu = fma(d1[n], F[n], accu);
  } else {
    // With t = TC r^2-type fits, a cartesian combination assigns each fit's +2 to one axis, i.e.
    // splits the set of fits into (Sx, Sy, Sz).  sum over combinations of L(Ax[Sx] Ay[Sy] Az[Sz])
    // is built axis by axis: Qxy[S] = sum_{Sx subset S} Ax[Sx] Ay[S \ Sx], then
    // sum_Sz L(Qxy[all \ Sz] Az[Sz]), L(p) = sum_n p[n] F_n.  Same per-axis polynomials (and
    // thresholds) as the enumeration of the 3^t combinations, 2^t final contractions instead of 3^t.
    constexpr int NS = 1 << TC;
    constexpr int full = NS - 1;
    Real Ax[NS][LT + 1], Qxy[NS][2 * LT + 1];
    int dAx[NS], dQ[NS];
#pragma unroll
    for (int ax = 0; ax < 3; ax++) {
      Real I[L + 1][LK + 1][LT + 1];
      const Real Cc = -fq * dP[ax];
      const Real Dd = fp * dP[ax];
      if (S.onec) rys_table_1c<L, LK>(R, S.amax[ax], S.cmax[ax], I);
      else rys_table<L, LK>(R, Cc, Dd, S.amax[ax], S.cmax[ax], I);
      if (ax == 1) {
#pragma unroll
        for (int t = 0; t < NS; t++) {
          dQ[t] = -1;
#pragma unroll
          for (int m = 0; m <= 2 * LT; m++) Qxy[t][m] = Real(0);
        }
      }
#pragma unroll
      for (int sa = 0; sa < NS; sa++) {
        int ob, oc;
        subset_options(S, sa, ob, oc);
        const int da = S.np[0][ax] + S.np[1][ax] + 2 * (ob & 1) + (ob & 2);
        const int dc = S.np[2][ax] + S.np[3][ax] + 2 * (oc & 1) + (oc & 2);
        Real Aa[LT + 1];
        axis_poly<L, LK>(Pn + (ax * NO + ob) * (L + 1), da, Qn + (ax * NO + oc) * (LK + 1), dc, I, ax == 0, Aa);
        const int dA = da + dc;
        if (ax == 0) {
#pragma unroll
          for (int m = 0; m <= LT; m++) Ax[sa][m] = Aa[m];
          dAx[sa] = dA;
        } else if (ax == 1) {
#pragma unroll
          for (int sx = 0; sx < NS; sx++) {
            if (sx & sa) continue;
            const int st = sx | sa;
            dQ[st] = max(dQ[st], dAx[sx] + dA);
#pragma unroll
            for (int a = 0; a <= LT; a++) {
              if (a > dAx[sx]) break;
#pragma unroll
              for (int c = 0; c <= LT; c++) {
                if (c > dA) break;
                Qxy[st][a + c] = fma(Aa[c], Ax[sx][a], Qxy[st][a + c]);
              }
            }
          }
        } else {
          const int st = full ^ sa;
          Real sum = Real(0);
#pragma unroll
          for (int c = 0; c <= LT; c++) {
            if (c > dA) break;
            Real g = Real(0);
#pragma unroll
            for (int a = 0; a <= 2 * LT; a++) {
              if (a > dQ[st] || a + c > NF) break;
              g = fma(Qxy[st][a], F[a + c], g);
            }
            sum = fma(Aa[c], g, sum);
          }
          accu = (sa == 0) ? sum : accu + sum;
        }
      }
    }
  }
  // src/general_primitive_integral.F90:192 without its constant 2 pi^{5/2}
  return (P.w * Q.w * rs_pq) * accu;
}

#ifdef __CUDACC__
// Work per CTA: one function quartet (ik|jl) and a slice of its bra primitive pairs against all
// its ket primitive pairs, the ket pairs staged in shared memory in tiles together with their
// recentred polynomials.
//
// Primitive screening (pre != nullptr): the primitive pairs of every function pair are sorted
// by decreasing Schwarz factor S; a primitive quartet with S_P S_Q < eps sqrt((ik|ik)(jl|jl))
// is skipped.  Each skipped term is bounded by that product, so the skipped part of an ERI is at
// most (number of primitive quartets) * eps * sqrt((ik|ik)(jl|jl)).
// FP32 tier (pre != nullptr): a kept primitive quartet with S_P S_Q < eps32 sqrt((ik|ik)(jl|jl))
// is evaluated in FP32 (PRIM_FP32_EPS in ss_common.cuh, the default eps32, gives the error
// bound); eps32 <= eps turns the tier off.
// For each bra pair the FP64 and the FP32 ket pairs of a tile are consecutive ranges from the
// start of the tile (the ket factors decrease along it); the items of each tier are numbered
// through an exclusive scan of the per-bra range lengths.  Without pre every item is FP64 and
// kept (the Schwarz diagonal itself).  The items of a tier are spread evenly over the threads
// (to within one).
//
// Schwarz-factor mode (self_out != nullptr; work = the quartets (ik|ik)): only the items (P, P)
// are evaluated and S_P = sqrt(c_P^2 (P|P)), the self-repulsion of the primitive pair's charge
// distribution (summed over the cartesian components of r^2-type fits) times its coefficient,
// is written to self_out[16 * (pair_off + P)] (PrimPair::pad[0] of the pair).  By
// Cauchy-Schwarz |c_P c_Q (P|Q)| <= S_P S_Q for every primitive quartet.
// TC: how many of the four functions are r^2-type fits (3 cartesian components sharing
// exponents), 0..4.  LK <= L bounds the per-axis degree of the ket pair (the bra's is L): the
// instances with LK < L serve quartets one of whose pairs is much lighter than the other, with
// smaller recursion tables and ket polynomials.  A work entry with bit 62 set is evaluated as
// (jl|ik), which has the same value, so that its lighter pair becomes the ket.
template <int L, int TC, int LK = L>
__global__ void __launch_bounds__(128, 1) eri_kernel(
    BasisDev B, const PrimPair* __restrict__ pp, const int64_t* __restrict__ pair_off,
    const int* __restrict__ pair_cnt, const int64_t* __restrict__ work, int split, int ktile,
    const int32_t* __restrict__ is, const int32_t* __restrict__ js, const int32_t* __restrict__ ks,
    const int32_t* __restrict__ ls, const double* __restrict__ pre, double eps, double eps32,
    double* __restrict__ partial,
    double* __restrict__ self_out, const PrimPairF* __restrict__ ppf) {
  constexpr bool T2 = TC > 0;
  constexpr int NO = T2 ? 4 : 1;        // options per axis: which of the pair's functions adds +2
  constexpr int QW = 3 * NO * (LK + 1);  // ket polynomial values per ket pair
  extern __shared__ double2 s_raw[];
  PrimPair* s_ket = reinterpret_cast<PrimPair*>(s_raw);
  double* s_q = reinterpret_cast<double*>(s_ket + ktile);
  PairView<float>* s_ketf = reinterpret_cast<PairView<float>*>(s_q + (size_t)ktile * QW);
  float* s_qf = reinterpret_cast<float*>(s_ketf + ktile);
  __shared__ double s_red[4];
  __shared__ int s_scan[SS_MAX_NG * SS_MAX_NG + 1];    // FP64 item offsets of the bra slice
  __shared__ int s_scan32[SS_MAX_NG * SS_MAX_NG + 1];  // FP32 item offsets
  __shared__ double s_boys[BOYS_SMEM_DOUBLES];
  __shared__ float s_boys32[BOYS32_K * BOYS32_N];
  const int64_t w = blockIdx.x / split;
  const int part = blockIdx.x % split;
  {  // the launch's dynamic shared memory must hold ktile staged ket pairs: checked, not assumed
    uint32_t dyn;
    asm("mov.u32 %0, %%dynamic_smem_size;" : "=r"(dyn));
    const size_t need =
        (size_t)ktile * (sizeof(PrimPair) + (size_t)QW * (sizeof(double) + sizeof(float)) + sizeof(PairView<float>));
    if (need > dyn) {  // block-uniform: no thread reaches a barrier
      if (threadIdx.x == 0) partial[w * split + part] = __longlong_as_double(0x7FF8000000000000LL);
      return;
    }
  }
  boys_tables_to_smem(s_boys);  // ordered before first use by the tile loop's barriers
  for (int t = threadIdx.x; t < BOYS32_K * BOYS32_N; t += blockDim.x) s_boys32[t] = boys32_tab[t];

  const int64_t wq = work[w];
  const int64_t q = wq & ((int64_t(1) << 62) - 1);
  const bool swp = (wq >> 62) & 1;  // evaluate (jl|ik)
  const int fi = (swp ? js[q] : is[q]) - 1, fk = (swp ? ls[q] : ks[q]) - 1;
  const int fj = (swp ? is[q] : js[q]) - 1, fl = (swp ? ks[q] : ls[q]) - 1;
  const int64_t pb = ss_pair_index(fi, fk), pk = ss_pair_index(fj, fl);
  const int nb = pair_cnt[pb], nk = pair_cnt[pk];
  const PrimPair* bra = pp + pair_off[pb];
  const PrimPair* ket = pp + pair_off[pk];
  const PrimPairF* braf = ppf + pair_off[pb];
  const PrimPairF* ketf = ppf + pair_off[pk];
  const QuartetShape S = quartet_shape<T2>(B, fi, fk, fj, fl);
  const int n = B.n;
  const double sch = pre ? sqrt(pre[fi + (int64_t)n * fk] * pre[fj + (int64_t)n * fl]) : 0.0;
  // the FP32 tier needs the Schwarz diagonal and the FP32 pair copies (not in self mode)
  const bool fp32_tier = pre != nullptr && ppf != nullptr && self_out == nullptr;
  const double tau = eps * sch, tau32 = (fp32_tier && eps32 > eps) ? eps32 * sch : 0.0;

  const int per = (nb + split - 1) / split;
  const int b0 = part * per;
  const int b1 = min(nb, b0 + per);
  const int nbs = max(b1 - b0, 0);
  if (nbs == 0) {  // an empty bra slice (more slices than bra pairs): block-uniform exit
    if (threadIdx.x == 0) partial[w * split + part] = 0.0;
    return;
  }
  double acc = 0.0;
  float acc32 = 0.f;

  for (int t0 = 0; t0 < nk; t0 += ktile) {
    const int kt = min(ktile, nk - t0);
    __syncthreads();
    {
      const double2* src = reinterpret_cast<const double2*>(ket + t0);
      for (int t = threadIdx.x; t < kt * 8; t += blockDim.x) s_raw[t] = src[t];
    }
    __syncthreads();
    // recentred ket polynomials, per (ket pair, axis, option), and their FP32 copies
    for (int kk = threadIdx.x; kk < kt; kk += blockDim.x) {
      double* qd = s_q + (size_t)kk * QW;
      pair_polys<LK, T2, double>(S, 1, s_ket[kk], qd);
      if (fp32_tier) {
        float* qf = s_qf + (size_t)kk * QW;
#pragma unroll
        for (int t = 0; t < QW; t++) qf[t] = (float)qd[t];
        s_ketf[kk] = view32(ketf[t0 + kk]);
      }
    }
    // per bra pair of the slice: the ket ranges [0, c64) in FP64 and [c64, c) in FP32
    for (int bi = threadIdx.x; bi < nbs; bi += blockDim.x) {
      int c = kt, c64 = kt;
      if (self_out) {
        c = c64 = (b0 + bi >= t0 && b0 + bi < t0 + kt) ? 1 : 0;  // the item (P, P) lies in this tile
      } else if (tau > 0.0) {
        const double sb = bra[b0 + bi].pad[0];
        // first index with sb * S_Q < thr (S_Q decreasing along the tile)
        auto first_below = [&](double thr) {
          int lo = 0, hi = kt;
          while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (sb * s_ket[mid].pad[0] < thr) hi = mid; else lo = mid + 1;
          }
          return lo;
        };
        c = first_below(tau);
        c64 = tau32 > tau ? first_below(tau32) : c;  // no FP32 tier: every kept item in FP64
      }
      s_scan[bi + 1] = c64;
      s_scan32[bi + 1] = c - c64;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      s_scan[0] = 0;
      s_scan32[0] = 0;
      for (int bi = 0; bi < nbs; bi++) {
        s_scan[bi + 1] += s_scan[bi];
        s_scan32[bi + 1] += s_scan32[bi];
      }
    }
    __syncthreads();

    // Without r^2-type fits each thread takes a contiguous run of items (bra-major), so its bra
    // polynomials change only when the run crosses a bra pair.  With them the items are dealt
    // round-robin (consecutive threads, consecutive ket pairs of one bra pair): the threads of a
    // warp then share their bra polynomials and the data-dependent branches of the option loops.
    // A thread locates its first item once (last bi with scan[bi] <= e) and then steps: the
    // position moves by the stride and carries over the bra pairs' range lengths.
    auto locate = [&](const int* scan, int e) {
      int lo = 0, hi = nbs - 1;
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (scan[mid] <= e) lo = mid; else hi = mid - 1;
      }
      return lo;
    };
    {  // FP64 tier
      const int nitems = s_scan[nbs];
      const int per_t = (nitems + (int)blockDim.x - 1) / (int)blockDim.x;
      const int e_begin = T2 ? (int)threadIdx.x : min(nitems, (int)threadIdx.x * per_t);
      const int e_end = T2 ? nitems : min(nitems, e_begin + per_t);
      const int e_step = T2 ? (int)blockDim.x : 1;
      int bcur = -1;
      double Pn[3 * NO * (L + 1)];
      PrimPair P;
      int bi = e_begin < e_end ? locate(s_scan, e_begin) : 0;
      int pos = e_begin < e_end ? e_begin - s_scan[bi] : 0;
      for (int e = e_begin; e < e_end; e += e_step) {
        while (pos >= s_scan[bi + 1] - s_scan[bi]) {
          pos -= s_scan[bi + 1] - s_scan[bi];
          bi++;
        }
        const int ib = b0 + bi, ik = self_out ? ib - t0 : pos;
        pos += e_step;
        if (ib != bcur) {
          P = bra[ib];
          bcur = ib;
          pair_polys<L, T2, double>(S, 0, P, Pn);
        }
        const PrimPair& Q = s_ket[ik];
        const double v =
            prim_quartet<L, TC, double, LK>(S, view64(P), Pn, view64(Q), s_q + (size_t)ik * QW, s_boys);
        if (self_out) {
          self_out[16 * (pair_off[pb] + ib)] = sqrt(fmax(PI_5_2 * v, 0.0));
          continue;
        }
        acc += v;
      }
    }
    {  // FP32 tier: the ket range [c64, c) of each bra pair
      const int nitems = s_scan32[nbs];
      const int per_t = (nitems + (int)blockDim.x - 1) / (int)blockDim.x;
      const int e_begin = T2 ? (int)threadIdx.x : min(nitems, (int)threadIdx.x * per_t);
      const int e_end = T2 ? nitems : min(nitems, e_begin + per_t);
      const int e_step = T2 ? (int)blockDim.x : 1;
      int bcur = -1;
      float Pn[3 * NO * (L + 1)];
      PairView<float> Pv;
      int bi = e_begin < e_end ? locate(s_scan32, e_begin) : 0;
      int pos = e_begin < e_end ? e_begin - s_scan32[bi] : 0;
      for (int e = e_begin; e < e_end; e += e_step) {
        while (pos >= s_scan32[bi + 1] - s_scan32[bi]) {
          pos -= s_scan32[bi + 1] - s_scan32[bi];
          bi++;
        }
        const int ib = b0 + bi;
        const int ik = (s_scan[bi + 1] - s_scan[bi]) + pos;
        pos += e_step;
        if (ib != bcur) {
          const PrimPairF P = braf[ib];
          bcur = ib;
          pair_polys<L, T2, float>(S, 0, P, Pn);
          Pv = view32(P);
        }
        acc32 += prim_quartet<L, TC, float, LK>(S, Pv, Pn, s_ketf[ik], s_qf + (size_t)ik * QW, s_boys32);
      }
    }
  }
  acc += (double)acc32;
  // block reduction in a fixed order
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) partial[w * split + part] = PI_5_2 * (((s_red[0] + s_red[1]) + s_red[2]) + s_red[3]);
}

#endif  // __CUDACC__

}  // namespace ss
