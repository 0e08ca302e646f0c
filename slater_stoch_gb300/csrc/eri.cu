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
constexpr double PI_5_2 = 34.9868366552;  // src/general_primitive_integral.F90:25

// (x - x_A)^a around x_P: coefficients of (x-x_P)^i, pw1 = x_P - x_A
// (src/give_explicit_poly_and_gaussian.F90:86-220, cases 0..4)
template <int L>
__device__ __forceinline__ void recentered(double pw1, int a, double (&P)[L + 1]) {
#pragma unroll
  for (int t = 0; t <= L; t++) P[t] = 0.0;
  if (a == 0) {
    P[0] = 1.0;
  } else if (a == 1) {
    P[0] = pw1;
    if (L >= 1) P[1 < L + 1 ? 1 : 0] = 1.0;
  } else if (a == 2) {
    double p2 = pw1 * pw1;
    P[0] = p2;
    if (L >= 2) { P[1 % (L + 1)] = 2.0 * pw1; P[2 % (L + 1)] = 1.0; }
  } else if (a == 3) {
    double p2 = pw1 * pw1, p3 = p2 * pw1;
    P[0] = p3;
    if (L >= 3) { P[1 % (L + 1)] = 3.0 * p2; P[2 % (L + 1)] = 3.0 * pw1; P[3 % (L + 1)] = 1.0; }
  } else {  // a == 4
    double p2 = pw1 * pw1, p3 = p2 * pw1, p4 = p2 * p2;
    P[0] = p4;
    if (L >= 4) {
      P[1 % (L + 1)] = 4.0 * p3; P[2 % (L + 1)] = 6.0 * p2; P[3 % (L + 1)] = 4.0 * pw1;
      P[4 % (L + 1)] = 1.0;
    }
  }
}

// P_new = recentered(A,a) * recentered(B,b) in multiply_poly's order (src/multiply_poly.F90:22-31)
template <int L>
__device__ __forceinline__ void pair_poly(double pa, int a, double pb, int b, double (&Pn)[L + 1]) {
  double Pa[L + 1], Pb[L + 1];
  recentered<L>(pa, a, Pa);
  recentered<L>(pb, b, Pb);
#pragma unroll
  for (int t = 0; t <= L; t++) Pn[t] = 0.0;
#pragma unroll
  for (int ib = 0; ib <= L; ib++)
#pragma unroll
    for (int ic = 0; ic <= L; ic++)
      if (ib + ic <= L && ib <= a && ic <= b) Pn[ib + ic] = Pn[ib + ic] + Pb[ic] * Pa[ib];
}

struct RecCoef {
  double p10_1, p10_2, p01_1, p01_2, pq_inv;
};

// Bottom-up table I(a,c)[m] (u-coefficients) for a <= amax, c <= cmax (both <= L).
template <int L>
__device__ __forceinline__ void rys_table(const RecCoef& R, double Cc, double Dd, int amax, int cmax,
                                          double (&I)[L + 1][L + 1][2 * L + 1]) {
#pragma unroll
  for (int c = 0; c <= L; c++) {
    if (c > cmax) break;
#pragma unroll
    for (int m = 0; m <= 2 * L; m++) {
      double v = 0.0;
      if (c == 0) {
        v = (m == 0) ? 1.0 : 0.0;
      } else {
        if (c >= 2) {
          // (c-1) B01 I(0,c-2): X scaled first, then d[m] += -p01_2 X[m-1]; d[m] += p01_1 X[m]
          if (m >= 1 && m - 1 <= c - 2) v = v + (-R.p01_2) * (I[0][c - 2][m - 1] * (double)(c - 1));
          if (m <= c - 2) v = v + R.p01_1 * (I[0][c - 2][m] * (double)(c - 1));
        }
        if (m >= 1 && m - 1 <= c - 1) v = v + Dd * I[0][c - 1][m - 1];
      }
      I[0][c][m] = v;
    }
  }
#pragma unroll
  for (int a = 1; a <= L; a++) {
    if (a > amax) break;
#pragma unroll
    for (int c = 0; c <= L; c++) {
      if (c > cmax) break;
#pragma unroll
      for (int m = 0; m <= 2 * L; m++) {
        double v = 0.0;
        if (a >= 2) {
          double s = (double)(a - 1);
          if (m >= 1 && m - 1 <= a - 2 + c) v = v + (-R.p10_2) * (I[a - 2][c][m - 1] * s);
          if (m <= a - 2 + c) v = v + R.p10_1 * (I[a - 2][c][m] * s);
        }
        if (c >= 1 && m >= 1 && m - 1 <= a - 1 + c - 1)
          v = v + R.pq_inv * (I[a - 1][c - 1][m - 1] * (double)c);
        if (m >= 1 && m - 1 <= a - 1 + c) v = v + Cc * I[a - 1][c][m - 1];
        I[a][c][m] = v;
      }
    }
  }
}

// Sum_{ix,jx} (Pn[ix] Qn[jx]) I(ix,jx) with the reference's thresholds; x_axis uses
// "skip if |P| < thresh", y/z "process if |P| > thresh".  Returns false if identically zero.
template <int L>
__device__ __forceinline__ bool axis_poly(const double (&Pn)[L + 1], int degP, const double (&Qn)[L + 1],
                                          int degQ, const double (&I)[L + 1][L + 1][2 * L + 1],
                                          bool x_axis, double (&out)[2 * L + 1]) {
#pragma unroll
  for (int m = 0; m <= 2 * L; m++) out[m] = 0.0;
  bool any = false;
#pragma unroll
  for (int ix = 0; ix <= L; ix++) {
    if (ix > degP) break;
    double a = Pn[ix];
    bool take = x_axis ? !(fabs(a) < THRESH) : (fabs(a) > THRESH);
    if (!take) continue;
#pragma unroll
    for (int jx = 0; jx <= L; jx++) {
      if (jx > degQ) break;
      double d = a * Qn[jx];
      if (fabs(d) < THRESH) continue;
      any = true;
#pragma unroll
      for (int m = 0; m <= 2 * L; m++)
        if (m <= ix + jx) out[m] = out[m] + d * I[ix][jx][m];
    }
  }
  if (!any) return false;
  bool nz = false;
#pragma unroll
  for (int m = 0; m <= 2 * L; m++) nz |= (out[m] != 0.0);
  return nz;
}

// Boys values F_0..F_nf(T) with the regimes of src/rint_sum.F90:27-65 (nf <= 20).
__device__ __forceinline__ void boys(double T, int nf, double* F) {
  const double sqpi = 1.7724538509055160273;  // dsqrt(dacos(-1.d0))
  if (T < 1.0) {
    if (T == 0.0) {
      F[0] = 1.0;
      for (int n = 1; n <= nf; n++) F[n] = 1.0 / (double)(n + n + 1);
      return;
    }
    double u_inv = 1.0 / sqrt(T);
    double u = T * u_inv;
    F[0] = 0.5 * u_inv * sqpi * erf(u);
    // rint1 (src/rint1.F90:29-41): sum_k (-T)^k/k! / (2(k+n)+1), stop at first |term| <= 1e-15
    double ak[21];
    double rt = 1.0, fk = 1.0;
#pragma unroll
    for (int k = 1; k <= 20; k++) {
      rt = -rt * T;
      fk = fk * (double)k;
      ak[k] = rt * (1.0 / fk);
    }
    for (int n = 1; n <= nf; n++) {
      double r = 1.0 / (double)(n + n + 1);
      for (int k = 1; k <= 20; k++) {
        double diff = ak[k] * (1.0 / (double)(2 * (k + n) + 1));
        r = r + diff;
        if (!(fabs(diff) > 1.e-15)) break;
      }
      F[n] = r;
    }
  } else {
    double v = (T > 80.0) ? 0.0 : exp(-T);
    double u_inv = 1.0 / sqrt(T);
    double u = T * u_inv;
    double two_rho_inv = 0.5 * u_inv * u_inv;
    double val0 = 0.5 * u_inv * sqpi * erf(u);
    F[0] = val0;
    double rt = (val0 - v) * two_rho_inv;
    double di = 3.0;
    for (int n = 1; n <= nf; n++) {
      F[n] = rt;
      rt = (rt * di - v) * two_rho_inv;
      di = di + 2.0;
    }
  }
}

struct QuartetDesc {
  int np[4][3];  // npower of i, k, j, l
  int t2[4];     // 1 if the function is an r^2-type fit (3 components)
  int nf;        // highest Boys order needed
};

__device__ __forceinline__ int comp_pow(const QuartetDesc& D, int f, int comp, int ax) {
  return D.np[f][ax] + ((D.t2[f] && comp == ax) ? 2 : 0);
}

template <int L>
__global__ void __launch_bounds__(128) eri_kernel(
    BasisDev B, const PrimPair* __restrict__ pp, const int64_t* __restrict__ pair_off,
    const int* __restrict__ pair_cnt, const int64_t* __restrict__ work, int split,
    const int32_t* __restrict__ is, const int32_t* __restrict__ js, const int32_t* __restrict__ ks,
    const int32_t* __restrict__ ls, double* __restrict__ partial) {
  extern __shared__ double2 s_raw[];
  PrimPair* s_ket = reinterpret_cast<PrimPair*>(s_raw);
  __shared__ double s_red[4];

  const int64_t w = blockIdx.x / split;
  const int part = blockIdx.x % split;
  const int64_t q = work[w];
  const int fi = is[q] - 1, fk = ks[q] - 1, fj = js[q] - 1, fl = ls[q] - 1;
  const int64_t pb = ss_pair_index(fi, fk), pk = ss_pair_index(fj, fl);
  const int nb = pair_cnt[pb], nk = pair_cnt[pk];
  const PrimPair* bra = pp + pair_off[pb];
  const PrimPair* ket = pp + pair_off[pk];

  {
    const double2* src = reinterpret_cast<const double2*>(ket);
    double2* dst = s_raw;
    for (int t = threadIdx.x; t < nk * 8; t += blockDim.x) dst[t] = src[t];
  }

  QuartetDesc D;
  const int fn[4] = {fi, fk, fj, fl};
  int ptot[4];
#pragma unroll
  for (int f = 0; f < 4; f++) {
    D.t2[f] = (B.i_type[fn[f]] == 2);
    ptot[f] = 0;
#pragma unroll
    for (int ax = 0; ax < 3; ax++) {
      D.np[f][ax] = B.npower[3 * fn[f] + ax];
      ptot[f] += D.np[f][ax];
    }
  }
  D.nf = ptot[0] + ptot[1] + ptot[2] + ptot[3] + 2 * (D.t2[0] + D.t2[1] + D.t2[2] + D.t2[3]);
  const int nci = D.t2[0] ? 3 : 1, nck = D.t2[1] ? 3 : 1, ncj = D.t2[2] ? 3 : 1, ncl = D.t2[3] ? 3 : 1;
  // per-axis maxima of a+b (bra) and c+d (ket)
  int amax[3], cmax[3];
#pragma unroll
  for (int ax = 0; ax < 3; ax++) {
    int am = 0, cm = 0;
    for (int ci = 0; ci < nci; ci++)
      for (int ck = 0; ck < nck; ck++) {
        int v = comp_pow(D, 0, ci, ax) + comp_pow(D, 1, ck, ax);
        am = v > am ? v : am;
      }
    for (int cj = 0; cj < ncj; cj++)
      for (int cl = 0; cl < ncl; cl++) {
        int v = comp_pow(D, 2, cj, ax) + comp_pow(D, 3, cl, ax);
        cm = v > cm ? v : cm;
      }
    amax[ax] = am;
    cmax[ax] = cm;
  }
  __syncthreads();

  double acc = 0.0;
  const int per = (nb + split - 1) / split;
  const int b0 = part * per;
  const int b1 = min(nb, b0 + per);
  for (int b = b0 + threadIdx.x; b < b1; b += blockDim.x) {
    const PrimPair P = bra[b];
    for (int kk = 0; kk < nk; kk++) {
      const PrimPair& Q = s_ket[kk];
      const double p = P.p, qq = Q.p;
      // src/general_primitive_integral.F90:54-60
      const double pq = P.p_inv * 0.5 * Q.p_inv;
      const double pq_inv = 0.5 / (p + qq);
      RecCoef R;
      R.p10_1 = qq * pq;
      R.p01_1 = p * pq;
      const double pq_inv_2 = pq_inv + pq_inv;
      R.p10_2 = pq_inv_2 * R.p10_1 * qq;
      R.p01_2 = pq_inv_2 * R.p01_1 * p;
      R.pq_inv = pq_inv;
      // src/general_primitive_integral.F90:142-146
      const double rho = p * qq * pq_inv_2;
      const double dx = P.P[0] - Q.P[0], dy = P.P[1] - Q.P[1], dz = P.P[2] - Q.P[2];
      const double dist = dx * dx + dy * dy + dz * dz;
      const double T = dist * rho;

      double I[3][L + 1][L + 1][2 * L + 1];
#pragma unroll
      for (int ax = 0; ax < 3; ax++) {
        const double Cc = -qq * (P.P[ax] - Q.P[ax]) * pq_inv_2;  // src/give_polynom_mult_center_x.F90:58
        const double Dd = -p * (Q.P[ax] - P.P[ax]) * pq_inv_2;   // :62
        rys_table<L>(R, Cc, Dd, amax[ax], cmax[ax], I[ax]);
      }
      double F[SS_MAX_NF + 1];
      boys(T, D.nf, F);
      double accu_all = 0.0;
      for (int ci = 0; ci < nci; ci++)
        for (int ck = 0; ck < nck; ck++)
          for (int cj = 0; cj < ncj; cj++)
            for (int cl = 0; cl < ncl; cl++) {
              double Ax[3][2 * L + 1];
              bool zero = false;
#pragma unroll
              for (int ax = 0; ax < 3; ax++) {
                const int a = comp_pow(D, 0, ci, ax), bb = comp_pow(D, 1, ck, ax);
                const int c = comp_pow(D, 2, cj, ax), d = comp_pow(D, 3, cl, ax);
                double Pn[L + 1], Qn[L + 1];
                pair_poly<L>(P.PA[ax], a, P.PB[ax], bb, Pn);
                pair_poly<L>(Q.PA[ax], c, Q.PB[ax], d, Qn);
                if (!axis_poly<L>(Pn, a + bb, Qn, c + d, I[ax], ax == 0, Ax[ax])) zero = true;
              }
              if (zero) continue;
              // d_poly = Ix*Iy, d1 = d_poly*Iz (src/general_primitive_integral.F90:148-161)
              double dp[4 * L + 1];
#pragma unroll
              for (int t = 0; t <= 4 * L; t++) dp[t] = 0.0;
#pragma unroll
              for (int ib = 0; ib <= 2 * L; ib++)
#pragma unroll
                for (int ic = 0; ic <= 2 * L; ic++) dp[ib + ic] = dp[ib + ic] + Ax[1][ic] * Ax[0][ib];
              double d1[6 * L + 1];
#pragma unroll
              for (int t = 0; t <= 6 * L; t++) d1[t] = 0.0;
#pragma unroll
              for (int ib = 0; ib <= 4 * L; ib++)
#pragma unroll
                for (int ic = 0; ic <= 2 * L; ic++) d1[ib + ic] = d1[ib + ic] + Ax[2][ic] * dp[ib];
              // rint_sum: F_0 term first, then increasing order (src/rint_sum.F90:27-65)
              double accu = d1[0] * F[0];
#pragma unroll
              for (int n = 1; n <= 6 * L; n++)
                if (n <= D.nf && n <= SS_MAX_NF) accu = accu + d1[n] * F[n];
              accu_all = accu_all + accu;
            }
      // src/general_primitive_integral.F90:192 and the coefficient product of src/gauss_ijkl.F90:137
      const double pref = P.fact * Q.fact * PI_5_2 * P.p_inv * Q.p_inv / sqrt(p + qq);
      acc = acc + (P.coef * Q.coef) * (pref * accu_all);
    }
  }
  // block reduction in a fixed order
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) partial[w * split + part] = ((s_red[0] + s_red[1]) + s_red[2]) + s_red[3];
}

// Primitive-pair table for function pair (i,k), i >= k: one thread per (m1,m2); compacts
// screened pairs away deterministically with a per-pair prefix over m1-rows.
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
  int local = 0;
  for (int t = threadIdx.x; t < ngi * ngk; t += blockDim.x) {
    int m1 = t / ngk, m2 = t % ngk;
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
  // sequential compaction in (m1, m2) order by thread 0 (ng <= 30: at most 900 entries)
  if (threadIdx.x != 0) return;
  int64_t o = off[pidx];
  for (int m1 = 0; m1 < ngi; m1++)
    for (int m2 = 0; m2 < ngk; m2++) {
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
      r.pad[0] = r.pad[1] = r.pad[2] = 0.0;
      out[o++] = r;
    }
}

// partial sums -> ERIs; diagonal reuse and Schwarz screening (src/two_e_slater.F90:264-279)
__global__ void eri_finalize(int64_t nint, const int32_t* __restrict__ is, const int32_t* __restrict__ js,
                             const int32_t* __restrict__ ks, const int32_t* __restrict__ ls,
                             const int64_t* __restrict__ slot, int split, const double* __restrict__ partial,
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
    for (int t = 0; t < split; t++) v = v + partial[s * split + t];
  }
  out[q] = v;
}

__global__ void precond_finalize(int n, int split, const double* __restrict__ partial,
                                 double* __restrict__ pre) {
  int64_t pidx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  int64_t np = (int64_t)n * (n + 1) / 2;
  if (pidx >= np) return;
  int i = (int)((sqrt(8.0 * pidx + 1.0) - 1.0) * 0.5);
  while ((int64_t)i * (i + 1) / 2 > pidx) i--;
  while ((int64_t)(i + 1) * (i + 2) / 2 <= pidx) i++;
  int k = (int)(pidx - (int64_t)i * (i + 1) / 2);
  double v = 0.0;
  for (int t = 0; t < split; t++) v = v + partial[pidx * split + t];
  pre[i + (int64_t)n * k] = v;
  pre[k + (int64_t)n * i] = v;
}

// Launch helpers ------------------------------------------------------------------------
size_t eri_smem_bytes(int max_cnt) { return (size_t)max_cnt * sizeof(PrimPair); }

cudaError_t launch_eri_class(int L, dim3 grid, size_t smem, cudaStream_t st, const BasisDev& B,
                             const PrimPair* pp, const int64_t* off, const int* cnt,
                             const int64_t* work, int split, const int32_t* is, const int32_t* js,
                             const int32_t* ks, const int32_t* ls, double* partial) {
#define SS_ERI_CASE(LL)                                                                          \
  case LL: {                                                                                     \
    cudaError_t e = cudaFuncSetAttribute(eri_kernel<LL>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                                         (int)smem);                                             \
    if (e != cudaSuccess) return e;                                                              \
    eri_kernel<LL><<<grid, 128, smem, st>>>(B, pp, off, cnt, work, split, is, js, ks, ls, partial); \
    return cudaGetLastError();                                                                   \
  }
  switch (L) {
    SS_ERI_CASE(0)
    SS_ERI_CASE(1)
    SS_ERI_CASE(2)
    SS_ERI_CASE(3)
    SS_ERI_CASE(4)
    default:
      return cudaErrorInvalidValue;
  }
#undef SS_ERI_CASE
}

}  // namespace ss
