// boys.cuh -- Boys function F_n(T) and exp(-T) of the analytic ERI kernel, table driven.
#pragma once
//
// FP64 is the roofline of the ERI stage, and one Boys evaluation per primitive quartet was
// about half of the FP64 instructions of the s-type classes.  These replace the library erf /
// exp and the term-by-term Taylor series with table-driven forms of the same quantities:
//
//  * exp_neg(x), x in [-745, 0]: Tang's table-driven method (ACM TOMS 15 (1989) 144-157):
//    k = rint(32 x / ln2), r = x - k ln2/32 (two-constant Cody-Waite reduction with FMA,
//    |r| <= ln2/64), exp(r) - 1 by its degree-6 Taylor polynomial (truncation < 3e-18),
//    2^(k/32) = 2^(k>>5) * 2^((k&31)/32) from a 32-entry table.  Error <= ~1 ulp.
//  * T >= 1, the reference's F_0 = sqrt(pi/T)/2 erf(sqrt T) (src/rint_sum.F90:44-61): for
//    T <= 36 F_0 comes from the Taylor series of F_0 around the nearest grid point T_k = 1+k/8,
//    F_0(T_k + d) = sum_{j<=8} F_j(T_k)/j! (-d)^j (d exact by Sterbenz, first omitted term
//    < 4e-17 relative); for T > 36 erf(sqrt T) is 1 in double and F_0 = sqrt(pi/T)/2 exactly as
//    in the reference.  The reference's upward recursion F_n = ((2n-1) F_{n-1} - e^-T)/(2T)
//    follows unchanged, so the F_n for n >= 1 carry the same recursion as the reference.
//  * T < 1 (the reference's per-order Taylor sums of src/rint1.F90): F_nf from the Taylor
//    series around T_k = k/16, F_nf(T_k + d) = sum_{j<8} F_{nf+j}(T_k) (-d)^j/j!, then the
//    stable downward recursion F_n = (2T F_{n+1} + e^-T)/(2n+1).
//
// The tables (boys_tables.cuh, from gen_boys_tables.py) are copied to shared memory once per
// CTA by boys_tables_to_smem.  Everything here is also valid host C++ (used by the host-side
// accuracy test of these functions against 40-digit values).
#include <math.h>
#include <stdint.h>
#include <string.h>

#include "boys_tables.cuh"

#ifdef __CUDACC__
#define SS_HD __host__ __device__ __forceinline__
#else
#define SS_HD inline
#endif

namespace ss {

constexpr int BOYS_SMEM_DOUBLES = BOYS_HI_K * BOYS_HI_J + BOYS_LO_K * BOYS_LO_N + 32;
constexpr double RINT_SHIFT = 6755399441055744.0;  // 1.5 * 2^52: x + SHIFT rounds x to an integer

SS_HD int64_t bits_of(double x) {
#ifdef __CUDA_ARCH__
  return __double_as_longlong(x);
#else
  int64_t v;
  memcpy(&v, &x, sizeof v);
  return v;
#endif
}
SS_HD double from_bits(int64_t v) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double(v);
#else
  double x;
  memcpy(&x, &v, sizeof x);
  return x;
#endif
}
SS_HD double rsqrt_d(double x) {
#ifdef __CUDA_ARCH__
  return rsqrt(x);
#else
  return 1.0 / sqrt(x);
#endif
}

// exp(x) for -745 < x <= 0 (normal results only: x >= -708)
SS_HD double exp_neg(double x, const double* e2) {
  const double t = fma(x, EXP_INV_LN2_32, RINT_SHIFT);
  const int k = (int)(bits_of(t) & 0xFFFFFFFFLL);  // low mantissa bits hold rint(32 x / ln2)
  const double kd = t - RINT_SHIFT;
  double r = fma(-kd, EXP_LN2_32_HI, x);
  r = fma(-kd, EXP_LN2_32_LO, r);
  double q = fma(r, 1.0 / 720.0, 1.0 / 120.0);
  q = fma(r, q, 1.0 / 24.0);
  q = fma(r, q, 1.0 / 6.0);
  q = fma(r, q, 0.5);
  q = fma(r, q, 1.0);
  const double tj = e2[k & 31];
  const double y = fma(tj, r * q, tj);
  // add k >> 5 (may be negative) to the exponent field; the shift is done on the unsigned bits
  return from_bits((int64_t)((uint64_t)bits_of(y) + ((uint64_t)(int64_t)(k >> 5) << 52)));
}

// F_0(T) for 1 <= T <= 36 from the grid Taylor table (rows of BOYS_HI_J coefficients)
SS_HD double boys0_hi(double T, const double* hi) {
  const double t = fma(T, 8.0, RINT_SHIFT - 8.0);
  const int k = (int)(bits_of(t) & 0xFFFFFFFFLL);  // rint(8 (T - 1))
  const double kd = t - RINT_SHIFT;
  const double x = fma(kd, 0.125, 1.0) - T;  // T_k - T, exact
  const double* a = hi + k * BOYS_HI_J;
  double s = a[8];
#pragma unroll
  for (int j = 7; j >= 0; j--) s = fma(s, x, a[j]);
  return s;
}

// F_nf(T) for 0 < T < 1 from the grid table of F_n(T_k)
SS_HD double boysn_lo(double T, int nf, const double* lo) {
  const double t = fma(T, 16.0, RINT_SHIFT);
  const int k = (int)(bits_of(t) & 0xFFFFFFFFLL);  // rint(16 T)
  const double kd = t - RINT_SHIFT;
  const double x = fma(kd, 0.0625, -T);  // T_k - T, exact
  const double* f = lo + k * BOYS_LO_N + nf;
  double s = f[7];
  s = fma(s, x * (1.0 / 7.0), f[6]);
  s = fma(s, x * (1.0 / 6.0), f[5]);
  s = fma(s, x * (1.0 / 5.0), f[4]);
  s = fma(s, x * (1.0 / 4.0), f[3]);
  s = fma(s, x * (1.0 / 3.0), f[2]);
  s = fma(s, x * 0.5, f[1]);
  s = fma(s, x, f[0]);
  return s;
}

// Boys values F_0..F_nf(T), nf <= NF <= BOYS_LO_N - 8.  tab = the shared-memory copy laid out
// as [hi | lo | exp2].
template <int NF>
SS_HD void boys_tab(double T, int nf, double (&F)[NF + 1], const double* tab) {
  static_assert(NF + 8 <= BOYS_LO_N, "Boys table too short for this order");
  const double* hi = tab;
  const double* lo = tab + BOYS_HI_K * BOYS_HI_J;
  const double* e2 = lo + BOYS_LO_K * BOYS_LO_N;
  const double sqpi = 1.7724538509055160273;  // dsqrt(dacos(-1.d0))
  // T >= 0: its range tests compare the bit pattern on the integer pipe (for non-negative
  // doubles the patterns order as the values), leaving the FP64 pipe to the arithmetic
  const int64_t tb = bits_of(T);
  if (tb < 0x3FF0000000000000LL) {  // T < 1
    if (tb == 0) {                   // T == +0
#pragma unroll
      for (int n = 0; n <= NF; n++) F[n] = 1.0 / (2 * n + 1);
      return;
    }
    const double s = boysn_lo(T, nf, lo);
    const double e = exp_neg(-T, e2);
    F[NF] = 0.0;
#pragma unroll
    for (int n = NF; n >= 0; n--) {
      if (n == nf) F[n] = s;
      else if (n < nf) F[n] = fma(T + T, F[n + 1 <= NF ? n + 1 : NF], e) * (1.0 / (2 * n + 1));
    }
  } else {
    const double v = (tb > 0x4054000000000000LL) ? 0.0 : exp_neg(-T, e2);  // T > 80
    const double u_inv = rsqrt_d(T);
    const double two_rho_inv = 0.5 * u_inv * u_inv;
    const double val0 = (tb > 0x4042000000000000LL) ? 0.5 * u_inv * sqpi : boys0_hi(T, hi);  // T > 36
    F[0] = val0;
    double rt = (val0 - v) * two_rho_inv;
    double di = 3.0;
#pragma unroll
    for (int n = 1; n <= NF; n++) {
      if (n > nf) break;
      F[n] = rt;
      rt = (rt * di - v) * two_rho_inv;
      di = di + 2.0;
    }
  }
}

// Single-precision Boys values F_0..F_nf(T) for the primitive quartets evaluated in FP32
// (relative error ~1e-7 plus the conditioning of T itself).  T < 30: F_nf from the Taylor series
// around T_k = k/8 with 6 terms (table rows F_n(T_k), n = 0..21, rounded to float), then the
// stable downward recursion F_n = (2T F_{n+1} + e^-T)/(2n+1).  T >= 30: F_0 = sqrt(pi/T)/2
// (erf(sqrt T) = 1 to 1e-14) and the upward recursion F_n = ((2n-1) F_{n-1} - e^-T)/(2T), stable
// there since (2n-1)/(2T) < 1.  tab32 = BOYS32_K x BOYS32_N floats.
template <int NF>
SS_HD void boys32(float T, int nf, float (&F)[NF + 1], const float* tab32) {
  static_assert(NF + 6 <= BOYS32_N, "FP32 Boys table too short for this order");
  if (T >= 30.f) {
    const float h = 0.5f / T;
    const float e = expf(-T);
    float f = 0.886226925452758f * sqrtf(h + h);  // sqrt(pi)/2 / sqrt(T)
    F[0] = f;
#pragma unroll
    for (int n = 1; n <= NF; n++) {
      if (n > nf) break;
      f = fmaf((float)(2 * n - 1), f, -e) * h;
      F[n] = f;
    }
    return;
  }
  const int k = (int)(T * 8.f + 0.5f);
  const float x = (float)k * 0.125f - T;  // T_k - T
  const float* f = tab32 + k * BOYS32_N + nf;
  float s = f[5];
  s = fmaf(s, x * 0.2f, f[4]);
  s = fmaf(s, x * 0.25f, f[3]);
  s = fmaf(s, x * (1.f / 3.f), f[2]);
  s = fmaf(s, x * 0.5f, f[1]);
  s = fmaf(s, x, f[0]);
  const float e = expf(-T);
  F[NF] = 0.f;
#pragma unroll
  for (int n = NF; n >= 0; n--) {
    if (n == nf) F[n] = s;
    else if (n < nf) F[n] = fmaf(T + T, F[n + 1 <= NF ? n + 1 : NF], e) * (1.f / (float)(2 * n + 1));
  }
}

#ifdef __CUDACC__
// cooperative copy of the three tables into shared memory (call before the first use, followed
// by a __syncthreads)
__device__ __forceinline__ void boys_tables_to_smem(double* s) {
  for (int t = threadIdx.x; t < BOYS_HI_K * BOYS_HI_J; t += blockDim.x) s[t] = boys_hi_tab[t];
  double* lo = s + BOYS_HI_K * BOYS_HI_J;
  for (int t = threadIdx.x; t < BOYS_LO_K * BOYS_LO_N; t += blockDim.x) lo[t] = boys_lo_tab[t];
  double* e2 = lo + BOYS_LO_K * BOYS_LO_N;
  for (int t = threadIdx.x; t < 32; t += blockDim.x) e2[t] = exp2_32_tab[t];
}
#endif

}  // namespace ss
