// one_e.cu -- one-electron integrals of the STO Gaussian fits: overlap S, nuclear attraction V
// and kinetic K for every function pair (i,k), as the reference's one_e_slater program computes
// them (src/one_e_slater.F90:81-89, src/one_elect.F90:1-105).
//
// One CTA per (i,k); its threads share the primitive products (m1, m2, cartesian component of
// each fit) and the block sums them in a fixed order, so results are run-to-run deterministic.
// Per primitive product:
//  * S: exp(-mu |A-B|^2) Ix Iy Iz, Ix = sqrt(pi/p) sum_{kx,lx} binomials (2k-1)!!/(2p)^k
//    (P-A)^kx (P-B)^lx (src/one_electron_sij.F90, src/one_electron_I.F90), skipped where
//    mu |A-B|^2 > -ln(1e-15) as the reference;
//  * K: the reference's three overlap terms (src/one_electron_Kij.F90);
//  * V: -sum_C Z_C NAI(A,B,C) (src/one_electron_Vij.F90, src/NAI_pol_mult.F90): per axis the
//    polynomial in t of I_x1_pol_mult_mono_elec, built bottom-up in the recursion's order
//      I(0,c) = (c-1) R2 I(0,c-2) + R1' I(0,c-1),  I(1,c) = c R2 I(0,c-1) + R1 I(0,c),
//      I(a,c) = (a-1) R2 I(a-2,c) + c R2 I(a-1,c-1) + R1 I(a-1,c)
//    with R1 = (P-A) - (P-C) t^2, R1' = (P-B) - (P-C) t^2, R2 = (1 - t^2)/(2p), then the product
//    of the three axes and sum_i d(2i) F_i(p |P-C|^2), coefficients below 1e-9 skipped as in
//    NAI_pol_mult.
#include <math.h>

#include <algorithm>

#include "boys.cuh"
#include "ss_common.cuh"
#include "ss_context.cuh"

namespace ss {

constexpr int OE_MAXP = 4;                     // per-axis power incl. the +2 of r^2 fits
constexpr int OE_DEG = 2 * (2 * OE_MAXP);      // degree in t of one axis polynomial (a + c <= 8)
constexpr int OE_TOT = 3 * OE_DEG;             // degree of the product of the three axes
constexpr int OE_NF = 8;                       // Boys orders: total power of the pair <= 8

__device__ double doublefact_d(int n) {  // src/doublefact.F90 (1 for n <= 2)
  if (n <= 2) return 1.0;
  double d = 1.0;
  for (int i = n; i >= 1; i -= 2) d = d * (double)i;
  return d;
}

__device__ double fact_d(int n) {
  double f = 1.0;
  for (int i = 2; i <= n; i++) f *= (double)i;
  return f;
}

__device__ double powi_d(double x, int k) {  // x**k by binary exponentiation
  double r = 1.0, b = x;
  while (k > 0) {
    if (k & 1) r *= b;
    b *= b;
    k >>= 1;
  }
  return r;
}

// src/one_electron_I.F90:1-29
__device__ double oe_I(int na, double ra, int nb, double rb, double gam, double rp) {
  double rint = 0.0;
  for (int kx = 0; kx <= na; kx++)
    for (int lx = 0; lx <= nb; lx++) {
      int kbig = na + nb - kx - lx;
      if (kbig % 2 == 1) continue;
      kbig = kbig / 2;
      const double f3 = doublefact_d(2 * kbig - 1);
      const double f2 = powi_d(1.0 / (2.0 * gam), kbig);
      const double bn = fact_d(na) / (fact_d(kx) * fact_d(na - kx));
      const double bl = fact_d(nb) / (fact_d(lx) * fact_d(nb - lx));
      rint = rint + f2 * f3 * bn * bl * powi_d(rp - ra, kx) * powi_d(rp - rb, lx);
    }
  return sqrt(3.14159265358979323846 / gam) * rint;
}

// src/one_electron_sij.F90:19-54
__device__ double oe_S(const int* na, const double* ra, double gamA, const int* nb, const double* rb, double gamB) {
  const double gamtot = gamA + gamB;
  const double rmu = gamA * gamB / gamtot;
  double rp[3];
  for (int l = 0; l < 3; l++) rp[l] = (gamA * ra[l] + gamB * rb[l]) / gamtot;
  const double x = ra[0] - rb[0], y = ra[1] - rb[1], z = ra[2] - rb[2];
  const double arg = rmu * (x * x + y * y + z * z);
  if (arg > 34.538776394910684) return 0.0;  // -ln(1e-15)
  double s = 1.0;
  for (int l = 0; l < 3; l++) s = s * oe_I(na[l], ra[l], nb[l], rb[l], gamtot, rp[l]);
  return exp(-arg) * s;
}

// src/one_electron_Kij.F90:1-46
__device__ double oe_K(const int* na, const double* ra, double gamA, const int* nb, const double* rb, double gamB) {
  int na2[3];
  const double sab = oe_S(na, ra, gamA, nb, rb, gamB);
  const double term1 = gamA * (3.0 + 2.0 * (na[0] + na[1] + na[2])) * sab;
  double sab_2 = 0.0;
  for (int l = 0; l < 3; l++) {
    for (int li = 0; li < 3; li++) na2[li] = na[li] + (li == l ? 2 : 0);
    sab_2 = sab_2 + oe_S(na2, ra, gamA, nb, rb, gamB);
  }
  const double term2 = -2.0 * gamA * gamA * sab_2;
  double sab_12 = 0.0;
  for (int l = 0; l < 3; l++) {
    for (int li = 0; li < 3; li++) na2[li] = (li == l && na[li] >= 2) ? na[li] - 2 : na[li];
    sab_12 = sab_12 + na[l] * (na[l] - 1) * oe_S(na2, ra, gamA, nb, rb, gamB);
  }
  return term1 + term2 + (-0.5 * sab_12);
}

// d += b (x) r with r = {r0, 0, r2} (multiply_poly_2 with a degree-2 polynomial in t)
__device__ __forceinline__ void oe_mul_add(const double* b, double r0, double r2, double* d) {
  for (int ib = 0; ib <= OE_DEG - 2; ib++) {
    if (b[ib] == 0.0) continue;
    d[ib] = d[ib] + r0 * b[ib];
    d[ib + 1] = d[ib + 1] + 0.0 * b[ib];
    d[ib + 2] = d[ib + 2] + r2 * b[ib];
  }
}

// per-axis polynomial I(a,c)(t) of I_x1_pol_mult_mono_elec (table over a' <= a, c' <= c)
__device__ void oe_axis(int a, int c, double r1_0, double r1p_0, double rpc, double p_inv_2,
                        double (&out)[OE_DEG + 1]) {
  double T[OE_MAXP + 1][OE_MAXP + 1][OE_DEG + 1];
  const double r1_2 = -rpc, r2_0 = p_inv_2, r2_2 = -p_inv_2;
  for (int cc = 0; cc <= c; cc++) {
    double* d = T[0][cc];
    for (int m = 0; m <= OE_DEG; m++) d[m] = 0.0;
    if (cc == 0) {
      d[0] = 1.0;
      continue;
    }
    double X[OE_DEG + 1];
    if (cc >= 2) {
      for (int m = 0; m <= OE_DEG; m++) X[m] = T[0][cc - 2][m] * (double)(cc - 1);
      oe_mul_add(X, r2_0, r2_2, d);
    }
    oe_mul_add(T[0][cc - 1], r1p_0, r1_2, d);
  }
  for (int aa = 1; aa <= a; aa++)
    for (int cc = 0; cc <= c; cc++) {
      double* d = T[aa][cc];
      for (int m = 0; m <= OE_DEG; m++) d[m] = 0.0;
      double X[OE_DEG + 1];
      if (aa == 1) {
        if (cc >= 1) {
          for (int m = 0; m <= OE_DEG; m++) X[m] = T[0][cc - 1][m] * (double)cc;
          oe_mul_add(X, r2_0, r2_2, d);
        }
        oe_mul_add(T[0][cc], r1_0, r1_2, d);
      } else {
        for (int m = 0; m <= OE_DEG; m++) X[m] = T[aa - 2][cc][m] * (double)(aa - 1);
        oe_mul_add(X, r2_0, r2_2, d);
        if (cc >= 1) {
          for (int m = 0; m <= OE_DEG; m++) X[m] = T[aa - 1][cc - 1][m] * (double)cc;
          oe_mul_add(X, r2_0, r2_2, d);
        }
        oe_mul_add(T[aa - 1][cc], r1_0, r1_2, d);
      }
    }
  for (int m = 0; m <= OE_DEG; m++) out[m] = T[a][c][m];
}

// src/NAI_pol_mult.F90:1-60
__device__ double oe_nai(const double* A, const double* B, const int* pA, const int* pB, double alpha, double beta,
                         const double* C, const double* s_boys) {
  const double two_pi = 2.0 * 3.14159265358979323846;
  const double p = alpha + beta, p_inv = 1.0 / p, rho = alpha * beta * p_inv;
  double dist = 0.0, dist_integral = 0.0, P[3];
  for (int i = 0; i < 3; i++) {
    P[i] = (alpha * A[i] + beta * B[i]) * p_inv;
    dist = dist + (A[i] - B[i]) * (A[i] - B[i]);
    dist_integral = dist_integral + (P[i] - C[i]) * (P[i] - C[i]);
  }
  const double cst = p * dist_integral;
  const double coeff = two_pi * exp(-(dist * rho)) * p_inv;
  double F[OE_NF + 1];
  const int n_pt = 2 * ((pA[0] + pB[0]) + (pA[1] + pB[1]) + (pA[2] + pB[2]));
  boys_tab<OE_NF>(cst, n_pt / 2, F, s_boys);
  if (n_pt == 0) return coeff * F[0];
  const double p_inv_2 = 0.5 / p;
  double dx[OE_DEG + 1], dy[OE_DEG + 1], dz[OE_DEG + 1];
  oe_axis(pA[0], pB[0], P[0] - A[0], P[0] - B[0], P[0] - C[0], p_inv_2, dx);
  oe_axis(pA[1], pB[1], P[1] - A[1], P[1] - B[1], P[1] - C[1], p_inv_2, dy);
  oe_axis(pA[2], pB[2], P[2] - A[2], P[2] - B[2], P[2] - C[2], p_inv_2, dz);
  double dxy[2 * OE_DEG + 1], d[OE_TOT + 1];
  for (int m = 0; m <= 2 * OE_DEG; m++) dxy[m] = 0.0;
  for (int m = 0; m <= OE_TOT; m++) d[m] = 0.0;
  for (int ib = 0; ib <= OE_DEG; ib++) {
    if (dx[ib] == 0.0) continue;
    for (int ic = 0; ic <= OE_DEG; ic++) dxy[ib + ic] = dxy[ib + ic] + dy[ic] * dx[ib];
  }
  for (int ib = 0; ib <= 2 * OE_DEG; ib++) {
    if (dxy[ib] == 0.0) continue;
    for (int ic = 0; ic <= OE_DEG; ic++) d[ib + ic] = d[ib + ic] + dz[ic] * dxy[ib];
  }
  double accu = 0.0;
  for (int i = 0; i <= n_pt; i += 2) {
    if (fabs(d[i]) < 1.e-9) continue;
    accu = accu + d[i] * F[i / 2];
  }
  return accu * coeff;
}

__global__ void __launch_bounds__(128) one_e_kernel(BasisDev B, int nat, const double* __restrict__ xyz,
                                                    const double* __restrict__ charge, double* __restrict__ S,
                                                    double* __restrict__ V, double* __restrict__ K) {
  __shared__ double s_boys[BOYS_SMEM_DOUBLES];
  __shared__ double s_red[3][4];
  boys_tables_to_smem(s_boys);
  __syncthreads();
  const int n = B.n;
  const int i = blockIdx.x % n, k = blockIdx.x / n;
  const int fn[2] = {i, k};
  int nc[2], ncomp[2][4][3], ct[2][4];
  for (int s = 0; s < 2; s++) {
    const int f = fn[s];
    const int* np = B.npower + 3 * f;
    const int it = B.i_type[f];
    if (it == 1) {
      nc[s] = 1;
      ct[s][0] = 0;
      for (int l = 0; l < 3; l++) ncomp[s][0][l] = np[l];
    } else if (it == 2) {
      nc[s] = 3;
      for (int ii = 0; ii < 3; ii++) {
        ct[s][ii] = 1;
        for (int l = 0; l < 3; l++) ncomp[s][ii][l] = np[l] + (l == ii ? 2 : 0);
      }
    } else {
      nc[s] = 4;
      for (int ii = 0; ii < 4; ii++) {
        ct[s][ii] = ii == 0 ? 0 : 1;
        for (int l = 0; l < 3; l++) ncomp[s][ii][l] = np[l] + (l == ii - 1 ? 2 : 0);
      }
    }
  }
  const double* A = B.center + 3 * i;
  const double* Bc = B.center + 3 * k;
  const int ngi = B.n_gauss[i], ngk = B.n_gauss[k];
  const int nitems = ngi * ngk * nc[0] * nc[1];
  double s = 0.0, v = 0.0, kin = 0.0;
  for (int e = threadIdx.x; e < nitems; e += blockDim.x) {
    int r = e;
    const int ii2 = r % nc[1]; r /= nc[1];
    const int ii1 = r % nc[0]; r /= nc[0];
    const int i2 = r % ngk;
    const int i1 = r / ngk;
    const double dd = B.c_gauss[i1 + (int64_t)B.ld * (i + (int64_t)n * ct[0][ii1])] *
                      B.c_gauss[i2 + (int64_t)B.ld * (k + (int64_t)n * ct[1][ii2])];
    const double ga = B.g_gauss[i1 + (int64_t)B.ld * i], gb = B.g_gauss[i2 + (int64_t)B.ld * k];
    s = s + dd * oe_S(ncomp[0][ii1], A, ga, ncomp[1][ii2], Bc, gb);
    double ac = 0.0;
    for (int kn = 0; kn < nat; kn++)
      ac = ac - charge[kn] * oe_nai(A, Bc, ncomp[0][ii1], ncomp[1][ii2], ga, gb, xyz + 3 * kn, s_boys);
    v = v + dd * ac;
    kin = kin + dd * oe_K(ncomp[0][ii1], A, ga, ncomp[1][ii2], Bc, gb);
  }
  double vals[3] = {s, v, kin};
  for (int t = 0; t < 3; t++) {
    double x = vals[t];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if ((threadIdx.x & 31) == 0) s_red[t][threadIdx.x >> 5] = x;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const int64_t o = i + (int64_t)n * k;
    S[o] = ((s_red[0][0] + s_red[0][1]) + s_red[0][2]) + s_red[0][3];
    V[o] = ((s_red[1][0] + s_red[1][1]) + s_red[1][2]) + s_red[1][3];
    K[o] = ((s_red[2][0] + s_red[2][1]) + s_red[2][2]) + s_red[2][3];
  }
}

int pool_get(ss_ctx* c, const char* name, size_t bytes, void** out);

}  // namespace ss

using namespace ss;

extern "C" {

int ss_nuclei_set(ss_ctx* c, int nat, const double* xyz, const double* charge) {
  if (!c) {
    ss_set_error_msg("null context");
    return SS_ERR_ARG;
  }
  if (nat < 0 || (nat > 0 && (!xyz || !charge))) {
    ss_set_error_msg("ss_nuclei_set: bad arguments (nat=%d)", nat);
    return SS_ERR_ARG;
  }
  c->h_nuc_xyz.assign(xyz, xyz + 3 * (size_t)nat);
  c->h_nuc_charge.assign(charge, charge + (size_t)nat);
  return SS_OK;
}

int ss_one_e(ss_ctx* c, double* S, double* V, double* K) {
  if (!c) {
    ss_set_error_msg("null context");
    return SS_ERR_ARG;
  }
  SS_CUDA_TRY(cudaSetDevice(c->device));
  if (!c->n) {
    ss_set_error_msg("ss_one_e needs ss_basis_set first");
    return SS_ERR_STATE;
  }
  for (int f = 0; f < c->n; f++) {
    int tot = c->h_itype[f] == 1 ? 0 : 2;
    for (int ax = 0; ax < 3; ax++) {
      tot += c->h_npower[3 * f + ax];
      if (c->h_npower[3 * f + ax] + (c->h_itype[f] == 1 ? 0 : 2) > OE_MAXP) {
        ss_set_error_msg("ss_one_e: function %d has a per-axis power above %d", f + 1, OE_MAXP);
        return SS_ERR_UNSUPPORTED;
      }
    }
    if (2 * tot > OE_NF) {
      ss_set_error_msg("ss_one_e: function %d has a total power above %d", f + 1, OE_NF / 2);
      return SS_ERR_UNSUPPORTED;
    }
  }
  const int n = c->n, nat = (int)c->h_nuc_charge.size();
  const size_t nn = (size_t)n * n;
  void *p_xyz, *p_ch, *p_out;
  int rc = pool_get(c, "oe_xyz", sizeof(double) * std::max<size_t>(3 * (size_t)nat, 1), &p_xyz);
  if (!rc) rc = pool_get(c, "oe_charge", sizeof(double) * std::max<size_t>((size_t)nat, 1), &p_ch);
  if (!rc) rc = pool_get(c, "oe_out", sizeof(double) * 3 * nn, &p_out);
  if (rc) return rc;
  if (nat) {
    SS_CUDA_TRY(cudaMemcpyAsync(p_xyz, c->h_nuc_xyz.data(), sizeof(double) * 3 * nat, cudaMemcpyHostToDevice,
                                c->stream));
    SS_CUDA_TRY(cudaMemcpyAsync(p_ch, c->h_nuc_charge.data(), sizeof(double) * nat, cudaMemcpyHostToDevice,
                                c->stream));
  }
  double* out = (double*)p_out;
  one_e_kernel<<<(unsigned)nn, 128, 0, c->stream>>>(c->basis, nat, (const double*)p_xyz, (const double*)p_ch, out,
                                                     out + nn, out + 2 * nn);
  SS_CUDA_TRY(cudaGetLastError());
  c->launches++;
  if (S) SS_CUDA_TRY(cudaMemcpyAsync(S, out, sizeof(double) * nn, cudaMemcpyDeviceToHost, c->stream));
  if (V) SS_CUDA_TRY(cudaMemcpyAsync(V, out + nn, sizeof(double) * nn, cudaMemcpyDeviceToHost, c->stream));
  if (K) SS_CUDA_TRY(cudaMemcpyAsync(K, out + 2 * nn, sizeof(double) * nn, cudaMemcpyDeviceToHost, c->stream));
  SS_CUDA_TRY(cudaStreamSynchronize(c->stream));
  return SS_OK;
}

}  // extern "C"
