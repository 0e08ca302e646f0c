// mc.cu -- ZV-MC correction kernels: walker sampler, faithful per-pair ZV map and densities,
// FP64 / REF32 accumulation, block statistics (replaces src/two_e_slater.F90:386-496).
#include <math.h>

#include "philox.cuh"
#include "ss_common.cuh"
#include "mc.cuh"

namespace ss {

// ---------------------------------------------------------------------------------------
// walkers
// ---------------------------------------------------------------------------------------
__device__ __forceinline__ void walker_normals(uint64_t seed, int64_t s, double (&n)[6]) {
#pragma unroll
  for (int j = 0; j < 3; j++) {
    uint32_t c[4] = {(uint32_t)s, (uint32_t)((uint64_t)s >> 32), (uint32_t)j, STREAM_WALKER};
    philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
    n[2 * j] = normcdfinv(u01_open(c[0], c[1]));
    n[2 * j + 1] = normcdfinv(u01_open(c[2], c[3]));
  }
}

// r1, r2: [3*S] walker-major.  Standard normals as draw_configuration returns.
__global__ void draw_walkers_kernel(uint64_t seed, int64_t first, int64_t S, double* __restrict__ r1,
                                    double* __restrict__ r2) {
  int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s >= S) return;
  double n[6];
  walker_normals(seed, first + s, n);
  r1[3 * s] = n[0]; r1[3 * s + 1] = n[1]; r1[3 * s + 2] = n[2];
  r2[3 * s] = n[3]; r2[3 * s + 1] = n[4]; r2[3 * s + 2] = n[5];
}

// per walker: |r1|, |r2|, pi_0 (src/compute_jacobian_and_pi0.F90:12-18)
__global__ void walker_aux_kernel(int64_t S, const double* __restrict__ r1, const double* __restrict__ r2,
                                  double* __restrict__ r1m, double* __restrict__ r2m, double* __restrict__ pi0) {
  int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s >= S) return;
  const double fpi0 = 1.0 / ((2.0 * M_PI) * (2.0 * M_PI) * (2.0 * M_PI));
  double a0 = r1[3 * s], a1 = r1[3 * s + 1], a2 = r1[3 * s + 2];
  double b0 = r2[3 * s], b1 = r2[3 * s + 1], b2 = r2[3 * s + 2];
  double m1 = a0 * a0 + a1 * a1 + a2 * a2;
  double m2 = b0 * b0 + b1 * b1 + b2 * b2;
  r1m[s] = sqrt(m1);
  r2m[s] = sqrt(m2);
  pi0[s] = exp(-0.5 * (m1 + m2)) * fpi0;
}

// ---------------------------------------------------------------------------------------
// pair densities (src/compute_densities.F90, src/u_orb.F90, src/u_gauss.F90)
// ---------------------------------------------------------------------------------------
__device__ __forceinline__ double u_orb(int nsto, double g, double r) {
  switch (nsto) {  // c_contract = 1 (src/read_basis.F90:35)
    case 0: return exp(-g * r);
    case 1: return r * exp(-g * r);
    case 2: return (r * r) * exp(-g * r);
    case 3: return (r * r) * r * exp(-g * r);
    case 4: { double r2 = r * r; return r2 * r2 * exp(-g * r); }
    default: return pow(r, (double)nsto) * exp(-g * r);
  }
}

__device__ __forceinline__ double u_gauss(const BasisDev& B, int i, double r) {
  const double r2 = r * r;
  double u = 0.0;
  const int ng = B.n_gauss[i];
  const double* c1 = B.c_gauss + (int64_t)B.ld * i;
  const double* c2 = B.c_gauss + (int64_t)B.ld * (i + (int64_t)B.n);
  const double* g = B.g_gauss + (int64_t)B.ld * i;
  for (int m = 0; m < ng; m++) u = u + (c1[m] + c2[m] * r2) * exp(-g[m] * r2);
  return u;
}

__device__ __forceinline__ void pair_density(const BasisDev& B, int i, int k, const double (&u)[3],
                                             double& rS, double& rG) {
  const double* ci = B.center + 3 * i;
  const double* ck = B.center + 3 * k;
  double dx = u[0] - ci[0], dy = u[1] - ci[1], dz = u[2] - ci[2];
  double poly_i = 1.0;
  for (int t = 0; t < B.npower[3 * i]; t++) poly_i = poly_i * dx;
  for (int t = 0; t < B.npower[3 * i + 1]; t++) poly_i = poly_i * dy;
  for (int t = 0; t < B.npower[3 * i + 2]; t++) poly_i = poly_i * dz;
  const double r_i = sqrt(dx * dx + dy * dy + dz * dz);
  dx = u[0] - ck[0]; dy = u[1] - ck[1]; dz = u[2] - ck[2];
  double poly_k = 1.0;
  for (int t = 0; t < B.npower[3 * k]; t++) poly_k = poly_k * dx;
  for (int t = 0; t < B.npower[3 * k + 1]; t++) poly_k = poly_k * dy;
  for (int t = 0; t < B.npower[3 * k + 2]; t++) poly_k = poly_k * dz;
  const double r_k = sqrt(dx * dx + dy * dy + dz * dz);
  const double poly_ik = poly_i * poly_k;
  rS = poly_ik * u_orb(B.n_sto[i], B.g_slater[i], r_i) * u_orb(B.n_sto[k], B.g_slater[k], r_k);
  rG = poly_ik * u_gauss(B, i, r_i) * u_gauss(B, k, r_k);
}

// One thread per (walker, used pair): ZV map (src/two_e_slater.F90:406-411), densities,
// Jacobians (src/compute_jacobian_and_pi0.F90:22-30).  FP64 mode folds the Jacobians and
// 1/pi_0 into the density columns; REF32 mode keeps them apart for the single-precision
// weight of src/two_e_slater.F90:442.
template <int MODE>
__global__ void zv_pair_kernel(BasisDev B, ZvPairs P, int64_t S, const double* __restrict__ r1,
                               const double* __restrict__ r2, const double* __restrict__ r1m,
                               const double* __restrict__ r2m, const double* __restrict__ pi0,
                               ZvChunk Z) {
  const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int p = blockIdx.y;
  if (s >= S) return;
  const int i = P.i[p], k = P.k[p];
  const double fzv = P.fzv[p], fjac = P.fjac[p];
  const double a1 = r1m[s], a2 = r2m[s];
  double u1[3], u2[3];
#pragma unroll
  for (int l = 0; l < 3; l++) {
    u1[l] = fzv * r1[3 * s + l] * a1 + P.G[3 * p + l];
    u2[l] = fzv * r2[3 * s + l] * a2 + P.G[3 * p + l];
  }
  double rs1, rg1, rs2, rg2;
  pair_density(B, i, k, u1, rs1, rg1);
  pair_density(B, i, k, u2, rs2, rg2);
  const double f1 = fjac * a1, f2 = fjac * a2;
  const double j1 = 0.25 * fabs(f1 * f1 * f1);
  const double j2 = 0.25 * fabs(f2 * f2 * f2);
  const int64_t o = (int64_t)p * Z.ld + s;
  Z.u1x[o] = u1[0]; Z.u1y[o] = u1[1]; Z.u1z[o] = u1[2];
  Z.u2x[o] = u2[0]; Z.u2y[o] = u2[1]; Z.u2z[o] = u2[2];
  if (MODE == SS_PREC_FP64) {
    const double ip = 1.0 / pi0[s];
    Z.a_s[o] = j1 * rs1;
    Z.a_g[o] = j1 * rg1;
    Z.b_s[o] = j2 * rs2 * ip;
    Z.b_g[o] = j2 * rg2 * ip;
  } else {
    Z.a_s[o] = rs1;
    Z.a_g[o] = rg1;
    Z.b_s[o] = rs2;
    Z.b_g[o] = rg2;
    Z.j1[o] = j1;
    Z.j2[o] = j2;
  }
}

// Accumulation (src/two_e_slater.F90:424-453).  One CTA per (bra pair, walker slice); each
// warp takes the quartets of the bra pair in turn, lanes stride over walkers.  Each
// quartet is summed by a single warp, so partials are deterministic.
template <int MODE>
__global__ void __launch_bounds__(256) zv_accum_kernel(int64_t S, ZvCsr Q, int nsplit, ZvChunk Z,
                                                       const double* __restrict__ pi0,
                                                       double* __restrict__ partS,
                                                       double* __restrict__ partG) {
  const int b = blockIdx.x / nsplit, sp = blockIdx.x % nsplit;
  const int p1 = Q.bra[b];
  const int64_t e0 = Q.off[b], e1 = Q.off[b + 1];
  const int64_t per = (S + nsplit - 1) / nsplit;
  const int64_t w0 = sp * per, w1 = min(S, w0 + per);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarp = blockDim.x >> 5;
  const int64_t o1 = (int64_t)p1 * Z.ld;
  for (int64_t e = e0 + warp; e < e1; e += nwarp) {
    const int64_t q = Q.q[e];
    const int64_t o2 = (int64_t)Q.ket[e] * Z.ld;
    double sS = 0.0, sG = 0.0;
    for (int64_t s = w0 + lane; s < w1; s += 32) {
      const double dx = Z.u1x[o1 + s] - Z.u2x[o2 + s];
      const double dy = Z.u1y[o1 + s] - Z.u2y[o2 + s];
      const double dz = Z.u1z[o1 + s] - Z.u2z[o2 + s];
      const double r12_2 = dx * dx + dy * dy + dz * dz;
      if (MODE == SS_PREC_FP64) {
        const double inv = rsqrt(r12_2);
        sS = fma(Z.a_s[o1 + s], Z.b_s[o2 + s] * inv, sS);
        sG = fma(Z.a_g[o1 + s], Z.b_g[o2 + s] * inv, sG);
      } else {
        const double rj = Z.j1[o1 + s] * Z.j2[o2 + s];
        const double factor = (double)(__fdiv_rn((float)rj, (float)pi0[s]));
        const double inv = (double)(__fdiv_rn(1.0f, __fsqrt_rn((float)r12_2)));
        const double wS = factor * Z.a_s[o1 + s] * Z.b_s[o2 + s];
        const double wG = factor * Z.a_g[o1 + s] * Z.b_g[o2 + s];
        sS = sS + wS * inv;
        sG = sG + wG * inv;
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      sS += __shfl_down_sync(0xffffffffu, sS, o);
      sG += __shfl_down_sync(0xffffffffu, sG, o);
    }
    if (lane == 0) {
      partS[q * nsplit + sp] = sS;
      partG[q * nsplit + sp] = sG;
    }
  }
}

__global__ void zv_reduce_partials(int64_t nint, int nsplit, const double* __restrict__ partS,
                                   const double* __restrict__ partG, double* __restrict__ eS,
                                   double* __restrict__ eG) {
  int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (q >= nint) return;
  double a = 0.0, g = 0.0;
  for (int t = 0; t < nsplit; t++) {
    a += partS[q * nsplit + t];
    g += partG[q * nsplit + t];
  }
  eS[q] += a;
  eG[q] += g;
}

// block moments (src/two_e_slater.F90:463-481)
__global__ void zv_block_stats(int64_t nint, int64_t npts, double* __restrict__ eS, double* __restrict__ eG,
                               double* __restrict__ acc, double* __restrict__ acc2) {
  int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (q >= nint) return;
  const double factor = 1.0 / (double)npts;
  const double x = eS[q] * factor - eG[q] * factor;
  acc[q] += x;
  acc2[q] += x * x;
  eS[q] = 0.0;
  eG[q] = 0.0;
}

// mean and error (src/two_e_slater.F90:488-492); unbiased=1 uses sqrt(var/(nb-1))
__global__ void zv_final(int64_t nint, int nb, int unbiased, const double* __restrict__ acc,
                         const double* __restrict__ acc2, double* __restrict__ mean,
                         double* __restrict__ sigma, unsigned long long* __restrict__ max_sigma_bits) {
  int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (q >= nint) return;
  const double m = acc[q] / nb, m2 = acc2[q] / nb;
  double e;
  if (unbiased)
    e = nb > 1 ? sqrt(fabs(m2 - m * m) / (double)(nb - 1)) : 0.0;
  else
    e = sqrt(fabs(m2 - m * m)) / sqrt((double)nb);
  mean[q] = m;
  sigma[q] = e;
  if (max_sigma_bits) atomicMax(max_sigma_bits, (unsigned long long)__double_as_longlong(e));
}

// ---------------------------------------------------------------------------------------
// launch wrappers
// ---------------------------------------------------------------------------------------
cudaError_t launch_draw_walkers(cudaStream_t st, uint64_t seed, int64_t first, int64_t S, double* r1,
                                double* r2) {
  if (S <= 0) return cudaSuccess;
  draw_walkers_kernel<<<(unsigned)((S + 255) / 256), 256, 0, st>>>(seed, first, S, r1, r2);
  return cudaGetLastError();
}

cudaError_t launch_walker_aux(cudaStream_t st, int64_t S, const double* r1, const double* r2, double* r1m,
                              double* r2m, double* pi0) {
  if (S <= 0) return cudaSuccess;
  walker_aux_kernel<<<(unsigned)((S + 255) / 256), 256, 0, st>>>(S, r1, r2, r1m, r2m, pi0);
  return cudaGetLastError();
}

cudaError_t launch_zv_pairs(cudaStream_t st, int mode, const BasisDev& B, const ZvPairs& P, int npairs,
                            int64_t S, const double* r1, const double* r2, const double* r1m,
                            const double* r2m, const double* pi0, const ZvChunk& Z) {
  dim3 grid((unsigned)((S + 127) / 128), (unsigned)npairs);
  if (mode == SS_PREC_FP64)
    zv_pair_kernel<SS_PREC_FP64><<<grid, 128, 0, st>>>(B, P, S, r1, r2, r1m, r2m, pi0, Z);
  else
    zv_pair_kernel<SS_PREC_REF32><<<grid, 128, 0, st>>>(B, P, S, r1, r2, r1m, r2m, pi0, Z);
  return cudaGetLastError();
}

cudaError_t launch_zv_accum(cudaStream_t st, int mode, int nbra, int nsplit, int64_t S, const ZvCsr& Q,
                            const ZvChunk& Z, const double* pi0, double* partS, double* partG) {
  dim3 grid((unsigned)(nbra * nsplit));
  if (mode == SS_PREC_FP64)
    zv_accum_kernel<SS_PREC_FP64><<<grid, 256, 0, st>>>(S, Q, nsplit, Z, pi0, partS, partG);
  else
    zv_accum_kernel<SS_PREC_REF32><<<grid, 256, 0, st>>>(S, Q, nsplit, Z, pi0, partS, partG);
  return cudaGetLastError();
}

cudaError_t launch_zv_reduce(cudaStream_t st, int64_t nint, int nsplit, const double* partS,
                             const double* partG, double* eS, double* eG) {
  zv_reduce_partials<<<(unsigned)((nint + 255) / 256), 256, 0, st>>>(nint, nsplit, partS, partG, eS, eG);
  return cudaGetLastError();
}

cudaError_t launch_zv_block_stats(cudaStream_t st, int64_t nint, int64_t npts, double* eS, double* eG,
                                  double* acc, double* acc2) {
  zv_block_stats<<<(unsigned)((nint + 255) / 256), 256, 0, st>>>(nint, npts, eS, eG, acc, acc2);
  return cudaGetLastError();
}

cudaError_t launch_zv_final(cudaStream_t st, int64_t nint, int nb, int unbiased, const double* acc,
                            const double* acc2, double* mean, double* sigma, unsigned long long* maxbits) {
  zv_final<<<(unsigned)((nint + 255) / 256), 256, 0, st>>>(nint, nb, unbiased, acc, acc2, mean, sigma,
                                                           maxbits);
  return cudaGetLastError();
}

}  // namespace ss
