// monocenter.cu -- exact one-centre Slater ERIs on the device (the do_exact_monocenter path of
// src/two_e_slater.F90:318-369).
//
// A quartet whose four functions sit on one centre has a closed form for the STOs themselves
// (src/compute_int_slater.F90:1-85): each x^nx y^ny z^nz / r^(nx+ny+nz) is expanded over
// complex spherical harmonics (src/ijkl_slater_xnynzn.F90:59-124, nx+ny+nz <= 2), and every
// term (n1 l1 m1 n2 l2 m2 | n3 l3 m3 n4 l4 m4) is the sum over the multipole order l of two Gaunt
// coefficients times the radial integral bigF (src/ijkl_slater.F90:49-103, src/bigF.F90,
// src/smallg.F90, src/compute_lmin_lmax.F90).  The Gaunt coefficient (src/gaunt.F90, a
// third-party routine) comes from its published definition through the Racah formula of the
// Wigner 3j symbol.  One thread per quartet; quartets on more than one centre are flagged 0.
// With ss_set_exact_monocenter the merged ERI of a one-centre quartet is this value and its MC
// error bar 0 (src/two_e_slater.F90:465-494, 558-562).
#include <math.h>
#include <string.h>

#include <algorithm>
#include <mutex>
#include <vector>

#include "ss_common.cuh"
#include "ss_context.cuh"

namespace ss {

int dev_alloc(ss_ctx* c, DevBuf& b, size_t bytes);

constexpr int MC_FACT = 32;
// factorials as the memoised product f(n) = f(n-1) n; x^n/r^n -> Y_l^m coefficients,
// [nx][ny][nz][l][m+2] real and imaginary parts
__constant__ double c_fact[MC_FACT];
__constant__ double c_ylm_re[3][3][3][3][5];
__constant__ double c_ylm_im[3][3][3][3][5];

__device__ __forceinline__ double mc_powi(double x, int k) {  // x**k by binary exponentiation
  double r = 1.0, b = x;
  while (k > 0) {
    if (k & 1) r *= b;
    b *= b;
    k >>= 1;
  }
  return r;
}

__device__ __forceinline__ double mc_sign(int k) { return (k & 1) ? -1.0 : 1.0; }

// Wigner 3j symbol (j1 j2 j3; m1 m2 m3), Racah's single-sum formula
__device__ double wigner3j(int j1, int j2, int j3, int m1, int m2, int m3) {
  if (m1 + m2 + m3 != 0) return 0.0;
  if (j3 < abs(j1 - j2) || j3 > j1 + j2) return 0.0;
  if (abs(m1) > j1 || abs(m2) > j2 || abs(m3) > j3) return 0.0;
  const double* f = c_fact;
  const double delta = f[j1 + j2 - j3] * f[j1 - j2 + j3] * f[-j1 + j2 + j3] / f[j1 + j2 + j3 + 1];
  const double pre = sqrt(delta * f[j1 + m1] * f[j1 - m1] * f[j2 + m2] * f[j2 - m2] * f[j3 + m3] * f[j3 - m3]);
  const int kmin = max(0, max(j2 - j3 - m1, j1 - j3 + m2));
  const int kmax = min(j1 + j2 - j3, min(j1 - m1, j2 + m2));
  double s = 0.0;
  for (int k = kmin; k <= kmax; k++) {
    const double t = 1.0 / (f[k] * f[j1 + j2 - j3 - k] * f[j1 - m1 - k] * f[j2 + m2 - k] * f[j3 - j2 + m1 + k] *
                            f[j3 - j1 - m2 + k]);
    s += (k & 1) ? -t : t;
  }
  return mc_sign(abs(j1 - j2 - m3)) * pre * s;
}

// int dOmega Y*_{l1 m1} Y_{l2 m2} Y_{l3 m3}, m1 = m2 + m3
__device__ double gaunt(int l1, int l2, int l3, int m1, int m2, int m3) {
  if (m1 - m2 - m3 != 0) return 0.0;
  if ((l1 + l2 + l3) & 1) return 0.0;
  const double c = sqrt((2.0 * l1 + 1.0) * (2.0 * l2 + 1.0) * (2.0 * l3 + 1.0) / (4.0 * M_PI));
  return mc_sign(abs(m1)) * c * wigner3j(l1, l2, l3, 0, 0, 0) * wigner3j(l1, l2, l3, -m1, m2, m3);
}

__device__ __forceinline__ double norm_sto(double gam, int n) {  // src/norm_sto.F90
  return sqrt(mc_powi(2.0 * gam, 2 * n + 1) / c_fact[n + n]);
}

__device__ double smallg(int n, int m, double g, double gp, int l) {  // src/smallg.F90
  double s = 0.0;
  for (int i = 0; i <= n + l; i++)
    s = s + c_fact[n + l] * c_fact[n + m - 1 - i] / c_fact[n + l - i] / mc_powi(g, i + 1) / mc_powi(gp, n + m - i);
  return s;
}

__device__ double bigF(int n12, double g12, int n34, double g34, int l) {  // src/bigF.F90:20-34
  const int l12 = -l, l34 = l + 1;
  const double g = g12 + g34;
  const double first =
      c_fact[n34 + l34 - 1] / mc_powi(g34, n34 + l34) * c_fact[n12 + l12 - 1] / mc_powi(g12, n12 + l12);
  return first + smallg(n34, n12, g34, g, l12 - 1) - smallg(n34, n12, g34, g, l34 - 1);
}

// src/ijkl_slater.F90:49-103 (with src/compute_lmin_lmax.F90)
__device__ double ijkl_slater(const int* ns, const int* ls, const int* ms, const double* gam) {
  const int l1 = ls[0], l2 = ls[1], l3 = ls[2], l4 = ls[3];
  if ((l1 + l2 + l3 + l4) & 1) return 0.0;
  const int m1 = ms[0], m2 = ms[1], m3 = ms[2], m4 = ms[3];
  if (m2 - m1 != m3 - m4) return 0.0;
  const int m = m2 - m1;
  double norm = 1.0;
  for (int i = 0; i < 4; i++) norm = norm * norm_sto(gam[i], ns[i]);
  const int lmax = min(l1 + l2, l3 + l4);
  const int mx12 = max(abs(l1 - l2), abs(m1 - m2));
  const int l12min = ((lmax + mx12) % 2 == 0) ? mx12 : mx12 + 1;
  const int mx34 = max(abs(l3 - l4), abs(m3 - m4));
  const int l34min = ((lmax + mx34) % 2 == 0) ? mx34 : mx34 + 1;
  const int lmin = max(l12min, l34min);
  const int n12 = ns[0] + ns[1], n34 = ns[2] + ns[3];
  const double g12 = gam[0] + gam[1], g34 = gam[2] + gam[3];
  double s = 0.0;
  for (int l = lmin; l <= lmax; l += 2)
    s = s + gaunt(l2, l, l1, m2, m, m1) * gaunt(l3, l, l4, m3, m, m4) * bigF(n12, g12, n34, g34, l) / (2.0 * l + 1.0);
  return 4.0 * M_PI * s * norm;
}

__global__ void monocenter_kernel(BasisDev B, int64_t nint, const int32_t* __restrict__ is,
                                  const int32_t* __restrict__ js, const int32_t* __restrict__ ks,
                                  const int32_t* __restrict__ ls, double* __restrict__ val,
                                  int32_t* __restrict__ mask, int* __restrict__ status) {
  const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (q >= nint) return;
  const int f[4] = {is[q] - 1, ks[q] - 1, js[q] - 1, ls[q] - 1};  // (i k | j l)
  bool same = true;
  for (int t = 1; t < 4; t++)
    for (int a = 0; a < 3; a++) same = same && B.center[3 * f[t] + a] == B.center[3 * f[0] + a];
  mask[q] = same ? 1 : 0;
  val[q] = 0.0;
  if (!same) return;
  int nx[4], ny[4], nz[4], ns[4], lmx[4];
  double gam[4];
  for (int t = 0; t < 4; t++) {
    nx[t] = B.npower[3 * f[t]];
    ny[t] = B.npower[3 * f[t] + 1];
    nz[t] = B.npower[3 * f[t] + 2];
    lmx[t] = nx[t] + ny[t] + nz[t];
    if (lmx[t] > 2) {  // the reference stops here (src/ijkl_slater_xnynzn.F90:41-44)
      atomicExch(status, 1);
      mask[q] = 0;
      return;
    }
    ns[t] = 1 + lmx[t] + B.n_sto[f[t]];
    gam[t] = B.g_slater[f[t]];
  }
  double rre = 0.0, rim = 0.0;
  for (int l1 = 0; l1 <= lmx[0]; l1++)
    for (int m1 = -l1; m1 <= l1; m1++)
      for (int l2 = 0; l2 <= lmx[1]; l2++)
        for (int m2 = -l2; m2 <= l2; m2++)
          for (int l3 = 0; l3 <= lmx[2]; l3++)
            for (int m3 = -l3; m3 <= l3; m3++)
              for (int l4 = 0; l4 <= lmx[3]; l4++)
                for (int m4 = -l4; m4 <= l4; m4++) {
                  const int lv[4] = {l1, l2, l3, l4}, mv[4] = {m1, m2, m3, m4};
                  double cr = 1.0, ci = 0.0;
                  for (int t = 0; t < 4; t++) {
                    const double ar = c_ylm_re[nx[t]][ny[t]][nz[t]][lv[t]][mv[t] + 2];
                    const double ai = c_ylm_im[nx[t]][ny[t]][nz[t]][lv[t]][mv[t] + 2];
                    const double nr = cr * ar - ci * ai, ni = cr * ai + ci * ar;
                    cr = nr;
                    ci = ni;
                  }
                  if (sqrt(cr * cr + ci * ci) > 1.e-20) {
                    const int ms[4] = {-m1, m2, -m3, m4};
                    const double v = mc_sign(abs(m1 + m3)) * ijkl_slater(ns, lv, ms, gam);
                    rre = rre + cr * v;
                    rim = rim + ci * v;
                  }
                }
  double norm = 1.0;
  for (int t = 0; t < 4; t++) norm = norm * norm_sto(gam[t], ns[t]);
  val[q] = rre / norm;
}

// merged ERI of the one-centre quartets = the exact value, MC mean and error bar 0
// (src/two_e_slater.F90:558-562 and :494); the others keep gauss + MC mean
__global__ void combine_mono_kernel(int64_t nint, const double* __restrict__ g, double* __restrict__ mean,
                                    double* __restrict__ sigma, const double* __restrict__ val,
                                    const int32_t* __restrict__ mask, double* __restrict__ out) {
  const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (q >= nint) return;
  if (mask[q]) {
    mean[q] = 0.0;
    sigma[q] = 0.0;
    out[q] = val[q];
  } else {
    out[q] = mean[q] + g[q];
  }
}

// once per device and process; job worker threads may get here together
static std::mutex g_tables_mu;
static bool g_tables_done[64] = {false};

static int upload_tables(ss_ctx* c) {
  std::lock_guard<std::mutex> lock(g_tables_mu);
  if (c->device >= 0 && c->device < 64 && g_tables_done[c->device]) return SS_OK;
  double f[MC_FACT];
  f[0] = 1.0;
  for (int i = 1; i < MC_FACT; i++) f[i] = f[i - 1] * i;
  f[1] = 1.0;
  static double re[3][3][3][3][5], im[3][3][3][3][5];
  memset(re, 0, sizeof re);
  memset(im, 0, sizeof im);
  const double pi = acos(-1.0);
  const double r4 = sqrt(4.0 * pi), r43 = sqrt(4.0 * pi / 3.0), r15 = sqrt(pi / 15.0), s2 = sqrt(2.0),
               s3 = sqrt(3.0);
  // src/ijkl_slater_xnynzn.F90:73-124
  re[0][0][0][0][2] = r4;
  re[1][0][0][1][1] = r43 / s2;
  re[1][0][0][1][3] = -r43 / s2;
  im[0][1][0][1][1] = r43 / s2;
  im[0][1][0][1][3] = r43 / s2;
  re[0][0][1][1][2] = r43;
  im[1][1][0][2][0] = r15 * s2;
  im[1][1][0][2][4] = -r15 * s2;
  im[0][1][1][2][1] = r15 * s2;
  im[0][1][1][2][3] = r15 * s2;
  re[1][0][1][2][1] = r15 * s2;
  re[1][0][1][2][3] = -r15 * s2;
  re[2][0][0][0][2] = r4 / 3.0;
  re[2][0][0][2][0] = r15 * s2;
  re[2][0][0][2][4] = r15 * s2;
  re[2][0][0][2][2] = -r15 * 2.0 / s3;
  re[0][2][0][0][2] = r4 / 3.0;
  re[0][2][0][2][0] = -r15 * s2;
  re[0][2][0][2][4] = -r15 * s2;
  re[0][2][0][2][2] = -r15 * 2.0 / s3;
  re[0][0][2][0][2] = r4 / 3.0;
  re[0][0][2][2][2] = r15 * 4.0 / s3;
  SS_CUDA_TRY(cudaMemcpyToSymbolAsync(c_fact, f, sizeof f, 0, cudaMemcpyHostToDevice, c->stream));
  SS_CUDA_TRY(cudaMemcpyToSymbolAsync(c_ylm_re, re, sizeof re, 0, cudaMemcpyHostToDevice, c->stream));
  SS_CUDA_TRY(cudaMemcpyToSymbolAsync(c_ylm_im, im, sizeof im, 0, cudaMemcpyHostToDevice, c->stream));
  SS_CUDA_TRY(cudaStreamSynchronize(c->stream));
  if (c->device >= 0 && c->device < 64) g_tables_done[c->device] = true;
  return SS_OK;
}

// exact values and one-centre mask of the context's quartets (cached until the basis or the
// quartets change)
int ensure_mono(ss_ctx* c) {
  if (c->have_mono) return SS_OK;
  int rc = upload_tables(c);
  if (rc) return rc;
  const int64_t nint = c->nint;
  rc = dev_alloc(c, c->d_mono_val, sizeof(double) * std::max<int64_t>(nint, 1));
  if (!rc) rc = dev_alloc(c, c->d_mono_mask, sizeof(int32_t) * std::max<int64_t>(nint, 1));
  if (!rc) rc = dev_alloc(c, c->d_mono_status, sizeof(int));
  if (rc) return rc;
  SS_CUDA_TRY(cudaMemsetAsync(c->d_mono_status.ptr, 0, sizeof(int), c->stream));
  if (nint > 0) {
    monocenter_kernel<<<(unsigned)((nint + 127) / 128), 128, 0, c->stream>>>(
        c->basis, nint, (const int32_t*)c->d_is.ptr, (const int32_t*)c->d_js.ptr, (const int32_t*)c->d_ks.ptr,
        (const int32_t*)c->d_ls.ptr, (double*)c->d_mono_val.ptr, (int32_t*)c->d_mono_mask.ptr,
        (int*)c->d_mono_status.ptr);
    SS_CUDA_TRY(cudaGetLastError());
    c->launches++;
  }
  int status = 0;
  SS_CUDA_TRY(cudaMemcpyAsync(&status, c->d_mono_status.ptr, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  SS_CUDA_TRY(cudaStreamSynchronize(c->stream));
  if (status) {
    ss_set_error_msg("exact one-centre Slater integrals: x^nx y^ny z^nz beyond d (nx+ny+nz > 2) not implemented");
    return SS_ERR_UNSUPPORTED;
  }
  int64_t cnt = 0;
  if (nint > 0) {
    std::vector<int32_t> m(nint);
    SS_CUDA_TRY(cudaMemcpyAsync(m.data(), c->d_mono_mask.ptr, sizeof(int32_t) * nint, cudaMemcpyDeviceToHost,
                                c->stream));
    SS_CUDA_TRY(cudaStreamSynchronize(c->stream));
    for (int32_t v : m) cnt += v;
  }
  c->n_mono = cnt;
  c->have_mono = true;
  return SS_OK;
}

int launch_combine_mono(ss_ctx* c, double* out) {
  combine_mono_kernel<<<(unsigned)((c->nint + 255) / 256), 256, 0, c->stream>>>(
      c->nint, (const double*)c->d_gauss.ptr, (double*)c->d_mean.ptr, (double*)c->d_sigma.ptr,
      (const double*)c->d_mono_val.ptr, (const int32_t*)c->d_mono_mask.ptr, out);
  SS_CUDA_TRY(cudaGetLastError());
  c->launches++;
  return SS_OK;
}

}  // namespace ss

using namespace ss;

extern "C" {

int ss_monocenter(ss_ctx* c, double* out, int32_t* mask, int64_t* n_mono) {
  if (!c) {
    ss_set_error_msg("null ss_ctx");
    return SS_ERR_ARG;
  }
  SS_CUDA_TRY(cudaSetDevice(c->device));
  if (!c->n || !c->nint) {
    ss_set_error_msg("basis and quartets must be set first");
    return SS_ERR_STATE;
  }
  int rc = ensure_mono(c);
  if (rc) return rc;
  if (out)
    SS_CUDA_TRY(cudaMemcpyAsync(out, c->d_mono_val.ptr, sizeof(double) * c->nint, cudaMemcpyDeviceToHost, c->stream));
  if (mask)
    SS_CUDA_TRY(
        cudaMemcpyAsync(mask, c->d_mono_mask.ptr, sizeof(int32_t) * c->nint, cudaMemcpyDeviceToHost, c->stream));
  SS_CUDA_TRY(cudaStreamSynchronize(c->stream));
  if (n_mono) *n_mono = c->n_mono;
  return SS_OK;
}

int ss_set_exact_monocenter(ss_ctx* c, int enable) {
  if (!c) {
    ss_set_error_msg("null ss_ctx");
    return SS_ERR_ARG;
  }
  c->exact_monocenter = enable != 0;
  return SS_OK;
}

}  // extern "C"
