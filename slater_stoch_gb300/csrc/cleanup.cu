// cleanup.cu -- PSD cleanup of the ERI matrix (svd_clean) and Davidson, FP64 on the device.
//
// ss_psd_clean restates src/svd_clean.F90:1-426 for one GPU: the ERIs are scattered into the
// symmetric matrix W (the reference's n^2 x n^2 <ij|kl> arrangement, or the packed Coulomb
// metric M[(ik),(jl)] = (ik|jl)); passes of a randomized SVD (Gaussian test matrix, q power
// iterations with Householder re-orthogonalisation, SVD of Y = Z^T W_work) find components
// U D V^T; the sign test <U_k, V_k> gives the eigenvalue sign and drops unresolved components;
// all found components are deflated from W_work and the negative ones are removed from W; the
// loop ends when npass >= N or max|D| < 1e-12; the cleaned ERIs are gathered back.  The SVD
// of Y comes from the eigen-decomposition of Y Y^T (Y Y^T = UY D^2 UY^T, V^T = D^-1 UY^T Y);
// components it cannot resolve relative to the largest one fail the sign test and are found
// in later passes, after the deflation has removed the large ones.
//
// Every product is the hand-written FP64 dgemm of linalg.cu, the orthonormalisations its blocked
// Householder QR and the eigenproblems its eigensolvers; each svd_clean pass reads back one
// small record (sign-test counts, largest |D|) to decide whether another pass is needed.
//
// ss_davidson restates src/davidson.F90:1-158 (lowest m eigenpairs, NMAX = min(10, N/m),
// diagonal preconditioner (E u - H u)/max(H_ii - E, 1e-2), convergence when the largest
// correction norm is < tol); the basis is kept orthonormal so the projected problem is a
// standard symmetric eigenproblem (the reference solves the equivalent generalized one with
// dsygv).
#include <math.h>
#include <string.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "linalg.cuh"
#include "philox.cuh"
#include "ss_common.cuh"
#include "ss_context.cuh"

namespace ss {

#define TRY(x)           \
  do {                   \
    int _rc = (x);       \
    if (_rc) return _rc; \
  } while (0)
// ---------------------------------------------------------------------------------------
// scatter / gather between the quartet list and the symmetric matrix
// ---------------------------------------------------------------------------------------
// REF_N2: W(ii,jj), ii = i + j n, jj = k + l n (0-based), the 8 permutations of
// src/svd_clean.F90:97-130; PACKED_PAIR: M(p(ik), p(jl)) and its transpose.
__device__ __forceinline__ void perm8(int t, int i, int j, int k, int l, int& a, int& b, int& c, int& d) {
  switch (t) {
    case 0: a = i; b = j; c = k; d = l; break;
    case 1: a = k; b = j; c = i; d = l; break;
    case 2: a = k; b = l; c = i; d = j; break;
    case 3: a = i; b = l; c = k; d = j; break;
    case 4: a = j; b = i; c = l; d = k; break;
    case 5: a = j; b = k; c = l; d = i; break;
    case 6: a = l; b = k; c = j; d = i; break;
    default: a = l; b = i; c = j; d = k; break;
  }
}

__global__ void scatter_kernel(int64_t nint, int layout, int n, int64_t N, const int32_t* __restrict__ is,
                               const int32_t* __restrict__ js, const int32_t* __restrict__ ks,
                               const int32_t* __restrict__ ls, const double* __restrict__ moy,
                               double* __restrict__ W) {
  const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (q >= nint) return;
  const int i = is[q] - 1, j = js[q] - 1, k = ks[q] - 1, l = ls[q] - 1;
  const double v = moy[q];
  if (layout == SS_LAYOUT_REF_N2) {
    for (int t = 0; t < 8; t++) {
      int a, b, c, d;
      perm8(t, i, j, k, l, a, b, c, d);
      const int64_t ii = a + (int64_t)b * n, jj = c + (int64_t)d * n;
      W[ii + jj * N] = v;  // column-major
    }
  } else {
    const int64_t p1 = ss_pair_index(i, k), p2 = ss_pair_index(j, l);
    W[p1 + p2 * N] = v;
    W[p2 + p1 * N] = v;
  }
}

__global__ void gather_kernel(int64_t nint, int layout, int n, int64_t N, const int32_t* __restrict__ is,
                              const int32_t* __restrict__ js, const int32_t* __restrict__ ks,
                              const int32_t* __restrict__ ls, const double* __restrict__ W,
                              double* __restrict__ moy) {
  const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (q >= nint) return;
  const int i = is[q] - 1, j = js[q] - 1, k = ks[q] - 1, l = ls[q] - 1;
  double v = 0.0;
  if (layout == SS_LAYOUT_REF_N2) {  // src/svd_clean.F90:372-405
    for (int t = 0; t < 8; t++) {
      int a, b, c, d;
      perm8(t, i, j, k, l, a, b, c, d);
      const int64_t ii = a + (int64_t)b * n, jj = c + (int64_t)d * n;
      v = v + W[ii + jj * N] * 0.125;
    }
  } else {
    const int64_t p1 = ss_pair_index(i, k), p2 = ss_pair_index(j, l);
    v = 0.5 * (W[p1 + p2 * N] + W[p2 + p1 * N]);
  }
  moy[q] = v;
}

// Gaussian test matrix (src/svd_clean.F90:159-171): Box-Muller from Philox, columns normalised
__global__ void gaussian_matrix_kernel(uint64_t seed, uint32_t pass, int N, int r, double* __restrict__ P) {
  const int k = blockIdx.x;
  __shared__ double sh[32];
  double ss = 0.0;
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    const uint64_t idx = (uint64_t)k * N + i;
    uint32_t c[4] = {(uint32_t)idx, (uint32_t)(idx >> 32), pass, STREAM_SVD};
    philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
    const double u1 = u01_open(c[0], c[1]), u2 = u01_open(c[2], c[3]);
    const double v = sqrt(-2.0 * log(u1)) * cos(6.283185307179586477 * u2);
    P[(size_t)k * N + i] = v;
    ss += v * v;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) ss += __shfl_down_sync(0xffffffffu, ss, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = ss;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += sh[w];
    sh[0] = 1.0 / sqrt(t);
  }
  __syncthreads();
  const double inv = sh[0];
  for (int i = threadIdx.x; i < N; i += blockDim.x) P[(size_t)k * N + i] *= inv;
}

// r_k = <U_k, Vt_k>; U (N x r col-major), Vt (r x N col-major, ld r)
__global__ void sign_test_kernel(int N, int r, const double* __restrict__ U, const double* __restrict__ Vt,
                                 double* __restrict__ rk) {
  const int k = blockIdx.x;
  __shared__ double sh[32];
  double s = 0.0;
  for (int i = threadIdx.x; i < N; i += blockDim.x) s += U[(size_t)k * N + i] * Vt[k + (size_t)i * r];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += sh[w];
    rk[k] = t;
  }
}

// columns of U scaled: out(:,k) = U(:,k) * s[k]
__global__ void scale_cols_kernel(int N, int r, const double* __restrict__ U, const double* __restrict__ s,
                                  double* __restrict__ out) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= (int64_t)N * r) return;
  out[e] = U[e] * s[e / N];
}

// Vt rows scaled by inv[k] (r x N col-major, ld r)
__global__ void scale_rows_kernel(int r, int N, double* __restrict__ Vt, const double* __restrict__ inv) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= (int64_t)N * r) return;
  Vt[e] *= inv[e % r];
}

static unsigned nb(int64_t n) { return (unsigned)((n + 255) / 256); }

// reverse the column order of the ascending eigenvectors V (r x r) into UY (largest first) and
// the singular values D_k = sqrt(max(ev[r-1-k], 0)) with their inverses
__global__ void svd_uy_kernel(int r, const double* __restrict__ V, const double* __restrict__ ev,
                              double* __restrict__ UY, double* __restrict__ D, double* __restrict__ invD) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= (int64_t)r * r) return;
  const int i = (int)(e % r), k = (int)(e / r);
  UY[e] = V[i + (size_t)(r - 1 - k) * r];
  if (i == 0) {
    const double d = sqrt(fmax(ev[r - 1 - k], 0.0));
    D[k] = d;
    invD[k] = d > 0.0 ? 1.0 / d : 0.0;
  }
}

struct SvdPassStats {
  int nbad, nneg;
  double dmax;
};

// the sign test of src/svd_clean.F90:286-296 on the device: D_k takes the sign of
// r_k = <U_k, Vt_k>, components with |r_k| < 0.99 are dropped; absD / negD are the deflation
// weights of W_work and W.  One CTA.
__global__ void svd_sign_kernel(int r, const double* __restrict__ rk, const double* __restrict__ D,
                                double* __restrict__ absD, double* __restrict__ negD, SvdPassStats* st) {
  __shared__ int s_bad, s_neg;
  __shared__ double s_max[32];
  if (threadIdx.x == 0) {
    s_bad = 0;
    s_neg = 0;
  }
  __syncthreads();
  double mx = 0.0;
  for (int k = threadIdx.x; k < r; k += blockDim.x) {
    double d = rk[k] < 0.0 ? -D[k] : D[k];
    if (fabs(rk[k]) < 0.99) {
      d = 0.0;
      atomicAdd(&s_bad, 1);
    }
    if (d < 0.0) atomicAdd(&s_neg, 1);
    absD[k] = fabs(d);
    negD[k] = d < 0.0 ? d : 0.0;
    mx = fmax(mx, fabs(d));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_down_sync(0xffffffffu, mx, o));
  if ((threadIdx.x & 31) == 0) s_max[threadIdx.x >> 5] = mx;
  __syncthreads();
  if (threadIdx.x == 0) {
    double m = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) m = fmax(m, s_max[w]);
    st->nbad = s_bad;
    st->nneg = s_neg;
    st->dmax = m;
  }
}

int psd_clean(ss_ctx* c, double* moy_host, int layout, int rank, int oversample, int q, uint64_t seed,
              int* n_removed) {
  const int n = c->n;
  const int64_t N64 = layout == SS_LAYOUT_REF_N2 ? (int64_t)n * n : (int64_t)n * (n + 1) / 2;
  if (N64 > 16384) {
    ss_set_error_msg("psd_clean: matrix dimension %lld too large for the dense device cleanup", (long long)N64);
    return SS_ERR_UNSUPPORTED;
  }
  const int N = (int)N64;
  const int r = std::min(rank + oversample, N);
  if (r < 1 || r > 2048) {
    ss_set_error_msg("psd_clean: rank + oversample must be in 1..2048 (got %d)", r);
    return SS_ERR_ARG;
  }
  void* p;
  double *W, *Ww, *P, *Z, *Y, *G, *ev, *UYv, *UY, *U, *Vt, *Us, *D, *invD, *absD, *negD, *rk, *moy, *qrw, *eigw, *gws;
  const size_t NN = (size_t)N * N, Nr = (size_t)N * r, rr = (size_t)r * r;
  const size_t gsz = std::max({dgemm_ws(N, r, N), dgemm_ws(r, N, N), dgemm_ws(r, r, N), dgemm_ws(r, N, r),
                               dgemm_ws(N, r, r), dgemm_ws(N, N, r), (size_t)1});
  TRY(pool_get(c, "cl_W", sizeof(double) * NN, &p)); W = (double*)p;
  TRY(pool_get(c, "cl_Ww", sizeof(double) * NN, &p)); Ww = (double*)p;
  TRY(pool_get(c, "cl_P", sizeof(double) * Nr, &p)); P = (double*)p;
  TRY(pool_get(c, "cl_Z", sizeof(double) * Nr, &p)); Z = (double*)p;
  TRY(pool_get(c, "cl_Y", sizeof(double) * Nr, &p)); Y = (double*)p;
  TRY(pool_get(c, "cl_G", sizeof(double) * rr, &p)); G = (double*)p;
  TRY(pool_get(c, "cl_ev", sizeof(double) * r, &p)); ev = (double*)p;
  TRY(pool_get(c, "cl_UYv", sizeof(double) * rr, &p)); UYv = (double*)p;
  TRY(pool_get(c, "cl_UY", sizeof(double) * rr, &p)); UY = (double*)p;
  TRY(pool_get(c, "cl_U", sizeof(double) * Nr, &p)); U = (double*)p;
  TRY(pool_get(c, "cl_Vt", sizeof(double) * Nr, &p)); Vt = (double*)p;
  TRY(pool_get(c, "cl_Us", sizeof(double) * Nr, &p)); Us = (double*)p;
  TRY(pool_get(c, "cl_D", sizeof(double) * 5 * r, &p)); D = (double*)p;
  invD = D + r; absD = D + 2 * r; negD = D + 3 * r; rk = D + 4 * r;
  TRY(pool_get(c, "cl_moy", sizeof(double) * c->nint, &p)); moy = (double*)p;
  TRY(pool_get(c, "cl_qr", sizeof(double) * ortho_qr_ws(N, r), &p)); qrw = (double*)p;
  TRY(pool_get(c, "cl_eig", sizeof(double) * std::max<size_t>(sym_eig_ws(r), 1), &p)); eigw = (double*)p;
  TRY(pool_get(c, "cl_gws", sizeof(double) * gsz, &p)); gws = (double*)p;
  TRY(pool_get(c, "cl_stats", 64, &p));
  SvdPassStats* dstats = (SvdPassStats*)p;
  int* derr = (int*)((char*)p + 32);
  int64_t* L = &c->launches;
  cudaStream_t st = c->stream;
  SS_CUDA_TRY(cudaMemsetAsync(derr, 0, sizeof(int), st));
  SS_CUDA_TRY(cudaMemcpyAsync(moy, moy_host, sizeof(double) * c->nint, cudaMemcpyHostToDevice, st));
  SS_CUDA_TRY(cudaMemsetAsync(Ww, 0, sizeof(double) * NN, st));
  scatter_kernel<<<nb(c->nint), 256, 0, st>>>(c->nint, layout, n, N, (const int32_t*)c->d_is.ptr,
                                               (const int32_t*)c->d_js.ptr, (const int32_t*)c->d_ks.ptr,
                                               (const int32_t*)c->d_ls.ptr, moy, Ww);
  SS_CUDA_TRY(cudaGetLastError());
  SS_CUDA_TRY(cudaMemcpyAsync(W, Ww, sizeof(double) * NN, cudaMemcpyDeviceToDevice, st));
  (*L)++;
  int npass = 0, removed = 0;
  uint32_t pass = 0;
  while (npass < N) {
    gaussian_matrix_kernel<<<r, 256, 0, st>>>(seed, pass, N, r, P);
    SS_CUDA_TRY(cudaGetLastError());
    (*L)++;
    // range finder (src/svd_clean.F90:183-255): Z = W_work P, q power iterations, each
    // product re-orthonormalised by Householder QR
    TRY(dgemm(st, 0, 0, N, r, N, 1.0, Ww, N, P, N, 0.0, Z, N, gws, L));
    TRY(ortho_qr(st, N, r, Z, N, qrw, L));
    for (int it = 0; it < q; it++) {
      TRY(dgemm(st, 1, 0, N, r, N, 1.0, Ww, N, Z, N, 0.0, P, N, gws, L));
      TRY(dgemm(st, 0, 0, N, r, N, 1.0, Ww, N, P, N, 0.0, Z, N, gws, L));
      TRY(ortho_qr(st, N, r, Z, N, qrw, L));
    }
    // SVD of Y = Z^T W_work (r x N) from Y Y^T = UY D^2 UY^T (src/svd.F90)
    TRY(dgemm(st, 1, 0, r, N, N, 1.0, Z, N, Ww, N, 0.0, Y, r, gws, L));
    TRY(dgemm(st, 0, 1, r, r, N, 1.0, Y, r, Y, r, 0.0, G, r, gws, L));
    TRY(sym_eig(st, r, G, UYv, ev, eigw, derr, L));
    svd_uy_kernel<<<nb((int64_t)r * r), 256, 0, st>>>(r, UYv, ev, UY, D, invD);
    SS_CUDA_TRY(cudaGetLastError());
    (*L)++;
    // Vt = D^-1 UY^T Y ; U = Z UY
    TRY(dgemm(st, 1, 0, r, N, r, 1.0, UY, r, Y, r, 0.0, Vt, r, gws, L));
    scale_rows_kernel<<<nb((int64_t)N * r), 256, 0, st>>>(r, N, Vt, invD);
    SS_CUDA_TRY(cudaGetLastError());
    TRY(dgemm(st, 0, 0, N, r, r, 1.0, Z, N, UY, r, 0.0, U, N, gws, L));
    sign_test_kernel<<<r, 256, 0, st>>>(N, r, U, Vt, rk);
    svd_sign_kernel<<<1, 1024, 0, st>>>(r, rk, D, absD, negD, dstats);
    SS_CUDA_TRY(cudaGetLastError());
    *L += 3;
    // W_work -= U |D| Vt ; W += U D_neg Vt   (src/svd_clean.F90:335-353)
    scale_cols_kernel<<<nb((int64_t)N * r), 256, 0, st>>>(N, r, U, absD, Us);
    SS_CUDA_TRY(cudaGetLastError());
    TRY(dgemm(st, 0, 0, N, N, r, -1.0, Us, N, Vt, r, 1.0, Ww, N, gws, L));
    scale_cols_kernel<<<nb((int64_t)N * r), 256, 0, st>>>(N, r, U, negD, Us);
    SS_CUDA_TRY(cudaGetLastError());
    TRY(dgemm(st, 0, 0, N, N, r, 1.0, Us, N, Vt, r, 1.0, W, N, gws, L));
    *L += 2;
    SvdPassStats hs;
    int herr = 0;
    SS_CUDA_TRY(cudaMemcpyAsync(&hs, dstats, sizeof hs, cudaMemcpyDeviceToHost, st));
    SS_CUDA_TRY(cudaMemcpyAsync(&herr, derr, sizeof(int), cudaMemcpyDeviceToHost, st));
    SS_CUDA_TRY(cudaStreamSynchronize(st));
    if (herr) {
      ss_set_error_msg("psd_clean: symmetric eigensolver %s (%d)", herr == 2 ? "grid barrier timed out" : "did not converge",
                       herr);
      return herr == 2 ? SS_ERR_TIMEOUT : SS_ERR_NUMERIC;
    }
    npass += r - hs.nbad;
    removed += hs.nneg;
    if (hs.dmax < 1.e-12) npass = N;  // src/svd_clean.F90:359
    pass++;
    if (pass > 1000) {
      ss_set_error_msg("psd_clean: no convergence after 1000 passes");
      return SS_ERR_NUMERIC;
    }
  }
  gather_kernel<<<nb(c->nint), 256, 0, st>>>(c->nint, layout, n, N, (const int32_t*)c->d_is.ptr,
                                              (const int32_t*)c->d_js.ptr, (const int32_t*)c->d_ks.ptr,
                                              (const int32_t*)c->d_ls.ptr, W, moy);
  SS_CUDA_TRY(cudaGetLastError());
  (*L)++;
  SS_CUDA_TRY(cudaMemcpyAsync(moy_host, moy, sizeof(double) * c->nint, cudaMemcpyDeviceToHost, st));
  SS_CUDA_TRY(cudaStreamSynchronize(st));
  if (n_removed) *n_removed = removed;
  return SS_OK;
}

// canonical read-back of src/davidson_clean.F90:108-112 (moy = W(ii,jj), no averaging)
__global__ void gather_canonical_kernel(int64_t nint, int layout, int n, int64_t N, const int32_t* __restrict__ is,
                                        const int32_t* __restrict__ js, const int32_t* __restrict__ ks,
                                        const int32_t* __restrict__ ls, const double* __restrict__ W,
                                        double* __restrict__ moy) {
  const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (q >= nint) return;
  const int i = is[q] - 1, j = js[q] - 1, k = ks[q] - 1, l = ls[q] - 1;
  if (layout == SS_LAYOUT_REF_N2)
    moy[q] = W[(i + (int64_t)j * n) + (k + (int64_t)l * n) * N];
  else
    moy[q] = W[ss_pair_index(i, k) + ss_pair_index(j, l) * N];
}

// columns of V scaled by min(lambda, 0) (the negative eigencomponents) and their count
__global__ void neg_scale_kernel(int N, const double* __restrict__ V, const double* __restrict__ ev,
                                 double* __restrict__ Vs, int* __restrict__ nneg) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= (int64_t)N * N) return;
  const int col = (int)(e / N);
  const double l = ev[col];
  Vs[e] = l < 0.0 ? V[e] * l : 0.0;
  if (e % N == 0 && l < 0.0) atomicAdd(nneg, 1);
}

// Remove the negative eigencomponents exactly (src/davidson_clean.F90:30-116, the path the
// reference takes for nbasis < 200): full FP64 eigen-decomposition of the ERI matrix, then
// W -= sum_{lambda_k < 0} lambda_k v_k v_k^T and the canonical entries are read back.  With the
// packed Coulomb metric the result is exactly PSD (to rounding, ~1e-15 of the largest eigenvalue).
int psd_project(ss_ctx* c, double* moy_host, int layout, int* n_removed) {
  const int n = c->n;
  const int64_t N64 = layout == SS_LAYOUT_REF_N2 ? (int64_t)n * n : (int64_t)n * (n + 1) / 2;
  if (N64 > 2048) {
    ss_set_error_msg("psd_project: matrix dimension %lld above the 2048 of the dense device eigensolver",
                     (long long)N64);
    return SS_ERR_UNSUPPORTED;
  }
  const int N = (int)N64;
  void* p;
  double *W, *V, *ev, *Vs, *moy, *eigw, *gws;
  const size_t NN = (size_t)N * N;
  TRY(pool_get(c, "pj_W", sizeof(double) * NN, &p)); W = (double*)p;
  TRY(pool_get(c, "pj_V", sizeof(double) * NN, &p)); V = (double*)p;
  TRY(pool_get(c, "pj_ev", sizeof(double) * N, &p)); ev = (double*)p;
  TRY(pool_get(c, "pj_Vs", sizeof(double) * NN, &p)); Vs = (double*)p;
  TRY(pool_get(c, "pj_moy", sizeof(double) * c->nint, &p)); moy = (double*)p;
  TRY(pool_get(c, "pj_eig", sizeof(double) * std::max<size_t>(sym_eig_ws(N), 1), &p)); eigw = (double*)p;
  TRY(pool_get(c, "pj_gws", sizeof(double) * std::max<size_t>(dgemm_ws(N, N, N), 1), &p)); gws = (double*)p;
  TRY(pool_get(c, "pj_ctl", 64, &p));
  int* derr = (int*)p;
  int* dneg = derr + 1;
  int64_t* L = &c->launches;
  cudaStream_t st = c->stream;
  SS_CUDA_TRY(cudaMemsetAsync(derr, 0, 2 * sizeof(int), st));
  SS_CUDA_TRY(cudaMemcpyAsync(moy, moy_host, sizeof(double) * c->nint, cudaMemcpyHostToDevice, st));
  SS_CUDA_TRY(cudaMemsetAsync(W, 0, sizeof(double) * NN, st));
  scatter_kernel<<<nb(c->nint), 256, 0, st>>>(c->nint, layout, n, N, (const int32_t*)c->d_is.ptr,
                                               (const int32_t*)c->d_js.ptr, (const int32_t*)c->d_ks.ptr,
                                               (const int32_t*)c->d_ls.ptr, moy, W);
  SS_CUDA_TRY(cudaGetLastError());
  (*L)++;
  TRY(sym_eig(st, N, W, V, ev, eigw, derr, L));
  neg_scale_kernel<<<nb((int64_t)NN), 256, 0, st>>>(N, V, ev, Vs, dneg);
  SS_CUDA_TRY(cudaGetLastError());
  (*L)++;
  TRY(dgemm(st, 0, 1, N, N, N, -1.0, Vs, N, V, N, 1.0, W, N, gws, L));
  gather_canonical_kernel<<<nb(c->nint), 256, 0, st>>>(c->nint, layout, n, N, (const int32_t*)c->d_is.ptr,
                                                        (const int32_t*)c->d_js.ptr, (const int32_t*)c->d_ks.ptr,
                                                        (const int32_t*)c->d_ls.ptr, W, moy);
  SS_CUDA_TRY(cudaGetLastError());
  (*L)++;
  int hctl[2] = {0, 0};
  SS_CUDA_TRY(cudaMemcpyAsync(hctl, derr, 2 * sizeof(int), cudaMemcpyDeviceToHost, st));
  SS_CUDA_TRY(cudaMemcpyAsync(moy_host, moy, sizeof(double) * c->nint, cudaMemcpyDeviceToHost, st));
  SS_CUDA_TRY(cudaStreamSynchronize(st));
  if (hctl[0]) {
    ss_set_error_msg("psd_project: symmetric eigensolver %s (%d)",
                     hctl[0] == 2 ? "grid barrier timed out" : "did not converge", hctl[0]);
    return hctl[0] == 2 ? SS_ERR_TIMEOUT : SS_ERR_NUMERIC;
  }
  if (n_removed) *n_removed = hctl[1];
  return SS_OK;
}

// ---------------------------------------------------------------------------------------
// Davidson
// ---------------------------------------------------------------------------------------
__global__ void diag_kernel(int N, const double* __restrict__ H, double* __restrict__ d) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < N) d[i] = H[i + (size_t)i * N];
}

// correction vectors (src/davidson.F90:132-140): c_j = (E_j x_j - w_j)/max(H_ii - E_j, 1e-2)
__global__ void davidson_correction(int N, int m, const double* __restrict__ X, const double* __restrict__ WX,
                                    const double* __restrict__ E, const double* __restrict__ Hd,
                                    double* __restrict__ Cout) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= (int64_t)N * m) return;
  const int i = (int)(e % N), j = (int)(e / N);
  Cout[e] = (E[j] * X[e] - WX[e]) / fmax(Hd[i] - E[j], 1.e-2);
}

__global__ void col_norms_kernel(int N, int m, const double* __restrict__ X, double* __restrict__ nrm) {
  const int k = blockIdx.x;
  __shared__ double sh[32];
  double s = 0.0;
  for (int i = threadIdx.x; i < N; i += blockDim.x) s += X[(size_t)k * N + i] * X[(size_t)k * N + i];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += sh[w];
    nrm[k] = sqrt(t);
  }
}

// largest of the m correction norms (one warp)
__global__ void max_norm_kernel(int m, const double* __restrict__ nrm, double* __restrict__ out) {
  double v = 0.0;
  for (int j = threadIdx.x; j < m; j += 32) v = fmax(v, nrm[j]);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
  if (threadIdx.x == 0) *out = v;
}

// symmetrised copy: out = (in + in^T) / 2, k x k col-major
__global__ void sym_copy_kernel(int k, const double* __restrict__ in, double* __restrict__ out) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= (int64_t)k * k) return;
  const int i = (int)(e % k), j = (int)(e / k);
  out[e] = 0.5 * (in[i + (size_t)j * k] + in[j + (size_t)i * k]);
}

int davidson(ss_ctx* c, const double* moy_host, int layout, int m, double tol, int max_iter, double* evals,
             double* evecs) {
  const int n = c->n;
  const int64_t N64 = layout == SS_LAYOUT_REF_N2 ? (int64_t)n * n : (int64_t)n * (n + 1) / 2;
  if (N64 > 16384 || m < 1 || m > N64) {
    ss_set_error_msg("davidson: bad sizes (N=%lld, m=%d)", (long long)N64, m);
    return SS_ERR_ARG;
  }
  const int N = (int)N64;
  const int nmax = std::max(2, std::min(10, N / m));  // src/davidson.F90:21
  const int kmax = nmax * m;
  if (kmax > N || kmax > 2048) {
    ss_set_error_msg("davidson: subspace %d larger than the matrix %d (or 2048)", kmax, N);
    return SS_ERR_ARG;
  }
  void* p;
  double *H, *Hd, *U, *WU, *S, *Sa, *Vk, *ev, *X, *WX, *Cc, *nrm, *tmp, *moy, *qrw, *eigw, *gws, *ctl;
  const size_t NN = (size_t)N * N, Nk = (size_t)N * kmax, kk2 = (size_t)kmax * kmax;
  const size_t gsz = std::max({dgemm_ws(N, m, N), dgemm_ws(kmax, kmax, N), dgemm_ws(N, m, kmax),
                               dgemm_ws(kmax, m, N), (size_t)1});
  TRY(pool_get(c, "dv_H", sizeof(double) * NN, &p)); H = (double*)p;
  TRY(pool_get(c, "dv_Hd", sizeof(double) * N, &p)); Hd = (double*)p;
  TRY(pool_get(c, "dv_U", sizeof(double) * Nk, &p)); U = (double*)p;
  TRY(pool_get(c, "dv_WU", sizeof(double) * Nk, &p)); WU = (double*)p;
  TRY(pool_get(c, "dv_S", sizeof(double) * kk2, &p)); S = (double*)p;
  TRY(pool_get(c, "dv_Sa", sizeof(double) * kk2, &p)); Sa = (double*)p;
  TRY(pool_get(c, "dv_Vk", sizeof(double) * kk2, &p)); Vk = (double*)p;
  TRY(pool_get(c, "dv_ev", sizeof(double) * kmax, &p)); ev = (double*)p;
  TRY(pool_get(c, "dv_X", sizeof(double) * (size_t)N * m, &p)); X = (double*)p;
  TRY(pool_get(c, "dv_WX", sizeof(double) * (size_t)N * m, &p)); WX = (double*)p;
  TRY(pool_get(c, "dv_C", sizeof(double) * (size_t)N * m, &p)); Cc = (double*)p;
  TRY(pool_get(c, "dv_nrm", sizeof(double) * m, &p)); nrm = (double*)p;
  TRY(pool_get(c, "dv_tmp", sizeof(double) * (size_t)kmax * m, &p)); tmp = (double*)p;
  TRY(pool_get(c, "dv_moy", sizeof(double) * c->nint, &p)); moy = (double*)p;
  TRY(pool_get(c, "dv_qr", sizeof(double) * ortho_qr_ws(N, m), &p)); qrw = (double*)p;
  TRY(pool_get(c, "dv_eig", sizeof(double) * std::max<size_t>(sym_eig_ws(kmax), 1), &p)); eigw = (double*)p;
  TRY(pool_get(c, "dv_gws", sizeof(double) * gsz, &p)); gws = (double*)p;
  TRY(pool_get(c, "dv_ctl", 64, &p)); ctl = (double*)p;  // [0] max correction norm, [1] error flag
  int* derr = (int*)(ctl + 1);
  int64_t* L = &c->launches;
  cudaStream_t st = c->stream;
  SS_CUDA_TRY(cudaMemsetAsync(derr, 0, sizeof(int), st));
  SS_CUDA_TRY(cudaMemcpyAsync(moy, moy_host, sizeof(double) * c->nint, cudaMemcpyHostToDevice, st));
  SS_CUDA_TRY(cudaMemsetAsync(H, 0, sizeof(double) * NN, st));
  scatter_kernel<<<nb(c->nint), 256, 0, st>>>(c->nint, layout, n, N, (const int32_t*)c->d_is.ptr,
                                               (const int32_t*)c->d_js.ptr, (const int32_t*)c->d_ks.ptr,
                                               (const int32_t*)c->d_ls.ptr, moy, H);
  diag_kernel<<<(N + 255) / 256, 256, 0, st>>>(N, H, Hd);
  // random normalised start vectors (src/davidson.F90:26-37), orthonormalised
  gaussian_matrix_kernel<<<m, 256, 0, st>>>(1, 0x44415649u, N, m, U);
  SS_CUDA_TRY(cudaGetLastError());
  *L += 3;
  TRY(ortho_qr(st, N, m, U, N, qrw, L));
  std::vector<double> hE(m);
  double hmax = 0.0;
  bool converged = false;
  int total = 0;
  while (!converged && total < max_iter) {
    for (int iter = 1; iter <= nmax - 1 && !converged && total < max_iter; iter++, total++) {
      const int shift = m * (iter - 1);
      // W(:, shift:shift+m) = H U(:, shift:shift+m)
      TRY(dgemm(st, 0, 0, N, m, N, 1.0, H, N, U + (size_t)shift * N, N, 0.0, WU + (size_t)shift * N, N, gws, L));
      const int k = shift + m;
      // projected matrix S = U^T W (k x k), symmetrised, eigen-decomposed (ascending)
      TRY(dgemm(st, 1, 0, k, k, N, 1.0, U, N, WU, N, 0.0, S, k, gws, L));
      sym_copy_kernel<<<nb((int64_t)k * k), 256, 0, st>>>(k, S, Sa);
      SS_CUDA_TRY(cudaGetLastError());
      (*L)++;
      TRY(sym_eig(st, k, Sa, Vk, ev, eigw, derr, L));
      // Ritz vectors X = U v, W X = W v of the lowest m (src/davidson.F90:118-126)
      TRY(dgemm(st, 0, 0, N, m, k, 1.0, U, N, Vk, k, 0.0, X, N, gws, L));
      TRY(dgemm(st, 0, 0, N, m, k, 1.0, WU, N, Vk, k, 0.0, WX, N, gws, L));
      davidson_correction<<<nb((int64_t)N * m), 256, 0, st>>>(N, m, X, WX, ev, Hd, Cc);
      col_norms_kernel<<<m, 256, 0, st>>>(N, m, Cc, nrm);
      max_norm_kernel<<<1, 32, 0, st>>>(m, nrm, ctl);
      SS_CUDA_TRY(cudaGetLastError());
      *L += 3;
      int herr = 0;
      SS_CUDA_TRY(cudaMemcpyAsync(&hmax, ctl, sizeof(double), cudaMemcpyDeviceToHost, st));
      SS_CUDA_TRY(cudaMemcpyAsync(&herr, derr, sizeof(int), cudaMemcpyDeviceToHost, st));
      SS_CUDA_TRY(cudaStreamSynchronize(st));
      if (herr) {
        ss_set_error_msg("davidson: projected eigenproblem %s", herr == 2 ? "timed out" : "did not converge");
        return herr == 2 ? SS_ERR_TIMEOUT : SS_ERR_NUMERIC;
      }
      converged = hmax < tol;  // src/davidson.F90:143
      if (converged || iter == nmax - 1) break;
      // new block: corrections orthogonalised against U (twice) and among themselves
      double* Un = U + (size_t)k * N;
      SS_CUDA_TRY(cudaMemcpyAsync(Un, Cc, sizeof(double) * N * m, cudaMemcpyDeviceToDevice, st));
      for (int rep = 0; rep < 2; rep++) {
        TRY(dgemm(st, 1, 0, k, m, N, 1.0, U, N, Un, N, 0.0, tmp, k, gws, L));
        TRY(dgemm(st, 0, 0, N, m, k, -1.0, U, N, tmp, k, 1.0, Un, N, gws, L));
      }
      TRY(ortho_qr(st, N, m, Un, N, qrw, L));
    }
    // restart with the current Ritz vectors (src/davidson.F90:151-155)
    SS_CUDA_TRY(cudaMemcpyAsync(U, X, sizeof(double) * N * m, cudaMemcpyDeviceToDevice, st));
    TRY(ortho_qr(st, N, m, U, N, qrw, L));
  }
  if (!converged) {
    ss_set_error_msg("davidson: not converged after %d iterations (largest correction %g)", max_iter, hmax);
    return SS_ERR_NUMERIC;
  }
  SS_CUDA_TRY(cudaMemcpyAsync(hE.data(), ev, sizeof(double) * m, cudaMemcpyDeviceToHost, st));
  if (evecs) SS_CUDA_TRY(cudaMemcpyAsync(evecs, X, sizeof(double) * N * m, cudaMemcpyDeviceToHost, st));
  SS_CUDA_TRY(cudaStreamSynchronize(st));
  if (evals) memcpy(evals, hE.data(), sizeof(double) * m);
  return SS_OK;
}

// ---------------------------------------------------------------------------------------
// Matrix-free Davidson cleanup (the nbasis >= 200 branch of src/davidson_clean.F90:120-323)
// ---------------------------------------------------------------------------------------
// The ERI matrix is never formed.  Each pass writes the quartet list once into the packed
// lower triangle of the pair metric, tri[P1 (P1+1)/2 + P2] = (ik|jl) with P1 = pair(i,k) >=
// P2 = pair(j,l): one double per canonical quartet, the reference's 8-fold list without its
// n^2 x n^2 expansion.  Both layouts read their elements from it: PACKED_PAIR M(p, q) =
// tri(max, min); REF_N2 W(a + b n, c + d n) = <ab|cd> = (ac|bd) = M(pair(a,c), pair(b,d)) --
// the same element the reference's 8 index permutations of one quartet reach
// (src/davidson_clean.F90:165-187).  Products H X are gathered row by row, so they carry no
// atomics and are reproducible.
__device__ __forceinline__ int64_t sym_pair(int64_t a, int64_t b) {
  return a >= b ? a * (a + 1) / 2 + b : b * (b + 1) / 2 + a;
}

__global__ void tri_fill_kernel(int64_t nint, const int32_t* __restrict__ is, const int32_t* __restrict__ js,
                                const int32_t* __restrict__ ks, const int32_t* __restrict__ ls,
                                const double* __restrict__ moy, double* __restrict__ tri) {
  const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (q >= nint) return;
  const int i = is[q] - 1, j = js[q] - 1, k = ks[q] - 1, l = ls[q] - 1;
  tri[sym_pair(sym_pair(i, k), sym_pair(j, l))] = moy[q];
}

__device__ __forceinline__ double op_element(int layout, int n, const double* __restrict__ tri, int r, int c) {
  if (layout == SS_LAYOUT_REF_N2) {
    const int a = r % n, b = r / n, cc = c % n, d = c / n;
    return tri[sym_pair(sym_pair(a, cc), sym_pair(b, d))];
  }
  return tri[sym_pair(r, c)];
}

constexpr int MF_ROWS = 16, MF_COLS = 32, MF_MAXM = 128;

// Y = H X, X and Y N x m column-major (leading dimension N), m <= MF_MAXM.  One CTA per 16
// rows; thread t owns row t % 16 and the columns t / 16 + 16 s.
__global__ void __launch_bounds__(256) op_apply_kernel(int layout, int n, int N, int m,
                                                       const double* __restrict__ tri,
                                                       const double* __restrict__ X, double* __restrict__ Y) {
  __shared__ double sE[MF_ROWS][MF_COLS + 1];
  __shared__ double sX[MF_COLS][MF_MAXM];
  const int r0 = blockIdx.x * MF_ROWS;
  const int t = threadIdx.x, rr = t & (MF_ROWS - 1), c16 = t >> 4;
  double acc[MF_MAXM / 16];
#pragma unroll
  for (int s = 0; s < MF_MAXM / 16; s++) acc[s] = 0.0;
  for (int c0 = 0; c0 < N; c0 += MF_COLS) {
    for (int e = t; e < MF_ROWS * MF_COLS; e += blockDim.x) {
      const int er = e / MF_COLS, ec = e % MF_COLS;
      sE[er][ec] = (r0 + er < N && c0 + ec < N) ? op_element(layout, n, tri, r0 + er, c0 + ec) : 0.0;
    }
    for (int e = t; e < MF_COLS * m; e += blockDim.x) {
      const int ec = e % MF_COLS, j = e / MF_COLS;
      sX[ec][j] = (c0 + ec < N) ? X[(c0 + ec) + (size_t)j * N] : 0.0;
    }
    __syncthreads();
#pragma unroll 4
    for (int cc = 0; cc < MF_COLS; cc++) {
      const double h = sE[rr][cc];
#pragma unroll
      for (int s = 0; s < MF_MAXM / 16; s++)
        if (c16 + 16 * s < m) acc[s] = fma(h, sX[cc][c16 + 16 * s], acc[s]);
    }
    __syncthreads();
  }
  if (r0 + rr < N) {
#pragma unroll
    for (int s = 0; s < MF_MAXM / 16; s++)
      if (c16 + 16 * s < m) Y[(r0 + rr) + (size_t)(c16 + 16 * s) * N] = acc[s];
  }
}


// residuals R_j = E_j X_j - (H X)_j (src/davidson_clean.F90:277-283)
__global__ void residual_kernel(int N, int m, const double* __restrict__ X, const double* __restrict__ WX,
                                const double* __restrict__ E, double* __restrict__ R) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= (int64_t)N * m) return;
  R[e] = E[e / N] * X[e] - WX[e];
}

// moy(kcp) -= E_j U(ii, j) U(jj, j) for the nneg negative pairs, canonical (ii, jj) of each
// quartet (src/davidson_clean.F90:310-317)
__global__ void deflate_kernel(int64_t nint, int layout, int n, int N, const int32_t* __restrict__ is,
                               const int32_t* __restrict__ js, const int32_t* __restrict__ ks,
                               const int32_t* __restrict__ ls, int nneg, const double* __restrict__ E,
                               const double* __restrict__ U, double* __restrict__ moy) {
  const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (q >= nint) return;
  const int i = is[q] - 1, j = js[q] - 1, k = ks[q] - 1, l = ls[q] - 1;
  int64_t ii, jj;
  if (layout == SS_LAYOUT_REF_N2) {
    ii = i + (int64_t)j * n;
    jj = k + (int64_t)l * n;
  } else {
    ii = sym_pair(i, k);
    jj = sym_pair(j, l);
  }
  double v = moy[q];
  for (int t = 0; t < nneg; t++) v = v - E[t] * U[ii + (size_t)t * N] * U[jj + (size_t)t * N];
  moy[q] = v;
}

static int op_apply(ss_ctx* c, int layout, int N, int m, const double* tri, const double* X, double* Y) {
  op_apply_kernel<<<(N + MF_ROWS - 1) / MF_ROWS, 256, 0, c->stream>>>(layout, c->n, N, m, tri, X, Y);
  SS_CUDA_TRY(cudaGetLastError());
  c->launches++;
  return SS_OK;
}

// V (N x b, leading dimension N) made orthonormal and orthogonal to U (N x k): two classical
// Gram-Schmidt passes against U, Householder QR of the block, then the pair once more (a block
// whose residuals vanished comes back from the first QR with unit columns that need not be
// orthogonal to U).
static int orthonormalize_block(ss_ctx* c, int N, int k, int b, const double* U, double* V, double* tmp,
                                double* qrw, double* gws) {
  for (int round = 0; round < 2; round++) {
    for (int rep = 0; rep < 2 && k > 0; rep++) {
      TRY(dgemm(c->stream, 1, 0, k, b, N, 1.0, U, N, V, N, 0.0, tmp, k, gws, &c->launches));
      TRY(dgemm(c->stream, 0, 0, N, b, k, -1.0, U, N, tmp, k, 1.0, V, N, gws, &c->launches));
    }
    TRY(ortho_qr(c->stream, N, b, V, N, qrw, &c->launches));
  }
  return SS_OK;
}

// Block Davidson for the lowest `m` eigenpairs (the reference's mmax = NMAX = nbasis unless
// given), plain residual expansion, basis of at most kmax = nmax m vectors (capped at N and at
// the 1024 of the device eigensolver) restarted from the Ritz vectors when full.  A search ends
// when the Ritz pairs up to the middle one (index m/2, the reference's test,
// src/davidson_clean.F90:286) and every negative Ritz pair have residual norm below tol, or
// when the basis spans the whole space; its negative Ritz pairs (below -1e-13 of the largest
// |ERI|, rounding level) are then deflated from moy and the search restarts from new random
// vectors, until a search finds none.  The reference also ends a search as soon as all m Ritz
// values are negative and deflates those pairs unconverged; converging them first makes the
// result with a basis that can span the whole space the exact projection's (for the packed
// metric, whose canonical read-back is exact).  The basis is kept orthonormal, so the
// projected problem is a standard symmetric one (the reference solves the equivalent
// generalized problem with dsygv).
int davidson_clean(ss_ctx* c, double* moy_host, int layout, int m, int nmax, double tol, int max_iter,
                   int* n_removed) {
  const int n = c->n;
  const int64_t N64 = layout == SS_LAYOUT_REF_N2 ? (int64_t)n * n : (int64_t)n * (n + 1) / 2;
  if (N64 < 2 || N64 > (1 << 26)) {
    ss_set_error_msg("davidson_clean: matrix dimension %lld out of range", (long long)N64);
    return SS_ERR_ARG;
  }
  const int N = (int)N64;
  // src/davidson_clean.F90:129-131: mmax = NMAX = nbasis; the default block is capped at the
  // MF_MAXM columns one product handles (a caller asking for more gets SS_ERR_UNSUPPORTED)
  if (m <= 0) m = std::min(n, MF_MAXM);
  if (nmax <= 0) nmax = n;
  m = std::min(m, std::max(1, N / 2));
  if (m > MF_MAXM) {
    ss_set_error_msg("davidson_clean: block of %d vectors above the %d supported", m, MF_MAXM);
    return SS_ERR_UNSUPPORTED;
  }
  int kmax = (int)std::min<int64_t>({(int64_t)m * std::max(nmax, 2), (int64_t)N, 1024});
  kmax = kmax / m * m;
  if (kmax < 2 * m) kmax = 2 * m;  // m <= N/2 and m <= 128: 2m <= min(N, 1024)
  double scale = 0.0;
  for (int64_t q = 0; q < c->nint; q++) scale = std::max(scale, fabs(moy_host[q]));
  const double neg_eps = 1e-13 * scale;
  void* p;
  double *tri, *U, *WU, *S, *Sa, *Vk, *ev, *X, *WX, *R, *nrm, *tmp, *moy, *qrw, *eigw, *gws;
  const int64_t T = (int64_t)(n * (n + 1) / 2) * (n * (n + 1) / 2 + 1) / 2;
  const size_t Nk = (size_t)N * kmax, Nm = (size_t)N * m, kk2 = (size_t)kmax * kmax;
  const size_t gsz = std::max({dgemm_ws(kmax, kmax, N), dgemm_ws(N, m, kmax), dgemm_ws(kmax, m, N), (size_t)1});
  TRY(pool_get(c, "dc_tri", sizeof(double) * T, &p)); tri = (double*)p;
  TRY(pool_get(c, "dc_U", sizeof(double) * Nk, &p)); U = (double*)p;
  TRY(pool_get(c, "dc_WU", sizeof(double) * Nk, &p)); WU = (double*)p;
  TRY(pool_get(c, "dc_S", sizeof(double) * kk2, &p)); S = (double*)p;
  TRY(pool_get(c, "dc_Sa", sizeof(double) * kk2, &p)); Sa = (double*)p;
  TRY(pool_get(c, "dc_Vk", sizeof(double) * kk2, &p)); Vk = (double*)p;
  TRY(pool_get(c, "dc_ev", sizeof(double) * kmax, &p)); ev = (double*)p;
  TRY(pool_get(c, "dc_X", sizeof(double) * Nm, &p)); X = (double*)p;
  TRY(pool_get(c, "dc_WX", sizeof(double) * Nm, &p)); WX = (double*)p;
  TRY(pool_get(c, "dc_R", sizeof(double) * Nm, &p)); R = (double*)p;
  TRY(pool_get(c, "dc_nrm", sizeof(double) * m, &p)); nrm = (double*)p;
  TRY(pool_get(c, "dc_tmp", sizeof(double) * (size_t)kmax * m, &p)); tmp = (double*)p;
  TRY(pool_get(c, "dc_moy", sizeof(double) * c->nint, &p)); moy = (double*)p;
  TRY(pool_get(c, "dc_qr", sizeof(double) * ortho_qr_ws(N, m), &p)); qrw = (double*)p;
  TRY(pool_get(c, "dc_eig", sizeof(double) * std::max<size_t>(sym_eig_ws(kmax), 1), &p)); eigw = (double*)p;
  TRY(pool_get(c, "dc_gws", sizeof(double) * gsz, &p)); gws = (double*)p;
  TRY(pool_get(c, "dc_ctl", 64, &p));
  int* derr = (int*)p;
  int64_t* L = &c->launches;
  cudaStream_t st = c->stream;
  const int32_t *d_is = (const int32_t*)c->d_is.ptr, *d_js = (const int32_t*)c->d_js.ptr,
                *d_ks = (const int32_t*)c->d_ks.ptr, *d_ls = (const int32_t*)c->d_ls.ptr;
  SS_CUDA_TRY(cudaMemsetAsync(derr, 0, sizeof(int), st));
  SS_CUDA_TRY(cudaMemcpyAsync(moy, moy_host, sizeof(double) * c->nint, cudaMemcpyHostToDevice, st));
  std::vector<double> hE(m), hn(m);
  int removed = 0, total = 0;
  for (int pass = 0;; pass++) {
    SS_CUDA_TRY(cudaMemsetAsync(tri, 0, sizeof(double) * T, st));
    tri_fill_kernel<<<nb(c->nint), 256, 0, st>>>(c->nint, d_is, d_js, d_ks, d_ls, moy, tri);
    // normalised Gaussian start vectors (src/davidson_clean.F90:137-149), orthonormalised
    gaussian_matrix_kernel<<<m, 256, 0, st>>>(1, 0x44434c00u + (uint32_t)pass, N, m, U);
    *L += 2;
    TRY(ortho_qr(st, N, m, U, N, qrw, L));
    TRY(op_apply(c, layout, N, m, tri, U, WU));
    int k = m;
    for (;;) {
      if (++total > max_iter) {
        ss_set_error_msg("davidson_clean: not converged after %d iterations (pass %d, residual %g)", max_iter,
                         pass, hn[m / 2]);
        return SS_ERR_NUMERIC;
      }
      // Rayleigh-Ritz on span(U): S = U^T H U, lowest m eigenpairs
      TRY(dgemm(st, 1, 0, k, k, N, 1.0, U, N, WU, N, 0.0, S, k, gws, L));
      sym_copy_kernel<<<nb((int64_t)k * k), 256, 0, st>>>(k, S, Sa);
      (*L)++;
      TRY(sym_eig(st, k, Sa, Vk, ev, eigw, derr, L));
      TRY(dgemm(st, 0, 0, N, m, k, 1.0, U, N, Vk, k, 0.0, X, N, gws, L));
      TRY(dgemm(st, 0, 0, N, m, k, 1.0, WU, N, Vk, k, 0.0, WX, N, gws, L));
      residual_kernel<<<nb((int64_t)N * m), 256, 0, st>>>(N, m, X, WX, ev, R);
      col_norms_kernel<<<m, 256, 0, st>>>(N, m, R, nrm);
      *L += 2;
      int herr = 0;
      SS_CUDA_TRY(cudaMemcpyAsync(hE.data(), ev, sizeof(double) * m, cudaMemcpyDeviceToHost, st));
      SS_CUDA_TRY(cudaMemcpyAsync(hn.data(), nrm, sizeof(double) * m, cudaMemcpyDeviceToHost, st));
      SS_CUDA_TRY(cudaMemcpyAsync(&herr, derr, sizeof(int), cudaMemcpyDeviceToHost, st));
      SS_CUDA_TRY(cudaStreamSynchronize(st));
      if (herr) {
        ss_set_error_msg("davidson_clean: projected eigenproblem %s", herr == 2 ? "timed out" : "did not converge");
        return herr == 2 ? SS_ERR_TIMEOUT : SS_ERR_NUMERIC;
      }
      double rmax = 0.0;
      for (int j = 0; j < m; j++)
        if (j <= m / 2 || hE[j] < -neg_eps) rmax = std::max(rmax, hn[j]);
      if (rmax < tol || k == N) break;
      if (k + m > kmax) {  // restart from the Ritz vectors (src/davidson_clean.F90:293-299)
        SS_CUDA_TRY(cudaMemcpyAsync(U, X, sizeof(double) * Nm, cudaMemcpyDeviceToDevice, st));
        TRY(ortho_qr(st, N, m, U, N, qrw, L));
        TRY(op_apply(c, layout, N, m, tri, U, WU));
        k = m;
        continue;
      }
      double* Un = U + (size_t)k * N;
      SS_CUDA_TRY(cudaMemcpyAsync(Un, R, sizeof(double) * Nm, cudaMemcpyDeviceToDevice, st));
      TRY(orthonormalize_block(c, N, k, m, U, Un, tmp, qrw, gws));
      TRY(op_apply(c, layout, N, m, tri, Un, WU + (size_t)k * N));
      k += m;
    }
    int nneg = 0;
    while (nneg < m && hE[nneg] < -neg_eps) nneg++;  // ascending
    if (nneg == 0) break;
    deflate_kernel<<<nb(c->nint), 256, 0, st>>>(c->nint, layout, n, N, d_is, d_js, d_ks, d_ls, nneg, ev, X, moy);
    SS_CUDA_TRY(cudaGetLastError());
    (*L)++;
    removed += nneg;
  }
  SS_CUDA_TRY(cudaMemcpyAsync(moy_host, moy, sizeof(double) * c->nint, cudaMemcpyDeviceToHost, st));
  SS_CUDA_TRY(cudaStreamSynchronize(st));
  if (n_removed) *n_removed = removed;
  return SS_OK;
}

}  // namespace ss

using namespace ss;

extern "C" {

int ss_psd_clean(ss_ctx* c, double* moy, int layout, int rank, int oversample, int q, uint64_t seed,
                 int* n_removed) {
  if (!c) {
    ss_set_error_msg("null ss_ctx");
    return SS_ERR_ARG;
  }
  SS_CUDA_TRY(cudaSetDevice(c->device));
  if (!c->n || !c->nint) {
    ss_set_error_msg("basis and quartets must be set first");
    return SS_ERR_STATE;
  }
  if (!moy || (layout != SS_LAYOUT_REF_N2 && layout != SS_LAYOUT_PACKED_PAIR) || rank < 1 || oversample < 0 ||
      q < 0) {
    ss_set_error_msg("ss_psd_clean: bad arguments");
    return SS_ERR_ARG;
  }
  return psd_clean(c, moy, layout, rank, oversample, q, seed, n_removed);
}

int ss_psd_project(ss_ctx* c, double* moy, int layout, int* n_removed) {
  if (!c) {
    ss_set_error_msg("null ss_ctx");
    return SS_ERR_ARG;
  }
  SS_CUDA_TRY(cudaSetDevice(c->device));
  if (!c->n || !c->nint) {
    ss_set_error_msg("basis and quartets must be set first");
    return SS_ERR_STATE;
  }
  if (!moy || (layout != SS_LAYOUT_REF_N2 && layout != SS_LAYOUT_PACKED_PAIR)) {
    ss_set_error_msg("ss_psd_project: bad arguments");
    return SS_ERR_ARG;
  }
  return psd_project(c, moy, layout, n_removed);
}

int ss_davidson(ss_ctx* c, const double* moy, int layout, int m, double tol, int max_iter, double* evals,
                double* evecs) {
  if (!c) {
    ss_set_error_msg("null ss_ctx");
    return SS_ERR_ARG;
  }
  SS_CUDA_TRY(cudaSetDevice(c->device));
  if (!c->n || !c->nint) {
    ss_set_error_msg("basis and quartets must be set first");
    return SS_ERR_STATE;
  }
  if (!moy || (layout != SS_LAYOUT_REF_N2 && layout != SS_LAYOUT_PACKED_PAIR) || !(tol > 0.0) || max_iter < 1) {
    ss_set_error_msg("ss_davidson: bad arguments");
    return SS_ERR_ARG;
  }
  return davidson(c, moy, layout, m, tol, max_iter, evals, evecs);
}

int ss_davidson_clean(ss_ctx* c, double* moy, int layout, int block, int max_blocks, double tol, int max_iter,
                      int* n_removed) {
  if (!c) {
    ss_set_error_msg("null ss_ctx");
    return SS_ERR_ARG;
  }
  SS_CUDA_TRY(cudaSetDevice(c->device));
  if (!c->n || !c->nint) {
    ss_set_error_msg("basis and quartets must be set first");
    return SS_ERR_STATE;
  }
  if (!moy || (layout != SS_LAYOUT_REF_N2 && layout != SS_LAYOUT_PACKED_PAIR) || !(tol > 0.0) || max_iter < 1) {
    ss_set_error_msg("ss_davidson_clean: bad arguments");
    return SS_ERR_ARG;
  }
  return davidson_clean(c, moy, layout, block, max_blocks, tol, max_iter, n_removed);
}

}  // extern "C"
