// linalg.cu -- FP64 dense linear algebra of the PSD cleanup, on the device.
//
//  * Householder QR of a tall N x r matrix and the explicit Q (the roles of dgeqrf/dorgqr in
//    src/ortho_qr.F90:1-39): one reflector kernel and one trailing-update kernel per column.
//  * Symmetric eigen-decomposition of an n x n matrix (n <= 1024) in one CTA: Householder
//    reduction to tridiagonal form with accumulated transformations, then implicit QL with
//    Wilkinson shifts on the tridiagonal (the classical tred2 / tql2 procedure), eigenvalues
//    ascending.  Used for the small SVD of svd_clean (src/svd.F90) and Davidson's projected
//    eigenproblem (src/davidson.F90:77-94).
#include <math.h>

#include "linalg.cuh"
#include "ss_common.cuh"

namespace ss {

// ---------------------------------------------------------------------------------------
// Householder QR, column-major Z (ld >= N)
// ---------------------------------------------------------------------------------------
__device__ __forceinline__ double block_sum(double v, double* sh) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) sh[w] = v;
  __syncthreads();
  if (w == 0) {
    v = (l < (int)(blockDim.x >> 5)) ? sh[l] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (l == 0) sh[0] = v;
  }
  __syncthreads();
  const double r = sh[0];
  __syncthreads();
  return r;
}

// reflector for column j: v = x - alpha e1 (stored in Z[j:,j] with v[0] = 1), tau, R_jj = alpha
__global__ void hh_reflector(int N, int j, double* Z, int ld, double* tau) {
  __shared__ double sh[32];
  double* x = Z + (size_t)j * ld;
  double ss = 0.0;
  for (int i = j + 1 + threadIdx.x; i < N; i += blockDim.x) ss += x[i] * x[i];
  const double sigma = block_sum(ss, sh);
  const double x0 = x[j];
  if (sigma == 0.0) {
    if (threadIdx.x == 0) tau[j] = 0.0;
    return;
  }
  const double mu = sqrt(x0 * x0 + sigma);
  const double alpha = x0 <= 0.0 ? mu : -mu;  // R_jj, sign chosen to avoid cancellation
  const double v0 = x0 - alpha;
  const double inv = 1.0 / v0;
  for (int i = j + 1 + threadIdx.x; i < N; i += blockDim.x) x[i] *= inv;
  if (threadIdx.x == 0) {
    tau[j] = -v0 / alpha;  // H = I - tau v v^T with v0 = 1
    x[j] = alpha;
  }
}

// apply H_j to columns c in [c0, c1): Z[j:,c] -= tau (v^T Z[j:,c]) v
__global__ void hh_apply(int N, int j, int c0, int c1, const double* V, int ldv, double* Z, int ld,
                         const double* tau) {
  __shared__ double sh[32];
  const int c = c0 + blockIdx.x;
  if (c >= c1) return;
  const double t = tau[j];
  if (t == 0.0) return;
  const double* v = V + (size_t)j * ldv;
  double* z = Z + (size_t)c * ld;
  double s = (threadIdx.x == 0) ? z[j] : 0.0;
  for (int i = j + 1 + threadIdx.x; i < N; i += blockDim.x) s += v[i] * z[i];
  const double w = t * block_sum(s, sh);
  if (threadIdx.x == 0) z[j] -= w;
  for (int i = j + 1 + threadIdx.x; i < N; i += blockDim.x) z[i] -= w * v[i];
}

__global__ void set_identity_cols(int N, int r, double* Q, int ld) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= (int64_t)N * r) return;
  const int i = (int)(e % N), c = (int)(e / N);
  Q[(size_t)c * ld + i] = (i == c) ? 1.0 : 0.0;
}

int ortho_qr(cudaStream_t st, int N, int r, double* Z, int ld, double* Qwork, double* tau, int64_t* launches) {
  if (r > N) {
    ss_set_error_msg("ortho_qr: more columns (%d) than rows (%d)", r, N);
    return SS_ERR_ARG;
  }
  const int T = 256;
  for (int j = 0; j < r; j++) {
    hh_reflector<<<1, T, 0, st>>>(N, j, Z, ld, tau);
    if (j + 1 < r) hh_apply<<<r - j - 1, T, 0, st>>>(N, j, j + 1, r, Z, ld, Z, ld, tau);
  }
  // explicit Q = H_0 ... H_{r-1} [I; 0]
  set_identity_cols<<<(unsigned)(((int64_t)N * r + 255) / 256), 256, 0, st>>>(N, r, Qwork, ld);
  for (int j = r - 1; j >= 0; j--) hh_apply<<<r - j, T, 0, st>>>(N, j, j, r, Z, ld, Qwork, ld, tau);
  SS_CUDA_TRY(cudaGetLastError());
  SS_CUDA_TRY(cudaMemcpy2DAsync(Z, sizeof(double) * ld, Qwork, sizeof(double) * ld, sizeof(double) * N, r,
                                cudaMemcpyDeviceToDevice, st));
  if (launches) *launches += 2 * r + 1;
  return SS_OK;
}

// ---------------------------------------------------------------------------------------
// symmetric eigen-decomposition, one CTA (blockDim 1024), row-major a[i*n+j]
// ---------------------------------------------------------------------------------------
__global__ void __launch_bounds__(1024) sym_eig_kernel(int n, double* __restrict__ a, double* __restrict__ d,
                                                       double* __restrict__ e, int* __restrict__ info) {
  __shared__ double sh[32];
  __shared__ double s_f, s_hh, s_anorm;
  __shared__ double s_c[1024], s_s[1024];
  __shared__ int s_m, s_cnt, s_stop;
  const int tid = threadIdx.x, nt = blockDim.x;
#define A(i, j) a[(size_t)(i) * n + (j)]
  // --- Householder tridiagonalisation with accumulated transformations -------------------
  for (int i = n - 1; i > 0; i--) {
    const int l = i - 1;
    double h = 0.0;
    if (l > 0) {
      double sc = 0.0;
      for (int k = tid; k <= l; k += nt) sc += fabs(A(i, k));
      const double scale = block_sum(sc, sh);
      if (scale == 0.0) {
        if (tid == 0) e[i] = A(i, l);
      } else {
        double hh = 0.0;
        for (int k = tid; k <= l; k += nt) {
          const double v = A(i, k) / scale;
          A(i, k) = v;
          hh += v * v;
        }
        h = block_sum(hh, sh);
        const double f0 = A(i, l);
        const double g0 = f0 >= 0.0 ? -sqrt(h) : sqrt(h);
        __syncthreads();  // every thread has read A(i,l) before it changes
        if (tid == 0) {
          e[i] = scale * g0;
          A(i, l) = f0 - g0;
        }
        h = h - f0 * g0;
        __syncthreads();
        // p = A u / h  (u = row i, entries 0..l), stored in e[0..l]
        double fpart = 0.0;
        for (int j = tid; j <= l; j += nt) {
          A(j, i) = A(i, j) / h;
          double g = 0.0;
          for (int k = 0; k <= j; k++) g += A(j, k) * A(i, k);
          for (int k = j + 1; k <= l; k++) g += A(k, j) * A(i, k);
          e[j] = g / h;
          fpart += e[j] * A(i, j);
        }
        const double f = block_sum(fpart, sh);
        const double hh2 = f / (h + h);
        for (int j = tid; j <= l; j += nt) e[j] = e[j] - hh2 * A(i, j);
        __syncthreads();
        // A -= u q^T + q u^T on the lower triangle
        for (int idx = tid; idx < (l + 1) * (l + 1); idx += nt) {
          const int j = idx / (l + 1), k = idx % (l + 1);
          if (k <= j) A(j, k) -= (A(i, j) * e[k] + e[j] * A(i, k));
        }
        __syncthreads();
      }
    } else {
      if (tid == 0) e[i] = A(i, l);
    }
    if (tid == 0) d[i] = h;
    __syncthreads();
  }
  if (tid == 0) {
    d[0] = 0.0;
    e[0] = 0.0;
  }
  __syncthreads();
  for (int i = 0; i < n; i++) {
    if (d[i] != 0.0) {
      // g_j = sum_k A(i,k) A(k,j); A(k,j) -= g_j A(k,i)   for j,k < i
      for (int j = tid; j < i; j += nt) {
        double g = 0.0;
        for (int k = 0; k < i; k++) g += A(i, k) * A(k, j);
        e[n + j] = g;  // scratch (e has 2n entries)
      }
      __syncthreads();
      for (int idx = tid; idx < i * i; idx += nt) {
        const int k = idx / i, j = idx % i;
        A(k, j) -= e[n + j] * A(k, i);
      }
      __syncthreads();
    }
    if (tid == 0) d[i] = A(i, i);
    __syncthreads();
    if (tid == 0) A(i, i) = 1.0;
    for (int j = tid; j < i; j += nt) {
      A(j, i) = 0.0;
      A(i, j) = 0.0;
    }
    __syncthreads();
  }
  // --- implicit QL on the tridiagonal (d, e), rotating the rows of A ------------------------
  if (tid == 0) {
    for (int i = 1; i < n; i++) e[i - 1] = e[i];
    e[n - 1] = 0.0;
    *info = 0;
    double an = 0.0;
    for (int i = 0; i < n; i++) an = fmax(an, fabs(d[i]) + fabs(e[i]));
    s_anorm = an;
  }
  __syncthreads();
  for (int l = 0; l < n; l++) {
    int iter = 0;
    while (true) {
      if (tid == 0) {
        int m;
        for (m = l; m < n - 1; m++) {
          const double dd = fabs(d[m]) + fabs(d[m + 1]);
          // split where e[m] is negligible next to its diagonal neighbours or to the whole
          // matrix (the absolute test deflates blocks of rounding-level entries, e.g. the
          // numerical null space of a rank-deficient Coulomb metric, that the relative test
          // alone would iterate on without converging)
          if (fabs(e[m]) <= 2.2204460492503131e-16 * dd || fabs(e[m]) <= 2.2204460492503131e-16 * s_anorm) break;
        }
        s_m = m;
        s_cnt = 0;
        s_stop = 0;
        if (m != l) {
          if (iter >= 60) {
            *info = l + 1;  // no convergence
            s_stop = 1;
          } else {
            double g = (d[l + 1] - d[l]) / (2.0 * e[l]);
            double r = hypot(g, 1.0);
            g = d[m] - d[l] + e[l] / (g + (g >= 0.0 ? fabs(r) : -fabs(r)));
            double s = 1.0, c = 1.0, p = 0.0;
            int i;
            bool underflow = false;
            for (i = m - 1; i >= l; i--) {
              double f = s * e[i], b = c * e[i];
              r = hypot(f, g);
              e[i + 1] = r;
              if (r == 0.0) {
                d[i + 1] -= p;
                e[m] = 0.0;
                underflow = true;
                break;
              }
              s = f / r;
              c = g / r;
              g = d[i + 1] - p;
              r = (d[i] - g) * s + 2.0 * c * b;
              p = s * r;
              d[i + 1] = g + p;
              g = c * r - b;
              s_c[s_cnt] = c;
              s_s[s_cnt] = s;
              s_cnt++;
            }
            if (!underflow) {
              d[l] -= p;
              e[l] = g;
              e[m] = 0.0;
            }
          }
        }
      }
      __syncthreads();
      const int m = s_m;
      if (m == l || s_stop) break;
      // rotations i = m-1, m-2, ... applied to columns (i, i+1) of the eigenvector matrix
      const int cnt = s_cnt;
      for (int k = tid; k < n; k += nt) {
        for (int t = 0; t < cnt; t++) {
          const int i = m - 1 - t;
          const double f = A(k, i + 1);
          A(k, i + 1) = s_s[t] * A(k, i) + s_c[t] * f;
          A(k, i) = s_c[t] * A(k, i) - s_s[t] * f;
        }
      }
      iter++;
      __syncthreads();
    }
    if (s_stop) break;
  }
  __syncthreads();
  // --- sort eigenvalues ascending (selection sort, columns swapped in parallel) -------------
  for (int i = 0; i < n - 1; i++) {
    if (tid == 0) {
      int k = i;
      double p = d[i];
      for (int j = i + 1; j < n; j++)
        if (d[j] < p) {
          k = j;
          p = d[j];
        }
      s_m = k;
      if (k != i) {
        d[k] = d[i];
        d[i] = p;
      }
    }
    __syncthreads();
    const int k = s_m;
    if (k != i)
      for (int j = tid; j < n; j += nt) {
        const double t = A(j, i);
        A(j, i) = A(j, k);
        A(j, k) = t;
      }
    __syncthreads();
  }
#undef A
}

int sym_eig(cudaStream_t st, int n, double* a, double* w, double* work, int* info, int64_t* launches) {
  if (n < 1 || n > 1024) {
    ss_set_error_msg("sym_eig: n=%d outside 1..1024", n);
    return SS_ERR_UNSUPPORTED;
  }
  sym_eig_kernel<<<1, 1024, 0, st>>>(n, a, w, work, info);
  SS_CUDA_TRY(cudaGetLastError());
  if (launches) (*launches)++;
  return SS_OK;
}

}  // namespace ss
