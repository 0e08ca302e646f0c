// linalg.cu -- FP64 dense linear algebra of the PSD cleanup and Davidson, on the device.
//
// GB300 runs FP64 at about 1/64 of its FP32 rate (two DFMA per clock per SM), so a one-SM
// solver of an n = 351 eigenproblem would take tens of milliseconds however it is written.
// The routines here spread the FP64 work over the whole GPU:
//  * dgemm: 32 x 32 output tiles, 256 threads with 2 x 2 accumulators each, 16-deep k steps
//    through shared memory; an inner dimension much longer than the output is split over
//    CTAs into a workspace and summed in a fixed order (no atomics: reproducible results);
//  * ortho_qr: blocked Householder QR (LAPACK's dgeqrf/dorgqr structure): one CTA factorises
//    each 32-column panel and forms its compact-WY factor T (H_1 ... H_b = I - V T V^T), the
//    trailing columns and the explicit Q are updated by three dgemm calls per panel;
//  * sym_eig, n > 128: cyclic two-sided Jacobi with the round-robin ("circle") pair order.  The
//    n/2 rotations of a round act on disjoint index pairs, so A' = J^T A J splits into
//    independent 2 x 2 blocks J_P^T A_PR J_R, written into a second buffer (no read-after-write
//    hazard inside a round), and V' = V J into independent row pairs.  One cooperative grid
//    does all rounds and sweeps with a bounded grid barrier per round;
//  * sym_eig, n <= 128: one CTA with the matrix in shared memory: Householder reduction to
//    tridiagonal form with accumulated transformations and implicit QL with Wilkinson shifts
//    (the classical tred2 / tql2 procedure), used for Davidson's small projected problems.
#include <math.h>

#include <algorithm>

#include "linalg.cuh"
#include "ss_common.cuh"

namespace ss {

namespace {

int sm_count() {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) !=
                                                  cudaSuccess || sms <= 0)
    sms = 152;
  return sms;
}

unsigned nblk(int64_t n, int t = 256) { return (unsigned)((n + t - 1) / t); }

}  // namespace

// ---------------------------------------------------------------------------------------
// GEMM
// ---------------------------------------------------------------------------------------
constexpr int GT = 32, GKS = 16;

// 32 x 32 output tile, 256 threads with 2 x 2 accumulators each (one FP64 FMA per shared-memory
// read pair: FP64 throughput, not shared-memory bandwidth, is the limit).  Small tiles waste
// little on the skinny products of the eigensolvers and Davidson (n = 10 columns).
__global__ void __launch_bounds__(256) dgemm_kernel(int ta, int tb, int m, int n, int k, int kper, double alpha,
                                                    const double* __restrict__ A, int lda,
                                                    const double* __restrict__ B, int ldb, double beta,
                                                    double* __restrict__ C, int ldc, double* __restrict__ ws) {
  __shared__ double As[GKS][GT + 1];  // As[kk][i] = op(A)(i0 + i, k0 + kk)
  __shared__ double Bs[GKS][GT + 1];  // Bs[kk][j] = op(B)(k0 + kk, j0 + j)
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int i0 = blockIdx.x * GT, j0 = blockIdx.y * GT;
  const int kb = blockIdx.z * kper, ke = min(k, kb + kper);
  double acc[2][2] = {{0.0, 0.0}, {0.0, 0.0}};
  for (int k0 = kb; k0 < ke; k0 += GKS) {
    for (int e = threadIdx.x; e < GT * GKS; e += 256) {
      // consecutive threads along the contiguous dimension of the source
      const int i = ta ? e / GKS : e % GT, kk = ta ? e % GKS : e / GT;
      const int gi = i0 + i, gk = k0 + kk;
      As[kk][i] = (gi < m && gk < ke) ? (ta ? A[gk + (size_t)gi * lda] : A[gi + (size_t)gk * lda]) : 0.0;
    }
    for (int e = threadIdx.x; e < GT * GKS; e += 256) {
      const int j = tb ? e % GT : e / GKS, kk = tb ? e / GT : e % GKS;
      const int gj = j0 + j, gk = k0 + kk;
      Bs[kk][j] = (gj < n && gk < ke) ? (tb ? B[gj + (size_t)gk * ldb] : B[gk + (size_t)gj * ldb]) : 0.0;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < GKS; kk++) {
      const double a0 = As[kk][tx], a1 = As[kk][tx + 16];
      const double b0 = Bs[kk][ty], b1 = Bs[kk][ty + 16];
      acc[0][0] = fma(a0, b0, acc[0][0]);
      acc[0][1] = fma(a0, b1, acc[0][1]);
      acc[1][0] = fma(a1, b0, acc[1][0]);
      acc[1][1] = fma(a1, b1, acc[1][1]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int r = 0; r < 2; r++)
#pragma unroll
    for (int c = 0; c < 2; c++) {
      const int gi = i0 + tx + 16 * r, gj = j0 + ty + 16 * c;
      if (gi >= m || gj >= n) continue;
      if (gridDim.z == 1) {
        double* cp = C + gi + (size_t)gj * ldc;
        *cp = beta == 0.0 ? alpha * acc[r][c] : fma(alpha, acc[r][c], beta * *cp);
      } else {
        ws[(size_t)blockIdx.z * m * n + gi + (size_t)gj * m] = acc[r][c];
      }
    }
}

__global__ void dgemm_reduce(int m, int n, int ks, double alpha, const double* __restrict__ ws, double beta,
                             double* __restrict__ C, int ldc) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= (int64_t)m * n) return;
  double s = 0.0;
  for (int z = 0; z < ks; z++) s += ws[(size_t)z * m * n + e];
  double* cp = C + (e % m) + (size_t)(e / m) * ldc;
  *cp = beta == 0.0 ? alpha * s : fma(alpha, s, beta * *cp);
}

// K split so that the grid has about two CTAs per SM, each K slice at least 32 deep
static void dgemm_split(int m, int n, int k, int* ks, int* kper) {
  const int64_t tiles = (int64_t)((m + GT - 1) / GT) * ((n + GT - 1) / GT);
  const int64_t target = 2 * (int64_t)sm_count();
  int s = (int)std::max<int64_t>(1, std::min<int64_t>((target + tiles - 1) / tiles, (k + 31) / 32));
  int per = (k + s - 1) / s;
  per = (per + GKS - 1) / GKS * GKS;
  *kper = std::max(per, GKS);
  *ks = (k + *kper - 1) / *kper;
}

size_t dgemm_ws(int m, int n, int k) {
  if (m <= 0 || n <= 0 || k <= 0) return 0;
  int ks, kper;
  dgemm_split(m, n, k, &ks, &kper);
  return ks > 1 ? (size_t)ks * m * n : 0;
}

int dgemm(cudaStream_t st, int ta, int tb, int m, int n, int k, double alpha, const double* A, int lda,
          const double* B, int ldb, double beta, double* C, int ldc, double* ws, int64_t* launches) {
  if (m <= 0 || n <= 0) return SS_OK;
  if (k <= 0) {  // C = beta C
    dgemm_reduce<<<nblk((int64_t)m * n), 256, 0, st>>>(m, n, 0, alpha, ws, beta, C, ldc);
    SS_CUDA_TRY(cudaGetLastError());
    if (launches) (*launches)++;
    return SS_OK;
  }
  int ks, kper;
  dgemm_split(m, n, k, &ks, &kper);
  if (!ws) {
    ks = 1;
    kper = k;
  }
  dim3 grid((unsigned)((m + GT - 1) / GT), (unsigned)((n + GT - 1) / GT), (unsigned)ks);
  dgemm_kernel<<<grid, 256, 0, st>>>(ta, tb, m, n, k, kper, alpha, A, lda, B, ldb, beta, C, ldc, ws);
  SS_CUDA_TRY(cudaGetLastError());
  if (launches) (*launches)++;
  if (ks > 1) {
    dgemm_reduce<<<nblk((int64_t)m * n), 256, 0, st>>>(m, n, ks, alpha, ws, beta, C, ldc);
    SS_CUDA_TRY(cudaGetLastError());
    if (launches) (*launches)++;
  }
  return SS_OK;
}

// ---------------------------------------------------------------------------------------
// Blocked Householder QR
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

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// r = sqrt(f^2 + g^2) and 1/r.  FP64 square roots and divisions take tens of FP64-pipe
// instructions, which GB300 issues at two per clock per SM; this takes the FP32 reciprocal
// square root of x = f^2 + g^2 as the seed and two Newton steps y <- y (3/2 - x y^2 / 2), each
// doubling the correct bits (24 -> 48 -> FP64 rounding), for a few FP64 fused multiply-adds.
// Outside the FP32 range of x it falls back to hypot and a division.
__device__ __forceinline__ void hypot_inv(double f, double g, double& r, double& rinv) {
  const double x = fma(f, f, g * g);
  if (!(x > 1e-36 && x < 1e36)) {
    r = hypot(f, g);
    rinv = r > 0.0 ? 1.0 / r : 0.0;
    return;
  }
  double y = (double)rsqrtf((float)x);
  const double hx = 0.5 * x;
  y = y * fma(-hx * y, y, 1.5);
  y = y * fma(-hx * y, y, 1.5);
  rinv = y;
  r = x * y;
}

// Panel j0 .. j0+b-1 of Z (rows j0 .. N-1): Householder vectors in place below the diagonal
// (unit leading entry implied), and explicitly into Vb(:, j0 .. j0+b-1) (zeros above, 1 on the
// diagonal); T (QR_NB x QR_NB col-major, upper triangular) with H_j0 ... H_{j0+b-1} =
// I - V T V^T (the forward column-wise recurrence of LAPACK's dlarft).  256 threads.  With
// SMEM the panel's mr = N - j0 rows are staged in shared memory (mr x b doubles), so the
// column-by-column steps read no global memory; otherwise it is factorised in place.
template <bool SMEM>
__global__ void __launch_bounds__(256) qr_panel_kernel(int N, int j0, int b, double* __restrict__ Z, int ld,
                                                        double* __restrict__ Vb, double* __restrict__ T) {
  extern __shared__ double s_panel[];
  __shared__ double sh[32];
  __shared__ double s_tau[QR_NB];
  __shared__ double s_G[QR_NB][QR_NB + 1];
  __shared__ double s_T[QR_NB][QR_NB + 1];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  const int mr = N - j0;
  double* X = SMEM ? s_panel : Z + j0 + (size_t)j0 * ld;  // X(i, jj), i < mr
  const int ldx = SMEM ? mr : ld;
  if (SMEM) {
    for (int e = threadIdx.x; e < mr * b; e += blockDim.x) {
      const int i = e % mr, jj = e / mr;
      X[i + (size_t)jj * ldx] = Z[j0 + i + (size_t)(j0 + jj) * ld];
    }
    __syncthreads();
  }
  for (int jj = 0; jj < b; jj++) {
    double* x = X + (size_t)jj * ldx;
    double ss = 0.0;
    for (int i = jj + 1 + threadIdx.x; i < mr; i += blockDim.x) ss += x[i] * x[i];
    const double sigma = block_sum(ss, sh);
    const double x0 = x[jj];
    double tau = 0.0;
    if (sigma != 0.0) {
      const double mu = sqrt(x0 * x0 + sigma);
      const double alpha = x0 <= 0.0 ? mu : -mu;  // R_cc, sign chosen against cancellation
      const double v0 = x0 - alpha;
      const double inv = 1.0 / v0;
      for (int i = jj + 1 + threadIdx.x; i < mr; i += blockDim.x) x[i] *= inv;
      tau = -v0 / alpha;
      __syncthreads();
      if (threadIdx.x == 0) x[jj] = alpha;
    }
    if (threadIdx.x == 0) s_tau[jj] = tau;
    __syncthreads();
    // H applied to the panel's remaining columns, one warp per column
    if (tau != 0.0)
      for (int cc = jj + 1 + warp; cc < b; cc += nw) {
        double* z = X + (size_t)cc * ldx;
        double s = lane == 0 ? z[jj] : 0.0;
        for (int i = jj + 1 + lane; i < mr; i += 32) s += x[i] * z[i];
        const double w = tau * warp_sum(s);
        if (lane == 0) z[jj] -= w;
        for (int i = jj + 1 + lane; i < mr; i += 32) z[i] -= w * x[i];
      }
    __syncthreads();
  }
  // factored panel back to Z; explicit V of the panel
  for (int e = threadIdx.x; e < N * b; e += blockDim.x) {
    const int i = e % N, jj = e / N, c = j0 + jj;
    const double v = i >= j0 ? X[(i - j0) + (size_t)jj * ldx] : 0.0;
    if (SMEM && i >= j0) Z[i + (size_t)c * ld] = v;
    Vb[i + (size_t)c * N] = i < c ? 0.0 : (i == c ? 1.0 : v);
  }
  __syncthreads();
  // G = V^T V of the panel, one warp per entry (from the staged rows when SMEM)
  for (int e = warp; e < b * b; e += nw) {
    const int r = e % b, cc = e / b;
    if (r > cc) continue;
    double s = 0.0;
    if (SMEM) {
      // V(i, r) = 1 at i = r, X(i, r) below, 0 above
      for (int i = cc + lane; i < mr; i += 32) {
        const double vr = i == r ? 1.0 : (i > r ? X[i + (size_t)r * ldx] : 0.0);
        const double vc = i == cc ? 1.0 : X[i + (size_t)cc * ldx];
        s += vr * vc;
      }
    } else {
      const double* vr = Vb + (size_t)(j0 + r) * N;
      const double* vc = Vb + (size_t)(j0 + cc) * N;
      for (int i = j0 + lane; i < N; i += 32) s += vr[i] * vc[i];
    }
    s = warp_sum(s);
    if (lane == 0) {
      s_G[r][cc] = s;
      s_G[cc][r] = s;
    }
  }
  __syncthreads();
  // T(0:jj, jj) = -tau_jj T(0:jj, 0:jj) G(0:jj, jj); T(jj, jj) = tau_jj (one warp, lane = row)
  if (warp == 0) {
    for (int jj = 0; jj < b; jj++) {
      double t = 0.0;
      if (lane < jj)
        for (int l = lane; l < jj; l++) t += s_T[lane][l] * s_G[l][jj];
      __syncwarp();
      if (lane < jj) s_T[lane][jj] = -s_tau[jj] * t;
      if (lane == jj) s_T[jj][jj] = s_tau[jj];
      if (lane > jj && lane < QR_NB) s_T[lane][jj] = 0.0;
      __syncwarp();
    }
  }
  __syncthreads();
  for (int e = threadIdx.x; e < QR_NB * QR_NB; e += blockDim.x) {
    const int r = e % QR_NB, cc = e / QR_NB;
    T[e] = (r < b && cc < b) ? s_T[r][cc] : 0.0;
  }
}

constexpr size_t QR_PANEL_SMEM_MAX = 200 * 1024;  // staged panel (doubles of mr x b)

__global__ void set_identity_cols(int N, int r, double* Q, int ld) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= (int64_t)N * r) return;
  const int i = (int)(e % N), c = (int)(e / N);
  Q[(size_t)c * ld + i] = (i == c) ? 1.0 : 0.0;
}

size_t ortho_qr_ws(int N, int r) {
  const int P = (r + QR_NB - 1) / QR_NB;
  size_t g = 0;
  for (int p = 0; p < P; p++) {  // the largest split-K workspace of the GEMMs ortho_qr issues
    const int j0 = p * QR_NB, b = std::min(QR_NB, r - j0), mr = N - j0;
    for (int nc : {r - j0 - b, r - j0})
      if (nc > 0) g = std::max({g, dgemm_ws(b, nc, mr), dgemm_ws(b, nc, b), dgemm_ws(mr, nc, b)});
  }
  return 2 * (size_t)N * r + (size_t)QR_NB * QR_NB * P + 2 * (size_t)QR_NB * r + g;
}

int ortho_qr(cudaStream_t st, int N, int r, double* Z, int ld, double* work, int64_t* launches) {
  if (r < 1 || r > N) {
    ss_set_error_msg("ortho_qr: need 1 <= columns (%d) <= rows (%d)", r, N);
    return SS_ERR_ARG;
  }
  const int P = (r + QR_NB - 1) / QR_NB;
  double* Q = work;                                    // N x r, ld N
  double* Vb = Q + (size_t)N * r;                      // N x r, ld N
  double* T = Vb + (size_t)N * r;                      // QR_NB x QR_NB per panel
  double* X1 = T + (size_t)QR_NB * QR_NB * P;          // QR_NB x r
  double* X2 = X1 + (size_t)QR_NB * r;                 // QR_NB x r
  double* gws = X2 + (size_t)QR_NB * r;
  for (int p = 0; p < P; p++) {
    const int j0 = p * QR_NB, b = std::min(QR_NB, r - j0), nc = r - j0 - b, mr = N - j0;
    double* Tp = T + (size_t)QR_NB * QR_NB * p;
    const size_t psmem = sizeof(double) * (size_t)mr * b;
    if (psmem <= QR_PANEL_SMEM_MAX) {
      SS_CUDA_TRY(cudaFuncSetAttribute(qr_panel_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)QR_PANEL_SMEM_MAX));
      qr_panel_kernel<true><<<1, 256, psmem, st>>>(N, j0, b, Z, ld, Vb, Tp);
    } else {
      qr_panel_kernel<false><<<1, 256, 0, st>>>(N, j0, b, Z, ld, Vb, Tp);
    }
    SS_CUDA_TRY(cudaGetLastError());
    if (launches) (*launches)++;
    if (nc > 0) {  // trailing columns: C <- (I - V T^T V^T) C
      const double* Vp = Vb + j0 + (size_t)j0 * N;
      double* Cc = Z + j0 + (size_t)(j0 + b) * ld;
      int rc = dgemm(st, 1, 0, b, nc, mr, 1.0, Vp, N, Cc, ld, 0.0, X1, b, gws, launches);
      if (!rc) rc = dgemm(st, 1, 0, b, nc, b, 1.0, Tp, QR_NB, X1, b, 0.0, X2, b, gws, launches);
      if (!rc) rc = dgemm(st, 0, 0, mr, nc, b, -1.0, Vp, N, X2, b, 1.0, Cc, ld, gws, launches);
      if (rc) return rc;
    }
  }
  // explicit Q = H_1 ... H_r [I; 0], panels applied last to first: Q <- (I - V T V^T) Q
  set_identity_cols<<<nblk((int64_t)N * r), 256, 0, st>>>(N, r, Q, N);
  SS_CUDA_TRY(cudaGetLastError());
  if (launches) (*launches)++;
  for (int p = P - 1; p >= 0; p--) {
    const int j0 = p * QR_NB, b = std::min(QR_NB, r - j0), nc = r - j0, mr = N - j0;
    const double* Vp = Vb + j0 + (size_t)j0 * N;
    const double* Tp = T + (size_t)QR_NB * QR_NB * p;
    double* Qs = Q + j0 + (size_t)j0 * N;
    int rc = dgemm(st, 1, 0, b, nc, mr, 1.0, Vp, N, Qs, N, 0.0, X1, b, gws, launches);
    if (!rc) rc = dgemm(st, 0, 0, b, nc, b, 1.0, Tp, QR_NB, X1, b, 0.0, X2, b, gws, launches);
    if (!rc) rc = dgemm(st, 0, 0, mr, nc, b, -1.0, Vp, N, X2, b, 1.0, Qs, N, gws, launches);
    if (rc) return rc;
  }
  SS_CUDA_TRY(cudaMemcpy2DAsync(Z, sizeof(double) * ld, Q, sizeof(double) * N, sizeof(double) * N, r,
                                cudaMemcpyDeviceToDevice, st));
  return SS_OK;
}

// ---------------------------------------------------------------------------------------
// Symmetric eigen-decomposition, n <= 128: one CTA, matrix in shared memory
// ---------------------------------------------------------------------------------------
constexpr int EIG_SMEM_MAX = 128;

__global__ void __launch_bounds__(256) sym_eig_smem_kernel(int n, const double* __restrict__ Ain,
                                                            double* __restrict__ Vout, double* __restrict__ w,
                                                            int* __restrict__ err) {
  extern __shared__ double s_dyn[];
  double* a = s_dyn;              // n x n, row-major view (symmetric input)
  double* d = a + n * n;          // n
  double* e = d + n;              // 2n (second half: scratch)
  double* s_c = e + 2 * n;        // n
  double* s_s = s_c + n;          // n
  __shared__ double sh[32];
  __shared__ double s_anorm;
  __shared__ int s_m, s_cnt, s_stop;
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int t = tid; t < n * n; t += nt) a[t] = Ain[t];
  __syncthreads();
#define A(i, j) a[(i) * n + (j)]
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
        const double sinv = 1.0 / scale;
        for (int k = tid; k <= l; k += nt) {
          const double v = A(i, k) * sinv;
          A(i, k) = v;
          hh += v * v;
        }
        h = block_sum(hh, sh);
        const double f0 = A(i, l);
        const double g0 = f0 >= 0.0 ? -sqrt(h) : sqrt(h);
        __syncthreads();
        if (tid == 0) {
          e[i] = scale * g0;
          A(i, l) = f0 - g0;
        }
        h = h - f0 * g0;
        const double hinv = 1.0 / h;
        __syncthreads();
        // p = A u / h (u = row i, entries 0..l) into e[0..l]: one warp per row j
        for (int j = tid >> 5; j <= l; j += nt >> 5) {
          double g = 0.0;
          for (int k = (tid & 31); k <= l; k += 32) g += (k <= j ? A(j, k) : A(k, j)) * A(i, k);
          g = warp_sum(g);
          if ((tid & 31) == 0) {
            A(j, i) = A(i, j) * hinv;
            e[j] = g * hinv;
          }
        }
        __syncthreads();
        double fpart = 0.0;
        for (int j = tid; j <= l; j += nt) fpart += e[j] * A(i, j);
        const double f = block_sum(fpart, sh);
        const double hh2 = f / (h + h);
        for (int j = tid; j <= l; j += nt) e[j] = e[j] - hh2 * A(i, j);
        __syncthreads();
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
      for (int j = tid >> 5; j < i; j += nt >> 5) {  // g_j = sum_k A(i,k) A(k,j), one warp per j
        double g = 0.0;
        for (int k = (tid & 31); k < i; k += 32) g += A(i, k) * A(k, j);
        g = warp_sum(g);
        if ((tid & 31) == 0) e[n + j] = g;
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
    double an = 0.0;
    for (int i = 0; i < n; i++) an = fmax(an, fabs(d[i]) + fabs(e[i]));
    s_anorm = an;
  }
  __syncthreads();
  int fail = 0;
  for (int l = 0; l < n && !fail; l++) {
    int iter = 0;
    while (true) {
      if (tid == 0) {
        int m;
        for (m = l; m < n - 1; m++) {
          const double dd = fabs(d[m]) + fabs(d[m + 1]);
          // negligible next to its neighbours or to the whole matrix (the absolute test deflates
          // runs of rounding-level entries, e.g. the numerical null space of a Coulomb metric)
          if (fabs(e[m]) <= 2.2204460492503131e-16 * dd || fabs(e[m]) <= 2.2204460492503131e-16 * s_anorm) break;
        }
        s_m = m;
        s_cnt = 0;
        s_stop = 0;
        if (m != l) {
          if (iter >= 60) {
            s_stop = 1;
          } else {
            double g = (d[l + 1] - d[l]) / (2.0 * e[l]);
            double r = hypot(g, 1.0);
            g = d[m] - d[l] + e[l] / (g + (g >= 0.0 ? fabs(r) : -fabs(r)));
            double s = 1.0, c = 1.0, p = 0.0;
            bool underflow = false;
            for (int i = m - 1; i >= l; i--) {
              double f = s * e[i], bb = c * e[i];
              double rinv;
              hypot_inv(f, g, r, rinv);
              e[i + 1] = r;
              if (r == 0.0) {
                d[i + 1] -= p;
                e[m] = 0.0;
                underflow = true;
                break;
              }
              s = f * rinv;
              c = g * rinv;
              g = d[i + 1] - p;
              r = (d[i] - g) * s + 2.0 * c * bb;
              p = s * r;
              d[i + 1] = g + p;
              g = c * r - bb;
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
      if (s_stop) {
        fail = 1;
        break;
      }
      if (m == l) break;
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
  }
  __syncthreads();
  if (fail) {
    if (tid == 0) atomicExch(err, 1);
    return;
  }
  // ascending order by rank (ties by index); eigenvector j = column j of the row-major A
  for (int j = tid; j < n; j += nt) {
    int rank = 0;
    for (int t = 0; t < n; t++) rank += (d[t] < d[j]) || (d[t] == d[j] && t < j);
    w[rank] = d[j];
    for (int i = 0; i < n; i++) Vout[i + (size_t)rank * n] = A(i, j);
  }
#undef A
}

// ---------------------------------------------------------------------------------------
// Symmetric eigen-decomposition, n > 128: cooperative round-robin Jacobi
// ---------------------------------------------------------------------------------------
constexpr uint32_t GRID_SPIN_LIMIT = 1u << 22;  // bounded grid barrier (seconds of L2 polling; a round takes microseconds)
constexpr int JACOBI_MAX_SWEEPS = 40;

struct JacobiCtl {
  unsigned int count, gen;  // grid barrier
  int rot[2];               // rotations of the current / previous sweep (by sweep parity)
  double amax;
  int sweeps;               // sweeps the last solve took
};

// Sense-free generation barrier over all CTAs of a cooperative launch (all co-resident).  A
// wait that runs past its limit sets *err = 2; every later barrier then returns at once.
__device__ bool grid_barrier(JacobiCtl* ctl, int* err) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned int* vgen = &ctl->gen;
    const unsigned int g = *vgen;
    __threadfence();
    const unsigned int arrived = atomicAdd(&ctl->count, 1u) + 1u;
    int ok = 1;
    if (arrived == gridDim.x) {
      ctl->count = 0;
      __threadfence();
      atomicAdd(&ctl->gen, 1u);
    } else {
      uint32_t it = 0;
      while (*vgen == g) {
        if (*(volatile int*)err) { ok = 0; break; }
        if (++it > GRID_SPIN_LIMIT) {
          atomicExch(err, 2);
          ok = 0;
          break;
        }
      }
    }
    __threadfence();
    s_ok = ok && *(volatile int*)err == 0;
  }
  __syncthreads();
  return s_ok != 0;
}

__device__ __forceinline__ int rr_player(int pos, int round, int np2) {  // circle method
  return pos == 0 ? 0 : 1 + (pos - 1 + round) % (np2 - 1);
}

__global__ void jacobi_maxabs(int64_t nn, const double* __restrict__ A, JacobiCtl* ctl) {
  __shared__ double sh[32];
  double m = 0.0;
  for (int64_t t = threadIdx.x; t < nn; t += blockDim.x) m = fmax(m, fabs(A[t]));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_down_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) t = fmax(t, sh[w]);
    ctl->amax = t;
    ctl->count = 0;
    ctl->gen = 0;
    ctl->rot[0] = ctl->rot[1] = 0;
  }
}

// A0 holds the matrix (it is overwritten), A1 the second buffer, V <- eigenvectors (unsorted),
// d <- eigenvalues (unsorted, diag of the converged matrix).
__global__ void __launch_bounds__(256) jacobi_kernel(int n, double* __restrict__ A0, double* __restrict__ A1,
                                                     double* __restrict__ V, double* __restrict__ d,
                                                     JacobiCtl* ctl, int* err) {
  extern __shared__ double s_cs[];  // c[np], s[np]
  __shared__ int s_rot;
  const int np = (n + 1) / 2, np2 = 2 * np;
  double* sc = s_cs;
  double* ss = sc + np;
  const double eps = 2.2204460492503131e-16;
  const double amax = ctl->amax;
  // entries at or below the rounding level of the matrix (eps max|A|): rounding in the other
  // rotations of their rows regenerates them at that size, so rotating them would never end
  const double tiny = eps * amax;
  const double inv_amax = amax > 0.0 ? 1.0 / amax : 0.0;
  const int64_t gthreads = (int64_t)gridDim.x * blockDim.x;
  const int64_t gtid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  // V = I
  for (int64_t e = gtid; e < (int64_t)n * n; e += gthreads) V[e] = (e % n == e / n) ? 1.0 : 0.0;
  if (!grid_barrier(ctl, err)) return;
  double* cur = A0;
  double* nxt = A1;
  int converged = 0, sweeps_done = 0;
  for (int sweep = 0; sweep < JACOBI_MAX_SWEEPS && !converged; sweep++) {
    sweeps_done = sweep + 1;
    for (int round = 0; round < np2 - 1; round++) {
      if (threadIdx.x == 0) s_rot = 0;
      if (round == 1 && blockIdx.x == 0 && threadIdx.x == 0) ctl->rot[(sweep + 1) & 1] = 0;
      __syncthreads();
      // rotation of every pair of this round, from the current 2 x 2 diagonal blocks
      int myrot = 0;
      for (int pi = threadIdx.x; pi < np; pi += blockDim.x) {
        int p = rr_player(pi, round, np2), q = rr_player(np2 - 1 - pi, round, np2);
        if (p > q) { const int t = p; p = q; q = t; }
        double c = 1.0, s = 0.0;
        if (q < n) {
          const double apq = cur[p + (size_t)q * n], app = cur[p + (size_t)p * n], aqq = cur[q + (size_t)q * n];
          // skip below the rounding level, or below eps of the diagonal pair (compared squared)
          if (fabs(apq) > tiny && apq * apq > eps * eps * fabs(app) * fabs(aqq)) {
            // the angle in FP32 on entries scaled by 1/max|A| (t = tan(theta) of the rotation that
            // zeroes apq; the symmetric Schur form of Golub and Van Loan), then (c, s) made
            // orthonormal in FP64: c^2 + s^2 = 1 - e, scaled by (1 - e)^(-1/2) = 1 + e/2 + 3e^2/8.
            // An FP32 angle leaves about 1e-7 of apq for the next sweep; the rotation itself is
            // orthogonal to FP64 precision.
            const float dq = (float)((aqq - app) * inv_amax), pq = (float)(apq * inv_amax);
            const float tau = dq / (2.0f * pq);
            const float at = fabsf(tau);
            const float t = at > 1e15f ? 0.5f / tau : copysignf(1.0f, tau) / (at + sqrtf(1.0f + at * at));
            const float cf = rsqrtf(1.0f + t * t);
            c = (double)cf;
            s = (double)(t * cf);
            const double e = 1.0 - fma(c, c, s * s);
            const double r = fma(e, fma(0.375, e, 0.5), 1.0);
            c *= r;
            s *= r;
            myrot++;
          }
        }
        sc[pi] = c;
        ss[pi] = s;
      }
      if (blockIdx.x == 0 && myrot) atomicAdd(&s_rot, myrot);
      __syncthreads();
      if (blockIdx.x == 0 && threadIdx.x == 0 && s_rot) atomicAdd(&ctl->rot[sweep & 1], s_rot);
      // A' = J^T A J by 2 x 2 blocks (pair P rows, pair R columns), P <= R; block (R, P) is
      // the transpose, written from the same values so the matrix stays exactly symmetric
      for (int64_t it = gtid; it < (int64_t)np * (np + 1) / 2; it += gthreads) {
        int R = (int)((sqrtf(8.0f * (float)it + 1.0f) - 1.0f) * 0.5f);  // corrected below
        while ((int64_t)R * (R + 1) / 2 > it) R--;
        while ((int64_t)(R + 1) * (R + 2) / 2 <= it) R++;
        const int P = (int)(it - (int64_t)R * (R + 1) / 2);
        int p = rr_player(P, round, np2), q = rr_player(np2 - 1 - P, round, np2);
        int r = rr_player(R, round, np2), s2 = rr_player(np2 - 1 - R, round, np2);
        if (p > q) { const int t = p; p = q; q = t; }
        if (r > s2) { const int t = r; r = s2; s2 = t; }
        const double cP = sc[P], sP = ss[P], cR = sc[R], sR = ss[R];
        const bool qv = q < n, sv = s2 < n;
        if (P == R) {  // diagonal block J^T A_PP J, its off-diagonal entry symmetrised
          const double app = cur[p + (size_t)p * n];
          if (!qv) {
            nxt[p + (size_t)p * n] = app;
            continue;
          }
          const double apq = cur[p + (size_t)q * n], aqq = cur[q + (size_t)q * n];
          const double xpp = cP * app - sP * apq, xpq = cP * apq - sP * aqq;
          const double xqp = sP * app + cP * apq, xqq = sP * apq + cP * aqq;
          nxt[p + (size_t)p * n] = cP * xpp - sP * xpq;
          nxt[q + (size_t)q * n] = sP * xqp + cP * xqq;
          const double bpq = 0.5 * ((sP * xpp + cP * xpq) + (cP * xqp - sP * xqq));
          nxt[p + (size_t)q * n] = bpq;
          nxt[q + (size_t)p * n] = bpq;
          continue;
        }
        const double a_pr = cur[p + (size_t)r * n];
        const double a_ps = sv ? cur[p + (size_t)s2 * n] : 0.0;
        const double a_qr = qv ? cur[q + (size_t)r * n] : 0.0;
        const double a_qs = (qv && sv) ? cur[q + (size_t)s2 * n] : 0.0;
        // rows: [x_p; x_q] = [[c, -s], [s, c]] [a_p; a_q]
        const double xpr = cP * a_pr - sP * a_qr, xps = cP * a_ps - sP * a_qs;
        const double xqr = sP * a_pr + cP * a_qr, xqs = sP * a_ps + cP * a_qs;
        // columns: [b_r, b_s] = [x_r, x_s] [[c, s], [-s, c]]
        const double bpr = cR * xpr - sR * xps, bps = sR * xpr + cR * xps;
        const double bqr = cR * xqr - sR * xqs, bqs = sR * xqr + cR * xqs;
        nxt[p + (size_t)r * n] = bpr;
        nxt[r + (size_t)p * n] = bpr;
        if (sv) {
          nxt[p + (size_t)s2 * n] = bps;
          nxt[s2 + (size_t)p * n] = bps;
        }
        if (qv) {
          nxt[q + (size_t)r * n] = bqr;
          nxt[r + (size_t)q * n] = bqr;
        }
        if (qv && sv) {
          nxt[q + (size_t)s2 * n] = bqs;
          nxt[s2 + (size_t)q * n] = bqs;
        }
      }
      // V' = V J, row pairs (each (row, pair) touches its own two entries: in place)
      for (int64_t it = gtid; it < (int64_t)n * np; it += gthreads) {
        const int i = (int)(it % n), P = (int)(it / n);
        if (ss[P] == 0.0) continue;
        int p = rr_player(P, round, np2), q = rr_player(np2 - 1 - P, round, np2);
        if (p > q) { const int t = p; p = q; q = t; }
        if (q >= n) continue;
        const double vp = V[i + (size_t)p * n], vq = V[i + (size_t)q * n];
        V[i + (size_t)p * n] = sc[P] * vp - ss[P] * vq;
        V[i + (size_t)q * n] = ss[P] * vp + sc[P] * vq;
      }
      if (!grid_barrier(ctl, err)) return;
      double* t = cur;
      cur = nxt;
      nxt = t;
    }
    converged = (*(volatile int*)&ctl->rot[sweep & 1] == 0);
  }
  if (gtid == 0) ctl->sweeps = sweeps_done;
  if (!converged) {
    if (gtid == 0) atomicExch(err, 1);
    return;
  }
  for (int64_t i = gtid; i < n; i += gthreads) d[i] = cur[i + (size_t)i * n];
}

// w = d ascending (ties by index), V columns permuted the same way (Vu -> V)
__global__ void eig_sort_kernel(int n, const double* __restrict__ d, const double* __restrict__ Vu,
                                double* __restrict__ w, double* __restrict__ V) {
  const int j = blockIdx.x;
  __shared__ int s_rank;
  if (threadIdx.x == 0) {
    int rank = 0;
    const double dj = d[j];
    for (int t = 0; t < n; t++) rank += (d[t] < dj) || (d[t] == dj && t < j);
    s_rank = rank;
    w[rank] = dj;
  }
  __syncthreads();
  const int rk = s_rank;
  for (int i = threadIdx.x; i < n; i += blockDim.x) V[i + (size_t)rk * n] = Vu[i + (size_t)j * n];
}

size_t sym_eig_ws(int n) {
  if (n <= EIG_SMEM_MAX) return 0;
  return 3 * (size_t)n * n + (size_t)n + 16;
}

int sym_eig(cudaStream_t st, int n, const double* A, double* V, double* w, double* work, int* d_err,
            int64_t* launches) {
  if (n < 1 || n > 4096) {
    ss_set_error_msg("sym_eig: n=%d outside 1..4096", n);
    return SS_ERR_UNSUPPORTED;
  }
  if (n <= EIG_SMEM_MAX) {
    const size_t smem = sizeof(double) * ((size_t)n * n + 5 * (size_t)n);
    // the opt-in is per kernel, not per launch: always the largest size, so that threads launching
    // different sizes at once never lower it under another's launch
    const int smem_max = (int)(sizeof(double) * (EIG_SMEM_MAX * EIG_SMEM_MAX + 5 * EIG_SMEM_MAX));
    SS_CUDA_TRY(cudaFuncSetAttribute(sym_eig_smem_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_max));
    // 256 threads: eight warps keep the FP64 pipe busy, and each of the many block-wide
    // barriers of the reduction gathers 8 warps instead of 32
    sym_eig_smem_kernel<<<1, 256, smem, st>>>(n, A, V, w, d_err);
    SS_CUDA_TRY(cudaGetLastError());
    if (launches) (*launches)++;
    return SS_OK;
  }
  double* A0 = work;
  double* A1 = A0 + (size_t)n * n;
  double* Vu = A1 + (size_t)n * n;
  double* d = Vu + (size_t)n * n;
  JacobiCtl* ctl = (JacobiCtl*)(d + n);
  static_assert(sizeof(JacobiCtl) <= 16 * sizeof(double), "control block fits its slot");
  SS_CUDA_TRY(cudaMemcpyAsync(A0, A, sizeof(double) * n * n, cudaMemcpyDeviceToDevice, st));
  jacobi_maxabs<<<1, 1024, 0, st>>>((int64_t)n * n, A0, ctl);
  SS_CUDA_TRY(cudaGetLastError());
  // one cooperative grid, all CTAs co-resident
  const int np = (n + 1) / 2;
  const size_t smem = sizeof(double) * 2 * np;
  SS_CUDA_TRY(cudaFuncSetAttribute(jacobi_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)(sizeof(double) * 2 * ((4096 + 1) / 2))));  // the largest n
  int per_sm = 0;
  SS_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, jacobi_kernel, 256, smem));
  const int64_t items = std::max<int64_t>((int64_t)np * (np + 1) / 2, (int64_t)n * np);  // 2x2 blocks, V rows
  const int64_t want = std::max<int64_t>(1, (items + 255) / 256);
  const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(want, (int64_t)sm_count() * std::max(per_sm, 1)));
  int nn = n;
  void* args[] = {&nn, &A0, &A1, &Vu, &d, &ctl, &d_err};
  SS_CUDA_TRY(cudaLaunchCooperativeKernel((const void*)jacobi_kernel, dim3(grid), dim3(256), args, smem, st));
  eig_sort_kernel<<<n, 128, 0, st>>>(n, d, Vu, w, V);
  SS_CUDA_TRY(cudaGetLastError());
  if (launches) *launches += 3;
  return SS_OK;
}

}  // namespace ss
