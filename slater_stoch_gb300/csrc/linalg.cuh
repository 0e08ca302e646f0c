// linalg.cuh -- FP64 dense linear algebra of the PSD cleanup and Davidson, on the device.
//
// All matrices are column-major with an explicit leading dimension.  Every routine enqueues its
// kernels on `st` and returns without synchronising; bounded device waits report through
// *d_err (a device int, 0 = ok), which the caller reads back with its next synchronisation.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace ss {

// C (m x n) = alpha op(A) op(B) + beta C; op(X) = X (trans = 0) or X^T (trans = 1);
// op(A) is m x k, op(B) is k x n.  The inner dimension is split over several CTAs when the
// output has few tiles; the partial products then go to `ws` (at least dgemm_ws(m, n, k)
// doubles) and are summed in a fixed order, so results are reproducible.  ws may be null when
// dgemm_ws returns 0.
size_t dgemm_ws(int m, int n, int k);
int dgemm(cudaStream_t st, int ta, int tb, int m, int n, int k, double alpha, const double* A, int lda,
          const double* B, int ldb, double beta, double* C, int ldc, double* ws, int64_t* launches);

// Z (N x r, leading dimension ld, r <= N) <- the Q factor of its Householder QR (the roles of
// dgeqrf / dorgqr in src/ortho_qr.F90:1-39), in blocks of QR_NB columns: one CTA factorises a
// panel and builds its compact-WY factor T, the rest of the matrix and the explicit Q are
// updated with dgemm.  work: at least ortho_qr_ws(N, r) doubles.
constexpr int QR_NB = 32;
size_t ortho_qr_ws(int N, int r);
int ortho_qr(cudaStream_t st, int N, int r, double* Z, int ld, double* work, int64_t* launches);

// Symmetric eigen-decomposition: A (n x n, col-major, ld n; only read) -> V (n x n col-major,
// V(:, j) the eigenvector of w[j]), w ascending.  n <= 128: one CTA with the matrix in shared
// memory (Householder tridiagonalisation with accumulated transformations, implicit QL with
// Wilkinson shifts: the tred2 / tql2 procedure).  n > 128: cyclic two-sided Jacobi with the
// round-robin pair order, all n/2 rotations of a round applied at once by a cooperative grid
// (A' = J^T A J by 2 x 2 blocks into a second buffer, V' = V J), one bounded grid barrier per
// round, until a sweep needs no rotation.  work: at least sym_eig_ws(n) doubles; *d_err is set
// to 1 on no convergence and 2 on a barrier timeout.
size_t sym_eig_ws(int n);
int sym_eig(cudaStream_t st, int n, const double* A, double* V, double* w, double* work, int* d_err,
            int64_t* launches);

}  // namespace ss
