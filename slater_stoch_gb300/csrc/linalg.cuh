// linalg.cuh -- FP64 device linear algebra used by the PSD cleanup and Davidson.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace ss {

// Z (N x r, column-major, leading dimension ld) <- Q of its Householder QR; Qwork same shape,
// tau >= r doubles.
int ortho_qr(cudaStream_t st, int N, int r, double* Z, int ld, double* Qwork, double* tau, int64_t* launches);

// a (n x n symmetric, row-major) <- eigenvectors as columns, w (n) <- eigenvalues ascending;
// work >= 2n doubles; *info != 0 on no convergence.  One CTA, n <= 1024.
int sym_eig(cudaStream_t st, int n, double* a, double* w, double* work, int* info, int64_t* launches);

}  // namespace ss
