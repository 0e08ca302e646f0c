// eri_k2c1k0.cu -- eri_kernel<2, 1, 0>: class (2, 1) quartets whose lighter pair has per-axis
// degree 0, evaluated with that pair as the ket (own translation unit).
#include "eri_kernel.cuh"

namespace ss {
cudaError_t launch_eri_L2c1k0(dim3 grid, int ktile, size_t smem, cudaStream_t st, const BasisDev& B,
                                  const PrimPair* pp, const int64_t* off, const int* cnt, const int64_t* work,
                                  int split, const int32_t* is, const int32_t* js, const int32_t* ks,
                                  const int32_t* ls, const double* pre, double eps, double eps32, double* partial,
                                  double* self_out, const PrimPairF* ppf) {
  cudaError_t e =
      cudaFuncSetAttribute(eri_kernel<2, 1, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, ERI_SMEM_MAX);
  if (e != cudaSuccess) return e;
  eri_kernel<2, 1, 0><<<grid, 128, smem, st>>>(B, pp, off, cnt, work, split, ktile, is, js, ks, ls, pre, eps, eps32,
                                                  partial, self_out, ppf);
  return cudaGetLastError();
}
}  // namespace ss
