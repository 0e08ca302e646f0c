// shared.cuh -- shared-walker estimator (one sample set for all orbital pairs).
//
// The faithful estimator maps one standard-normal walker per pair through the pair's own
// ZV map, so 1/|u1_ik - u2_jl| couples (ik, jl, s) and the sum is not a matrix product.
// The shared estimator draws u1, u2 once per sample from a mixture of those ZV-map densities
// (pi(u) = sum_c w_c p_c(u)), which makes the weight w_s = 1/(|u1-u2| pi(u1) pi(u2)) pair
// independent.  With Delta = rhoS - rhoG and the identity
//   rhoS_ik rhoS_jl - rhoG_ik rhoG_jl = Delta_ik rhoS_jl + rhoG_ik Delta_jl
// the block sum is C = [Delta1 | rhoG1] . diag(w) . [rhoS2 | Delta2]^T, a GEMM with K = 2S,
// computed on tcgen05 tensor cores in BF16 with a hi+lo split (3 products) and FP32
// accumulation.  Both estimators are unbiased for the same integrals.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

struct ss_ctx;

namespace ss {

int run_shared(ss_ctx* c, double a_zv, uint64_t seed, int64_t npts, int nblocks, int prec,
               double sigma_target);

// C_partial[ks][P][P] (fp32) = sum over the ks-th K slice of Ahi Bhi^T + Ahi Blo^T + Alo Bhi^T;
// A*, B*: [P][K] bf16 row-major (K contiguous), K a multiple of 64.  err_flag is set non-zero
// when a bounded wait gives up.
int launch_split_bf16_gemm(cudaStream_t st, const void* a_hi, const void* a_lo, const void* b_hi,
                           const void* b_lo, int P, int64_t K, int ksplit, float* c_partial,
                           int* err_flag);

}  // namespace ss
