// ss_common.cuh -- shared definitions for the sm_103a kernels of the two-electron path.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/slaterstoch.h"

#define SS_CUDA_TRY(expr)                          \
  do {                                             \
    cudaError_t _e = (expr);                       \
    if (_e != cudaSuccess) {                       \
      ss_set_cuda_error(_e, #expr, __FILE__, __LINE__); \
      return SS_ERR_CUDA;                          \
    }                                              \
  } while (0)

void ss_set_cuda_error(cudaError_t e, const char* what, const char* file, int line);
void ss_set_error_msg(const char* fmt, ...);

namespace ss {

// Limits of the device kernels (checked on the host before any launch).
constexpr int SS_MAX_POW = 4;        // per-function per-axis power, incl. the +2 of r^2 fits
constexpr int SS_MAX_NG = 30;        // Gaussians per fit (src/common_data.F90:7)
constexpr int SS_MAX_NF = 24;        // highest Boys order F_n used by one primitive quartet
// Primitive screening of the analytic ERIs: a primitive quartet whose Schwarz bound S_P S_Q is
// below PRIM_SCREEN_EPS * sqrt((ik|ik)(jl|jl)) is skipped.  With at most 30 x 30 primitive pairs
// per function pair the skipped part of an ERI is below 8.1e5 * 1e-18 = 8.1e-13 of its Schwarz
// bound sqrt((ik|ik)(jl|jl)), and in practice far below (the bound is loose, the signs vary).
constexpr double PRIM_SCREEN_EPS = 1e-18;
// Dynamic shared memory of one ERI-kernel CTA (ket tiles and their polynomials) never exceeds
// this; every launch opts in to exactly this much, so concurrent launches from several host
// threads (jobs) all set the same per-kernel attribute (a per-launch size would race).
constexpr int ERI_SMEM_MAX = 60 * 1024;
// Light-ket rule: the ket degree bound LK of the instance that evaluates a quartet whose pairs
// have per-axis degree bounds L (the larger) and lmin (the smaller), the lighter pair taking the
// ket; -1 for the full-L instance.  Instances exist for LK = lmin < L <= 3, and for L = 4 with
// LK = max(lmin, 1) <= 2.
__host__ __device__ inline int ss_light_ket(int L, int lmin) {
  if (lmin >= L) return -1;
  if (L == 4) return lmin <= 2 ? (lmin < 1 ? 1 : lmin) : -1;
  return lmin;
}
// Where a quartet's partial sums (one per bra slice) live: slot code = offset << SLOT_SPLIT_BITS |
// split, the partials being entries offset .. offset + split - 1 (split < 2^SLOT_SPLIT_BITS).
constexpr int SLOT_SPLIT_BITS = 7;
__host__ __device__ inline int64_t slot_offset(int64_t code) { return code >> SLOT_SPLIT_BITS; }
__host__ __device__ inline int slot_split(int64_t code) { return (int)(code & ((1 << SLOT_SPLIT_BITS) - 1)); }
// Mixed precision: a kept primitive quartet whose Schwarz bound S_P S_Q is below
// PRIM_FP32_EPS * sqrt((ik|ik)(jl|jl)) is evaluated in FP32 (the default of ss_set_eri_tiers).
// Its value is off by about kappa * 6e-8 * S_P S_Q (kappa the cancellation amplification of its
// evaluation), or by its whole value when its FP32 prefactor K_AB c_P c_Q underflows -- terms of
// ~1e-40 then.  Summed over a quartet's tier the difference from FP64 was measured at 1.8e-15 of
// the Schwarz bound (20-Gaussian fits, host build of the kernel arithmetic), and on the device
// the largest deviation from the oracle over a stratified sample of the 26-function H2O basis
// was 6.4e-3 of the 1e-12 gate (1.1e-3 with a 1e-13 threshold).  The tier takes 40 % of the
// primitive quartets there (28 % at 1e-13), leaving 30 % in FP64.
constexpr double PRIM_FP32_EPS = 1e-11;

// One primitive pair of a function pair (i,k): the Gaussian product of
// g_gauss(m1,i) and g_gauss(m2,k) (src/gaussian_product.F90:1-33), padded to 128 bytes.
struct __align__(16) PrimPair {
  double p, p_inv;       // alpha+beta, 1/(alpha+beta)
  double P[3];           // product centre
  double fact;           // K_AB (0 pairs are not stored)
  double coef;           // c(m1,i) * c(m2,k)
  double PA[3];          // P - A  (pows_a(1) of src/give_explicit_poly_and_gaussian.F90:125)
  double PB[3];          // P - B
  double pad[3];         // [0] Schwarz factor sqrt(coef^2 (P|P)), [1] index m1*ng(k)+m2,
                         // [2] w = fact * coef * p_inv
};
static_assert(sizeof(PrimPair) == 16 * sizeof(double), "PrimPair is 16 doubles (the kernels stride by 16)");

// FP32 copy of a primitive pair for the primitive quartets evaluated in FP32: fc = w = K_AB c p_inv.
struct __align__(16) PrimPairF {
  float p, p_inv, P[3], fc, PA[3], PB[3], pad[2];
};
static_assert(sizeof(PrimPairF) == 16 * sizeof(float), "PrimPairF is 16 floats");

// The fields of a primitive pair that one primitive quartet reads, in the arithmetic type of the
// evaluation (FP64, or FP32 for the quartets below the FP32 bound); the ERI kernel keeps the FP32
// views of a ket tile in shared memory.  w = K_AB c p_inv, the pair's factor of the primitive
// quartet's prefactor (the constant 2 pi^{5/2} of src/general_primitive_integral.F90:192 is
// applied once to the contracted sum); hp = p_inv / 2 (exact).
template <typename Real>
struct PairView {
  Real p, p_inv, hp, P[3], w;
};

// Shared memory of the ERI kernel per staged ket pair: the FP64 record and its recentred
// polynomials (3 axes x options x (LK + 1)), the FP32 view and the FP32 polynomials -- the
// kernel's carve-up of its dynamic shared memory, in the same order.
inline size_t eri_ket_bytes(int LK, bool t2) {
  const size_t qw = 3 * (t2 ? 4 : 1) * (size_t)(LK + 1);
  return sizeof(PrimPair) + sizeof(double) * qw + sizeof(PairView<float>) + sizeof(float) * qw;
}

// Device view of the fitted basis (Fortran layouts, 0-based).
struct BasisDev {
  int n, ld;
  const double* center;   // [3n]
  const int* npower;      // [3n]
  const int* n_sto;       // [n]
  const int* i_type;      // [n]
  const int* n_gauss;     // [n]
  const double* c_gauss;  // [ld*n*2]
  const double* g_gauss;  // [ld*n]
  const double* g_slater; // [n]
  const int* sys;         // [n] system of each function when several systems share the basis
                          // (ss_basis_systems; pairs across systems are never formed), or null
};

__host__ __device__ inline int64_t ss_pair_index(int i, int k) {  // i >= k, 0-based
  return (int64_t)i * (i + 1) / 2 + k;
}

}  // namespace ss
