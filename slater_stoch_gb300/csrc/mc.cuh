// mc.cuh -- device views and launchers of the ZV-MC kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "ss_common.cuh"

namespace ss {

// used pairs (i,k), i >= k, with the per-pair ZV-map constants (src/two_e_slater.F90:339-348,406)
struct ZvPairs {
  const int* i;
  const int* k;
  const double* G;     // [3*npairs] centre of the map
  const double* fzv;   // 0.5 a_ZV / (zeta_i + zeta_k)
  const double* fjac;  // a_ZV / (zeta_i + zeta_k)
};

// per-chunk pair columns, [pair][walker] with leading dimension ld (walker fastest)
struct ZvChunk {
  int64_t ld;
  double *u1x, *u1y, *u1z, *u2x, *u2y, *u2z;
  double *a_s, *a_g, *b_s, *b_g;  // FP64: J1 rhoS1, J1 rhoG1, J2 rhoS2/pi0, J2 rhoG2/pi0; REF32: raw densities
  double *j1, *j2;                // REF32 only
};

// quartets grouped by bra pair: for CTA b, entries off[b]..off[b+1] give (quartet, ket pair)
struct ZvCsr {
  const int* bra;
  const int64_t* off;
  const int64_t* q;
  const int* ket;
};

cudaError_t launch_draw_walkers(cudaStream_t st, uint64_t seed, int64_t first, int64_t S, double* r1,
                                double* r2);
cudaError_t launch_walker_aux(cudaStream_t st, int64_t S, const double* r1, const double* r2, double* r1m,
                              double* r2m, double* pi0);
cudaError_t launch_zv_pairs(cudaStream_t st, int mode, const BasisDev& B, const ZvPairs& P, int npairs,
                            int64_t S, const double* r1, const double* r2, const double* r1m,
                            const double* r2m, const double* pi0, const ZvChunk& Z);
cudaError_t launch_zv_accum(cudaStream_t st, int mode, int nbra, int nsplit, int64_t S, const ZvCsr& Q,
                            const ZvChunk& Z, const double* pi0, double* partS, double* partG);
cudaError_t launch_zv_reduce(cudaStream_t st, int64_t nint, int nsplit, const double* partS,
                             const double* partG, double* eS, double* eG);
cudaError_t launch_zv_block_stats(cudaStream_t st, int64_t nint, int64_t npts, double* eS, double* eG,
                                  double* acc, double* acc2);
cudaError_t launch_zv_final(cudaStream_t st, int64_t nint, int nb, int unbiased, const double* acc,
                            const double* acc2, double* mean, double* sigma, unsigned long long* maxbits);

}  // namespace ss
