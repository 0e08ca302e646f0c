// philox.cuh -- counter-based Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11) and the
// standard-normal walker draw used by both estimators.  Replaces draw_configuration
// (src/draw_configuration.F90:1-29), whose r = sqrt(2) erfcinv(2 - 2U) is the inverse
// normal CDF of U; here U comes from Philox keyed by (seed, sample index) so any sample
// can be regenerated independently (resume, sharding, parity checks).
#pragma once
#include <stdint.h>

namespace ss {

__host__ __device__ __forceinline__ void philox_round(uint32_t (&c)[4], const uint32_t (&k)[2]) {
  const uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
  const uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
  const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
  const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
  const uint32_t n0 = hi1 ^ c[1] ^ k[0];
  const uint32_t n2 = hi0 ^ c[3] ^ k[1];
  c[0] = n0;
  c[1] = lo1;
  c[2] = n2;
  c[3] = lo0;
}

__host__ __device__ __forceinline__ void philox4x32_10(uint32_t (&c)[4], uint32_t k0, uint32_t k1) {
  uint32_t k[2] = {k0, k1};
#pragma unroll
  for (int r = 0; r < 10; r++) {
    philox_round(c, k);
    k[0] += 0x9E3779B9u;
    k[1] += 0xBB67AE85u;
  }
}

// 53-bit uniform in the open interval (0,1) from two 32-bit words
__host__ __device__ __forceinline__ double u01_open(uint32_t hi, uint32_t lo) {
  const uint64_t b = (((uint64_t)hi << 32) | lo) >> 11;
  return ((double)b + 0.5) * 1.1102230246251565404e-16;  // 2^-53
}

// stream tags keep the faithful walkers, the shared-walker proposal and the SVD test
// matrices on disjoint Philox counters
constexpr uint32_t STREAM_WALKER = 0x57414C4Bu;   // "WALK"
constexpr uint32_t STREAM_SHARED = 0x53484152u;   // "SHAR"
constexpr uint32_t STREAM_SVD = 0x53564443u;      // "SVDC"

}  // namespace ss
