// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as
// easy as 1, 2, 3", SC'11), the counter-based stream behind every Monte
// Carlo step of this library.
//
// Stream convention, one Philox block per Monte Carlo step:
//   block b of chain c = philox4x32_10({b_lo, b_hi, c, 0}, {seed_lo, seed_hi})
//   w0 -> move selection (w0 * n) >> 32, w1 -> trial magnitude w1 * 2^-32,
//   w2 -> Metropolis uniform w2 * 2^-32, w3 -> spare.
// It stands in for the reference's GSL gsl_rng_taus2 draws
// (src/jmmMCState.cpp:779-781, :1762-1763, :1370, :2252).
#pragma once
#include <stdint.h>

namespace jmm {

struct Words4 {
  uint32_t w[4];
};

__host__ __device__ __forceinline__ void mulhilo32(uint32_t a, uint32_t b, uint32_t &hi,
                                                   uint32_t &lo) {
#if defined(__CUDA_ARCH__)
  hi = __umulhi(a, b);
  lo = a * b;
#else
  uint64_t p = (uint64_t)a * (uint64_t)b;
  hi = (uint32_t)(p >> 32);
  lo = (uint32_t)p;
#endif
}

__host__ __device__ __forceinline__ Words4 philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2,
                                                        uint32_t c3, uint32_t k0, uint32_t k1) {
  constexpr uint32_t kM0 = 0xD2511F53u, kM1 = 0xCD9E8D57u;
  constexpr uint32_t kW0 = 0x9E3779B9u, kW1 = 0xBB67AE85u;
#pragma unroll
  for (int round = 0; round < 10; ++round) {
    uint32_t hi0, lo0, hi1, lo1;
    mulhilo32(kM0, c0, hi0, lo0);
    mulhilo32(kM1, c2, hi1, lo1);
    uint32_t n0 = hi1 ^ c1 ^ k0;
    uint32_t n2 = hi0 ^ c3 ^ k1;
    c0 = n0;
    c1 = lo1;
    c2 = n2;
    c3 = lo0;
    k0 += kW0;
    k1 += kW1;
  }
  Words4 out;
  out.w[0] = c0;
  out.w[1] = c1;
  out.w[2] = c2;
  out.w[3] = c3;
  return out;
}

// The four words of Monte Carlo step `block` of chain `chain`.
__host__ __device__ __forceinline__ Words4 step_words(uint64_t seed, uint64_t block,
                                                     uint32_t chain) {
  return philox4x32_10((uint32_t)block, (uint32_t)(block >> 32), chain, 0u, (uint32_t)seed,
                       (uint32_t)(seed >> 32));
}

__host__ __device__ __forceinline__ uint64_t word_to_index(uint32_t w, uint64_t n) {
  // n < 2^32 always holds here (particle counts), so the product fits 64 bits.
#if defined(__CUDA_ARCH__)
  return __umulhi(w, (uint32_t)n);
#else
  return ((uint64_t)w * n) >> 32;
#endif
}

__host__ __device__ __forceinline__ double word_to_unit(uint32_t w) {
  return (double)w * (1.0 / 4294967296.0);
}

__host__ __device__ __forceinline__ float word_to_unit_f(uint32_t w) {
  // top 24 bits: exactly representable, in [0, 1)
  return (float)(w >> 8) * (1.0f / 16777216.0f);
}

}  // namespace jmm
