/*
 * oracle/philox.h -- TEST INFRASTRUCTURE (the oracle), never shipped.
 *
 * Philox4x32-10 counter-based generator, restated from its publication:
 *   J. K. Salmon, M. A. Moraes, R. O. Dror, D. E. Shaw,
 *   "Parallel random numbers: as easy as 1, 2, 3", SC'11 (2011).
 * Round function: two 32x32->64 multiplies by M0=0xD2511F53 and
 * M1=0xCD9E8D57, a lane swap and an xor with the key; the key is bumped by
 * the Weyl constants (0x9E3779B9, 0xBB67AE85) between the ten rounds.
 *
 * The reference draws from GSL's gsl_rng_taus2 (src/jmmMCState.cpp:779-781),
 * a third-party dependency that is not vendored and has no pinned version
 * (src/Makefile:5, "-lgsl").  The oracle replaces that stream by this
 * counter-based one, with the slot convention below; the CUDA product code
 * carries its own implementation of the same generator.
 *
 * Stream convention ("one Philox block per Monte Carlo step"):
 *   block b of chain c  = philox4x32_10({b_lo, b_hi, c, 0}, {seed_lo, seed_hi})
 *   word 0 -> move selection   : (w0 * n) >> 32          in [0, n)
 *   word 1 -> trial magnitude  : w1 * 2^-32              in [0, 1)
 *   word 2 -> Metropolis draw  : w2 * 2^-32              in [0, 1)
 *   word 3 -> spare (domain offsets of the alternating sweep)
 */
#ifndef JMM_ORACLE_PHILOX_H
#define JMM_ORACLE_PHILOX_H

#include <stdint.h>

#define JMMO_PHILOX_M0 0xD2511F53u
#define JMMO_PHILOX_M1 0xCD9E8D57u
#define JMMO_PHILOX_W0 0x9E3779B9u
#define JMMO_PHILOX_W1 0xBB67AE85u

static inline void jmmo_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2],
                                      uint32_t out[4]) {
  uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
  uint32_t k0 = key[0], k1 = key[1];
  for (int round = 0; round < 10; ++round) {
    if (round > 0) {
      k0 += JMMO_PHILOX_W0;
      k1 += JMMO_PHILOX_W1;
    }
    uint64_t p0 = (uint64_t)JMMO_PHILOX_M0 * (uint64_t)c0;
    uint64_t p1 = (uint64_t)JMMO_PHILOX_M1 * (uint64_t)c2;
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    uint32_t n0 = hi1 ^ c1 ^ k0;
    uint32_t n2 = hi0 ^ c3 ^ k1;
    c0 = n0;
    c1 = lo1;
    c2 = n2;
    c3 = lo0;
  }
  out[0] = c0;
  out[1] = c1;
  out[2] = c2;
  out[3] = c3;
}

/* The four words of Monte Carlo step `block` of chain `chain`. */
static inline void jmmo_step_words(uint64_t seed, uint64_t block, uint32_t chain,
                                   uint32_t out[4]) {
  uint32_t ctr[4] = {(uint32_t)block, (uint32_t)(block >> 32), chain, 0u};
  uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
  jmmo_philox4x32_10(ctr, key, out);
}

static inline uint64_t jmmo_word_to_index(uint32_t w, uint64_t n) {
  return (uint64_t)(((unsigned __int128)w * (unsigned __int128)n) >> 32);
}

static inline double jmmo_word_to_unit(uint32_t w) {
  return (double)w * (1.0 / 4294967296.0);
}

#endif
