/*
 * oracle/gsl_shim/gsl/gsl_rng.h -- TEST INFRASTRUCTURE (the oracle).
 *
 * A project-written stand-in for the four GSL calls the reference makes
 * (src/jmmMCState.cpp:779-781 gsl_rng_alloc/gsl_rng_set,
 *  :1762-1763 gsl_rng_uniform_int/gsl_rng_uniform, :1370 and :2252
 *  gsl_rng_uniform).  GSL itself is not installed and not vendored; this
 * header is NOT GSL and does not reproduce taus2.  It hands out the
 * project's Philox4x32-10 stream with the "one block per Monte Carlo step"
 * convention of oracle/philox.h:
 *
 *   gsl_rng_uniform_int(r, n)  opens the next block b (b = 1, 2, ...) and
 *                              returns (w0 * n) >> 32;
 *   gsl_rng_uniform(r)         returns the next word of the open block
 *                              (w1, then w2, then w3) times 2^-32.
 *
 * The reference's Step() draws exactly one uniform_int per step
 * (src/jmmMCState.cpp:1762), so block b is step number b, and the
 * data-dependent extra draw (dE > 0, :1367-1370; bf < 1, :2251-2252) takes
 * word 2 of the same block.  A uniform() with no block open (never the case
 * in the reference's driver) opens one and starts at word 1.
 *
 * Setting JMM_SHIM_LOG=<path> appends one binary record per draw
 * (uint64 block, uint32 slot, uint32 word) so that a run of the reference
 * can be replayed draw for draw.
 */
#ifndef JMM_GSL_SHIM_RNG_H
#define JMM_GSL_SHIM_RNG_H

#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>

#include "../../philox.h"

typedef struct {
  const char *name;
} gsl_rng_type;

typedef struct {
  uint64_t seed;
  uint64_t block;   /* last opened block, 0 = none yet */
  uint32_t words[4];
  int slot;         /* next unused word of the open block; 4 = exhausted */
  FILE *log;
} gsl_rng;

static const gsl_rng_type jmm_shim_philox_type = {"philox4x32-10 (jmm shim)"};
static const gsl_rng_type *gsl_rng_taus2 = &jmm_shim_philox_type;

static inline gsl_rng *gsl_rng_alloc(const gsl_rng_type *t) {
  (void)t;
  gsl_rng *r = (gsl_rng *)calloc(1, sizeof(gsl_rng));
  r->slot = 4;
  const char *path = getenv("JMM_SHIM_LOG");
  if (path && path[0]) r->log = fopen(path, "wb");
  return r;
}

static inline void gsl_rng_free(gsl_rng *r) {
  if (!r) return;
  if (r->log) fclose(r->log);
  free(r);
}

static inline void gsl_rng_set(gsl_rng *r, unsigned long seed) {
  r->seed = (uint64_t)seed;
  r->block = 0;
  r->slot = 4;
}

static inline void jmm_shim_open_block(gsl_rng *r) {
  r->block += 1;
  jmmo_step_words(r->seed, r->block, 0u, r->words);
  r->slot = 0;
}

static inline uint32_t jmm_shim_take(gsl_rng *r) {
  uint32_t w = r->words[r->slot];
  if (r->log) {
    uint32_t slot = (uint32_t)r->slot;
    fwrite(&r->block, sizeof(uint64_t), 1, r->log);
    fwrite(&slot, sizeof(uint32_t), 1, r->log);
    fwrite(&w, sizeof(uint32_t), 1, r->log);
  }
  r->slot += 1;
  return w;
}

static inline unsigned long gsl_rng_uniform_int(gsl_rng *r, unsigned long n) {
  jmm_shim_open_block(r);
  return (unsigned long)jmmo_word_to_index(jmm_shim_take(r), (uint64_t)n);
}

static inline double gsl_rng_uniform(gsl_rng *r) {
  if (r->slot >= 4) {
    jmm_shim_open_block(r);
    r->slot = 1;
  }
  return jmmo_word_to_unit(jmm_shim_take(r));
}

#endif
