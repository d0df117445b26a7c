/*
 * oracle/jmm_oracle.h -- TEST INFRASTRUCTURE (the oracle), never shipped.
 * CPU restatements used only by tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py.  The structs are the product's public ones
 * (include/jmm_gpu.h) so that one ctypes layout serves both sides.
 */
#ifndef JMM_ORACLE_H
#define JMM_ORACLE_H

#include <stdint.h>

#include "../include/jmm_gpu.h"
#include "philox.h"

typedef struct jmmo_plain jmmo_plain;

jmmo_plain *jmmo_plain_create(const jmm_params *prm);
int jmmo_plain_set_config(jmmo_plain *h, const double *r, uint64_t n, double l, uint64_t sn);
int jmmo_plain_fad(jmmo_plain *h, uint64_t nm, double d);
int jmmo_plain_steps(jmmo_plain *h, uint64_t n_steps, const jmm_draw *replay,
                     jmm_step_record *log);
int jmmo_plain_update_thermo(jmmo_plain *h);
int jmmo_plain_reset_thermo(jmmo_plain *h);
int jmmo_plain_echeck(jmmo_plain *h, double *e_test, int32_t *reset);
int jmmo_plain_set_step_sizes(jmmo_plain *h, double max_step, double max_dl);
int jmmo_plain_get_state(jmmo_plain *h, jmm_state *out);
int jmmo_plain_get_positions(jmmo_plain *h, double *r, uint64_t n);
int jmmo_plain_get_separations(jmmo_plain *h, double *rij, uint64_t n_pairs);
void jmmo_plain_destroy(jmmo_plain *h);

void jmmo_philox_raw(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
void jmmo_step_words_export(uint64_t seed, uint64_t block, uint32_t chain, uint32_t out[4]);

#endif
