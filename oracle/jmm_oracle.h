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
int jmmo_plain_move(jmmo_plain *h, int32_t kind, uint64_t nm, double rn, jmm_step_record *rec);
/* The plain form's pair functions alone (phiLJcut / phiLJinfcutoff /
 * phiHarmoniccut): phi[0..8] of separation d. */
void jmmo_phi(int32_t potential, double d, double cut, int32_t virial, double l, double *phi);
int jmmo_plain_update_thermo(jmmo_plain *h);
int jmmo_plain_reset_thermo(jmmo_plain *h);
int jmmo_plain_echeck(jmmo_plain *h, double *e_test, int32_t *reset);
int jmmo_plain_set_step_sizes(jmmo_plain *h, double max_step, double max_dl);
int jmmo_plain_get_state(jmmo_plain *h, jmm_state *out);
int jmmo_plain_get_positions(jmmo_plain *h, double *r, uint64_t n);
int jmmo_plain_get_separations(jmmo_plain *h, double *rij, uint64_t n_pairs);
void jmmo_plain_destroy(jmmo_plain *h);
int jmmo_plain_histograms(jmmo_plain *h, uint64_t rhonb, double rbw, int32_t gns, double gsw,
                          uint64_t gnb, double gbw);
int jmmo_plain_take_rho(jmmo_plain *h, int32_t *out, uint64_t rhonb);
int jmmo_plain_take_g(jmmo_plain *h, int32_t *out, uint64_t n);
int jmmo_plain_hist_counts(jmmo_plain *h, int32_t *rho, uint64_t rhonb, int32_t *g,
                           uint64_t ng);
double jmmo_plain_trial_volume_energy(jmmo_plain *h, double dl);
int jmmo_plain_move_volume(jmmo_plain *h, double l);
int jmmo_plain_relax_volume(jmmo_plain *h, jmm_relax_step *log, int32_t *n_steps);

void jmmo_philox_raw(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
void jmmo_step_words_export(uint64_t seed, uint64_t block, uint32_t chain, uint32_t out[4]);

typedef struct jmmo_batch jmmo_batch;

jmmo_batch *jmmo_batch_create(const jmm_batch_config *cfg, const jmm_chain_desc *chains,
                              uint32_t n_chains, int fp64);
void jmmo_batch_destroy(jmmo_batch *b);
int jmmo_batch_run(jmmo_batch *b, uint64_t n_sweeps);
int jmmo_batch_run_chain(jmmo_batch *b, uint32_t chain, uint64_t n_sweeps);
int jmmo_batch_results(jmmo_batch *b, jmm_chain_result *out, uint32_t n_chains);
int jmmo_batch_get_positions(jmmo_batch *b, uint32_t chain, double *x, uint32_t n);
int jmmo_batch_set_positions(jmmo_batch *b, uint32_t chain, const double *x, uint32_t n,
                             double l);
int jmmo_batch_energies(jmmo_batch *b, double *e, uint32_t n_chains);
double jmmo_energy64(const jmm_chain_desc *c, const double *x, double l, int periodic);
void jmmo_batch_hist_sample(const float *x, uint32_t n, float l, int periodic, uint32_t rhonb,
                            float rbw, uint32_t gns, float gsw, uint32_t gnb, float gbw,
                            uint64_t *row);
void jmmo_energy_grad64(const jmm_chain_desc *c, const double *x, double l, int periodic,
                        double out[4]);
float jmmo_portable_logf(float x);
float jmmo_portable_expf(float x);

#endif
