/*
 * oracle/plain_oracle.c -- TEST INFRASTRUCTURE (the oracle), never shipped.
 *
 * CPU FP64 restatement of the reference's single-chain move loop, written to
 * be bit-identical to the reference built with oracle/gsl_shim (checked in
 * tests/test_oracle_vs_reference.py against tests/golden/).  Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg use it.
 *
 *   phiLJcut / phiLJinfcutoff  src/pot.cpp:19-108
 *   phiHarmoniccut             src/pot.cpp:110-141
 *   setupMCS (lattice, rij)    src/jmmMCState.cpp:261-790 (:559-562, :767-769)
 *   fad                        src/jmmMCState.cpp:853-1003
 *   qad2                       src/jmmMCState.cpp:1160-1464
 *   qavLJ                      src/jmmMCState.cpp:1648-1730
 *   incrementStep / Step       src/jmmMCState.cpp:1734-1811
 *   updateThermo               src/jmmMCState.cpp:1941-1961
 *   ECheck                     src/jmmMCState.cpp:1965-2095
 *   fav                        src/jmmMCState.cpp:2161-2293
 *   fgrho / ugrho              src/jmmMCState.cpp:1069-1149
 *   qagrho                     src/jmmMCState.cpp:2297-2384
 *   relaxVolume                src/jmmMCState.cpp:2396-2643
 *   calculateEnergyOfTrialVolumeChange / moveVolume   :2756-2905
 *
 * Every FP64 expression keeps the reference's operand order; the file is
 * compiled with -ffp-contract=off so no multiply-add is fused.
 * Pair (i, j), i < j, lives at the reference's packed index
 * i(N-1) - i(i+1)/2 + j - 1 (pidx) of the pair arrays.
 */
#include "jmm_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

struct jmmo_plain {
  jmm_params prm;
  uint64_t n;
  uint64_t num_trial_types;
  double l;
  double max_step, max_dl;
  uint64_t sn;
  uint64_t rng_block;
  uint32_t rng_slot;
  uint32_t words[4];
  double tot[9];
  double bf;      /* persists across calls like mcs->bf              */
  double ran;     /* persists across calls like the file-static ran  */
  uint64_t d_acc[2], v_acc[2];
  double thermo[12];
  uint64_t echeck_count, echeck_resets;
  double echeck_e, echeck_e_before;
  double *r;
  double *r_trial;
  double *rij;          /* N(N-1)/2 packed, stored separations     */
  double *q;            /* 9 x N(N-1)/2 stored pair quantities     */
  double *rij_trial;    /* N(N-1)/2                                 */
  double *q_trial;      /* 9 x N(N-1)/2                             */
  /* rho(x) and g(x) histograms: current counts (rhol, gl) and their sums
   * since the last take (rhoA, gA), int as in the reference, g slice-major */
  int hist_on;
  uint64_t rhonb, gnb;
  int32_t gns;
  double rbw, gsw, gbw;
  int32_t *rhol, *rhoA, *gl, *gA;
};

/* ---- pair potentials ---------------------------------------------------- */

/* phiLJcut, src/pot.cpp:19-101.  `virial` is the params[0] > 0.1 test. */
static void phi_lj(double d, double cut, int virial, double *phi) {
  double rij3 = d * d * d;
  double rij6 = 1 / (rij3 * rij3);
  double rij12 = rij6 * rij6;
  double phitot = 0, phi6 = 0, phi12 = 0, vir6 = 0, vir12 = 0, virtot = 0;
  double hv6 = 0, hv12 = 0, hvtot = 0;
  if (d <= cut) {
    phi6 = 4 * rij6;
    phi12 = 4 * rij12;
    phitot = phi12 - phi6;
    if (virial) {
      vir6 = 24 * rij6;
      vir12 = 48 * rij12;
      virtot = vir12 - vir6;
      hv6 = 144 * rij6;
      hv12 = 576 * rij12;
      hvtot = hv12 - hv6;
    }
  }
  phi[0] = phitot;
  phi[2] = phi12;
  phi[4] = phi6;
  phi[1] = virtot;
  phi[3] = vir12;
  phi[5] = vir6;
  phi[6] = hvtot;
  phi[7] = hv12;
  phi[8] = hv6;
}

/* phiHarmoniccut, src/pot.cpp:110-141.  The reference leaves phi[2..8]
 * unwritten (and phi[1] undefined when params[0] != 1); they are 0 here. */
static void phi_harmonic(double d, double cut, int virial, double l, double *phi) {
  for (int k = 0; k < 9; ++k) phi[k] = 0;
  if (d <= 0) {
    phi[0] = 10E10;
    phi[1] = 10E10;
  } else if (d < cut) {
    double rijm = d - 1.0;
    phi[0] = rijm * rijm;
    phi[1] = virial ? (2 / l) * d * rijm : 0;
  }
}

static void phi_eval(const jmmo_plain *h, double d, int virial, double l, double *phi) {
  if (h->prm.potential == JMM_POT_HARMONIC)
    phi_harmonic(d, h->prm.cutoff, virial, l, phi);
  else
    phi_lj(d, h->prm.potential == JMM_POT_LJ ? INFINITY : h->prm.cutoff, virial, phi);
}

/* The pair functions alone, for their tests: potential and cut-off as in
 * jmm_params, virial the params[0] > 0.1 test, l phiHarmoniccut's box. */
void jmmo_phi(int32_t potential, double d, double cut, int32_t virial, double l, double *phi) {
  jmmo_plain h;
  memset(&h, 0, sizeof(h));
  h.prm.potential = potential;
  h.prm.cutoff = cut;
  phi_eval(&h, d, virial, l, phi);
}

/* Index of pair (i < j) in the packed row-major triangle, the reference's
 * ind(i, j) = i(N-1) - i(i+1)/2 + j - 1 (src/jmmMCState.cpp:142-148): the
 * pair state takes N(N-1)/2 entries per quantity, as in the reference. */
static inline uint64_t pidx(uint64_t n, uint64_t i, uint64_t j) {
  return i * (n - 1) - i * (i + 1) / 2 + j - 1;
}

/* Pairs beyond the neighbour-number limit carry zeros (jmmMCState.cpp:1217). */
static int pair_cut(const jmmo_plain *h, uint64_t i, uint64_t j) {
  return h->prm.nbn >= 0 && (j - i) > (uint64_t)h->prm.nbn;
}

/* ---- the shim's stream -------------------------------------------------- */

static void open_block(jmmo_plain *h) {
  h->rng_block += 1;
  jmmo_step_words(h->prm.seed, h->rng_block, 0u, h->words);
  h->rng_slot = 0;
}

static uint64_t draw_int(jmmo_plain *h, uint64_t n) {
  open_block(h);
  uint32_t w = h->words[0];
  h->rng_slot = 1;
  return jmmo_word_to_index(w, n);
}

static double draw_uniform(jmmo_plain *h) {
  if (h->rng_slot >= 4) {
    open_block(h);
    h->rng_slot = 1;
  }
  uint32_t w = h->words[h->rng_slot];
  h->rng_slot += 1;
  return jmmo_word_to_unit(w);
}

/* ---- set-up ------------------------------------------------------------- */

static void rebuild_separations(jmmo_plain *h) {
  uint64_t n = h->n;
  for (uint64_t i = 0; i < n; ++i)
    for (uint64_t j = i + 1; j < n; ++j) h->rij[pidx(n, i, j)] = h->r[j] - h->r[i];
}

jmmo_plain *jmmo_plain_create(const jmm_params *prm) {
  if (!prm || prm->n < 2) return NULL;
  if (prm->potential != JMM_POT_LJCUT && prm->potential != JMM_POT_LJ &&
      prm->potential != JMM_POT_HARMONIC)
    return NULL;
  jmmo_plain *h = (jmmo_plain *)calloc(1, sizeof(jmmo_plain));
  h->prm = *prm;
  h->n = prm->n;
  uint64_t n = h->n;
  h->num_trial_types = prm->ensemble == JMM_NPT ? n + 1 : n;
  h->l = prm->ensemble == JMM_NPT ? (double)n : prm->l;
  h->max_step = prm->max_step;
  h->max_dl = prm->max_dl;
  h->rng_slot = 4;
  h->r = (double *)calloc(n, sizeof(double));
  h->r_trial = (double *)calloc(n, sizeof(double));
  h->rij = (double *)calloc(n * (n - 1) / 2, sizeof(double));
  h->rij_trial = (double *)calloc(n * (n - 1) / 2, sizeof(double));
  h->q = (double *)calloc(9 * (n * (n - 1) / 2), sizeof(double));
  h->q_trial = (double *)calloc(9 * (n * (n - 1) / 2), sizeof(double));
  if (!h->r || !h->r_trial || !h->rij || !h->rij_trial || !h->q || !h->q_trial) {
    jmmo_plain_destroy(h);
    return NULL;
  }
  h->tot[JMM_Q_E] = 10E10;
  h->tot[JMM_Q_VIR] = 10E10;
  h->tot[JMM_Q_HV] = 10E10;
  h->tot[JMM_Q_E6] = -5E10;
  h->tot[JMM_Q_E12] = 5E10;
  h->tot[JMM_Q_VIR6] = -5E10;
  h->tot[JMM_Q_VIR12] = 5E10;
  h->tot[JMM_Q_HV6] = -5E10;
  h->tot[JMM_Q_HV12] = 5E10;
  for (uint64_t i = 0; i < n; ++i) h->r[i] = ((i + 0.5) / n - 0.5) * h->l;
  rebuild_separations(h);
  return h;
}

int jmmo_plain_set_config(jmmo_plain *h, const double *r, uint64_t n, double l,
                          uint64_t sn) {
  if (!h || n != h->n) return JMM_ERR_INVALID;
  memcpy(h->r, r, n * sizeof(double));
  h->l = l;
  h->sn = sn;
  h->tot[JMM_Q_E] = 10.0E10;
  h->tot[JMM_Q_VIR] = 10.0E10;
  h->tot[JMM_Q_HV] = 10.0E10;
  rebuild_separations(h);
  return JMM_OK;
}

void jmmo_plain_destroy(jmmo_plain *h) {
  if (!h) return;
  free(h->rhol);
  free(h->rhoA);
  free(h->gl);
  free(h->gA);
  free(h->r);
  free(h->r_trial);
  free(h->rij);
  free(h->rij_trial);
  free(h->q);
  free(h->q_trial);
  free(h);
}

/* ---- rho(x) and g(x) histograms ------------------------------------------ */

/* Counts are int in the reference; sums wrap as its int arithmetic does on
 * the platforms it runs on. */
static int32_t wrap_add(int32_t a, int32_t b) { return (int32_t)((uint32_t)a + (uint32_t)b); }

static long rho_bin(const jmmo_plain *h, double x) {
  return (long)floor(x / h->rbw + h->rhonb / 2.0);
}

static long slice_of(const jmmo_plain *h, double x) {
  return (long)floor(x / h->gsw + h->gns / 2.0);
}

/* fgrho, src/jmmMCState.cpp:1069-1127: counts of the current positions
 * (density) and of the stored separations (g(x), each pair in the slices of
 * both particles).  A negative separation (particles that passed each
 * other) gives a negative bin, which the reference writes out of bounds;
 * here it is not counted. */
static void fgrho(jmmo_plain *h) {
  uint64_t n = h->n;
  memset(h->rhol, 0, h->rhonb * sizeof(int32_t));
  for (uint64_t i = 0; i < n; ++i) {
    long rb = rho_bin(h, h->r[i]);
    if (rb >= 0 && rb < (long)h->rhonb) h->rhol[rb]++;
  }
  memset(h->gl, 0, (uint64_t)h->gns * h->gnb * sizeof(int32_t));
  for (uint64_t i = 0; i < n; ++i) {
    for (uint64_t j = i + 1; j < n; ++j) {
      long gs1 = slice_of(h, h->r[i]);
      long gs2 = slice_of(h, h->r[j]);
      long gb = (long)floor(h->rij[pidx(n, i, j)] / h->gbw);
      if (gb >= 0 && gb < (long)h->gnb) {
        if (gs1 >= 0 && gs1 < h->gns) h->gl[gs1 * h->gnb + gb]++;
        if (gs2 >= 0 && gs2 < h->gns) h->gl[gs2 * h->gnb + gb]++;
      }
    }
  }
}

/* ugrho, src/jmmMCState.cpp:1131-1149 */
static void ugrho(jmmo_plain *h) {
  for (uint64_t b = 0; b < h->rhonb; ++b) h->rhoA[b] = wrap_add(h->rhoA[b], h->rhol[b]);
  for (uint64_t b = 0; b < (uint64_t)h->gns * h->gnb; ++b) h->gA[b] = wrap_add(h->gA[b], h->gl[b]);
}

/* qagrho, src/jmmMCState.cpp:2297-2384: particle nm moved by md (r[nm] is
 * the new position; the old one is formed as r[nm] - md). */
static void qagrho(jmmo_plain *h, uint64_t nm, double md) {
  uint64_t n = h->n;
  long rb1 = rho_bin(h, h->r[nm] - md);
  long rb2 = rho_bin(h, h->r[nm]);
  if (rb1 >= 0 && rb1 < (long)h->rhonb) h->rhol[rb1]--;
  if (rb2 >= 0 && rb2 < (long)h->rhonb) h->rhol[rb2]++;
  long gs11 = slice_of(h, h->r[nm] - md);
  long gs12 = slice_of(h, h->r[nm]);
  int v11 = gs11 >= 0 && gs11 < h->gns, v12 = gs12 >= 0 && gs12 < h->gns;
  for (uint64_t i = 0; i < n; ++i) {
    if (i == nm) continue;
    long gs2 = slice_of(h, h->r[i]);
    int v2 = gs2 >= 0 && gs2 < h->gns;
    long gb1 = (long)(unsigned long)floor(fabs(h->r[nm] - md - h->r[i]) / h->gbw);
    long gb2 = (long)(unsigned long)floor(fabs(h->r[nm] - h->r[i]) / h->gbw);
    int vb1 = gb1 >= 0 && gb1 < (long)h->gnb, vb2 = gb2 >= 0 && gb2 < (long)h->gnb;
    if (v11 && vb1) h->gl[gs11 * h->gnb + gb1]--;
    if (v12 && vb2) h->gl[gs12 * h->gnb + gb2]++;
    if (v2 && vb1) h->gl[gs2 * h->gnb + gb1]--;
    if (v2 && vb2) h->gl[gs2 * h->gnb + gb2]++;
  }
}

int jmmo_plain_histograms(jmmo_plain *h, uint64_t rhonb, double rbw, int32_t gns, double gsw,
                          uint64_t gnb, double gbw) {
  if (!h || rhonb < 1 || gns < 1 || gnb < 1 || !(rbw > 0) || !(gsw > 0) || !(gbw > 0))
    return JMM_ERR_INVALID;
  free(h->rhol);
  free(h->rhoA);
  free(h->gl);
  free(h->gA);
  h->rhonb = rhonb;
  h->rbw = rbw;
  h->gns = gns;
  h->gsw = gsw;
  h->gnb = gnb;
  h->gbw = gbw;
  h->rhol = (int32_t *)calloc(rhonb, sizeof(int32_t));
  h->rhoA = (int32_t *)calloc(rhonb, sizeof(int32_t));
  h->gl = (int32_t *)calloc((uint64_t)gns * gnb, sizeof(int32_t));
  h->gA = (int32_t *)calloc((uint64_t)gns * gnb, sizeof(int32_t));
  if (!h->rhol || !h->rhoA || !h->gl || !h->gA) return JMM_ERR_NOMEM;
  h->hist_on = 1;
  fgrho(h); /* set-up: current counts, accumulated once (jmmMCState.cpp:773-776) */
  ugrho(h);
  return JMM_OK;
}

int jmmo_plain_take_rho(jmmo_plain *h, int32_t *out, uint64_t rhonb) {
  if (!h->hist_on || rhonb != h->rhonb) return JMM_ERR_INVALID;
  memcpy(out, h->rhoA, rhonb * sizeof(int32_t));
  memset(h->rhoA, 0, rhonb * sizeof(int32_t));
  return JMM_OK;
}

int jmmo_plain_take_g(jmmo_plain *h, int32_t *out, uint64_t n) {
  if (!h->hist_on || n != (uint64_t)h->gns * h->gnb) return JMM_ERR_INVALID;
  memcpy(out, h->gA, n * sizeof(int32_t));
  memset(h->gA, 0, n * sizeof(int32_t));
  return JMM_OK;
}

int jmmo_plain_hist_counts(jmmo_plain *h, int32_t *rho, uint64_t rhonb, int32_t *g,
                           uint64_t ng) {
  if (!h->hist_on || rhonb != h->rhonb || ng != (uint64_t)h->gns * h->gnb)
    return JMM_ERR_INVALID;
  memcpy(rho, h->rhol, rhonb * sizeof(int32_t));
  memcpy(g, h->gl, ng * sizeof(int32_t));
  return JMM_OK;
}

/* ---- moves -------------------------------------------------------------- */

static void commit_pair(jmmo_plain *h, uint64_t ind) {
  uint64_t nn = h->n * (h->n - 1) / 2;
  h->rij[ind] = h->rij_trial[ind];
  for (int k = 0; k < 9; ++k) h->q[k * nn + ind] = h->q_trial[k * nn + ind];
}

/* fad, src/jmmMCState.cpp:853-1003 */
int jmmo_plain_fad(jmmo_plain *h, uint64_t nm, double d) {
  if (!h || nm >= h->n) return JMM_ERR_INVALID;
  uint64_t n = h->n, nn = n * (n - 1) / 2;
  double rn = d;
  memcpy(h->r_trial, h->r, n * sizeof(double));
  double md = (rn - 0.5) * 2 * h->max_step;
  h->r_trial[nm] = h->r[nm] + md;
  if (fabs(h->r_trial[nm]) > (h->l / 2.0)) {
    h->d_acc[1]++;
    return JMM_OK;
  }
  double sum[9] = {0};
  double phi[9];
  for (uint64_t i = 0; i < n; ++i) {
    for (uint64_t j = i + 1; j < n; ++j) {
      uint64_t ind = pidx(n, i, j);
      h->rij_trial[ind] = h->r_trial[j] - h->r_trial[i];
      if (pair_cut(h, i, j)) {
        for (int k = 0; k < 9; ++k) h->q_trial[k * nn + ind] = 0;
      } else {
        phi_eval(h, h->rij_trial[ind], 1, h->l, phi);
        for (int k = 0; k < 9; ++k) {
          h->q_trial[k * nn + ind] = phi[k];
          sum[k] += phi[k];
        }
      }
    }
  }
  if (sum[JMM_Q_E] > h->tot[JMM_Q_E]) {
    h->ran = draw_uniform(h);
    h->bf = exp((h->tot[JMM_Q_E] - sum[JMM_Q_E]) / h->prm.t);
  }
  if (sum[JMM_Q_E] < h->tot[JMM_Q_E] || h->bf > h->ran) {
    h->d_acc[0]++;
    for (int k = 0; k < 9; ++k) h->tot[k] = sum[k];
    h->r[nm] = h->r_trial[nm];
    for (uint64_t i = 0; i < n; ++i)
      for (uint64_t j = i + 1; j < n; ++j) commit_pair(h, pidx(n, i, j));
  } else {
    h->d_acc[1]++;
  }
  return JMM_OK;
}

static void set_record(jmm_step_record *rec, const jmmo_plain *h, uint64_t nm, double rn,
                       double ran, double bf, int kind, int outcome) {
  if (!rec) return;
  rec->sn = h->sn;
  rec->nm = nm;
  rec->rn = rn;
  rec->ran = ran;
  rec->bf = bf;
  rec->e = h->tot[JMM_Q_E];
  rec->vir = h->tot[JMM_Q_VIR];
  rec->hv = h->tot[JMM_Q_HV];
  rec->l = h->l;
  rec->kind = kind;
  rec->outcome = outcome;
}

/* qad2, src/jmmMCState.cpp:1160-1464 (the histogram updates of :1431 and
 * :1453 in qad2 below) */
static int qad2_move(jmmo_plain *h, uint64_t nm, double rn, const jmm_draw *rp,
                     double *ran_out, double *bf_out) {
  uint64_t n = h->n, nn = n * (n - 1) / 2;
  double md = (rn - 0.5) * 2 * h->max_step;
  h->r_trial[nm] = h->r[nm] + md;
  if (fabs(h->r_trial[nm]) > h->l / 2.0) {
    h->d_acc[1]++;
    return JMM_OUT_REJECT_WALL;
  }
  double phi[9];
  double da[9] = {0}, db[9] = {0}, dsum[9];
  /* loop A: partners i < nm, separation r[nm] - r[i] grows by md */
  for (uint64_t i = 0; i < nm; ++i) {
    uint64_t ind = pidx(n, i, nm);
    h->rij_trial[ind] = h->rij[ind] + md;
    if (pair_cut(h, i, nm)) {
      for (int k = 0; k < 9; ++k) h->q_trial[k * nn + ind] = 0;
    } else {
      phi_eval(h, h->rij_trial[ind], 1, h->l, phi);
      for (int k = 0; k < 9; ++k) h->q_trial[k * nn + ind] = phi[k];
    }
    for (int k = 0; k < 9; ++k)
      da[k] = da[k] - h->q[k * nn + ind] + h->q_trial[k * nn + ind];
  }
  /* loop B: partners i > nm, separation r[i] - r[nm] shrinks by md */
  for (uint64_t i = nm + 1; i < n; ++i) {
    uint64_t ind = pidx(n, nm, i);
    h->rij_trial[ind] = h->rij[ind] - md;
    if (pair_cut(h, nm, i)) {
      for (int k = 0; k < 9; ++k) h->q_trial[k * nn + ind] = 0;
    } else {
      phi_eval(h, h->rij_trial[ind], 1, h->l, phi);
      for (int k = 0; k < 9; ++k) h->q_trial[k * nn + ind] = phi[k];
    }
    for (int k = 0; k < 9; ++k)
      db[k] = db[k] - h->q[k * nn + ind] + h->q_trial[k * nn + ind];
  }
  for (int k = 0; k < 9; ++k) dsum[k] = da[k] + db[k];
  double de = dsum[JMM_Q_E];
  if (de > 0) {
    h->ran = rp ? rp->ran : draw_uniform(h);
    h->bf = exp(-de / h->prm.t);
    *ran_out = h->ran;
    *bf_out = h->bf;
  }
  if (de <= 0 || h->bf > h->ran) {
    h->d_acc[0]++;
    for (int k = 0; k < 9; ++k) h->tot[k] += dsum[k];
    h->r[nm] = h->r_trial[nm];
    for (uint64_t i = 0; i < nm; ++i) commit_pair(h, pidx(n, i, nm));
    for (uint64_t i = nm + 1; i < n; ++i) commit_pair(h, pidx(n, nm, i));
    if (h->hist_on) qagrho(h, nm, md);
    return JMM_OUT_ACCEPT;
  }
  h->d_acc[1]++;
  return JMM_OUT_REJECT;
}

/* qad2 accumulates the histograms once whatever the outcome, the wall
 * rejection included (ugrho at src/jmmMCState.cpp:1453). */
static int qad2(jmmo_plain *h, uint64_t nm, double rn, const jmm_draw *rp,
                double *ran_out, double *bf_out) {
  int outcome = qad2_move(h, nm, rn, rp, ran_out, bf_out);
  if (h->hist_on) ugrho(h);
  return outcome;
}

/* fav, src/jmmMCState.cpp:2161-2293 */
static int fav(jmmo_plain *h, double rn, const jmm_draw *rp, double *ran_out,
               double *bf_out) {
  uint64_t n = h->n, nn = n * (n - 1) / 2;
  double dl = (rn - 0.5) * 2 * h->max_dl;
  double lnew = h->l + dl;
  double lrat1 = lnew / h->l;
  for (uint64_t i = 0; i < n; ++i) h->r_trial[i] = h->r[i] * lrat1;
  double sum[9] = {0};
  double phi[9];
  for (uint64_t i = 0; i < n; ++i) {
    for (uint64_t j = i + 1; j < n; ++j) {
      uint64_t ind = pidx(n, i, j);
      if (pair_cut(h, i, j)) {
        for (int k = 0; k < 9; ++k) h->q_trial[k * nn + ind] = 0;
      } else {
        double d = h->r_trial[j] - h->r_trial[i];
        phi_eval(h, d, 1, lnew, phi);
        for (int k = 0; k < 9; ++k) {
          h->q_trial[k * nn + ind] = phi[k];
          sum[k] += phi[k];
        }
      }
    }
  }
  h->bf = exp(-(sum[JMM_Q_E] - h->tot[JMM_Q_E] + h->prm.p * dl) / h->prm.t +
              h->n * log(lrat1));
  *bf_out = h->bf;
  if (h->bf < 1.0) {
    h->ran = rp ? rp->ran : draw_uniform(h);
    *ran_out = h->ran;
  }
  if (h->bf >= 1.0 || h->bf > h->ran) {
    h->v_acc[0]++;
    h->l = h->l + dl;
    for (int k = 0; k < 9; ++k) h->tot[k] = sum[k];
    memcpy(h->r, h->r_trial, n * sizeof(double));
    for (uint64_t i = 0; i < n; ++i) {
      for (uint64_t j = i + 1; j < n; ++j) {
        uint64_t ind = pidx(n, i, j);
        h->rij[ind] = h->r[j] - h->r[i];
        for (int k = 0; k < 9; ++k) h->q[k * nn + ind] = h->q_trial[k * nn + ind];
      }
    }
    return JMM_OUT_ACCEPT;
  }
  h->v_acc[1]++;
  return JMM_OUT_REJECT;
}

/* qavLJ, src/jmmMCState.cpp:1648-1730, restated with a 9-entry phi buffer.
 * The reference passes a 6-entry buffer to a 9-entry writer
 * (jmmMCState.cpp:1651 vs pot.cpp:90-100) and aborts on the first accepted
 * volume move, so nothing here is pinned to it. */
static int qav_lj(jmmo_plain *h, double rn, const jmm_draw *rp, double *ran_out,
                  double *bf_out) {
  uint64_t n = h->n, nn = n * (n - 1) / 2;
  double dl = (rn - 0.5) * 2 * h->max_dl;
  double lrat1 = (h->l + dl) / h->l;
  double lrat3 = lrat1 * lrat1 * lrat1;
  double lrat6 = 1 / (lrat3 * lrat3);
  double lrat12 = lrat6 * lrat6;
  double e12t = lrat12 * h->tot[JMM_Q_E12];
  double e6t = lrat6 * h->tot[JMM_Q_E6];
  double de = e12t - e6t - h->tot[JMM_Q_E];
  h->bf = exp(-(de + h->prm.p * dl) / h->prm.t + h->n * log(lrat1));
  *bf_out = h->bf;
  if (h->bf < 1.0) {
    h->ran = rp ? rp->ran : draw_uniform(h);
    *ran_out = h->ran;
  }
  if (h->bf >= 1.0 || h->bf > h->ran) {
    h->v_acc[0]++;
    h->tot[JMM_Q_E] = h->tot[JMM_Q_E] + de;
    h->tot[JMM_Q_E12] = e12t;
    h->tot[JMM_Q_E6] = e6t;
    h->l = h->l + dl;
    double lrat7 = lrat6 / lrat1;
    double lrat13 = lrat12 / lrat1;
    h->tot[JMM_Q_VIR6] = lrat7 * h->tot[JMM_Q_VIR6];
    h->tot[JMM_Q_VIR12] = lrat13 * h->tot[JMM_Q_VIR12];
    h->tot[JMM_Q_VIR] = h->n * h->prm.t / h->l + h->tot[JMM_Q_VIR12] - h->tot[JMM_Q_VIR6];
    for (uint64_t i = 0; i < n; ++i) h->r[i] = lrat1 * h->r[i];
    double phi[9];
    for (uint64_t i = 0; i < n; ++i) {
      for (uint64_t j = i + 1; j < n; ++j) {
        uint64_t ind = pidx(n, i, j);
        h->rij[ind] = lrat1 * h->rij[ind];
        phi_eval(h, h->rij[ind], 1, h->l, phi);
        for (int k = 0; k < 9; ++k) h->q[k * nn + ind] = phi[k];
      }
    }
    if (h->hist_on) { /* fgrho, then ugrho (src/jmmMCState.cpp:1717, :1726) */
      fgrho(h);
      ugrho(h);
    }
    return JMM_OUT_ACCEPT;
  }
  h->v_acc[1]++;
  if (h->hist_on) ugrho(h);
  return JMM_OUT_REJECT;
}

/* ECheck, src/jmmMCState.cpp:1965-2095 */
int jmmo_plain_echeck(jmmo_plain *h, double *e_test_out, int32_t *reset_out) {
  uint64_t n = h->n, nn = n * (n - 1) / 2;
  double phi[9];
  double etest = 0;
  for (uint64_t i = 0; i < n; ++i) {
    for (uint64_t j = i + 1; j < n; ++j) {
      if (pair_cut(h, i, j)) continue;
      phi_eval(h, h->r[j] - h->r[i], 0, h->l, phi);
      etest += phi[0];
    }
  }
  h->echeck_count++;
  h->echeck_e = etest;
  h->echeck_e_before = h->tot[JMM_Q_E];
  int reset = fabs(etest - h->tot[JMM_Q_E]) > 0.0001;
  if (reset) {
    h->echeck_resets++;
    double sum[9] = {0};
    for (uint64_t i = 0; i < n; ++i) {
      for (uint64_t j = i + 1; j < n; ++j) {
        uint64_t ind = pidx(n, i, j);
        if (pair_cut(h, i, j)) {
          for (int k = 0; k < 9; ++k) h->q[k * nn + ind] = 0;
        } else {
          h->rij[ind] = h->r[j] - h->r[i];
          phi_eval(h, h->rij[ind], 1, h->l, phi);
          for (int k = 0; k < 9; ++k) {
            h->q[k * nn + ind] = phi[k];
            sum[k] += phi[k];
          }
        }
      }
    }
    for (int k = 0; k < 9; ++k) h->tot[k] = sum[k];
  }
  if (e_test_out) *e_test_out = etest;
  if (reset_out) *reset_out = reset;
  return JMM_OK;
}

/* updateThermo, src/jmmMCState.cpp:1941-1961 */
int jmmo_plain_update_thermo(jmmo_plain *h) {
  double *a = h->thermo;
  double l = h->l, e = h->tot[JMM_Q_E], vir = h->tot[JMM_Q_VIR], hv = h->tot[JMM_Q_HV];
  double rho = h->n / l;
  a[0] = a[0] + rho;
  a[1] = a[1] + rho * rho;
  a[2] = a[2] + l;
  a[3] = a[3] + l * l;
  a[4] = a[4] + e;
  a[5] = a[5] + e * e;
  a[6] = a[6] + l * e;
  a[7] = a[7] + vir;
  a[8] = a[8] + vir * vir;
  a[9] = a[9] + e * vir;
  a[10] = a[10] + hv;
  a[11] = a[11] + hv * hv;
  return JMM_OK;
}

int jmmo_plain_reset_thermo(jmmo_plain *h) {
  memset(h->thermo, 0, sizeof(h->thermo));
  return JMM_OK;
}

/* incrementStep + Step, src/jmmMCState.cpp:1734-1811 */
int jmmo_plain_steps(jmmo_plain *h, uint64_t n_steps, const jmm_draw *replay,
                     jmm_step_record *log) {
  for (uint64_t s = 0; s < n_steps; ++s) {
    h->sn++;
    const jmm_draw *rp = replay ? &replay[s] : NULL;
    uint64_t nm;
    double rn;
    if (rp) {
      nm = rp->nm;
      rn = rp->rn;
    } else {
      nm = draw_int(h, h->num_trial_types);
      rn = draw_uniform(h);
    }
    double ran = NAN, bf = NAN;
    int kind = JMM_KIND_DISPLACEMENT, outcome;
    if (nm < h->n) {
      outcome = qad2(h, nm, rn, rp, &ran, &bf);
    } else if (nm == h->n) {
      kind = JMM_KIND_VOLUME;
      if (h->prm.potential == JMM_POT_LJ && h->prm.nbn < 0)
        outcome = qav_lj(h, rn, rp, &ran, &bf);
      else
        outcome = fav(h, rn, rp, &ran, &bf);
    } else {
      return JMM_ERR_INVALID;
    }
    if (h->prm.eci && h->sn % h->prm.eci == 0) jmmo_plain_echeck(h, NULL, NULL);
    jmmo_plain_update_thermo(h);
    set_record(log ? &log[s] : NULL, h, nm, rn, ran, bf, kind, outcome);
  }
  return JMM_OK;
}

int jmmo_plain_set_step_sizes(jmmo_plain *h, double max_step, double max_dl) {
  h->max_step = max_step;
  h->max_dl = max_dl;
  return JMM_OK;
}

int jmmo_plain_get_state(jmmo_plain *h, jmm_state *s) {
  memset(s, 0, sizeof(*s));
  s->sn = h->sn;
  s->rng_block = h->rng_block;
  s->rng_slot = h->rng_slot;
  s->l = h->l;
  memcpy(s->tot, h->tot, sizeof(h->tot));
  s->d_acc[0] = h->d_acc[0];
  s->d_acc[1] = h->d_acc[1];
  s->v_acc[0] = h->v_acc[0];
  s->v_acc[1] = h->v_acc[1];
  s->max_step = h->max_step;
  s->max_dl = h->max_dl;
  memcpy(s->thermo, h->thermo, sizeof(h->thermo));
  s->echeck_count = h->echeck_count;
  s->echeck_resets = h->echeck_resets;
  s->echeck_e = h->echeck_e;
  s->echeck_e_before = h->echeck_e_before;
  return JMM_OK;
}

int jmmo_plain_get_positions(jmmo_plain *h, double *r, uint64_t n) {
  if (n != h->n) return JMM_ERR_INVALID;
  memcpy(r, h->r, n * sizeof(double));
  return JMM_OK;
}

int jmmo_plain_get_separations(jmmo_plain *h, double *rij, uint64_t n_pairs) {
  uint64_t n = h->n;
  if (n_pairs != n * (n - 1) / 2) return JMM_ERR_INVALID;
  uint64_t k = 0;
  for (uint64_t i = 0; i < n; ++i)
    for (uint64_t j = i + 1; j < n; ++j) rij[k++] = h->rij[pidx(n, i, j)];
  return JMM_OK;
}

/* The raw Philox4x32-10 block and the per-step words, for the RNG tests. */
void jmmo_philox_raw(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  jmmo_philox4x32_10(ctr, key, out);
}

void jmmo_step_words_export(uint64_t seed, uint64_t block, uint32_t chain, uint32_t out[4]) {
  jmmo_step_words(seed, block, chain, out);
}

/* One trial outside Step (the reference's qad2/fav/qavLJ called directly). */
int jmmo_plain_move(jmmo_plain *h, int32_t kind, uint64_t nm, double rn, jmm_step_record *rec) {
  double ran = NAN, bf = NAN;
  int outcome;
  if (kind == JMM_KIND_DISPLACEMENT) {
    if (nm >= h->n) return JMM_ERR_INVALID;
    outcome = qad2(h, nm, rn, NULL, &ran, &bf);
  } else if (h->prm.potential == JMM_POT_LJ && h->prm.nbn < 0) {
    outcome = qav_lj(h, rn, NULL, &ran, &bf);
  } else {
    outcome = fav(h, rn, NULL, &ran, &bf);
  }
  set_record(rec, h, kind == JMM_KIND_VOLUME ? h->n : nm, rn, ran, bf, kind, outcome);
  return JMM_OK;
}

/* ---- volume relaxation ----------------------------------------------------- */

/* calculateEnergyOfTrialVolumeChange, src/jmmMCState.cpp:2756-2800: E of the
 * positions scaled to L + dl, summed in pair order, pairs beyond NBN zero. */
double jmmo_plain_trial_volume_energy(jmmo_plain *h, double dl) {
  uint64_t n = h->n;
  double lrat1 = (h->l + dl) / h->l;
  for (uint64_t i = 0; i < n; ++i) h->r_trial[i] = h->r[i] * lrat1;
  double e = 0, phi[9];
  for (uint64_t i = 0; i < n; ++i) {
    for (uint64_t j = i + 1; j < n; ++j) {
      if (pair_cut(h, i, j)) continue;
      phi_eval(h, h->r_trial[j] - h->r_trial[i], 0, h->l, phi);
      e += phi[0];
    }
  }
  return e;
}

/* moveVolume, src/jmmMCState.cpp:2803-2905: positions scaled to the box
 * length l, every pair and total recomputed (separations of pairs beyond NBN
 * are left as they were). */
int jmmo_plain_move_volume(jmmo_plain *h, double l) {
  uint64_t n = h->n, nn = n * (n - 1) / 2;
  double lrat1 = l / h->l;
  for (uint64_t i = 0; i < n; ++i) h->r[i] = h->r[i] * lrat1;
  h->l = l;
  double sum[9] = {0}, phi[9];
  for (uint64_t i = 0; i < n; ++i) {
    for (uint64_t j = i + 1; j < n; ++j) {
      uint64_t ind = pidx(n, i, j);
      if (pair_cut(h, i, j)) {
        for (int k = 0; k < 9; ++k) h->q[k * nn + ind] = 0;
        continue;
      }
      h->rij[ind] = h->r[j] - h->r[i];
      phi_eval(h, h->rij[ind], 1, l, phi);
      for (int k = 0; k < 9; ++k) {
        h->q[k * nn + ind] = phi[k];
        sum[k] += phi[k];
      }
    }
  }
  memcpy(h->tot, sum, sizeof(sum));
  return JMM_OK;
}

/* relaxVolume, src/jmmMCState.cpp:2396-2643: up to 20 Newton steps on
 * E(L) + P L - N T ln L from central differences at +-0.1, each clamped to
 * 0.1 N and to the bracket of lengths seen, until a step is below 0.0025 N.
 * One record per step; returns 1 when converged, 0 after 20 steps. */
int jmmo_plain_relax_volume(jmmo_plain *h, jmm_relax_step *log, int32_t *n_steps) {
  double ltrymin = 0, ltrymax = 1E10;
  const double hh = 0.1;
  for (int count = 0; count < 20; ++count) {
    double eup = jmmo_plain_trial_volume_energy(h, hh);
    double edown = jmmo_plain_trial_volume_energy(h, -hh);
    double e = h->tot[JMM_Q_E];
    double first = (eup - edown) / (2 * hh);
    double second = (eup - 2.0 * e + edown) / (hh * hh);
    double dle = -(h->prm.p - ((double)h->n / h->l) * h->prm.t + first) / second;
    double relax_max = (double)0.10 * h->n;
    if (fabs(dle) > relax_max) dle = dle < 0 ? -relax_max : relax_max;
    if (h->l + dle > ltrymax)
      dle = 0.5 * (ltrymax - h->l);
    else if (h->l + dle < ltrymin)
      dle = 0.5 * (ltrymin - h->l);
    if (dle > 0.0)
      ltrymin = h->l;
    else
      ltrymax = h->l;
    int done = fabs(dle) < 0.0025 * h->n;
    jmmo_plain_move_volume(h, h->l + dle);
    if (log) {
      log[count].e_up = eup;
      log[count].e_down = edown;
      log[count].dl = dle;
      log[count].l = h->l;
      log[count].e = h->tot[JMM_Q_E];
    }
    if (n_steps) *n_steps = count + 1;
    if (done) return 1;
  }
  return 0;
}
