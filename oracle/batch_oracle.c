/*
 * oracle/batch_oracle.c -- TEST INFRASTRUCTURE (the oracle), never shipped.
 *
 * CPU restatement of the batched chain form (include/jmm_gpu.h, jmm_batch_*).
 * Each chain is the reference's sequential single-particle Metropolis chain
 * (Step src/jmmMCState.cpp:1758-1811, qad2 :1160-1464, fav :2161-2293,
 * updateThermo :1941-1961) with the batched form's choices: Philox block
 * (step, chain) per step, ordered particles, windowed neighbours, ln L or
 * linear volume moves, FP64 re-summation at volume moves.
 *
 * Two modes:
 *  - FP32 (fp64 = 0): the kernel's EXACT precision mode operation for
 *    operation -- the lane-to-neighbour map of a group of G lanes, the
 *    butterfly order of the group sums, the FP32 running offset and its FP64
 *    folds -- so that positions, energies and statistics match bit for bit.
 *  - FP64 (fp64 = 1): the same chain with FP64 positions and pair energies and
 *    libm exp/log: the FP64 reference for energies and ensemble averages.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "jmm_fp32.h"
#include "jmm_oracle.h"

struct jmmo_batch {
  jmm_batch_config cfg;
  uint32_t n_chains;
  int fp64;
  uint32_t g;      /* window lanes G of one trial move          */
  uint32_t lanes;  /* lanes per chain G*S: energy-sum partition */
  jmm_chain_desc *chains;
  jmm_chain_result *res;
  float **xf;
  double **xd;
};

typedef struct {
  uint32_t n, pot, ensemble, spsw, id;
  float eps4, sigma2, inv_sigma2, rc2, beta, two_max_step, vol_step, rc;
  double beta_d, p;
  /* FP64 copies */
  double eps4_d, sigma2_d, inv_sigma2_d, rc2_d, two_max_step_d, vol_step_d;
} chain_prm;

static chain_prm make_prm(const jmm_chain_desc *c, uint32_t id) {
  chain_prm P;
  memset(&P, 0, sizeof(P));
  P.id = id;
  P.n = c->n;
  P.pot = (uint32_t)c->potential;
  P.ensemble = (uint32_t)c->ensemble;
  P.spsw = c->ensemble == JMM_NPT ? c->n + 1 : c->n;
  P.eps4 = c->potential == JMM_POT_LJCUT ? (float)(4.0 * c->eps) : (float)c->eps;
  P.sigma2 = (float)(c->sigma * c->sigma);
  P.inv_sigma2 = (float)(1.0 / (c->sigma * c->sigma));
  P.rc2 = (float)(c->cutoff * c->cutoff);
  P.rc = (float)c->cutoff;
  P.beta = (float)(1.0 / c->t);
  P.beta_d = 1.0 / c->t;
  P.p = c->p;
  P.two_max_step = (float)(2.0 * c->max_step);
  P.vol_step = (float)c->vol_step;
  P.eps4_d = c->potential == JMM_POT_LJCUT ? 4.0 * c->eps : c->eps;
  P.sigma2_d = c->sigma * c->sigma;
  P.inv_sigma2_d = 1.0 / (c->sigma * c->sigma);
  P.rc2_d = c->cutoff * c->cutoff;
  P.two_max_step_d = 2.0 * c->max_step;
  P.vol_step_d = c->vol_step;
  return P;
}

/* ---- pair energies ------------------------------------------------------ */

static float pair_e32(float d2, const chain_prm *P) {
  if (!(d2 <= P->rc2)) return 0.0f;
  if (P->pot == JMM_POT_GAUSS) return P->eps4 * jmmo_expf(-(d2 * P->inv_sigma2));
  float inv2 = P->sigma2 * (1.0f / d2);
  float inv6 = (inv2 * inv2) * inv2;
  if (P->pot == JMM_POT_SOFTSPHERE) return P->eps4 * (inv6 * inv6);
  return P->eps4 * (inv6 * (inv6 - 1.0f));
}

static double pair_e64(double d2, const chain_prm *P) {
  if (!(d2 <= P->rc2_d)) return 0.0;
  if (P->pot == JMM_POT_GAUSS) return P->eps4_d * exp(-d2 * P->inv_sigma2_d);
  double inv2 = P->sigma2_d / d2;
  double inv6 = inv2 * inv2 * inv2;
  if (P->pot == JMM_POT_SOFTSPHERE) return P->eps4_d * inv6 * inv6;
  return P->eps4_d * inv6 * (inv6 - 1.0);
}

static float butterfly32(float *v, uint32_t g) {
  float tmp[32];
  for (uint32_t m = 1; m < g; m <<= 1) {
    for (uint32_t k = 0; k < g; ++k) tmp[k] = v[k] + v[k ^ m];
    memcpy(v, tmp, g * sizeof(float));
  }
  return v[0];
}

static double butterfly64(double *v, uint32_t g) {
  double tmp[32];
  for (uint32_t m = 1; m < g; m <<= 1) {
    for (uint32_t k = 0; k < g; ++k) tmp[k] = v[k] + v[k ^ m];
    memcpy(v, tmp, g * sizeof(double));
  }
  return v[0];
}

/* U_old and (scaled) U_new with the kernel's lane partition (FP32 mode). */
static void energies32(const float *xs, const chain_prm *P, uint32_t g, int periodic, float lf,
                       int scaled, float s, float lnf, double *u_old, double *u_new,
                       uint64_t *pairs, uint32_t *err) {
  const int n = (int)P->n;
  double uo[32], un[32];
  uint64_t cnt = 0;
  for (uint32_t gl = 0; gl < g; ++gl) {
    uo[gl] = 0.0;
    un[gl] = 0.0;
    for (int i = (int)gl; i < n; i += (int)g) {
      float xi = xs[i];
      float xin = scaled ? xi * s : xi;
      float eo = 0.0f, en = 0.0f;
      for (int k = 1;; ++k) {
        int j = i + k;
        float shift = 0.0f, shiftn = 0.0f;
        if (!periodic) {
          if (j >= n) break;
        } else {
          if (2 * k > n - 1) {
            *err = JMM_ERR_INVALID;
            break;
          }
          if (j >= n) {
            j -= n;
            shift = lf;
            shiftn = lnf;
          }
        }
        float xj = xs[j];
        float d = (xj + shift) - xi;
        float d2 = d * d;
        float dn2 = d2;
        if (scaled) {
          float dn = ((xj * s) + shiftn) - xin;
          dn2 = dn * dn;
        }
        if (d2 > P->rc2 && dn2 > P->rc2) break;
        eo = eo + pair_e32(d2, P);
        if (scaled) en = en + pair_e32(dn2, P);
        cnt += scaled ? 2 : 1;
      }
      uo[gl] = uo[gl] + (double)eo;
      if (scaled) un[gl] = un[gl] + (double)en;
    }
  }
  *u_old = butterfly64(uo, g);
  *u_new = scaled ? butterfly64(un, g) : *u_old;
  *pairs += cnt;
}

static void energies64(const double *xs, const chain_prm *P, int periodic, double l, double s,
                       double lnew, double *u_old, double *u_new, uint64_t *pairs) {
  const int n = (int)P->n;
  double uo = 0.0, un = 0.0;
  for (int i = 0; i < n; ++i) {
    for (int k = 1;; ++k) {
      int j = i + k;
      double shift = 0.0, shiftn = 0.0;
      if (!periodic) {
        if (j >= n) break;
      } else {
        if (2 * k > n - 1) break;
        if (j >= n) {
          j -= n;
          shift = l;
          shiftn = lnew;
        }
      }
      double d = xs[j] + shift - xs[i];
      double dn = xs[j] * s + shiftn - xs[i] * s;
      double d2 = d * d, dn2 = dn * dn;
      if (d2 > P->rc2_d && dn2 > P->rc2_d) break;
      uo += pair_e64(d2, P);
      un += pair_e64(dn2, P);
      *pairs += 2;
    }
  }
  *u_old = uo;
  *u_new = un;
}

/* ---- statistics ------------------------------------------------------------ */

typedef struct {
  double e0;
  float delta, sd, sd2;
  uint32_t nseg;
  double delta_d, sd_d, sd2_d; /* FP64 mode */
} seg_t;

static void fold(seg_t *g, jmm_chain_result *R, double l, uint32_t n, int fp64) {
  double nd = (double)g->nseg;
  double sdd = fp64 ? g->sd_d : (double)g->sd;
  double sd2d = fp64 ? g->sd2_d : (double)g->sd2;
  double lin = nd * g->e0 + sdd;
  R->sum_e = R->sum_e + lin;
  R->sum_e2 = R->sum_e2 + (((nd * g->e0) * g->e0 + (2.0 * g->e0) * sdd) + sd2d);
  R->sum_l = R->sum_l + nd * l;
  R->sum_l2 = R->sum_l2 + (nd * l) * l;
  R->sum_le = R->sum_le + l * lin;
  double rho = (double)n / l;
  R->sum_rho = R->sum_rho + nd * rho;
  R->sum_rho2 = R->sum_rho2 + (nd * rho) * rho;
  R->samples += g->nseg;
  g->e0 = g->e0 + (fp64 ? g->delta_d : (double)g->delta);
  g->delta = g->sd = g->sd2 = 0.0f;
  g->delta_d = g->sd_d = g->sd2_d = 0.0;
  g->nseg = 0;
}

static float threshold32(uint32_t w) {
  float u = ((float)(w >> 9) + 0.5f) * 1.1920929e-07f;
  return -jmmo_logf(u);
}

static double threshold64(uint32_t w) {
  double u = ((double)(w >> 9) + 0.5) * (1.0 / 8388608.0);
  return -log(u);
}

/* One launch of n_sweeps for one chain. */
/* One displacement step of the FP32 chain (the EXACT kernel's arithmetic):
 * particle nm of xs[0..n) with the step's Philox words w, G window lanes of
 * W neighbours per side; moves the particle when accepted and returns the
 * accepted energy change (0 when rejected).  Counts accepted moves, window
 * extensions and window pair slots (4 W per step and per extension). */
static float disp32(float *xs, int n, int nm, const uint32_t w[4], const chain_prm *P,
                    int periodic, float lf, float half_l, uint32_t G, uint32_t W, uint64_t *pairs,
                    uint32_t *err, jmm_chain_result *R) {
  const float u1 = (float)(w[1] >> 8) * (1.0f / 16777216.0f);
  const float thr = threshold32(w[2]);
  const float md = (u1 - 0.5f) * P->two_max_step;
  const float xo = xs[nm];
  const float xn = xo + md;
  float left, right;
  if (periodic) {
    left = nm > 0 ? xs[nm - 1] : xs[n - 1] - lf;
    right = nm + 1 < n ? xs[nm + 1] : xs[0] + lf;
  } else {
    left = nm > 0 ? xs[nm - 1] : -INFINITY;
    right = nm + 1 < n ? xs[nm + 1] : INFINITY;
  }
  int ok = (xn > left) && (xn < right);
  if (!periodic) ok = ok && !(fabsf(xn) > half_l);
  /* the step's lanes evaluate its window (4 W pair slots) whether or not
   * the trial keeps its place */
  if (!ok) {
    *pairs += 4 * W;
    return 0.0f;
  }
  /* lane w of the G lanes of a step: side -1 for w < G/2; offsets
   * kb, kb + G/2, ... (kb = w % (G/2) + 1) up to the window W,
   * summed in offset order, then the butterfly over the G lanes */
  const int H2 = (int)G / 2;
  const int KPL = (int)W / H2;
  float de = 0.0f;
  for (int chunk = 0;; ++chunk) {
    float v[32] = {0};
    int any_sat = 0;
    for (uint32_t gl = 0; gl < G; ++gl) {
      const int side = (int)gl < H2 ? -1 : 1;
      const int kb = (int)gl % H2 + 1;
      float tl = 0.0f;
      for (int q = 0; q < KPL; ++q) {
        const int k = chunk * (int)W + kb + q * H2;
        int j = nm + side * k;
        int valid = 1;
        float shift = 0.0f;
        if (!periodic) {
          valid = j >= 0 && j < n;
        } else if (j < 0) {
          j += n;
          shift = -lf;
        } else if (j >= n) {
          j -= n;
          shift = lf;
        }
        float tq = 0.0f;
        if (valid) {
          const float xj = xs[j] + shift;
          const float dnw = side > 0 ? xj - xn : xn - xj;
          const float dol = side > 0 ? xj - xo : xo - xj;
          const float dn2 = dnw * dnw, do2 = dol * dol;
          tq = pair_e32(dn2, P) - pair_e32(do2, P);
          if (k == (chunk + 1) * (int)W && (dn2 <= P->rc2 || do2 <= P->rc2)) any_sat = 1;
        }
        tl = q == 0 ? tq : tl + tq;
      }
      v[gl] = tl;
    }
    de = de + butterfly32(v, G);
    *pairs += 4 * W;
    if (!any_sat) break;
    if (chunk == 0) R->window_overflows += 1;
    if (periodic && 2 * (chunk + 2) * (int)W > n - 1) {
      *err = JMM_ERR_INVALID;
      break;
    }
  }
  const int acc = (de <= 0.0f) || (de * P->beta < thr);
  if (!acc) return 0.0f;
  xs[nm] = xn;
  R->disp_acc += 1;
  return de;
}

static void run_chain(jmmo_batch *b, uint32_t c, uint64_t n_sweeps) {
  const jmm_batch_config *cfg = &b->cfg;
  const chain_prm Pv = make_prm(&b->chains[c], c);
  const chain_prm *P = &Pv;
  const int fp64 = b->fp64;
  const uint32_t G = b->g, W = b->cfg.window ? b->cfg.window : (G <= 8 ? 4 : G / 2);
  const int n = (int)P->n;
  float *xs = fp64 ? NULL : b->xf[c];
  double *xd = fp64 ? b->xd[c] : NULL;
  jmm_chain_result *R = &b->res[c];
  const int periodic = cfg->boundary == JMM_BOUNDARY_PERIODIC;
  const int npt = P->ensemble == JMM_NPT;
  const int per_sweep = cfg->vol_schedule == JMM_VOLSCHED_SWEEP;
  double L = R->l;
  float lf = (float)L, half_l = (float)(L * 0.5);
  seg_t g;
  memset(&g, 0, sizeof(g));
  g.e0 = R->e;
  const uint32_t spsw = P->spsw;
  uint32_t sweep_pos = (uint32_t)(R->steps % spsw);
  uint32_t sweeps_since_resum = 0;
  uint32_t err = R->error;
  uint64_t pairs = R->pair_evals;
  const uint64_t total = n_sweeps * (uint64_t)spsw;
  const uint64_t step0 = R->steps;

  for (uint64_t t = 0; t < total; ++t) {
    uint32_t w[4];
    jmmo_step_words(cfg->seed, step0 + t + 1, P->id, w);
    const uint32_t w0 = w[0];
    int vol = 0, nm;
    ++sweep_pos;
    if (npt && !per_sweep) {
      nm = (int)jmmo_word_to_index(w0, (uint64_t)n + 1);
      vol = nm == n;
    } else {
      nm = (int)jmmo_word_to_index(w0, (uint64_t)n);
      vol = npt && sweep_pos == spsw;
    }
    const int sweep_end = sweep_pos == spsw;
    if (sweep_end) sweep_pos = 0;

    if (!vol) {
      R->disp_att += 1;
      if (!fp64) {
        g.delta = g.delta + disp32(xs, n, nm, w, P, periodic, lf, half_l, G, W, &pairs, &err, R);
      } else {
        const double u1 = (double)(w[1] >> 8) * (1.0 / 16777216.0);
        const double thr = threshold64(w[2]);
        const double md = (u1 - 0.5) * P->two_max_step_d;
        const double xo = xd[nm], xn = xo + md;
        double left, right;
        if (periodic) {
          left = nm > 0 ? xd[nm - 1] : xd[n - 1] - L;
          right = nm + 1 < n ? xd[nm + 1] : xd[0] + L;
        } else {
          left = nm > 0 ? xd[nm - 1] : -INFINITY;
          right = nm + 1 < n ? xd[nm + 1] : INFINITY;
        }
        int ok = (xn > left) && (xn < right);
        if (!periodic) ok = ok && !(fabs(xn) > 0.5 * L);
        if (ok) {
          double de = 0.0;
          for (int side = -1; side <= 1; side += 2) {
            for (int k = 1; k < n; ++k) {
              int j = nm + side * k;
              double shift = 0.0;
              if (!periodic) {
                if (j < 0 || j >= n) break;
              } else {
                if (2 * k > n - 1) break;
                if (j < 0) {
                  j += n;
                  shift = -L;
                } else if (j >= n) {
                  j -= n;
                  shift = L;
                }
              }
              const double xj = xd[j] + shift;
              const double dnw = side > 0 ? xj - xn : xn - xj;
              const double dol = side > 0 ? xj - xo : xo - xj;
              const double dn2 = dnw * dnw, do2 = dol * dol;
              if (dn2 > P->rc2_d && do2 > P->rc2_d) break;
              de += pair_e64(dn2, P) - pair_e64(do2, P);
              pairs += 2;
            }
          }
          if (de <= 0.0 || de * P->beta_d < thr) {
            xd[nm] = xn;
            g.delta_d += de;
            R->disp_acc += 1;
          }
        }
      }
    } else {
      /* volume move */
      double lnew, logw, uo, un;
      if (!fp64) {
        const float u1 = (float)(w[1] >> 8) * (1.0f / 16777216.0f);
        const float v = 2.0f * u1 - 1.0f;
        float s;
        if (cfg->vol_move == JMM_VOLMOVE_LNL) {
          const float lns = P->vol_step * v;
          s = jmmo_expf(lns);
          lnew = L * (double)s;
          logw = (double)(n + 1) * (double)lns;
        } else {
          const double dl = (double)(P->vol_step * v);
          lnew = L + dl;
          const double ratio = lnew / L;
          s = (float)ratio;
          logw = lnew > 0.0 ? (double)n * log(ratio) : -INFINITY;
        }
        const float lnf = (float)lnew;
        energies32(xs, P, b->lanes, periodic, lf, 1, s, lnf, &uo, &un, &pairs, &err);
        const double drift = fabs((g.e0 + (double)g.delta) - uo);
        if (drift > R->max_drift) R->max_drift = drift;
        const double du = un - uo;
        const double arg = P->beta_d * (du + P->p * (lnew - L)) - logw;
        int acc = arg < (double)threshold32(w[2]);
        if (!(lnew > 0.0)) acc = 0;
        if (periodic && !(lnew > 2.0 * (double)P->rc)) acc = 0;
        fold(&g, R, L, (uint32_t)n, 0);
        R->vol_att += 1;
        if (acc) {
          for (int i = 0; i < n; ++i) xs[i] = xs[i] * s;
          L = lnew;
          lf = (float)L;
          half_l = (float)(L * 0.5);
          g.e0 = un;
          R->vol_acc += 1;
        } else {
          g.e0 = uo;
        }
      } else {
        const double u1 = (double)(w[1] >> 8) * (1.0 / 16777216.0);
        const double v = 2.0 * u1 - 1.0;
        double s;
        if (cfg->vol_move == JMM_VOLMOVE_LNL) {
          const double lns = P->vol_step_d * v;
          s = exp(lns);
          lnew = L * s;
          logw = (double)(n + 1) * lns;
        } else {
          lnew = L + P->vol_step_d * v;
          s = lnew / L;
          logw = lnew > 0.0 ? (double)n * log(s) : -INFINITY;
        }
        energies64(xd, P, periodic, L, s, lnew, &uo, &un, &pairs);
        const double drift = fabs((g.e0 + g.delta_d) - uo);
        if (drift > R->max_drift) R->max_drift = drift;
        const double arg = P->beta_d * ((un - uo) + P->p * (lnew - L)) - logw;
        int acc = arg < threshold64(w[2]);
        if (!(lnew > 0.0)) acc = 0;
        if (periodic && !(lnew > 2.0 * (double)P->rc)) acc = 0;
        fold(&g, R, L, (uint32_t)n, 1);
        R->vol_att += 1;
        if (acc) {
          for (int i = 0; i < n; ++i) xd[i] = xd[i] * s;
          L = lnew;
          g.e0 = un;
          R->vol_acc += 1;
        } else {
          g.e0 = uo;
        }
      }
    }
    /* per-step sample */
    if (!fp64) {
      g.sd = g.sd + g.delta;
      g.sd2 = fmaf(g.delta, g.delta, g.sd2);
    } else {
      g.sd_d += g.delta_d;
      g.sd2_d += g.delta_d * g.delta_d;
    }
    g.nseg += 1;
    if (sweep_end && !npt && cfg->resum_sweeps > 0 &&
        ++sweeps_since_resum >= cfg->resum_sweeps) {
      sweeps_since_resum = 0;
      double uo, un;
      if (!fp64) {
        energies32(xs, P, b->lanes, periodic, lf, 0, 1.0f, lf, &uo, &un, &pairs, &err);
        const double drift = fabs((g.e0 + (double)g.delta) - uo);
        if (drift > R->max_drift) R->max_drift = drift;
      } else {
        energies64(xd, P, periodic, L, 1.0, L, &uo, &un, &pairs);
        const double drift = fabs((g.e0 + g.delta_d) - uo);
        if (drift > R->max_drift) R->max_drift = drift;
      }
      fold(&g, R, L, (uint32_t)n, fp64);
      g.e0 = uo;
    }
  }
  fold(&g, R, L, (uint32_t)n, fp64);
  R->e = g.e0;
  R->l = L;
  R->steps = step0 + total;
  R->pair_evals = pairs;
  if (!isfinite(R->e)) err = JMM_ERR_NUMERIC;
  R->error = err;
}

/* ---- split chains (jmm_batch_config.split_n) -------------------------------
 * The GPU runs a long constant-L chain between walls as alternating domains:
 * per sweep, domains of B particles from a random offset, the domains of one
 * colour at once, then the other.  Domains of one phase share no pair, so
 * replaying them one after another in index order gives the GPU's result
 * bit for bit: each domain's steps are the EXACT kernel's displacement steps
 * on the chain's positions (G = 4 lanes, the split window), its Philox
 * blocks those of the chain's steps lo + 1 .. hi of the sweep, its energy
 * change an FP32 sum over its steps; the chain's FP64 energy takes the
 * domains' changes in index order and is sampled once per sweep. */
static uint32_t split_domain_size(uint32_t n) {
  const uint32_t b = 32u * ((n + 479u) / 480u);
  return b < 32u ? 32u : b;
}

static int is_split(const jmmo_batch *b, const jmm_chain_desc *c) {
  return !b->fp64 && b->cfg.split_n > 0 && c->n >= b->cfg.split_n && c->ensemble == JMM_NLT &&
         b->cfg.boundary == JMM_BOUNDARY_WALLS;
}

static void run_split32(jmmo_batch *b, uint32_t c, uint64_t n_sweeps) {
  const jmm_batch_config *cfg = &b->cfg;
  const chain_prm Pv = make_prm(&b->chains[c], c);
  const chain_prm *P = &Pv;
  const int n = (int)P->n;
  float *xs = b->xf[c];
  jmm_chain_result *R = &b->res[c];
  const uint32_t W0 = cfg->window ? cfg->window : (b->g <= 8 ? 4u : b->g / 2u);
  const uint32_t W = W0 > 8 ? 16u : (W0 > 4 ? 8u : 4u);
  const uint32_t B = split_domain_size((uint32_t)n);
  const double L = R->l;
  const float lf = (float)L, half_l = (float)(L * 0.5);
  const double rho = (double)n / L;
  uint64_t steps = R->steps, pairs = R->pair_evals;
  uint32_t err = R->error, since_resum = 0;
  double e = R->e;
  double *dde = (double *)calloc((size_t)n / B + 2, sizeof(double));
  for (uint64_t sw = 0; sw < n_sweeps; ++sw) {
    uint32_t lw[4];
    jmmo_step_words(cfg->seed, steps + 1, P->id, lw);
    const int off = (int)jmmo_word_to_index(lw[3], B);
    const uint32_t first = lw[3] & 1u;
    const int n_dom = (n - off + (int)B - 1) / (int)B + 1;
    for (int phase = 0; phase < 2; ++phase) {
      const int colour = (int)((first + (uint32_t)phase) & 1u);
      for (int d = colour; d < n_dom; d += 2) {
        const int lo = off + (d - 1) * (int)B < 0 ? 0 : off + (d - 1) * (int)B;
        const int hi = off + d * (int)B > n ? n : off + d * (int)B;
        dde[d] = 0.0;
        if (hi <= lo) continue;
        int fits = 1;
        if (lo >= 16) fits = fits && (xs[lo - 1] - xs[lo - 16]) > P->rc;
        if (hi + 16 <= n) fits = fits && (xs[hi + 15] - xs[hi]) > P->rc;
        if (!fits) {
          err |= JMM_ERR_INVALID;
          continue;
        }
        float delta = 0.0f;
        const int nd = hi - lo;
        for (int t = 0; t < nd; ++t) {
          uint32_t w[4];
          jmmo_step_words(cfg->seed, steps + (uint64_t)lo + (uint64_t)t + 1, P->id, w);
          const int nm = lo + (int)jmmo_word_to_index(w[0], (uint64_t)nd);
          R->disp_att += 1;
          delta = delta + disp32(xs, n, nm, w, P, 0, lf, half_l, 4, W, &pairs, &err, R);
        }
        dde[d] = (double)delta;
      }
    }
    for (int d = 0; d < n_dom; ++d) e = e + dde[d];
    R->sum_e = R->sum_e + e;
    R->sum_e2 = R->sum_e2 + e * e;
    R->sum_l = R->sum_l + L;
    R->sum_l2 = R->sum_l2 + L * L;
    R->sum_le = R->sum_le + L * e;
    R->sum_rho = R->sum_rho + rho;
    R->sum_rho2 = R->sum_rho2 + rho * rho;
    R->samples += 1;
    steps += (uint64_t)n;
    if (cfg->resum_sweeps > 0 && ++since_resum >= cfg->resum_sweeps) {
      since_resum = 0;
      double uo, un;
      energies32(xs, P, 32, 0, lf, 0, 1.0f, lf, &uo, &un, &pairs, &err);
      const double drift = fabs(e - uo);
      if (drift > R->max_drift) R->max_drift = drift;
      e = uo;
    }
  }
  free(dde);
  R->e = e;
  R->steps = steps;
  R->pair_evals = pairs;
  if (!isfinite(e)) err |= JMM_ERR_NUMERIC;
  R->error = err;
}

static void run_any(jmmo_batch *b, uint32_t c, uint64_t n_sweeps) {
  if (is_split(b, &b->chains[c]))
    run_split32(b, c, n_sweeps);
  else
    run_chain(b, c, n_sweeps);
}

/* ---- API ------------------------------------------------------------------- */

static double chain_energy(jmmo_batch *b, uint32_t c) {
  const chain_prm P = make_prm(&b->chains[c], c);
  const int periodic = b->cfg.boundary == JMM_BOUNDARY_PERIODIC;
  double uo, un;
  uint64_t pairs = 0;
  uint32_t err = 0;
  const double L = b->res[c].l;
  if (b->fp64) {
    energies64(b->xd[c], &P, periodic, L, 1.0, L, &uo, &un, &pairs);
  } else {
    const float lf = (float)L;
    energies32(b->xf[c], &P, 32, periodic, lf, 0, 1.0f, lf, &uo, &un, &pairs, &err);
    if (err) uo = NAN;
  }
  return uo;
}

jmmo_batch *jmmo_batch_create(const jmm_batch_config *cfg, const jmm_chain_desc *chains,
                              uint32_t n_chains, int fp64) {
  if (!cfg || !chains || n_chains == 0) return NULL;
  jmmo_batch *b = (jmmo_batch *)calloc(1, sizeof(jmmo_batch));
  b->cfg = *cfg;
  b->n_chains = n_chains;
  b->fp64 = fp64;
  b->g = cfg->lanes_per_chain ? cfg->lanes_per_chain : 4;
  b->lanes = b->g * (cfg->steps_per_round ? cfg->steps_per_round : 32 / b->g);
  b->chains = (jmm_chain_desc *)malloc(n_chains * sizeof(jmm_chain_desc));
  memcpy(b->chains, chains, n_chains * sizeof(jmm_chain_desc));
  b->res = (jmm_chain_result *)calloc(n_chains, sizeof(jmm_chain_result));
  b->xf = (float **)calloc(n_chains, sizeof(float *));
  b->xd = (double **)calloc(n_chains, sizeof(double *));
  for (uint32_t c = 0; c < n_chains; ++c) {
    const jmm_chain_desc *d = &chains[c];
    b->xf[c] = (float *)malloc(d->n * sizeof(float));
    b->xd[c] = (double *)malloc(d->n * sizeof(double));
    for (uint32_t i = 0; i < d->n; ++i) {
      double r = ((i + 0.5) / d->n - 0.5) * d->l0;
      if (cfg->init == JMM_INIT_JITTER) {
        uint32_t w[4];
        jmmo_step_words(cfg->seed, (1ull << 63) | i, c, w);
        r += cfg->jitter * (2.0 * jmmo_word_to_unit(w[0]) - 1.0);
      }
      b->xf[c][i] = (float)r;
      b->xd[c][i] = fp64 ? r : (double)(float)r;
    }
    b->res[c].l = d->l0;
  }
  for (uint32_t c = 0; c < n_chains; ++c) b->res[c].e = chain_energy(b, c);
  return b;
}

void jmmo_batch_destroy(jmmo_batch *b) {
  if (!b) return;
  for (uint32_t c = 0; c < b->n_chains; ++c) {
    free(b->xf[c]);
    free(b->xd[c]);
  }
  free(b->xf);
  free(b->xd);
  free(b->res);
  free(b->chains);
  free(b);
}

int jmmo_batch_run(jmmo_batch *b, uint64_t n_sweeps) {
  for (uint32_t c = 0; c < b->n_chains; ++c) run_any(b, c, n_sweeps);
  return JMM_OK;
}

int jmmo_batch_run_chain(jmmo_batch *b, uint32_t chain, uint64_t n_sweeps) {
  if (chain >= b->n_chains) return JMM_ERR_INVALID;
  run_any(b, chain, n_sweeps);
  return JMM_OK;
}

int jmmo_batch_results(jmmo_batch *b, jmm_chain_result *out, uint32_t n_chains) {
  if (n_chains != b->n_chains) return JMM_ERR_INVALID;
  memcpy(out, b->res, n_chains * sizeof(jmm_chain_result));
  return JMM_OK;
}

int jmmo_batch_get_positions(jmmo_batch *b, uint32_t chain, double *x, uint32_t n) {
  if (chain >= b->n_chains || n != b->chains[chain].n) return JMM_ERR_INVALID;
  for (uint32_t i = 0; i < n; ++i) x[i] = b->fp64 ? b->xd[chain][i] : (double)b->xf[chain][i];
  return JMM_OK;
}

int jmmo_batch_set_positions(jmmo_batch *b, uint32_t chain, const double *x, uint32_t n,
                             double l) {
  if (chain >= b->n_chains || n != b->chains[chain].n) return JMM_ERR_INVALID;
  for (uint32_t i = 0; i < n; ++i) {
    b->xf[chain][i] = (float)x[i];
    b->xd[chain][i] = b->fp64 ? x[i] : (double)(float)x[i];
  }
  b->res[chain].l = l;
  b->res[chain].e = chain_energy(b, chain);
  return JMM_OK;
}

int jmmo_batch_energies(jmmo_batch *b, double *e, uint32_t n_chains) {
  if (n_chains != b->n_chains) return JMM_ERR_INVALID;
  for (uint32_t c = 0; c < n_chains; ++c) e[c] = chain_energy(b, c);
  return JMM_OK;
}

/* FP64 energy of arbitrary positions of one chain description (any mode). */
double jmmo_energy64(const jmm_chain_desc *c, const double *x, double l, int periodic) {
  chain_prm P = make_prm(c, 0);
  double uo, un;
  uint64_t pairs = 0;
  energies64(x, &P, periodic, l, 1.0, l, &uo, &un, &pairs);
  return uo;
}

float jmmo_portable_logf(float x) { return jmmo_logf(x); }
float jmmo_portable_expf(float x) { return jmmo_expf(x); }

/* U, dU/deps, dU/dsigma, dU/dL (positions scaled with the box) of one
 * configuration in FP64: the reference for the gradient kernel. */
void jmmo_energy_grad64(const jmm_chain_desc *c, const double *x, double l, int periodic,
                        double out[4]) {
  const int n = (int)c->n;
  const double eps = c->eps, sig = c->sigma, rc2 = c->cutoff * c->cutoff;
  double u = 0, ge = 0, gs = 0, rd = 0;
  for (int i = 0; i < n; ++i) {
    for (int k = 1;; ++k) {
      int j = i + k;
      double shift = 0;
      if (!periodic) {
        if (j >= n) break;
      } else {
        if (2 * k > n - 1) break;
        if (j >= n) {
          j -= n;
          shift = l;
        }
      }
      const double d = x[j] + shift - x[i];
      const double r2 = d * d;
      if (r2 > rc2) break;
      double e, g_eps, r_dphi, g_sig;
      if (c->potential == JMM_POT_GAUSS) {
        const double a = r2 / (sig * sig);
        const double ex = exp(-a);
        g_eps = ex;
        e = eps * ex;
        r_dphi = -2.0 * e * a;
        g_sig = 2.0 * e * a / sig;
      } else {
        const double inv2 = sig * sig / r2;
        const double inv6 = inv2 * inv2 * inv2;
        const double inv12 = inv6 * inv6;
        if (c->potential == JMM_POT_SOFTSPHERE) {
          g_eps = inv12;
          e = eps * inv12;
          r_dphi = -12.0 * e;
        } else {
          g_eps = 4.0 * (inv12 - inv6);
          e = eps * g_eps;
          r_dphi = -24.0 * eps * (2.0 * inv12 - inv6);
        }
        g_sig = -r_dphi / sig;
      }
      u += e;
      ge += g_eps;
      gs += g_sig;
      rd += r_dphi;
    }
  }
  out[0] = u;
  out[1] = ge;
  out[2] = gs;
  out[3] = rd / l;
}

/* One histogram sample of one chain (the batched form's
 * jmm_batch_sample_histograms): row[0] += 1; position bins
 * floor(x / rbw + rhonb/2) and slice bins floor(x / gsw + gns/2) in FP32;
 * pairs to the right of each particle (on a ring through the wrap, at most
 * half way round) until the FP32 separation reaches gnb * gbw, bin
 * floor(d / gbw), counted in the slice of both particles.  The layout and
 * bin rules are those of the reference's printRho / printG and fgrho
 * (src/jmmMCState.cpp:1021-1061, :1069-1127). */
static int hist_bin32(float x, float w, uint32_t nb) {
  const float f = floorf(x / w + 0.5f * (float)nb);
  return (f >= 0.0f && f < (float)nb) ? (int)f : -1;
}

void jmmo_batch_hist_sample(const float *x, uint32_t n, float l, int periodic, uint32_t rhonb,
                            float rbw, uint32_t gns, float gsw, uint32_t gnb, float gbw,
                            uint64_t *row) {
  uint64_t *g = row + 1 + rhonb;
  const float range = (float)gnb * gbw;
  row[0] += 1;
  for (uint32_t i = 0; i < n; ++i) {
    const float xi = x[i];
    const int rb = hist_bin32(xi, rbw, rhonb);
    if (rb >= 0) row[1 + rb] += 1;
    const int si = hist_bin32(xi, gsw, gns);
    for (uint32_t k = 1; k < n; ++k) {
      if (periodic && 2 * k > n) break;
      uint32_t j = i + k;
      float shift = 0.0f;
      if (j >= n) {
        if (!periodic) break;
        j -= n;
        shift = l;
      }
      const float xj = x[j];
      const float d = (xj + shift) - xi;
      if (!(d < range)) break;
      const float gf = floorf(d / gbw);
      if (!(gf < (float)gnb)) continue;
      const int gb = (int)gf;
      if (si >= 0) g[(uint64_t)si * gnb + gb] += 1;
      const int sj = hist_bin32(xj, gsw, gns);
      if (sj >= 0) g[(uint64_t)sj * gnb + gb] += 1;
    }
  }
}
