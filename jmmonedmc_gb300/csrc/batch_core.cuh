// batch_core.cuh -- device code of the batched chain kernel.
//
// One chain is the reference's sequential single-particle Metropolis chain
// (Step/qad2/fav, src/jmmMCState.cpp:1758-1811, :1160-1464, :2161-2293),
// re-cast for many chains per GPU:
//  * a group of G lanes owns one chain; lane g looks at neighbour
//    side(g)*k(g) of the moved particle, side = -1 for g < W = G/2, k =
//    g % W + 1, and evaluates that pair at the old and the trial position;
//  * positions are FP32 in shared memory and stay ordered along the line,
//    so the partners within the cut-off are index neighbours; when the
//    W-th neighbour on a side is still within the cut-off the window is
//    extended in further chunks of W;
//  * the energy change is the group's butterfly sum (xor 1, 2, 4, ...);
//  * Philox words of 32 steps are drawn ahead, one step per lane, and
//    handed out with shuffles;
//  * the running energy is an FP64 base plus an FP32 offset that is folded
//    into FP64 at every volume move, re-summation and launch end, together
//    with the per-step accumulators (sum E, E^2, L, L^2, LE, rho, rho^2).
// Every FP32/FP64 operation is an explicit round-to-nearest intrinsic so
// that the EXACT precision mode can be replayed bit for bit by the oracle;
// the FAST mode differs only in using the hardware reciprocal and exp.
#pragma once
#include <math.h>
#include <stdint.h>

#include "../../include/jmm_gpu.h"
#include "fp32math.cuh"
#include "philox.cuh"

namespace jmm {
namespace batch {

struct ChainParams {
  uint32_t id;               // user index: Philox stream and result slot
  uint32_t n;
  uint32_t pot;
  uint32_t ensemble;
  uint32_t steps_per_sweep;  // n, or n+1 with volume moves
  uint32_t s_off;            // float offset of the chain in its block's shared memory
  uint64_t x_off;            // float offset of the chain's positions in HBM
  float eps4;                // LJ: 4 eps; soft sphere and Gaussian: eps
  float sigma2;
  float inv_sigma2;
  float rc2;
  float beta;                // 1/T
  float two_max_step;
  float vol_step;
  float rc;
  double beta_d, p;
};

struct KernelCfg {
  uint64_t seed;
  uint64_t n_sweeps;
  int32_t boundary, vol_move, vol_schedule, resum_sweeps;
  uint32_t n_chains;
  uint32_t chains_per_block;
};

template <bool kExact>
__device__ __forceinline__ float rcp32(float x) {
  if (kExact) return __frcp_rn(x);
  float y;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

template <bool kExact>
__device__ __forceinline__ float exp32(float x) {
  if (kExact) return portable_expf(x);
  return __expf(x);
}

// Pair energy from the squared separation; 0 beyond the cut-off.
template <bool kExact>
__device__ __forceinline__ float pair_energy(float d2, const ChainParams &P) {
  if (!(d2 <= P.rc2)) return 0.0f;
  if (P.pot == JMM_POT_GAUSS)
    return __fmul_rn(P.eps4, exp32<kExact>(-__fmul_rn(d2, P.inv_sigma2)));
  const float inv2 = __fmul_rn(P.sigma2, rcp32<kExact>(d2));
  const float inv6 = __fmul_rn(__fmul_rn(inv2, inv2), inv2);
  if (P.pot == JMM_POT_SOFTSPHERE) return __fmul_rn(P.eps4, __fmul_rn(inv6, inv6));
  return __fmul_rn(P.eps4, __fmul_rn(inv6, __fsub_rn(inv6, 1.0f)));  // LJ 12-6
}

template <int G>
__device__ __forceinline__ float group_sum(float v, unsigned mask) {
#pragma unroll
  for (int m = 1; m < G; m <<= 1) v = __fadd_rn(v, __shfl_xor_sync(mask, v, m, G));
  return v;
}

template <int G>
__device__ __forceinline__ double group_sum_d(double v, unsigned mask) {
#pragma unroll
  for (int m = 1; m < G; m <<= 1) v = __dadd_rn(v, __shfl_xor_sync(mask, v, m, G));
  return v;
}

// Total pair energy of the chain at positions xs (U_old) and at positions
// scaled by s with box length lnew (U_new): lane g takes particles g, g+G, ...
// and their right-hand neighbours in order until both separations exceed the
// cut-off; per-particle sums are FP32, the lane and group sums FP64.
template <int G, bool kExact, bool kScaled>
__device__ void group_energies(const float *xs, const ChainParams &P, int gl, unsigned gmask,
                               bool periodic, float lf, float s, float lnf, double &u_old,
                               double &u_new, uint64_t &pairs, uint32_t &err) {
  const int n = (int)P.n;
  double uo = 0.0, un = 0.0;
  uint32_t cnt = 0;
  for (int i = gl; i < n; i += G) {
    const float xi = xs[i];
    const float xin = kScaled ? __fmul_rn(xi, s) : xi;
    float eo = 0.0f, en = 0.0f;
    for (int k = 1;; ++k) {
      int j = i + k;
      float shift = 0.0f, shiftn = 0.0f;
      if (!periodic) {
        if (j >= n) break;
      } else {
        if (2 * k > n - 1) {  // the window reached half the ring: images would overlap
          err = JMM_ERR_INVALID;
          break;
        }
        if (j >= n) {
          j -= n;
          shift = lf;
          shiftn = lnf;
        }
      }
      const float xj = xs[j];
      const float d = __fsub_rn(__fadd_rn(xj, shift), xi);
      const float d2 = __fmul_rn(d, d);
      float dn2 = d2;
      if (kScaled) {
        const float dn = __fsub_rn(__fadd_rn(__fmul_rn(xj, s), shiftn), xin);
        dn2 = __fmul_rn(dn, dn);
      }
      if (d2 > P.rc2 && dn2 > P.rc2) break;
      eo = __fadd_rn(eo, pair_energy<kExact>(d2, P));
      if (kScaled) en = __fadd_rn(en, pair_energy<kExact>(dn2, P));
      cnt += kScaled ? 2 : 1;
    }
    uo = __dadd_rn(uo, (double)eo);
    if (kScaled) un = __dadd_rn(un, (double)en);
  }
  u_old = group_sum_d<G>(uo, gmask);
  u_new = kScaled ? group_sum_d<G>(un, gmask) : u_old;
  pairs += __reduce_add_sync(gmask, cnt);
}

// Running statistics of one chain between folds.
struct Seg {
  double e0;       // FP64 energy at the start of the segment
  float delta;     // FP32 energy change since then
  float sd, sd2;   // sums of delta and delta^2 over the segment's steps
  uint32_t nseg;   // steps sampled in the segment
};

__device__ __forceinline__ void fold(Seg &g, jmm_chain_result &R, double l, uint32_t n) {
  const double nd = (double)g.nseg;
  const double sdd = (double)g.sd, sd2d = (double)g.sd2;
  const double lin = __dadd_rn(__dmul_rn(nd, g.e0), sdd);
  R.sum_e = __dadd_rn(R.sum_e, lin);
  R.sum_e2 = __dadd_rn(R.sum_e2, __dadd_rn(__dadd_rn(__dmul_rn(__dmul_rn(nd, g.e0), g.e0),
                                                     __dmul_rn(__dmul_rn(2.0, g.e0), sdd)),
                                           sd2d));
  R.sum_l = __dadd_rn(R.sum_l, __dmul_rn(nd, l));
  R.sum_l2 = __dadd_rn(R.sum_l2, __dmul_rn(__dmul_rn(nd, l), l));
  R.sum_le = __dadd_rn(R.sum_le, __dmul_rn(l, lin));
  const double rho = __ddiv_rn((double)n, l);
  R.sum_rho = __dadd_rn(R.sum_rho, __dmul_rn(nd, rho));
  R.sum_rho2 = __dadd_rn(R.sum_rho2, __dmul_rn(__dmul_rn(nd, rho), rho));
  R.samples += g.nseg;
  g.e0 = __dadd_rn(g.e0, (double)g.delta);
  g.delta = 0.0f;
  g.sd = 0.0f;
  g.sd2 = 0.0f;
  g.nseg = 0;
}

// The Metropolis threshold -ln u, u the midpoint of the 23-bit cell of w
// (exact in FP32, strictly inside (0, 1)).
__device__ __forceinline__ float threshold_of(uint32_t w) {
  const float u = __fmul_rn(__fadd_rn((float)(w >> 9), 0.5f), 1.1920929e-07f);  // 2^-23
  return -portable_logf(u);
}

template <int G, bool kExact>
__global__ void __launch_bounds__(256) chains_kernel(const ChainParams *__restrict__ prm,
                                                     jmm_chain_result *__restrict__ res,
                                                     float *__restrict__ xg, KernelCfg cfg) {
  constexpr int W = G / 2;
  constexpr int KS = 32 / G;  // steps each lane draws ahead per batch of 32
  extern __shared__ float smem[];
  const int gl = threadIdx.x % G;
  const int gw = (threadIdx.x & 31) / G;
  const unsigned gmask = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << (gw * G));
  const uint32_t slot = blockIdx.x * cfg.chains_per_block + threadIdx.x / G;
  if (slot >= cfg.n_chains) return;
  const ChainParams P = prm[slot];
  const int n = (int)P.n;
  float *xs = smem + P.s_off;
  for (int i = gl; i < n; i += G) xs[i] = xg[P.x_off + i];
  __syncwarp(gmask);

  jmm_chain_result R = res[P.id];
  const bool periodic = cfg.boundary == JMM_BOUNDARY_PERIODIC;
  const bool npt = P.ensemble == JMM_NPT;
  const bool per_sweep = cfg.vol_schedule == JMM_VOLSCHED_SWEEP;
  double L = R.l;
  float lf = (float)L, half_l = (float)__dmul_rn(L, 0.5);
  Seg g;
  g.e0 = R.e;
  g.delta = 0.0f;
  g.sd = 0.0f;
  g.sd2 = 0.0f;
  g.nseg = 0;
  const uint32_t spsw = P.steps_per_sweep;
  uint32_t sweep_pos = (uint32_t)(R.steps % spsw);
  uint32_t sweeps_since_resum = 0;
  uint32_t err = R.error;
  uint64_t pairs = R.pair_evals;
  const int side = gl < W ? -1 : 1;
  const int kk = gl % W + 1;
  const uint64_t total = cfg.n_sweeps * (uint64_t)spsw;
  const uint64_t step0 = R.steps;

  for (uint64_t t = 0; t < total; t += 32) {
    uint32_t r_w0[KS];
    float r_u1[KS], r_thr[KS];
#pragma unroll
    for (int k = 0; k < KS; ++k) {
      const uint64_t s = step0 + t + (uint64_t)(gl + G * k) + 1;
      const Words4 w = step_words(cfg.seed, s, P.id);
      r_w0[k] = w.w[0];
      r_u1[k] = word_to_unit_f(w.w[1]);
      r_thr[k] = threshold_of(w.w[2]);
    }
#pragma unroll
    for (int k = 0; k < KS; ++k) {
      for (int src = 0; src < G; ++src) {
        if (t + (uint64_t)(k * G + src) >= total) break;
        const uint32_t w0 = __shfl_sync(gmask, r_w0[k], src, G);
        const float u1 = __shfl_sync(gmask, r_u1[k], src, G);
        const float thr = __shfl_sync(gmask, r_thr[k], src, G);
        bool vol = false;
        int nm;
        ++sweep_pos;
        if (npt && !per_sweep) {
          nm = (int)word_to_index(w0, (uint64_t)n + 1);
          vol = nm == n;
        } else {
          nm = (int)word_to_index(w0, (uint64_t)n);
          vol = npt && sweep_pos == spsw;
        }
        const bool sweep_end = sweep_pos == spsw;
        if (sweep_end) sweep_pos = 0;

        if (!vol) {
          // ---- displacement (qad2) ----
          const float md = __fmul_rn(__fsub_rn(u1, 0.5f), P.two_max_step);
          const float xo = xs[nm];
          const float xn = __fadd_rn(xo, md);
          float left, right;
          if (periodic) {
            left = nm > 0 ? xs[nm - 1] : __fsub_rn(xs[n - 1], lf);
            right = nm + 1 < n ? xs[nm + 1] : __fadd_rn(xs[0], lf);
          } else {
            left = nm > 0 ? xs[nm - 1] : -INFINITY;
            right = nm + 1 < n ? xs[nm + 1] : INFINITY;
          }
          bool ok = (xn > left) && (xn < right);
          if (!periodic) ok = ok && !(fabsf(xn) > half_l);
          R.disp_att += 1;
          if (ok) {
            float de = 0.0f;
            for (int chunk = 0;; ++chunk) {
              const int k = chunk * W + kk;
              int j = nm + side * k;
              bool valid = true;
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
              float t_pair = 0.0f;
              bool sat = false;
              if (valid) {
                const float xj = __fadd_rn(xs[j], shift);
                const float dnw = side > 0 ? __fsub_rn(xj, xn) : __fsub_rn(xn, xj);
                const float dol = side > 0 ? __fsub_rn(xj, xo) : __fsub_rn(xo, xj);
                const float dn2 = __fmul_rn(dnw, dnw), do2 = __fmul_rn(dol, dol);
                t_pair = __fsub_rn(pair_energy<kExact>(dn2, P), pair_energy<kExact>(do2, P));
                sat = (k == (chunk + 1) * W) && (dn2 <= P.rc2 || do2 <= P.rc2);
              }
              de = __fadd_rn(de, group_sum<G>(t_pair, gmask));
              pairs += 2 * G;
              if (!__any_sync(gmask, sat)) break;
              if (chunk == 0) R.window_overflows += 1;
              if (periodic && 2 * (chunk + 2) * W > n - 1) {
                err = JMM_ERR_INVALID;
                break;
              }
            }
            const bool acc = (de <= 0.0f) || (__fmul_rn(de, P.beta) < thr);
            if (acc) {
              if (gl == 0) xs[nm] = xn;
              g.delta = __fadd_rn(g.delta, de);
              R.disp_acc += 1;
            }
            __syncwarp(gmask);
          }
        } else {
          // ---- volume move (fav), ln L or linear ----
          double lnew;
          float s;
          double logw;  // weight term: (N+1) ln s or N ln(L'/L)
          const float v = __fsub_rn(__fmul_rn(2.0f, u1), 1.0f);
          if (cfg.vol_move == JMM_VOLMOVE_LNL) {
            const float lns = __fmul_rn(P.vol_step, v);
            s = portable_expf(lns);
            lnew = __dmul_rn(L, (double)s);
            logw = __dmul_rn((double)(n + 1), (double)lns);
          } else {
            const double dl = (double)__fmul_rn(P.vol_step, v);
            lnew = __dadd_rn(L, dl);
            const double ratio = __ddiv_rn(lnew, L);
            s = (float)ratio;
            logw = lnew > 0.0 ? __dmul_rn((double)n, log(ratio)) : -INFINITY;
          }
          double uo, un;
          const float lnf = (float)lnew;
          group_energies<G, kExact, true>(xs, P, gl, gmask, periodic, lf, s, lnf, uo, un, pairs,
                                          err);
          const double drift = fabs(__dsub_rn(__dadd_rn(g.e0, (double)g.delta), uo));
          if (drift > R.max_drift) R.max_drift = drift;
          const double du = __dsub_rn(un, uo);
          const double arg = __dsub_rn(
              __dmul_rn(P.beta_d, __dadd_rn(du, __dmul_rn(P.p, __dsub_rn(lnew, L)))), logw);
          bool acc = arg < (double)thr;
          if (!(lnew > 0.0)) acc = false;
          if (periodic && !(lnew > 2.0 * (double)P.rc)) acc = false;
          fold(g, R, L, (uint32_t)n);
          R.vol_att += 1;
          if (acc) {
            for (int i = gl; i < n; i += G) xs[i] = __fmul_rn(xs[i], s);
            L = lnew;
            lf = (float)L;
            half_l = (float)__dmul_rn(L, 0.5);
            g.e0 = un;
            R.vol_acc += 1;
          } else {
            g.e0 = uo;
          }
          __syncwarp(gmask);
        }
        // ---- per-step sample (updateThermo) ----
        g.sd = __fadd_rn(g.sd, g.delta);
        g.sd2 = __fmaf_rn(g.delta, g.delta, g.sd2);
        g.nseg += 1;
        // ---- FP64 re-summation of constant-L chains ----
        if (sweep_end && !npt && cfg.resum_sweeps > 0 &&
            ++sweeps_since_resum >= (uint32_t)cfg.resum_sweeps) {
          sweeps_since_resum = 0;
          double uo, un;
          group_energies<G, kExact, false>(xs, P, gl, gmask, periodic, lf, 1.0f, lf, uo, un,
                                           pairs, err);
          const double drift = fabs(__dsub_rn(__dadd_rn(g.e0, (double)g.delta), uo));
          if (drift > R.max_drift) R.max_drift = drift;
          fold(g, R, L, (uint32_t)n);
          g.e0 = uo;
        }
      }
    }
  }
  fold(g, R, L, (uint32_t)n);
  R.e = g.e0;
  R.l = L;
  R.steps = step0 + total;
  R.pair_evals = pairs;
  if (!isfinite(R.e)) err = JMM_ERR_NUMERIC;
  R.error = err;
  __syncwarp(gmask);
  for (int i = gl; i < n; i += G) xg[P.x_off + i] = xs[i];
  if (gl == 0) res[P.id] = R;
}

// Fresh FP64 energies of every chain (32 lanes per chain).
template <bool kExact>
__global__ void energies_kernel(const ChainParams *__restrict__ prm, const float *__restrict__ xg,
                                const jmm_chain_result *__restrict__ res, double *__restrict__ e_out,
                                uint32_t n_chains, int32_t boundary) {
  const uint32_t c = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
  if (c >= n_chains) return;
  const ChainParams P = prm[c];
  const float *x = xg + P.x_off;
  const float lf = (float)res[P.id].l;
  double uo, un;
  uint64_t pairs = 0;
  uint32_t err = 0;
  group_energies<32, kExact, false>(x, P, threadIdx.x & 31, 0xffffffffu,
                                    boundary == JMM_BOUNDARY_PERIODIC, lf, 1.0f, lf, uo, un,
                                    pairs, err);
  if ((threadIdx.x & 31) == 0) e_out[P.id] = err ? (double)NAN : uo;
}

}  // namespace batch
}  // namespace jmm
