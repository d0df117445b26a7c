// batch_core.cuh -- device code of the batched chain kernel.
//
// One chain is the reference's sequential single-particle Metropolis chain
// (Step/qad2/fav, src/jmmMCState.cpp:1758-1811, :1160-1464, :2161-2293),
// re-cast for many chains per GPU.  A chain owns L = G*S lanes (16 or 32):
//
//  * Window.  Particles stay ordered along the line, so the partners within
//    the cut-off of the moved particle are index neighbours.  G lanes
//    evaluate one trial move against W neighbours per side: lane w takes
//    side -1 for w < G/2, +1 otherwise, and the offsets k = w % (G/2) + 1,
//    k + G/2, ... up to W, at the old and the trial position; the energy
//    change is the butterfly sum (xor 1, 2, 4, ...) of the G lanes.  When
//    the W-th neighbour on a side is still within the cut-off the window is
//    extended in chunks of W (a rare slow path).
//  * Speculative rounds.  The S lane segments of a chain evaluate the next S
//    steps of the chain at once, all from the current positions.  Step s of
//    the round is kept if no earlier kept step of the round was accepted
//    within W index positions of it (its window would have seen the moved
//    particle) — with walls, only if the two particles are neighbours or
//    their old-to-trial spans come within the cut-off; the first step that
//    fails is re-evaluated at the start of the next round.  Kept steps are
//    committed in order, so every step's outcome, the running energy and the
//    statistics are those of the sequential chain, operation for operation.
//  * Philox words of 32 steps ahead are drawn by the chain's lanes into a
//    small shared buffer.
//  * The running energy is an FP64 base plus an FP32 offset, folded into
//    FP64 at every volume move, re-summation and launch end together with
//    the per-step accumulators (sum E, E^2, L, L^2, LE, rho, rho^2).
// Every FP32/FP64 operation is an explicit round-to-nearest intrinsic so
// that the EXACT precision mode can be replayed bit for bit by the oracle;
// the FAST mode differs in using the hardware reciprocal, exp and log, in
// scaling a window's summed pair shapes by the potential's strength once, in
// forming a volume move's U_new - U_old from per-pair differences (FP32 in
// a lane, FP64 across lanes), and in summing a round's per-step statistics by a scan over
// its slots into per-lane shares instead of step by step (the same
// quantities, rounded in another order).
#pragma once
#include <math.h>
#include <stddef.h>
#include <stdint.h>

#include "../../include/jmm_gpu.h"
#include "fp32math.cuh"
#include "philox.cuh"

namespace jmm {
namespace batch {

constexpr int kRingSteps = 32;  // Philox words drawn ahead per chain
// One 16-byte record per step (particle index, displacement or volume
// uniform, Metropolis threshold, unused), read with one shared-memory load.
constexpr int kRingWords = 4 * kRingSteps;
// Ghost slots on each side of a chain's positions in shared memory: far
// sentinels between hard walls, periodic images on a ring, so that the
// neighbour window is read without bounds tests.
constexpr int kGhost = 16;
constexpr float kFar = 1e30f;

struct ChainParams {
  uint32_t id;               // user index: Philox stream and result slot
  uint32_t n;
  uint32_t pot;
  uint32_t ensemble;
  uint32_t steps_per_sweep;  // n, or n+1 with volume moves
  uint32_t s_off;            // float offset of the chain's positions in block shared memory
  uint64_t x_off;            // float offset of the chain's positions in HBM
  float eps4;                // LJ: 4 eps; soft sphere and Gaussian: eps
  float sigma2;
  float inv_sigma2;
  float rc2;
  float beta;                // 1/T
  float two_max_step;
  float vol_step;
  float rc;
  float grid;                // domain sweeps: position grid step 2^-k, displacements
                             // snapped to it; 0 (unused) for whole chains
  uint32_t dom;              // split chains: domain size B; 0 for whole chains
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

// Pair energy from the squared separation; 0 beyond the cut-off (a select,
// not a branch).  Runtime potential, for the rarely executed paths.
template <bool kExact>
__device__ __forceinline__ float pair_energy(float d2, const ChainParams &P) {
  float e;
  if (P.pot == JMM_POT_GAUSS) {
    e = __fmul_rn(P.eps4, exp32<kExact>(-__fmul_rn(d2, P.inv_sigma2)));
  } else {
    const float inv2 = __fmul_rn(P.sigma2, rcp32<kExact>(d2));
    const float inv6 = __fmul_rn(__fmul_rn(inv2, inv2), inv2);
    e = (P.pot == JMM_POT_SOFTSPHERE) ? __fmul_rn(P.eps4, __fmul_rn(inv6, inv6))
                                      : __fmul_rn(P.eps4, __fmul_rn(inv6, __fsub_rn(inv6, 1.0f)));
  }
  return d2 <= P.rc2 ? e : 0.0f;
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
// scaled by s with box length lnew (U_new): lane g of the chain's L lanes
// takes particles g, g+L, ... and their right-hand neighbours in order until
// both separations exceed the cut-off; per-particle sums are FP32, the lane
// and chain sums FP64.
template <int L, bool kExact, bool kScaled>
__device__ void group_energies(const float *xs, const ChainParams &P, int gl, unsigned gmask,
                               bool periodic, float lf, float s, float lnf, double &u_old,
                               double &u_new, uint64_t &pairs, uint32_t &err) {
  const int n = (int)P.n;
  double uo = 0.0, un = 0.0;
  uint32_t cnt = 0;
  for (int i = gl; i < n; i += L) {
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
  u_old = group_sum_d<L>(uo, gmask);
  u_new = kScaled ? group_sum_d<L>(un, gmask) : u_old;
  pairs += __reduce_add_sync(gmask, cnt);
}

// Running statistics of one chain between folds.
struct Seg {
  double e0;       // FP64 energy at the start of the segment
  float delta;     // FP32 energy change since then
  float sd, sd2;   // sums of delta and delta^2 over the segment's steps
  uint32_t nseg;   // steps sampled in the segment
};

// Folds the segment into the chain's FP64 sums at box length l and density
// rho = n / l; the record lives in HBM and only the chain's first lane
// (`writer`) updates it.
__device__ __forceinline__ void fold(Seg &g, jmm_chain_result *__restrict__ rp, bool writer,
                                     double l, double rho) {
  if (writer) {
    const double nd = (double)g.nseg;
    const double sdd = (double)g.sd, sd2d = (double)g.sd2;
    const double lin = __dadd_rn(__dmul_rn(nd, g.e0), sdd);
    rp->sum_e = __dadd_rn(rp->sum_e, lin);
    rp->sum_e2 = __dadd_rn(rp->sum_e2,
                           __dadd_rn(__dadd_rn(__dmul_rn(__dmul_rn(nd, g.e0), g.e0),
                                               __dmul_rn(__dmul_rn(2.0, g.e0), sdd)),
                                     sd2d));
    rp->sum_l = __dadd_rn(rp->sum_l, __dmul_rn(nd, l));
    rp->sum_l2 = __dadd_rn(rp->sum_l2, __dmul_rn(__dmul_rn(nd, l), l));
    rp->sum_le = __dadd_rn(rp->sum_le, __dmul_rn(l, lin));
    rp->sum_rho = __dadd_rn(rp->sum_rho, __dmul_rn(nd, rho));
    rp->sum_rho2 = __dadd_rn(rp->sum_rho2, __dmul_rn(__dmul_rn(nd, rho), rho));
    rp->samples += g.nseg;
  }
  g.e0 = __dadd_rn(g.e0, (double)g.delta);
  g.delta = 0.0f;
  g.sd = 0.0f;
  g.sd2 = 0.0f;
  g.nseg = 0;
}

static_assert(offsetof(jmm_chain_result, sum_rho2) - offsetof(jmm_chain_result, sum_e) ==
                  6 * sizeof(double),
              "the seven sums are consecutive doubles");

// FAST precision: lanes 0-6 of the chain fold one sum each (sum_e ..
// sum_rho2, consecutive doubles of the record) as one product and a term,
// a * b + c, from the segment's sum of E, lin = nd e0 + sd, and of E^2,
// e0 (lin + sd) + sd2; lane 0 adds the sample count.
__device__ __forceinline__ void fold_spread(Seg &g, jmm_chain_result *__restrict__ rp, int cl,
                                            double l, double rho) {
  const double nd = (double)g.nseg, sdd = (double)g.sd;
  const double lin = fma(nd, g.e0, sdd);
  if (cl < 7) {
    const double ndx = nd * (cl == 3 ? l : rho);
    const double a = cl == 1 ? g.e0 : (cl == 4 ? lin : ((cl == 3 || cl == 6) ? ndx : nd));
    const double b = cl == 0 ? g.e0 : (cl == 1 ? lin + sdd : (cl <= 4 ? l : rho));
    const double c = cl == 0 ? sdd : (cl == 1 ? (double)g.sd2 : 0.0);
    double *sum = &rp->sum_e + cl;
    *sum = *sum + fma(a, b, c);
  }
  if (cl == 0) rp->samples += g.nseg;
  g.e0 = __dadd_rn(g.e0, (double)g.delta);
  g.delta = 0.0f;
  g.sd = 0.0f;
  g.sd2 = 0.0f;
  g.nseg = 0;
}

// The spread fold as a call of its own: the step loops of two-lane slots
// (2 x 16) keep fewer registers live with it out of line.
static __device__ __noinline__ void fold_spread_call(Seg &g, jmm_chain_result *__restrict__ rp,
                                                     int cl, double l, double rho) {
  fold_spread(g, rp, cl, l, rho);
}

// The fold of a chain of L lanes: spread over seven lanes in FAST precision,
// by the first lane in EXACT (the order the oracle replays).
template <int L, bool kExact, bool kOutOfLine = false>
__device__ __forceinline__ void fold_run(Seg &g, jmm_chain_result *__restrict__ rp, int cl,
                                         double l, double rho) {
  if (kExact || L < 8)
    fold(g, rp, cl == 0, l, rho);
  else if (kOutOfLine)
    fold_spread_call(g, rp, cl, l, rho);
  else
    fold_spread(g, rp, cl, l, rho);
}

__device__ __forceinline__ void note_drift(jmm_chain_result *__restrict__ rp, bool writer,
                                           double drift) {
  if (writer && drift > rp->max_drift) rp->max_drift = drift;
}

// In FAST precision each slot leader keeps its steps' share of the segment
// sums (sum of delta, of delta^2) in its own registers; the shares join the
// chain's sums before every fold.
template <int L>
__device__ __forceinline__ void gather_shares(Seg &g, float &sd_loc, float &sd2_loc, unsigned gmask) {
  g.sd = __fadd_rn(g.sd, group_sum<L>(sd_loc, gmask));
  g.sd2 = __fadd_rn(g.sd2, group_sum<L>(sd2_loc, gmask));
  sd_loc = 0.0f;
  sd2_loc = 0.0f;
}

// The per-chain constants of the step loop, kept in registers.
struct Hot {
  float eps4, sigma2, inv_sigma2, rc2, beta, two_max_step;
};

template <int POT, bool kExact>
__device__ __forceinline__ float pair_energy_h(float d2, const Hot &H) {
  float e;
  if (POT == JMM_POT_GAUSS) {
    e = __fmul_rn(H.eps4, exp32<kExact>(-__fmul_rn(d2, H.inv_sigma2)));
  } else {
    const float inv2 = __fmul_rn(H.sigma2, rcp32<kExact>(d2));
    const float inv6 = __fmul_rn(__fmul_rn(inv2, inv2), inv2);
    e = (POT == JMM_POT_SOFTSPHERE) ? __fmul_rn(H.eps4, __fmul_rn(inv6, inv6))
                                    : __fmul_rn(H.eps4, __fmul_rn(inv6, __fsub_rn(inv6, 1.0f)));
  }
  return d2 <= H.rc2 ? e : 0.0f;
}

// The pair energy over its strength (eps4): the FAST step loop sums these
// and scales the chain's energy change once.  LJ's (s^6)^2 - s^6 is one fused
// multiply-add here (FAST only).
template <int POT>
__device__ __forceinline__ float pair_shape_fast(float d2, const Hot &H) {
  float e;
  if (POT == JMM_POT_GAUSS) {
    e = __expf(-__fmul_rn(d2, H.inv_sigma2));
  } else {
    const float inv2 = __fmul_rn(H.sigma2, rcp32<false>(d2));
    const float inv6 = __fmul_rn(__fmul_rn(inv2, inv2), inv2);
    e = (POT == JMM_POT_SOFTSPHERE) ? __fmul_rn(inv6, inv6) : __fmaf_rn(inv6, inv6, -inv6);
  }
  return d2 <= H.rc2 ? e : 0.0f;
}

// Energy change of one window pair, old separation^2 do2 to trial dn2: in
// EXACT precision the difference of the two pair energies; in FAST the
// difference of their shapes, scaled by eps4 after the window sum.
template <int POT, bool kExact>
__device__ __forceinline__ float pair_change(float dn2, float do2, const Hot &H) {
  if (kExact) return __fsub_rn(pair_energy_h<POT, true>(dn2, H), pair_energy_h<POT, true>(do2, H));
  return __fsub_rn(pair_shape_fast<POT>(dn2, H), pair_shape_fast<POT>(do2, H));
}

// The Metropolis threshold -ln u, u the midpoint of the 23-bit cell of w
// (exact in FP32, strictly inside (0, 1)); the portable log in EXACT
// precision, the hardware one otherwise.
template <bool kExact>
__device__ __forceinline__ float threshold_of(uint32_t w) {
  const float u = __fmul_rn(__fadd_rn((float)(w >> 9), 0.5f), 1.1920929e-07f);  // 2^-23
  return kExact ? -portable_logf(u) : -__logf(u);
}

// group_energies for the step loop: potential and boundary fixed at compile
// time.  EXACT precision sums in the same order (per-particle FP32, lane and
// chain FP64) and forms U_new - U_old as the difference of the two FP64 sums.
// FAST sums each lane's pair shapes in FP32 and, apart, the differences of
// its scaled and unscaled pair shapes (each a small fraction of its pair's
// energy, so that their FP32 sum carries an error far below that of the
// shapes' own), scales both by eps4 in FP64 and sums the lanes in FP64:
// U_new - U_old is the FP64 sum of the per-pair differences, and
// U_new = U_old + du (a caller's U_new - U_old gives du back to within an
// ulp of U).
// kPair: FAST sums U_old and U_new - U_old in one butterfly (below); the
// step loops of two-lane slots (2 x 16) run faster with two separate ones.
template <int L, int POT, bool PER, bool kExact, bool kScaled, bool kPair = true>
__device__ __noinline__ void chain_energies(const float *xs, const Hot &H, int n, int gl,
                                               unsigned gmask, float lf, float s, float lnf,
                                               double &u_old, double &u_new, uint64_t &pairs,
                                               uint32_t &err) {
  double uo = 0.0, un = 0.0;   // EXACT: U_old and U_new lane sums
  float fo = 0.0f, fd = 0.0f;  // FAST: the lane's shapes and shape differences
  uint32_t cnt = 0;
  for (int i = gl; i < n; i += L) {
    const float xi = xs[i];
    const float xin = kScaled ? __fmul_rn(xi, s) : xi;
    float eo = 0.0f, en = 0.0f;
    for (int k = 1;; ++k) {
      int j = i + k;
      float shift = 0.0f, shiftn = 0.0f;
      if (!PER) {
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
      // with walls the shifts are 0 and adding them changes no bit
      const float d = __fsub_rn(PER ? __fadd_rn(xj, shift) : xj, xi);
      const float d2 = __fmul_rn(d, d);
      float dn2 = d2;
      if (kScaled) {
        const float xjs = __fmul_rn(xj, s);
        const float dn = __fsub_rn(PER ? __fadd_rn(xjs, shiftn) : xjs, xin);
        dn2 = __fmul_rn(dn, dn);
      }
      if (d2 > H.rc2 && dn2 > H.rc2) break;
      if (kExact) {
        eo = __fadd_rn(eo, pair_energy_h<POT, true>(d2, H));
        if (kScaled) en = __fadd_rn(en, pair_energy_h<POT, true>(dn2, H));
      } else {
        const float so = pair_shape_fast<POT>(d2, H);
        fo = __fadd_rn(fo, so);
        if (kScaled) fd = __fadd_rn(fd, __fsub_rn(pair_shape_fast<POT>(dn2, H), so));
      }
      cnt += kScaled ? 2 : 1;
    }
    if (kExact) {
      uo = __dadd_rn(uo, (double)eo);
      if (kScaled) un = __dadd_rn(un, (double)en);
    }
  }
  if (!kExact && kScaled && kPair && L >= 2) {
    // both FAST sums over the lanes in one FP64 butterfly: after the first
    // exchange even lanes carry sums of shapes, odd lanes of differences
    const bool odd = gl & 1;
    double r = __dadd_rn(odd ? (double)fd : (double)fo,
                         __shfl_xor_sync(gmask, odd ? (double)fo : (double)fd, 1, L));
#pragma unroll
    for (int m = 2; m < L; m <<= 1) r = __dadd_rn(r, __shfl_xor_sync(gmask, r, m, L));
    u_old = __dmul_rn((double)H.eps4, __shfl_sync(gmask, r, 0, L));
    u_new = __dadd_rn(u_old, __dmul_rn((double)H.eps4, __shfl_sync(gmask, r, 1, L)));
    pairs += __reduce_add_sync(gmask, cnt);
    return;
  }
  if (!kExact) {
    uo = __dmul_rn((double)H.eps4, (double)fo);
    un = __dmul_rn((double)H.eps4, (double)fd);
  }
  u_old = group_sum_d<L>(uo, gmask);
  if (!kScaled) {
    u_new = u_old;
  } else {
    const double x = group_sum_d<L>(un, gmask);
    u_new = kExact ? x : __dadd_rn(u_old, x);
  }
  pairs += __reduce_add_sync(gmask, cnt);
}

// Neighbour index of window lane (side, k), clamped for loads, and its
// periodic shift.  With HALO the chain is one domain of a longer chain and
// the kGhost slots on each side hold the neighbouring domains' particles.
template <bool PER, bool HALO = false>
__device__ __forceinline__ int window_index(int nm, int side, int k, int n, float lf, bool &inr,
                                            float &shift) {
  int j = nm + side * k;
  shift = 0.0f;
  if (HALO) {
    inr = j >= -kGhost && j < n + kGhost;
    j = j < -kGhost ? -kGhost : (j >= n + kGhost ? n + kGhost - 1 : j);
  } else if (!PER) {
    inr = j >= 0 && j < n;
    j = j < 0 ? 0 : (j >= n ? n - 1 : j);
  } else {
    inr = true;
    if (j < 0) {
      j += n;
      shift = -lf;
    } else if (j >= n) {
      j -= n;
      shift = lf;
    }
  }
  return j;
}

// Ghost slots: far sentinels (hard walls) or the periodic images of the last
// and first kGhost particles, x - L and x + L, as the wrap of the window
// computes them.
template <bool PER>
__device__ __forceinline__ void set_ghosts(float *xs, int n, float lf, int cl, int lanes) {
  for (int k = cl; k < kGhost; k += lanes) {
    if (PER) {
      xs[-1 - k] = k < n ? __fsub_rn(xs[n - 1 - k], lf) : -kFar;
      xs[n + k] = k < n ? __fadd_rn(xs[k], lf) : kFar;
    } else {
      xs[-1 - k] = -kFar;
      xs[n + k] = kFar;
    }
  }
}

// The default number of neighbours looked at on each side of a moved
// particle for G lanes per step: 4 for G <= 8 (two lanes per side each take
// two offsets when G = 4), G/2 beyond.  A shape may widen it to any multiple
// of G/2 up to kGhost.
__host__ __device__ constexpr int window_of(int g) { return g <= 8 ? 4 : g / 2; }

__host__ __device__ constexpr unsigned leader_bits(int g, int s) {
  unsigned m = 0;
  for (int k = 0; k < s; ++k) m |= 1u << (k * g);
  return m;
}

// One chain for one launch: n_sweeps sweeps in speculative rounds of S steps.
// rp is the chain's record (state and statistics); P.id keys its Philox
// stream.  HALO: the chain is one domain of a longer chain, whose neighbouring
// particles fill the kGhost slots on each side; SNAP: trial displacements are
// snapped to the position grid P.grid (large chains' integer positions).
template <int G, int S, int POT, bool PER, bool kExact, bool HALO = false, int WIN = window_of(G),
          bool SNAP = HALO>
__device__ __forceinline__ void run_chain(const ChainParams &P, jmm_chain_result *__restrict__ rp,
                                          float *__restrict__ xg, float *xs, uint32_t *ring,
                                          const KernelCfg &cfg, int cl, unsigned gmask) {
  constexpr int W = WIN;            // neighbours looked at on each side
  static_assert(W >= G / 2 && W % (G / 2) == 0 && W <= kGhost, "window: multiple of G/2, <= kGhost");
  constexpr int H2 = G / 2;         // lanes per side
  constexpr int KPL = W / H2;       // neighbours per lane
  constexpr int L = G * S;
  constexpr unsigned kSlotBits = (G == 32) ? 0xffffffffu : ((1u << G) - 1u);
  constexpr unsigned kLeaders = leader_bits(G, S);  // lane s*G of every slot
  const int n = (int)P.n;
  const int slot = cl / G;
  const int wl = cl % G;
  const int side = wl < H2 ? -1 : 1;
  const int kb = wl % H2 + 1;  // this lane's offsets: kb, kb + H2, ...
  const int lane_shift = (int)(threadIdx.x & 31) - cl;  // first lane of the chain in the warp
  constexpr unsigned kChainBits = (L == 32) ? 0xffffffffu : ((1u << L) - 1u);
  // The conflict test gives each lane R pairs (s1 < s2) of the round's
  // slots: pair number cl + r*L in the order of s2 and then s1, so that the
  // lowest lane of the first set r with a conflict names the first slot to
  // drop.  Packed as src1 | src2 << 8 | s2 << 16 (lanes of slots s1, s2);
  // s2 = S marks an idle entry.
  constexpr int kPairs = S * (S - 1) / 2;
  constexpr int R = kPairs > L ? (kPairs + L - 1) / L : 1;
  uint32_t ptab[R];
#pragma unroll
  for (int r = 0; r < R; ++r) {
    int c = cl + r * L, p1 = 0, p2 = S;
    for (int s2 = 1; s2 < S; ++s2) {
      if (c < s2) {
        p1 = c;
        p2 = s2;
        break;
      }
      c -= s2;
    }
    ptab[r] = (uint32_t)(p1 * G) | ((uint32_t)((p2 < S ? p2 : 0) * G) << 8) | ((uint32_t)p2 << 16);
  }
  const bool writer = cl == 0;
  uint4 *ring_rec = reinterpret_cast<uint4 *>(ring);  // 16-byte aligned: see kRingWords
  Hot H;
  H.eps4 = P.eps4;
  H.sigma2 = P.sigma2;
  H.inv_sigma2 = P.inv_sigma2;
  H.rc2 = P.rc2;
  H.beta = P.beta;
  H.two_max_step = P.two_max_step;

  const bool npt = P.ensemble == JMM_NPT;
  const bool per_sweep = cfg.vol_schedule == JMM_VOLSCHED_SWEEP;
  double L_box = rp->l;
  float lf = (float)L_box, half_l = (float)__dmul_rn(L_box, 0.5);
  // n / L, renewed when L changes; a domain (HALO) keeps no statistics of
  // its own: its caller samples the whole chain once per sweep
  double rho_box = HALO ? 0.0 : __ddiv_rn((double)n, L_box);
  Seg g;
  g.e0 = rp->e;
  g.delta = 0.0f;
  g.sd = 0.0f;
  g.sd2 = 0.0f;
  g.nseg = 0;
  constexpr bool kShares = !kExact && S > 1 && !HALO;
  float sd_loc = 0.0f, sd2_loc = 0.0f;  // this lane's shares (kShares)
  const float inv_grid = SNAP ? __frcp_rn(P.grid) : 0.0f;
  const uint32_t spsw = P.steps_per_sweep;
  const uint64_t step0 = rp->steps;
  // a domain's pass is one sweep of its particles from wherever its caller's
  // step count stands (where rounds end does not change a step's outcome)
  uint32_t sweep_pos = HALO ? 0u : (uint32_t)(step0 % spsw);
  uint32_t sweeps_since_resum = 0;
  uint32_t err = rp->error;
  uint64_t pairs = rp->pair_evals;
  // window pair slots: 4 W for every kept displacement step (its lanes
  // evaluate the window whether or not the trial keeps its place) and for
  // every chunk an extended window adds
  uint32_t chunks_extra = 0;
  uint32_t d_acc = 0, d_att = 0, v_acc = 0, v_att = 0, overflows = 0;
  const uint32_t total = (uint32_t)(cfg.n_sweeps * (uint64_t)spsw);
  __syncwarp(gmask);  // every lane has read the record before lane 0 updates it

  uint32_t base = 0, pbase = 0;
  bool ring_valid = false;
  while (base < total) {
    if (!ring_valid || base + S > pbase + kRingSteps) {
      pbase = base;
      __syncwarp(gmask);
      // ring offset of the next sweep-closing volume step; later ones follow
      // every spsw steps
      const uint32_t e_vol = spsw - 1u - sweep_pos;
      for (int e = cl; e < kRingSteps; e += L) {
        const Words4 w = step_words(cfg.seed, step0 + pbase + e + 1, P.id);
        const float u1 = word_to_unit_f(w.w[1]);
        int nm_e;
        if (npt && !per_sweep) {
          nm_e = (int)word_to_index(w.w[0], (uint64_t)n + 1);
        } else {
          nm_e = (int)word_to_index(w.w[0], (uint64_t)n);
          if (npt && (uint32_t)e >= e_vol &&
              (spsw >= (uint32_t)kRingSteps ? (uint32_t)e == e_vol : ((uint32_t)e - e_vol) % spsw == 0))
            nm_e = n;  // the sweep's volume step
        }
        float md_e = __fmul_rn(__fsub_rn(u1, 0.5f), H.two_max_step);
        if (SNAP) md_e = __fmul_rn(rintf(__fmul_rn(md_e, inv_grid)), P.grid);  // exact: 2^k scales
        ring_rec[e] = make_uint4((uint32_t)nm_e, __float_as_uint(nm_e == n ? u1 : md_e),
                                 __float_as_uint(threshold_of<kExact>(w.w[2])), 0u);
      }
      __syncwarp(gmask);
      ring_valid = true;
    }
    uint32_t rem = total - base;
    if (rem > (uint32_t)S) rem = S;
    if (rem > spsw - sweep_pos) rem = spsw - sweep_pos;
    const uint4 rec = ring_rec[base + slot - pbase];  // offset < 32
    const int nm = (int)rec.x;
    const float u1 = __uint_as_float(rec.y);  // md of a displacement, u1 of a volume step
    const float thr = __uint_as_float(rec.z);
    const bool isvol = nm == n;
    const unsigned volbits =
        (__ballot_sync(gmask, isvol && wl == 0 && (uint32_t)slot < rem) >> lane_shift & kChainBits);

    if (volbits & 1u) {
      // ---- volume move (fav), ln L or linear: all L lanes ----
      double lnew;
      float s;
      double logw;  // weight term: (N+1) ln s or N ln(L'/L)
      // the volume step is slot 0's: every lane takes its uniforms
      const float u1_0 = __shfl_sync(gmask, u1, 0, L);
      const float thr_0 = __shfl_sync(gmask, thr, 0, L);
      const float v = __fsub_rn(__fmul_rn(2.0f, u1_0), 1.0f);
      if (cfg.vol_move == JMM_VOLMOVE_LNL) {
        const float lns = __fmul_rn(P.vol_step, v);
        s = portable_expf(lns);
        lnew = __dmul_rn(L_box, (double)s);
        logw = __dmul_rn((double)(n + 1), (double)lns);
      } else {
        const double dl = (double)__fmul_rn(P.vol_step, v);
        lnew = __dadd_rn(L_box, dl);
        const double ratio = __ddiv_rn(lnew, L_box);
        s = (float)ratio;
        logw = lnew > 0.0 ? __dmul_rn((double)n, log(ratio)) : -INFINITY;
      }
      double uo, un;
      const float lnf = (float)lnew;
      chain_energies<L, POT, PER, kExact, true, (G >= 4)>(xs, H, n, cl, gmask, lf, s, lnf, uo, un,
                                                         pairs, err);
      const double drift = fabs(__dsub_rn(__dadd_rn(g.e0, (double)g.delta), uo));
      note_drift(rp, writer, drift);
      if (kShares) gather_shares<L>(g, sd_loc, sd2_loc, gmask);
      const double du = __dsub_rn(un, uo);
      const double arg = __dsub_rn(
          __dmul_rn(P.beta_d, __dadd_rn(du, __dmul_rn(P.p, __dsub_rn(lnew, L_box)))), logw);
      bool acc = arg < (double)thr_0;
      if (!(lnew > 0.0)) acc = false;
      if (PER && !(lnew > 2.0 * (double)P.rc)) acc = false;
      fold_run<L, kExact, (G < 4)>(g, rp, cl, L_box, rho_box);
      v_att += 1;
      if (acc) {
        for (int i = cl; i < n; i += L) xs[i] = __fmul_rn(xs[i], s);
        L_box = lnew;
        rho_box = __ddiv_rn((double)n, L_box);
        lf = (float)L_box;
        half_l = (float)__dmul_rn(L_box, 0.5);
        if (PER) {
          __syncwarp(gmask);
          set_ghosts<PER>(xs, n, lf, cl, L);
        }
        g.e0 = un;
        v_acc += 1;
      } else {
        g.e0 = uo;
      }
      __syncwarp(gmask);
      g.sd = __fadd_rn(g.sd, g.delta);
      g.sd2 = __fmaf_rn(g.delta, g.delta, g.sd2);
      g.nseg += 1;
      base += 1;
      sweep_pos += 1;
    } else {
      if (volbits) rem = min(rem, (uint32_t)(__ffs(volbits) - 1) / G);
      // ---- S displacement steps (qad2) from the current positions ----
      const int nmc = nm < n ? nm : n - 1;
      const float md = u1;
      const float xo = xs[nmc];
      const float xn = __fadd_rn(xo, md);
      const float left = xs[nmc - 1], right = xs[nmc + 1];  // ghosts at the ends
      bool ok = (xn > left) && (xn < right);
      if (!PER) ok = ok && !(fabsf(xn) > half_l);
      // this lane's KPL neighbours, summed in offset order
      float t_lane = 0.0f;
      bool sat = false;
#pragma unroll
      for (int q = 0; q < KPL; ++q) {
        const int k = kb + q * H2;
        const float xj = xs[nmc + side * k];  // a ghost beyond either end
        // xj - x and x - xj round to the same magnitude: the side needs no sign
        const float dnw = __fsub_rn(xj, xn), dol = __fsub_rn(xj, xo);
        const float dn2 = __fmul_rn(dnw, dnw), do2 = __fmul_rn(dol, dol);
        const float tq = pair_change<POT, kExact>(dn2, do2, H);
        t_lane = q == 0 ? tq : __fadd_rn(t_lane, tq);
        if (q == KPL - 1) sat = ok && k == W && (dn2 <= H.rc2 || do2 <= H.rc2);
      }
      float de = group_sum<G>(t_lane, gmask);
      const unsigned satbits = (__ballot_sync(gmask, sat) >> lane_shift & kChainBits);
      uint32_t f = rem;
      if (satbits & kSlotBits) {
        // slow path: slot 0's window reaches beyond W; extend it chunk by chunk
        for (int chunk = 1;; ++chunk) {
          float t2 = 0.0f;
          bool sat2 = false;
#pragma unroll
          for (int q = 0; q < KPL; ++q) {
            const int k = chunk * W + kb + q * H2;
            bool inr2;
            float shift2;
            const int j2 = window_index<PER, HALO>(nmc, side, k, n, lf, inr2, shift2);
            const float xj2 = __fadd_rn(xs[j2], shift2);
            const float dn_2 = __fsub_rn(xj2, xn), do_2 = __fsub_rn(xj2, xo);
            const float dn22 = __fmul_rn(dn_2, dn_2), do22 = __fmul_rn(do_2, do_2);
            const float tq = inr2 ? pair_change<POT, kExact>(dn22, do22, H) : 0.0f;
            t2 = q == 0 ? tq : __fadd_rn(t2, tq);
            if (q == KPL - 1)
              sat2 = inr2 && k == (chunk + 1) * W && (dn22 <= H.rc2 || do22 <= H.rc2);
          }
          de = __fadd_rn(de, group_sum<G>(t2, gmask));
          chunks_extra += 1;
          if (!(((__ballot_sync(gmask, sat2) >> lane_shift & kChainBits)) & kSlotBits)) break;
          if (PER && 2 * (chunk + 2) * W > n - 1) {
            err = JMM_ERR_INVALID;
            break;
          }
        }
        f = 1;
        overflows += 1;
      }
      if (!kExact) de = __fmul_rn(de, H.eps4);  // the window sum of pair shapes
      const bool acc = ok && ((de <= 0.0f) || (__fmul_rn(de, H.beta) < thr));
      const unsigned accbits = (__ballot_sync(gmask, acc) >> lane_shift & kChainBits);
      if (S > 1 && f > 1) {
        // Step s2 is dropped, with every later one, if an earlier step s1 of
        // the round was accepted within W index positions of its particle.
        // With walls, a neighbour two or more places away matters only if
        // the spans [old, trial] of the two particles come within the
        // cut-off: otherwise every pair term between them is 0 before and
        // after (FP32 rounding is monotone, so fl(gap)^2 > rc^2 bounds all
        // four), and beyond W nothing changes since no particle passes
        // another.  Each lane tests its pairs, set by set.
#pragma unroll
        for (int r = 0; r < R; ++r) {
          const int src1 = (int)(ptab[r] & 0xffu), src2 = (int)((ptab[r] >> 8) & 0xffu);
          const int s2 = (int)(ptab[r] >> 16);
          const int nm1 = __shfl_sync(gmask, nmc, src1, L);
          const int nm2 = __shfl_sync(gmask, nmc, src2, L);
          int dist = nm1 - nm2;
          dist = dist < 0 ? -dist : dist;
          if (PER) dist = min(dist, n - dist);
          bool cand = s2 < S && ((accbits >> src1) & 1u) && dist <= W;
          const bool far = !PER && cand && dist >= 2;
          // the spans are compared only when some pair is such a candidate
          if (!PER && __any_sync(gmask, far)) {
            const float a0 = __shfl_sync(gmask, xo, src1, L);
            const float a1 = __shfl_sync(gmask, xn, src1, L);
            const float b0 = __shfl_sync(gmask, xo, src2, L);
            const float b1 = __shfl_sync(gmask, xn, src2, L);
            const float gap = fmaxf(__fsub_rn(fminf(a0, a1), fmaxf(b0, b1)),
                                    __fsub_rn(fminf(b0, b1), fmaxf(a0, a1)));
            if (far && gap > 0.0f && __fmul_rn(gap, gap) > H.rc2) cand = false;
          }
          const unsigned pbits = (__ballot_sync(gmask, cand) >> lane_shift & kChainBits);
          if (pbits) {  // later sets hold later pairs
            f = min(f, (uint32_t)__shfl_sync(gmask, s2, __ffs(pbits) - 1, L));
            break;
          }
        }
        const unsigned late = satbits & ~kSlotBits;  // windows of slots 1 .. S-1 beyond W
        if (late) f = min(f, (uint32_t)(__ffs(late) - 1) / G);
      }
      // commit steps 0 .. f-1 in order: positions by every slot leader at
      // once (their particles are distinct or unmoved), statistics in order
      const unsigned committed = f >= (uint32_t)S ? kLeaders : (kLeaders & ((1u << (f * G)) - 1u));
      if (wl == 0 && (uint32_t)slot < f && acc) {
        xs[nmc] = xn;
        if (PER) {  // keep the periodic images of the first and last W particles
          if (nmc < kGhost) xs[n + nmc] = __fadd_rn(xn, lf);
          if (nmc >= n - kGhost) xs[nmc - n] = __fsub_rn(xn, lf);
        }
      }
      const float de_acc = acc ? de : 0.0f;
      if (kExact || S == 1) {
        // step by step, the order the oracle replays
#pragma unroll
        for (int s2 = 0; s2 < S; ++s2) {
          const float d_s = __shfl_sync(gmask, de_acc, s2 * G, L);
          if ((uint32_t)s2 < f) {
            g.delta = __fadd_rn(g.delta, d_s);
            if (!HALO) {
              g.sd = __fadd_rn(g.sd, g.delta);
              g.sd2 = __fmaf_rn(g.delta, g.delta, g.sd2);
            }
          }
        }
      } else {
        // the energy change after each kept step by a scan over the slots
        float x = de_acc;
#pragma unroll
        for (int o = 1; o < S; o <<= 1) {
          const float y = __shfl_up_sync(gmask, x, o * G, L);
          if (slot >= o) x = __fadd_rn(x, y);
        }
        // the slot leaders of kept steps add their step's share
        if (!HALO) {
          const float v = ((uint32_t)slot < f && wl == 0) ? __fadd_rn(g.delta, x) : 0.0f;
          sd_loc = __fadd_rn(sd_loc, v);
          sd2_loc = __fmaf_rn(v, v, sd2_loc);
        }
        g.delta = __fadd_rn(g.delta, __shfl_sync(gmask, x, (int)(f - 1) * G, L));
      }
      __syncwarp(gmask);
      d_acc += __popc(accbits & committed);
      d_att += f;
      g.nseg += f;
      base += f;
      sweep_pos += f;
    }
    if (sweep_pos == spsw) {
      sweep_pos = 0;
      if (!npt && cfg.resum_sweeps > 0 && ++sweeps_since_resum >= (uint32_t)cfg.resum_sweeps) {
        sweeps_since_resum = 0;
        double uo, un;
        chain_energies<L, POT, PER, kExact, false>(xs, H, n, cl, gmask, lf, 1.0f, lf, uo, un, pairs,
                                                   err);
        const double drift = fabs(__dsub_rn(__dadd_rn(g.e0, (double)g.delta), uo));
        note_drift(rp, writer, drift);
        if (kShares) gather_shares<L>(g, sd_loc, sd2_loc, gmask);
        fold_run<L, kExact, (G < 4)>(g, rp, cl, L_box, rho_box);
        g.e0 = uo;
      }
    }
  }
  if (kShares) gather_shares<L>(g, sd_loc, sd2_loc, gmask);
  if (HALO)
    g.e0 = __dadd_rn(g.e0, (double)g.delta);
  else
    fold_run<L, kExact, (G < 4)>(g, rp, cl, L_box, rho_box);
  if (!isfinite(g.e0)) err = JMM_ERR_NUMERIC;
  if (writer) {
    rp->e = g.e0;
    rp->l = L_box;
    rp->steps = step0 + total;
    rp->pair_evals = pairs + (uint64_t)(4 * W) * (d_att + chunks_extra);
    rp->disp_acc += d_acc;
    rp->disp_att += d_att;
    rp->vol_acc += v_acc;
    rp->vol_att += v_att;
    rp->window_overflows += overflows;
    rp->error = err;
  }
  __syncwarp(gmask);
  if (!HALO)  // a domain's caller writes back its own (moved) particles
    for (int i = cl; i < n; i += L) xg[P.x_off + i] = xs[i];
}

// One kernel per (shape, potential, boundary, precision): the chains of one
// potential class, L lanes each, chains_per_block chains per block.
// A single-warp chain is held to REG = 72 registers so that 27 of them stay
// resident per SM (4096 chains on 152 SMs in one wave); chains that share a
// warp (G*S < 32) may use 128, and so may single-warp chains of a batch
// with at most 16 of them per SM (the REG = 128 instantiations,
// csrc/batch_wide.cu), which then spill nothing.
template <int G, int S, int POT, bool PER, bool kExact, int WIN, int REG = (G * S == 32 ? 72 : 128)>
__global__ void __maxnreg__(REG) chains_kernel(const ChainParams *__restrict__ prm,
                                                     jmm_chain_result *__restrict__ res,
                                                     float *__restrict__ xg, KernelCfg cfg) {
  constexpr int L = G * S;
  extern __shared__ __align__(16) float smem[];
  const int cl = threadIdx.x % L;
  const int cw = (threadIdx.x & 31) / L;
  const unsigned gmask = (L == 32) ? 0xffffffffu : (((1u << L) - 1u) << (cw * L));
  const uint32_t local = threadIdx.x / L;
  const uint32_t slot = blockIdx.x * cfg.chains_per_block + local;
  if (slot >= cfg.n_chains) return;
  const ChainParams P = prm[slot];
  uint32_t *ring = reinterpret_cast<uint32_t *>(smem) + local * kRingWords;
  float *xs = smem + P.s_off + kGhost;
  for (int i = cl; i < (int)P.n; i += L) xs[i] = xg[P.x_off + i];
  __syncwarp(gmask);
  set_ghosts<PER>(xs, (int)P.n, (float)res[P.id].l, cl, L);
  __syncwarp(gmask);
  run_chain<G, S, POT, PER, kExact, false, WIN>(P, res + P.id, xg, xs, ring, cfg, cl, gmask);
}

// ---- split chains: one chain's sweep over several warps ---------------------
//
// A long constant-L chain between walls runs as one block of M warps.  Per
// sweep its index range is cut into domains of B particles from a random
// offset o in [0, B) -- domain d = [o + (d-1)B, o + dB) clipped to [0, N) --
// and the domains of one colour (d even or d odd; which colour first drawn
// per sweep) make their steps at the same time, one warp each, on the
// chain's positions in shared memory, then the other colour, with a block
// barrier between.  A domain is the batched step loop (run_chain with HALO)
// on its own particles, its 16 neighbours on each side frozen for the phase.
// Two active domains are separated by a frozen interior domain of B >= 32
// particles, and a domain runs only if the 16th frozen neighbour on each
// interior side lies beyond the cut-off from the first (else it is skipped
// and the chain flagged JMM_ERR_INVALID), so active domains share no pair: a
// phase is a product of independent Metropolis chains on the conditional
// distribution of each domain given the rest, which leaves the Boltzmann
// distribution invariant; the random offset and colour make the layout
// itself random.  Domains of one phase share no pair, so the order in which
// they run does not change a bit of the result.
//
// Domain [lo, hi) of a sweep takes the chain's Philox blocks steps + lo + 1
// .. steps + hi (steps counted before the sweep), so a sweep draws the N
// blocks a whole sweep would, and the layout comes from the fourth word
// (unused by a step) of block steps + 1: offset from its high bits, colour
// from its lowest.  Each domain's energy change is summed in FP32 over its
// steps; after the sweep the chain's FP64 energy takes the domains' changes
// in index order, and the statistics sample the energy once per sweep
// (samples count sweeps; thread 0 takes a sweep's sample while the other
// warps start the next sweep).  Constant-L chains re-sum every resum_sweeps
// sweeps over the whole chain (32 lanes of warp 0).

constexpr uint32_t kSplitWarps = 8;  // warps of a split chain's block, at most

// B for a chain of n particles: a multiple of 32 of at least 2 kGhost, and
// at least n / 15, so that a sweep has at most 16 non-empty domains and a
// colour at most kSplitWarps.
__host__ __device__ constexpr uint32_t split_domain_size(uint32_t n) {
  return 32u * ((n + 479u) / 480u) < 2u * (uint32_t)kGhost ? 2u * (uint32_t)kGhost
                                                          : 32u * ((n + 479u) / 480u);
}

// Shared memory of a split chain's block: per warp a step ring and a domain
// record, the domains' energy changes of two sweeps, then the positions with
// their ghosts.
__host__ __device__ constexpr uint64_t split_smem_bytes(uint32_t n, uint32_t warps) {
  return (uint64_t)warps * (kRingWords * 4u + sizeof(jmm_chain_result)) +
         16u * (uint64_t)(n / split_domain_size(n) + 2u) + 4u * ((uint64_t)n + 2u * kGhost);
}

// Held to 64 registers: more split blocks stay resident per SM, which beat
// the extra spills on the uneven batch (1.25e10 moves/s against 1.15e10 at
// 72, four interleaved runs each).
template <int G, int S, int POT, bool kExact, int WIN>
__global__ void __maxnreg__(64) split_kernel(const ChainParams *__restrict__ prm,
                                             jmm_chain_result *__restrict__ res,
                                             float *__restrict__ xg, KernelCfg cfg) {
  static_assert(G * S == 32, "one warp per domain");
  extern __shared__ __align__(16) float smem[];
  __shared__ unsigned long long tally[kSplitWarps][4];  // accepted, attempted, pairs, overflows
  __shared__ uint32_t tally_err[kSplitWarps];
  if (blockIdx.x >= cfg.n_chains) return;
  const uint32_t nwarps = blockDim.x >> 5, warp = threadIdx.x >> 5;
  const int cl = threadIdx.x & 31;
  const ChainParams P = prm[blockIdx.x];
  const int n = (int)P.n;
  const uint32_t B = P.dom;
  uint32_t *ring = reinterpret_cast<uint32_t *>(smem) + warp * kRingWords;
  jmm_chain_result *drec =
      reinterpret_cast<jmm_chain_result *>(reinterpret_cast<uint32_t *>(smem) + nwarps * kRingWords);
  // the domains' energy changes (n / B + 2 domains at most), one buffer per
  // sweep parity: thread 0 adds a sweep's changes while the next sweep runs
  const int dstride = n / (int)B + 2;
  double *dde = reinterpret_cast<double *>(drec + nwarps);
  float *xs = reinterpret_cast<float *>(dde + 2 * dstride) + kGhost;
  jmm_chain_result *rp = res + P.id;
  const double L = rp->l;
  const float lf = (float)L;
  for (int i = threadIdx.x; i < n; i += blockDim.x) xs[i] = xg[P.x_off + i];
  if (warp == 0) set_ghosts<false>(xs, n, lf, cl, 32);
  unsigned long long acc = 0, att = 0, pairs = 0, ovf = 0;
  uint32_t err = 0;
  uint64_t steps = rp->steps;
  double e = rp->e;  // thread 0's running energy
  const double rho = __ddiv_rn((double)n, L);
  KernelCfg dcfg = cfg;  // one pass over a domain, no re-summation inside
  dcfg.n_sweeps = 1;
  dcfg.resum_sweeps = 0;
  ChainParams Pd = P;
  Pd.ensemble = JMM_NLT;
  uint32_t since_resum = 0;
  // thread 0: the chain's energy after a sweep (its domains' changes in
  // index order) into the per-sweep samples
  int pend_dom = 0;         // domains of the sweep whose sample is pending (0: none)
  const double *pend_dde = dde;
  auto sample = [&]() {
    for (int d = 0; d < pend_dom; ++d) e = __dadd_rn(e, pend_dde[d]);
    rp->sum_e = __dadd_rn(rp->sum_e, e);
    rp->sum_e2 = __dadd_rn(rp->sum_e2, __dmul_rn(e, e));
    rp->sum_l = __dadd_rn(rp->sum_l, L);
    rp->sum_l2 = __dadd_rn(rp->sum_l2, __dmul_rn(L, L));
    rp->sum_le = __dadd_rn(rp->sum_le, __dmul_rn(L, e));
    rp->sum_rho = __dadd_rn(rp->sum_rho, rho);
    rp->sum_rho2 = __dadd_rn(rp->sum_rho2, __dmul_rn(rho, rho));
    rp->samples += 1;
  };
  __syncthreads();
  for (uint64_t sw = 0; sw < cfg.n_sweeps; ++sw) {
    const Words4 lw = step_words(cfg.seed, steps + 1, P.id);
    const int off = (int)word_to_index(lw.w[3], (uint64_t)B);
    const uint32_t first = lw.w[3] & 1u;
    const int n_dom = (n - off + (int)B - 1) / (int)B + 1;
    double *dd = dde + (sw & 1u) * dstride;
    for (int phase = 0; phase < 2; ++phase) {
      // the previous sweep's sample, by thread 0 ahead of its first domain
      // (the other warps go on; the previous sweep's buffer stays untouched
      // until the sweep after this one)
      if (phase == 0 && pend_dom > 0) {
        if (threadIdx.x == 0) sample();
        pend_dom = 0;
      }
      const int colour = (int)((first + (uint32_t)phase) & 1u);
      for (int d = colour + 2 * (int)warp; d < n_dom; d += 2 * (int)nwarps) {
        const int lo = max(0, off + (d - 1) * (int)B);
        const int hi = min(n, off + d * (int)B);
        double de_d = 0.0;
        if (hi > lo) {
          // the 16th frozen neighbour beyond each interior edge lies beyond
          // the cut-off (where the chain goes on past the halo)
          bool fits = true;
          if (lo >= kGhost) fits = fits && __fsub_rn(xs[lo - 1], xs[lo - kGhost]) > P.rc;
          if (hi + kGhost <= n) fits = fits && __fsub_rn(xs[hi + kGhost - 1], xs[hi]) > P.rc;
          if (!fits) {
            err |= JMM_ERR_INVALID;
          } else {
            jmm_chain_result *dr = drec + warp;
            static_assert(sizeof(jmm_chain_result) % 8 == 0 && sizeof(jmm_chain_result) <= 256,
                          "a record is at most 32 eight-byte words");
            if (cl < (int)(sizeof(jmm_chain_result) / 8))
              reinterpret_cast<unsigned long long *>(dr)[cl] = 0ull;
            __syncwarp();
            if (cl == 0) {
              dr->l = L;
              dr->steps = steps + (uint64_t)lo;
            }
            __syncwarp();
            Pd.n = (uint32_t)(hi - lo);
            Pd.steps_per_sweep = (uint32_t)(hi - lo);
            run_chain<G, S, POT, false, kExact, true, WIN, false>(Pd, dr, nullptr, xs + lo, ring,
                                                                  dcfg, cl, 0xffffffffu);
            __syncwarp();
            de_d = dr->e;
            acc += dr->disp_acc;
            att += dr->disp_att;
            pairs += dr->pair_evals;
            ovf += dr->window_overflows;
            err |= dr->error;
            __syncwarp();
          }
        }
        if (cl == 0) dd[d] = de_d;
      }
      __syncthreads();
    }
    pend_dom = n_dom;
    pend_dde = dd;
    steps += (uint64_t)n;
    if (cfg.resum_sweeps > 0 && ++since_resum >= (uint32_t)cfg.resum_sweeps) {
      since_resum = 0;
      // the sample first, then the fresh sum replaces the running energy
      if (threadIdx.x == 0) sample();
      pend_dom = 0;
      if (warp == 0) {
        Hot H;
        H.eps4 = P.eps4;
        H.sigma2 = P.sigma2;
        H.inv_sigma2 = P.inv_sigma2;
        H.rc2 = P.rc2;
        H.beta = P.beta;
        H.two_max_step = P.two_max_step;
        double uo, un;
        uint64_t rpairs = 0;
        uint32_t rerr = 0;
        chain_energies<32, POT, false, kExact, false>(xs, H, n, cl, 0xffffffffu, lf, 1.0f, lf, uo,
                                                      un, rpairs, rerr);
        if (cl == 0) {
          const double drift = fabs(__dsub_rn(e, uo));
          if (drift > rp->max_drift) rp->max_drift = drift;
          e = uo;
          pairs += rpairs;
          err |= rerr;
        }
      }
      __syncthreads();  // the re-sum reads every position before the next sweep moves any
    }
  }
  if (pend_dom > 0 && threadIdx.x == 0) sample();
  for (int i = threadIdx.x; i < n; i += blockDim.x) xg[P.x_off + i] = xs[i];
  if (cl == 0) {
    tally[warp][0] = acc;
    tally[warp][1] = att;
    tally[warp][2] = pairs;
    tally[warp][3] = ovf;
    tally_err[warp] = err;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t e_all = rp->error;
    for (uint32_t w = 0; w < nwarps; ++w) {
      rp->disp_acc += tally[w][0];
      rp->disp_att += tally[w][1];
      rp->pair_evals += tally[w][2];
      rp->window_overflows += (uint32_t)tally[w][3];
      e_all |= tally_err[w];
    }
    if (!isfinite(e)) e_all |= JMM_ERR_NUMERIC;
    rp->e = e;
    rp->steps = steps;
    rp->error = e_all;
  }
}

typedef void (*ChainsKernelFn)(const ChainParams *, jmm_chain_result *, float *, KernelCfg);

// The 128-register FAST instantiations of the single-warp shapes
// (csrc/batch_wide.cu); nullptr for a shape that has none.
ChainsKernelFn pick_kernel_wide(uint32_t g, uint32_t s, uint32_t w, int pot, bool per);

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
