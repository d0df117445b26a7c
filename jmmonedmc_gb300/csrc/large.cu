// large.cu -- chains too long for one SM's shared memory (N up to 2^24),
// behind the jmm_large_* entry points of include/jmm_gpu.h.  Constant L,
// hard walls at +-L/2, ordered particles (LJ, soft sphere or Gaussian with
// the cut-off window of the batched kernel).
//
// Positions live in HBM as int64 multiples of a grid step 2^-k chosen per
// chain so that a domain with its halo spans fewer than 2^22 steps (an
// absolute FP32 coordinate on a chain 1.5e6 long would have an ulp of
// 0.0625).  Converting them to FP32 coordinates about a domain's origin is
// then exact, every separation within the cut-off is the same FP32 number
// in every kernel, and trial displacements are snapped to the grid.  Two
// ways to run the same chain:
//
//  * Sequential plain sweep (sequential_kernel).  One warp per chain makes
//    the chain's N single-particle Metropolis steps in order on the HBM
//    positions, 16 neighbours per side per pass.  This is the conventional
//    sweep, latency bound (one dependent HBM round trip per step).
//  * Alternating-domain sweep (domain_kernel).  Per sweep the index range
//    is cut into domains of B particles from a random offset o in [0, B):
//    domain d = [o + (d-1)B, o + dB) clipped to [0, N).  The domains of one
//    colour (d even, or d odd; which colour goes first is random per sweep)
//    run at the same time, one warp each, then the other colour.  A domain
//    copies its particles and kGhost = 16 of each neighbour's (frozen for
//    the phase; far sentinels beyond the chain's ends) into shared memory as
//    FP32 coordinates about a local origin, makes B single-particle
//    Metropolis steps on its own particles with the batched kernel's step
//    loop and writes its particles back.  Two active domains are separated
//    by a frozen interior domain of B >= 2 kGhost particles, and the kernel
//    checks that the halo reaches beyond the cut-off and that the domain
//    fits the FP32 frame (else it flags JMM_ERR_INVALID and skips the
//    domain), so they share no pair: a phase is a product of independent
//    Metropolis chains on the conditional distribution of each domain given
//    the rest, which leaves the Boltzmann distribution invariant, and the
//    random offset and colour order make every particle's position in the
//    layout random.
//
// Energies: each step-loop record accumulates its own energy changes (FP32
// within a launch, FP64 across launches); a chain's running energy is its
// last FP64 re-summation plus its records' changes, sampled once per sweep
// into FP64 sums of E and E^2.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <new>
#include <vector>

#include "batch_core.cuh"
#include "common.cuh"

using namespace jmm;
using namespace jmm::batch;

namespace {

constexpr int kG = 2, kS = 16;  // a domain's step loop: 2 window lanes x 16 steps per round
constexpr int kWarpsPerBlock = 4;
// Shared words of one domain warp: its step ring, then its particles with
// their halo, padded to 16 bytes so that the next warp's ring records stay
// aligned.
__host__ __device__ constexpr uint32_t warp_words(uint32_t b) {
  return (uint32_t)kRingWords + ((b + 2u * kGhost + 3u) & ~3u);
}
constexpr int kSeqSide = 16;   // neighbours per side per pass, sequential sweep
constexpr uint32_t kStatWarps = 8;

constexpr int64_t kFarQ = 1ll << 60;      // sentinel positions beyond the chain's ends
constexpr int64_t kFrame = 1ll << 24;     // grid steps an FP32 frame holds exactly

struct LargeChain {
  uint64_t x_base;  // offset of the chain's particle 0 in the padded position buffer
  uint32_t n;
  uint32_t pot;
  uint32_t rec0;    // first domain record of the chain
  uint32_t n_dom;   // domain records: N/B rounded up, plus one for the offset
  float eps4, sigma2, inv_sigma2, rc2, beta, two_max_step, rc;
  float grid;       // position grid step 2^-k
  int64_t wall_q;   // walls at +-wall_q grid steps: |x| <= L/2
  double l;
};

struct LargeState {
  double e_base;    // FP64 energy at the last re-summation
  double sum_e, sum_e2;
  double max_drift; // largest |running E - fresh FP64 sum| at a re-summation
  uint64_t sweeps;  // sweeps done: the index of the sweep's layout draw
  uint64_t samples;
};

__device__ __forceinline__ ChainParams domain_params(const LargeChain &c, uint32_t id, uint32_t n) {
  ChainParams P;
  P.grid = c.grid;
  P.id = id;
  P.n = n;
  P.pot = c.pot;
  P.ensemble = JMM_NLT;
  P.steps_per_sweep = n;
  P.s_off = 0;
  P.x_off = 0;
  P.eps4 = c.eps4;
  P.sigma2 = c.sigma2;
  P.inv_sigma2 = c.inv_sigma2;
  P.rc2 = c.rc2;
  P.beta = c.beta;
  P.two_max_step = c.two_max_step;
  P.vol_step = 0.0f;
  P.rc = c.rc;
  P.beta_d = 0.0;
  P.p = 0.0;
  return P;
}

__device__ __forceinline__ Hot hot_of(const LargeChain &c) {
  Hot H;
  H.eps4 = c.eps4;
  H.sigma2 = c.sigma2;
  H.inv_sigma2 = c.inv_sigma2;
  H.rc2 = c.rc2;
  H.beta = c.beta;
  H.two_max_step = c.two_max_step;
  return H;
}

// Offset and first colour of sweep `s` of chain `chain`: Philox block
// 2^62 + s of stream `chain` (step counters stay below 2^62).
__device__ __forceinline__ void sweep_layout(uint64_t seed, uint32_t chain, uint64_t s,
                                             uint32_t b, uint32_t *off, uint32_t *first) {
  const Words4 w = step_words(seed, (1ull << 62) | s, chain);
  *off = (uint32_t)word_to_index(w.w[0], b);
  *first = w.w[1] & 1u;
}

// Grid steps to an FP32 coordinate (exact below kFrame steps).
__device__ __forceinline__ float q_to_f(int64_t dq, float grid) {
  return __fmul_rn(__ll2float_rn(dq), grid);
}

template <int POT, int WIN>
__global__ void __maxnreg__(72)
    domain_kernel(const LargeChain *__restrict__ chains, const LargeState *__restrict__ states,
                  jmm_chain_result *__restrict__ rec, int64_t *__restrict__ q, uint32_t n_chains,
                  uint32_t b, uint32_t phase, uint32_t doms_per_chain, KernelCfg cfg) {
  extern __shared__ __align__(16) float smem[];
  const uint32_t wib = threadIdx.x / 32;
  const uint64_t warp = (uint64_t)blockIdx.x * kWarpsPerBlock + wib;
  const uint32_t c = (uint32_t)(warp / doms_per_chain);
  if (c >= n_chains) return;
  const LargeChain ch = chains[c];
  if (ch.pot != (uint32_t)POT) return;
  uint32_t off, first;
  sweep_layout(cfg.seed, c, states[c].sweeps, b, &off, &first);
  const uint32_t d = 2 * (uint32_t)(warp % doms_per_chain) + ((first + phase) & 1u);
  if (d >= ch.n_dom) return;
  const int64_t lo = max((int64_t)0, (int64_t)off + ((int64_t)d - 1) * (int64_t)b);
  const int64_t hi = min((int64_t)ch.n, (int64_t)off + (int64_t)d * (int64_t)b);
  if (hi <= lo) return;
  const int n = (int)(hi - lo);
  const int cl = threadIdx.x & 31;
  int64_t *qc = q + ch.x_base + lo;  // qc[-kGhost .. n + kGhost - 1] are valid (padding)
  jmm_chain_result *rp = rec + ch.rec0 + d;
  const bool left_wall = lo == 0, right_wall = hi == (int64_t)ch.n;

  // local origin O and half-width H (grid steps): the walls at +-L/2 map to
  // +-H in the step loop's symmetric wall test; an interior domain has none
  int64_t O, H = 0;
  if (left_wall && right_wall) {
    O = 0;
    H = ch.wall_q;
  } else if (left_wall) {
    H = (qc[n] + ch.wall_q + 1) >> 1;
    O = H - ch.wall_q;
  } else if (right_wall) {
    H = (ch.wall_q - qc[-1] + 1) >> 1;
    O = ch.wall_q - H;
  } else {
    O = (qc[0] + qc[n - 1]) >> 1;
  }
  // the halo must reach beyond the cut-off (unloaded neighbours are then
  // farther than the last halo particle from every particle of the domain),
  // and every real particle loaded must fit the FP32 frame
  const double reach = 1.0001 * (double)ch.rc / (double)ch.grid;
  const int il = lo >= kGhost ? -kGhost : -(int)lo;
  const int ir = (int64_t)ch.n - 1 - lo >= n + kGhost - 1 ? n + kGhost - 1 : (int)((int64_t)ch.n - 1 - lo);
  bool fits = H < kFrame && qc[ir] - O < kFrame && O - qc[il] < kFrame;
  if (!right_wall) fits = fits && (double)(qc[n + kGhost - 1] - qc[n]) > reach;
  if (!left_wall) fits = fits && (double)(qc[-1] - qc[-kGhost]) > reach;
  if (!fits) {
    if (cl == 0) rp->error |= JMM_ERR_INVALID;
    return;
  }
  uint32_t *ring = reinterpret_cast<uint32_t *>(smem) + wib * warp_words(b);
  float *xs = reinterpret_cast<float *>(ring + kRingWords) + kGhost;
  for (int i = cl - kGhost; i < n + kGhost; i += 32) xs[i] = q_to_f(qc[i] - O, ch.grid);
  if (cl == 0) rp->l = (left_wall || right_wall) ? __dmul_rn(2.0, (double)q_to_f(H, ch.grid)) : 2e30;
  __syncwarp();
  const ChainParams P = domain_params(ch, ch.rec0 + d, (uint32_t)n);
  run_chain<kG, kS, POT, false, false, true, WIN>(P, rec + P.id, nullptr, xs, ring, cfg, cl,
                                                  0xffffffffu);
  __syncwarp();
  const float inv_grid = __frcp_rn(ch.grid);
  for (int i = cl; i < n; i += 32) qc[i] = O + __float2ll_rn(__fmul_rn(xs[i], inv_grid));
}

template <int POT>
__global__ void __launch_bounds__(32)
    sequential_kernel(const LargeChain *__restrict__ chains, jmm_chain_result *__restrict__ rec,
                      int64_t *__restrict__ q, uint32_t n_chains, uint32_t id_base, KernelCfg cfg) {
  const uint32_t c = blockIdx.x;
  if (c >= n_chains) return;
  const LargeChain ch = chains[c];
  if (ch.pot != (uint32_t)POT) return;
  const int lane = threadIdx.x & 31;
  const int side = lane < kSeqSide ? -1 : 1;
  const int k0 = (lane % kSeqSide) + 1;
  const int n = (int)ch.n;
  const uint32_t id = id_base + c;
  jmm_chain_result *rp = rec + id;
  int64_t *qc = q + ch.x_base;  // qc[-kGhost .. n + kGhost - 1] are valid (padding)
  const Hot H = hot_of(ch);
  const float grid = ch.grid, inv_grid = __frcp_rn(ch.grid);
  const uint64_t step0 = rp->steps;
  double e_acc = 0.0;
  uint32_t n_acc = 0, chunks = 0;
  uint32_t err = rp->error;
  __syncwarp();
  for (int s = 0; s < n; ++s) {
    const Words4 w = step_words(cfg.seed, step0 + (uint64_t)s + 1, id);
    const int nm = (int)word_to_index(w.w[0], (uint64_t)n);
    const float md = __fmul_rn(__fsub_rn(word_to_unit_f(w.w[1]), 0.5f), H.two_max_step);
    const float thr = threshold_of<false>(w.w[2]);
    const int64_t qo = qc[nm];
    const int64_t qn = qo + __float2ll_rn(__fmul_rn(md, inv_grid));  // snapped to the grid
    const int64_t qj = qc[nm + side * k0];  // a padding sentinel beyond either end
    const float dn = q_to_f(side > 0 ? qj - qn : qn - qj, grid);
    const float dd = q_to_f(side > 0 ? qj - qo : qo - qj, grid);
    const float dn2 = __fmul_rn(dn, dn), do2 = __fmul_rn(dd, dd);
    const float t = __fsub_rn(pair_energy_h<POT, false>(dn2, H), pair_energy_h<POT, false>(do2, H));
    bool sat = k0 == kSeqSide && (dn2 <= H.rc2 || do2 <= H.rc2);
    float de = group_sum<32>(t, 0xffffffffu);
    for (int chunk = 1; __any_sync(0xffffffffu, sat); ++chunk) {
      const int k = chunk * kSeqSide + k0;
      const int j = nm + side * k;
      float t2 = 0.0f;
      sat = false;
      if (j >= 0 && j < n) {
        const int64_t qj2 = qc[j];
        const float dn_2 = q_to_f(side > 0 ? qj2 - qn : qn - qj2, grid);
        const float do_2 = q_to_f(side > 0 ? qj2 - qo : qo - qj2, grid);
        const float dn22 = __fmul_rn(dn_2, dn_2), do22 = __fmul_rn(do_2, do_2);
        t2 = __fsub_rn(pair_energy_h<POT, false>(dn22, H), pair_energy_h<POT, false>(do22, H));
        sat = k0 == kSeqSide && (dn22 <= H.rc2 || do22 <= H.rc2);
      }
      de = __fadd_rn(de, group_sum<32>(t2, 0xffffffffu));
      chunks += 1;
    }
    const bool ok = qn > qc[nm - 1] && qn < qc[nm + 1] && qn <= ch.wall_q && qn >= -ch.wall_q;
    const bool acc = ok && ((de <= 0.0f) || (__fmul_rn(de, H.beta) < thr));
    if (acc) {
      e_acc = __dadd_rn(e_acc, (double)de);
      n_acc += 1;
      __syncwarp();  // every lane has read q[nm] before it changes
      if (lane == 0) qc[nm] = qn;
    }
    __syncwarp();
  }
  if (!isfinite(e_acc)) err = JMM_ERR_NUMERIC;
  if (lane == 0) {
    rp->e = __dadd_rn(rp->e, e_acc);
    rp->steps = step0 + (uint64_t)n;
    rp->disp_acc += n_acc;
    rp->disp_att += (uint64_t)n;
    rp->pair_evals += (uint64_t)(4 * kSeqSide) * ((uint64_t)n + chunks);
    rp->window_overflows += chunks;
    rp->error = err;
  }
}

// Sum of a chain's open energy changes over its records (32 lanes).
__device__ __forceinline__ double open_changes(const jmm_chain_result *__restrict__ rec, uint32_t r0,
                                               uint32_t nr, int lane) {
  double s = 0.0;
  for (uint32_t r = lane; r < nr; r += 32) s = __dadd_rn(s, rec[r0 + r].e);
  return group_sum_d<32>(s, 0xffffffffu);
}

// Once per sweep: the chain's running energy into its sums.
__global__ void sweep_stats_kernel(const LargeChain *__restrict__ chains,
                                   LargeState *__restrict__ states,
                                   const jmm_chain_result *__restrict__ rec, uint32_t n_chains,
                                   int32_t seq_base) {
  const uint32_t c = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
  if (c >= n_chains) return;
  const LargeChain ch = chains[c];
  const int lane = threadIdx.x & 31;
  const double s = seq_base < 0 ? open_changes(rec, ch.rec0, ch.n_dom, lane)
                                : open_changes(rec, (uint32_t)seq_base + c, 1, lane);
  if (lane == 0) {
    LargeState st = states[c];
    const double e = __dadd_rn(st.e_base, s);
    st.sum_e = __dadd_rn(st.sum_e, e);
    st.sum_e2 = __dadd_rn(st.sum_e2, __dmul_rn(e, e));
    st.samples += 1;
    st.sweeps += 1;
    states[c] = st;
  }
}

// FP64 energies of the chains in two passes: warp (chain c, segment g) sums
// the pair energies of particles [g kEnergySeg, (g + 1) kEnergySeg) with their
// right-hand partners (FP32 pair terms, FP64 lane and warp sums); then one
// warp per chain adds its segments in order.  Both orders are fixed, so the
// sums are the same on every run.
constexpr uint32_t kEnergySeg = 4096;

__global__ void energy_part_kernel(const LargeChain *__restrict__ chains,
                                   const int64_t *__restrict__ q, double *__restrict__ part,
                                   uint32_t n_chains, uint32_t n_seg) {
  const uint64_t w = (uint64_t)blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
  const uint32_t c = (uint32_t)(w / n_seg), g = (uint32_t)(w % n_seg);
  if (c >= n_chains) return;
  const LargeChain ch = chains[c];
  const ChainParams P = domain_params(ch, 0, ch.n);
  const int64_t *qc = q + ch.x_base;
  const int lane = threadIdx.x & 31;
  const int n = (int)ch.n;
  const int i0 = (int)(g * kEnergySeg);
  const int i1 = min(n, i0 + (int)kEnergySeg);
  double u = 0.0;
  for (int i = i0 + lane; i < i1; i += 32) {
    const int64_t qi = qc[i];
    float e = 0.0f;
    for (int j = i + 1; j < n; ++j) {
      const float d = q_to_f(qc[j] - qi, ch.grid);
      const float d2 = __fmul_rn(d, d);
      if (d2 > P.rc2) break;
      e = __fadd_rn(e, pair_energy<false>(d2, P));
    }
    u = __dadd_rn(u, (double)e);
  }
  u = group_sum_d<32>(u, 0xffffffffu);
  if (lane == 0) part[(uint64_t)c * n_seg + g] = u;
}

__global__ void energy_sum_kernel(const double *__restrict__ part, double *__restrict__ e_out,
                                  uint32_t n_chains, uint32_t n_seg) {
  const uint32_t c = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
  if (c >= n_chains) return;
  const int lane = threadIdx.x & 31;
  double u = 0.0;
  for (uint32_t g = lane; g < n_seg; g += 32) u = __dadd_rn(u, part[(uint64_t)c * n_seg + g]);
  u = group_sum_d<32>(u, 0xffffffffu);
  if (lane == 0) e_out[c] = u;
}

// After a re-summation: the new base; the records' open changes back to 0.
__global__ void rebase_kernel(const LargeChain *__restrict__ chains, LargeState *__restrict__ states,
                              jmm_chain_result *__restrict__ rec, const double *__restrict__ e,
                              uint32_t n_chains, int32_t seq_base, bool note) {
  const uint32_t c = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
  if (c >= n_chains) return;
  const LargeChain ch = chains[c];
  const int lane = threadIdx.x & 31;
  const uint32_t r0 = seq_base < 0 ? ch.rec0 : (uint32_t)seq_base + c;
  const uint32_t nr = seq_base < 0 ? ch.n_dom : 1;
  const double s = open_changes(rec, r0, nr, lane);
  __syncwarp();
  for (uint32_t r = lane; r < nr; r += 32) rec[r0 + r].e = 0.0;
  if (lane == 0) {
    const double drift = fabs(__dsub_rn(__dadd_rn(states[c].e_base, s), e[c]));
    if (note && drift > states[c].max_drift) states[c].max_drift = drift;
    states[c].e_base = e[c];
  }
}

// ---- positions: lattice, host values snapped to the grid, checks ---------
// One block row per chain (blockIdx.y), particles along x.

__global__ void lattice_kernel(const LargeChain *__restrict__ chains, int64_t *__restrict__ q,
                               uint32_t c0, uint64_t seed, int32_t init, double jitter) {
  const uint32_t c = c0 + blockIdx.y;
  const LargeChain ch = chains[c];
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x - kGhost;
  if (i >= (int64_t)ch.n + kGhost) return;
  int64_t v;
  if (i < 0) {
    v = -kFarQ;
  } else if (i >= (int64_t)ch.n) {
    v = kFarQ;
  } else {
    // r_i = ((i + 0.5)/N - 0.5) L (jmmMCState.cpp:559-562), plus the
    // batched chains' jitter draw
    double r = __dmul_rn(__dsub_rn(__ddiv_rn((double)i + 0.5, (double)ch.n), 0.5), ch.l);
    if (init == JMM_INIT_JITTER) {
      const Words4 w = step_words(seed, (1ull << 63) | (uint64_t)i, c);
      r = __dadd_rn(r, __dmul_rn(jitter, __dsub_rn(__dmul_rn(2.0, word_to_unit(w.w[0])), 1.0)));
    }
    v = __double2ll_rn(__dmul_rn(r, 1.0 / (double)ch.grid));
    v = v > ch.wall_q ? ch.wall_q : (v < -ch.wall_q ? -ch.wall_q : v);
  }
  q[ch.x_base + i] = v;
}

// Host values (staged in the padded layout) to grid steps; flags values
// outside the walls.
__global__ void snap_kernel(const LargeChain *__restrict__ chains, const double *__restrict__ x,
                            int64_t *__restrict__ q, uint32_t c0, uint32_t *__restrict__ bad) {
  const LargeChain ch = chains[c0 + blockIdx.y];
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ch.n) return;
  const double v = __dmul_rn(x[ch.x_base + i], 1.0 / (double)ch.grid);  // exact: 2^k
  if (!(fabs(v) <= (double)ch.wall_q)) {
    atomicOr(bad, 1u);
    return;
  }
  q[ch.x_base + i] = __double2ll_rn(v);
}

// Particles strictly increasing along each chain, else a flag.
__global__ void order_kernel(const LargeChain *__restrict__ chains, const int64_t *__restrict__ q,
                             uint32_t c0, uint32_t *__restrict__ bad) {
  const LargeChain ch = chains[c0 + blockIdx.y];
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x + 1;
  if (i >= ch.n) return;
  if (!(q[ch.x_base + i] > q[ch.x_base + i - 1])) atomicOr(bad, 2u);
}

__global__ void unsnap_kernel(const LargeChain *__restrict__ chains, const int64_t *__restrict__ q,
                              double *__restrict__ x, uint32_t c0) {
  const LargeChain ch = chains[c0 + blockIdx.y];
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ch.n) return;
  x[ch.x_base + i] = __dmul_rn((double)q[ch.x_base + i], (double)ch.grid);
}

typedef void (*DomainKernel)(const LargeChain *, const LargeState *, jmm_chain_result *, int64_t *,
                             uint32_t, uint32_t, uint32_t, uint32_t, KernelCfg);

// Neighbours per side a domain step looks at before it extends its window,
// for a potential class: 3, 4 or 8, from the densest chain's neighbours
// within the cut-off (as the batched form's defaults: rc / 0.85 sigma for a
// 12-power core, 1.5 rho rc for the Gaussian core).
uint32_t window_for(double need) { return need <= 3.0 ? 3u : (need <= 4.0 ? 4u : 8u); }

template <int POT>
DomainKernel domain_kernel_for(uint32_t win) {
  return win <= 3 ? domain_kernel<POT, 3> : (win <= 4 ? domain_kernel<POT, 4> : domain_kernel<POT, 8>);
}

template <int POT>
void launch_phase(const LargeChain *d_chains, const LargeState *d_states, jmm_chain_result *d_rec,
                  int64_t *d_q, uint32_t n_chains, uint32_t b, uint32_t phase, uint32_t doms_per_chain,
                  uint32_t win, const KernelCfg &kc, cudaStream_t s) {
  const uint64_t warps = (uint64_t)n_chains * doms_per_chain;
  const uint32_t blocks = (uint32_t)((warps + kWarpsPerBlock - 1) / kWarpsPerBlock);
  const size_t smem = (size_t)kWarpsPerBlock * warp_words(b) * sizeof(float);
  domain_kernel_for<POT>(win)<<<blocks, 32 * kWarpsPerBlock, smem, s>>>(
      d_chains, d_states, d_rec, d_q, n_chains, b, phase, doms_per_chain, kc);
}

}  // namespace

struct jmm_large {
  jmm_batch_config cfg;
  uint32_t n_chains = 0, b = 0, doms_per_chain = 0, records = 0;
  std::vector<LargeChain> host_chains;
  uint64_t total = 0;        // doubles in the padded position buffer
  bool pots[3] = {false, false, false};
  uint32_t win[3] = {3, 3, 3};  // domain window per potential class (window_for)
  double need[3] = {0.0, 0.0, 0.0};
  LargeChain *d_chains = nullptr;
  LargeState *d_states = nullptr;
  jmm_chain_result *d_rec = nullptr;  // domain records, then one per chain for the sequential sweep
  int64_t *d_q = nullptr;    // positions in grid steps, padded with sentinels
  double *d_stage = nullptr; // host-format positions (same layout), allocated on first use
  uint32_t *d_bad = nullptr; // flags of the position checks
  double *d_e = nullptr;
  double *d_part = nullptr;  // per-segment partial energies (energy_sums)
  uint32_t max_n = 0;
  cudaStream_t stream = nullptr;
  uint64_t sweeps_since_resum = 0;
  int mode = 0;              // records holding the open changes: 0 domains, 1 sequential
};

// A handle's device memory comes from the device's stream-ordered pool,
// which keeps up to 16 GiB of freed blocks for the next handle, so that
// repeated one-call runs (jmm_large_run_host) do not map and unmap
// gigabytes each time.
static cudaError_t pool_alloc(void **p, size_t bytes, cudaStream_t s) {
  static bool configured = false;
  if (!configured) {
    int dev = 0;
    cudaMemPool_t pool;
    if (cudaGetDevice(&dev) == cudaSuccess && cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
      uint64_t keep = 16ull << 30;
      cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
      if (keep < (16ull << 30)) {
        keep = 16ull << 30;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
      }
    }
    configured = true;
  }
  return cudaMallocAsync(p, bytes, s);
}

static void large_free(jmm_large *h) {
  if (!h) return;
  void *bufs[8] = {h->d_chains, h->d_states, h->d_rec, h->d_q,
                   h->d_stage,  h->d_bad,    h->d_e,   h->d_part};
  for (void *p : bufs)
    if (p) cudaFreeAsync(p, h->stream);
  if (h->stream) {
    cudaStreamSynchronize(h->stream);
    cudaStreamDestroy(h->stream);
  }
  delete h;
}

static KernelCfg large_cfg(const jmm_large *h) {
  KernelCfg kc;
  kc.seed = h->cfg.seed;
  kc.n_sweeps = 1;
  kc.boundary = JMM_BOUNDARY_WALLS;
  kc.vol_move = JMM_VOLMOVE_LNL;
  kc.vol_schedule = JMM_VOLSCHED_SWEEP;
  kc.resum_sweeps = 0;
  kc.n_chains = h->n_chains;
  kc.chains_per_block = 1;
  return kc;
}

static int32_t seq_base_of(const jmm_large *h, int mode) {
  return mode == 0 ? -1 : (int32_t)h->records;
}

// FP64 re-summation on stream s: new base energies, open changes folded.
// The chains' FP64 energies into d_e, on stream s.
static int energy_sums(jmm_large *h, cudaStream_t s) {
  const uint32_t n_seg = (h->max_n + kEnergySeg - 1) / kEnergySeg;
  const uint64_t warps = (uint64_t)h->n_chains * n_seg;
  energy_part_kernel<<<(uint32_t)((warps + kStatWarps - 1) / kStatWarps), 32 * kStatWarps, 0, s>>>(
      h->d_chains, h->d_q, h->d_part, h->n_chains, n_seg);
  energy_sum_kernel<<<(h->n_chains + kStatWarps - 1) / kStatWarps, 32 * kStatWarps, 0, s>>>(
      h->d_part, h->d_e, h->n_chains, n_seg);
  JMM_CUDA(cudaGetLastError());
  return JMM_OK;
}

static int resum(jmm_large *h, cudaStream_t s, bool note) {
  const uint32_t blocks = (h->n_chains + kStatWarps - 1) / kStatWarps;
  const int rc = energy_sums(h, s);
  if (rc) return rc;
  rebase_kernel<<<blocks, 32 * kStatWarps, 0, s>>>(h->d_chains, h->d_states, h->d_rec, h->d_e,
                                                   h->n_chains, seq_base_of(h, h->mode), note);
  JMM_CUDA(cudaGetLastError());
  h->sweeps_since_resum = 0;
  return JMM_OK;
}

static dim3 chain_grid(const jmm_large *h, uint32_t c0, uint32_t c1, uint32_t extra) {
  return dim3((h->max_n + extra + 255) / 256, c1 - c0);
}

// Orders and walls of chains [c0, c1) checked on the device: JMM_OK or
// JMM_ERR_INVALID with the reason.
static int check_positions(jmm_large *h, uint32_t c0, uint32_t c1, const char *what) {
  order_kernel<<<chain_grid(h, c0, c1, 0), 256, 0, h->stream>>>(h->d_chains, h->d_q, c0, h->d_bad);
  JMM_CUDA(cudaGetLastError());
  uint32_t bad = 0;
  JMM_CUDA(cudaMemcpyAsync(&bad, h->d_bad, sizeof(bad), cudaMemcpyDeviceToHost, h->stream));
  JMM_CUDA(cudaStreamSynchronize(h->stream));
  if (bad & 1u) return fail(JMM_ERR_INVALID, "%s: a position lies outside the walls", what);
  if (bad & 2u)
    return fail(JMM_ERR_INVALID, "%s: positions must increase by at least one grid step", what);
  return JMM_OK;
}

// Host positions (compact, chain after chain) of chains [c0, c1) to the
// device: one copy per chain into the staging buffer, then snapped.
static int upload_positions(jmm_large *h, const double *x, uint32_t c0, uint32_t c1,
                            const char *what) {
  if (!h->d_stage) JMM_CUDA(pool_alloc((void **)&h->d_stage, h->total * sizeof(double), h->stream));
  JMM_CUDA(cudaMemsetAsync(h->d_bad, 0, sizeof(uint32_t), h->stream));
  uint64_t src = 0;
  for (uint32_t k = c0; k < c1; ++k) {
    const LargeChain &lc = h->host_chains[k];
    JMM_CUDA(cudaMemcpyAsync(h->d_stage + lc.x_base, x + src, lc.n * sizeof(double),
                             cudaMemcpyHostToDevice, h->stream));
    src += lc.n;
  }
  snap_kernel<<<chain_grid(h, c0, c1, 0), 256, 0, h->stream>>>(h->d_chains, h->d_stage, h->d_q, c0,
                                                               h->d_bad);
  return check_positions(h, c0, c1, what);
}

static int download_positions(jmm_large *h, double *x, uint32_t c0, uint32_t c1) {
  if (!h->d_stage) JMM_CUDA(pool_alloc((void **)&h->d_stage, h->total * sizeof(double), h->stream));
  unsnap_kernel<<<chain_grid(h, c0, c1, 0), 256, 0, h->stream>>>(h->d_chains, h->d_q, h->d_stage, c0);
  JMM_CUDA(cudaGetLastError());
  uint64_t dst = 0;
  for (uint32_t k = c0; k < c1; ++k) {
    const LargeChain &lc = h->host_chains[k];
    JMM_CUDA(cudaMemcpyAsync(x + dst, h->d_stage + lc.x_base, lc.n * sizeof(double),
                             cudaMemcpyDeviceToHost, h->stream));
    dst += lc.n;
  }
  JMM_CUDA(cudaStreamSynchronize(h->stream));
  return JMM_OK;
}

static int enqueue(jmm_large *h, uint64_t n_sweeps, int mode, cudaStream_t s) {
  if (h->mode != mode) {
    const int rc = resum(h, s, true);  // fold the other records' changes into the base
    if (rc) return rc;
    h->mode = mode;
  }
  const KernelCfg kc = large_cfg(h);
  const uint32_t sblocks = (h->n_chains + kStatWarps - 1) / kStatWarps;
  for (uint64_t sw = 0; sw < n_sweeps; ++sw) {
    if (mode == 0) {
      for (uint32_t phase = 0; phase < 2; ++phase) {
        if (h->pots[0])
          launch_phase<JMM_POT_LJCUT>(h->d_chains, h->d_states, h->d_rec, h->d_q, h->n_chains, h->b,
                                      phase, h->doms_per_chain, h->win[0], kc, s);
        if (h->pots[1])
          launch_phase<JMM_POT_SOFTSPHERE>(h->d_chains, h->d_states, h->d_rec, h->d_q, h->n_chains,
                                           h->b, phase, h->doms_per_chain, h->win[1], kc, s);
        if (h->pots[2])
          launch_phase<JMM_POT_GAUSS>(h->d_chains, h->d_states, h->d_rec, h->d_q, h->n_chains, h->b,
                                      phase, h->doms_per_chain, h->win[2], kc, s);
      }
    } else {
      const uint32_t base = h->records;
      if (h->pots[0])
        sequential_kernel<JMM_POT_LJCUT><<<h->n_chains, 32, 0, s>>>(h->d_chains, h->d_rec, h->d_q,
                                                                   h->n_chains, base, kc);
      if (h->pots[1])
        sequential_kernel<JMM_POT_SOFTSPHERE><<<h->n_chains, 32, 0, s>>>(h->d_chains, h->d_rec,
                                                                        h->d_q, h->n_chains, base, kc);
      if (h->pots[2])
        sequential_kernel<JMM_POT_GAUSS><<<h->n_chains, 32, 0, s>>>(h->d_chains, h->d_rec, h->d_q,
                                                                   h->n_chains, base, kc);
    }
    sweep_stats_kernel<<<sblocks, 32 * kStatWarps, 0, s>>>(h->d_chains, h->d_states, h->d_rec,
                                                           h->n_chains, seq_base_of(h, mode));
    JMM_CUDA(cudaGetLastError());
    if (h->cfg.resum_sweeps && ++h->sweeps_since_resum >= h->cfg.resum_sweeps) {
      const int rc = resum(h, s, true);
      if (rc) return rc;
    }
  }
  return JMM_OK;
}

// Creates the chains; with x_in (host FP64 positions, chains back to back)
// they start there instead of on the configured lattice.
static int large_create(const jmm_batch_config *cfg, const jmm_chain_desc *chains,
                        uint32_t n_chains, uint32_t domain_size, jmm_large **out,
                        const double *x_in) {
  clear_error();
  JMM_CHECK_ARG(cfg && chains && out && n_chains > 0, "null argument or no chains");
  JMM_CHECK_ARG(n_chains <= 65535, "at most 65535 chains");
  *out = nullptr;
  JMM_CHECK_ARG(domain_size >= 2 * kGhost && domain_size <= 8192,
                "domain_size must be in [32, 8192]");
  JMM_CHECK_ARG(cfg->boundary == JMM_BOUNDARY_WALLS, "hard walls only");
  JMM_CHECK_ARG(cfg->precision == JMM_PREC_FAST, "JMM_PREC_FAST only");
  for (uint32_t k = 0; k < n_chains; ++k) {
    const jmm_chain_desc &c = chains[k];
    if (c.n < domain_size || c.n > (1u << 24))
      return fail(JMM_ERR_INVALID, "jmm_large_create: chain %u: N must be in [domain_size, 2^24]", k);
    if (c.ensemble != JMM_NLT)
      return fail(JMM_ERR_INVALID, "jmm_large_create: chain %u: constant-L chains only", k);
    if (c.potential != JMM_POT_LJCUT && c.potential != JMM_POT_SOFTSPHERE &&
        c.potential != JMM_POT_GAUSS)
      return fail(JMM_ERR_INVALID, "jmm_large_create: chain %u: unknown potential", k);
    if (!(c.t > 0) || !(c.l0 > 0) || !(c.sigma > 0) || !(c.cutoff > 0) || !(c.max_step > 0))
      return fail(JMM_ERR_INVALID,
                  "jmm_large_create: chain %u: T, L, sigma, cut-off and step must be positive", k);
    if (!isfinite(c.t) || !isfinite(c.l0) || !isfinite(c.sigma) || !isfinite(c.cutoff) ||
        !isfinite(c.max_step) || !isfinite(c.eps))
      return fail(JMM_ERR_INVALID, "jmm_large_create: chain %u: parameters must be finite", k);
  }
  if (!jmm_device_available()) return fail(JMM_ERR_CUDA, "jmm_large_create: no CUDA device");
  jmm_large *h = new (std::nothrow) jmm_large();
  if (!h) return fail(JMM_ERR_NOMEM, "jmm_large_create: host allocation failed");
  h->cfg = *cfg;
  h->n_chains = n_chains;
  h->b = domain_size;
  uint32_t max_dom = 0;
  uint64_t off = 0;
  uint64_t rec = 0;
  for (uint32_t k = 0; k < n_chains; ++k) {
    const jmm_chain_desc &c = chains[k];
    LargeChain lc;
    memset(&lc, 0, sizeof(lc));
    lc.x_base = off + kGhost;
    lc.n = c.n;
    lc.pot = (uint32_t)c.potential;
    lc.n_dom = (c.n + domain_size - 1) / domain_size + 1;
    lc.rec0 = (uint32_t)rec;
    lc.eps4 = c.potential == JMM_POT_LJCUT ? (float)(4.0 * c.eps) : (float)c.eps;
    lc.sigma2 = (float)(c.sigma * c.sigma);
    lc.inv_sigma2 = (float)(1.0 / (c.sigma * c.sigma));
    lc.rc2 = (float)(c.cutoff * c.cutoff);
    lc.rc = (float)c.cutoff;
    lc.beta = (float)(1.0 / c.t);
    lc.two_max_step = (float)(2.0 * c.max_step);
    lc.l = c.l0;
    // grid step 2^-k: a domain with both halos spans about (B + 2 kGhost) L/N,
    // kept below 2^23 steps (half the exact FP32 frame on either side)
    const double span = (domain_size + 2.0 * kGhost) * c.l0 / c.n;
    const int kexp = std::min(40, (int)floor(log2(8388608.0 / span)));
    if (kexp < 8) {
      large_free(h);
      return fail(JMM_ERR_INVALID,
                  "jmm_large_create: chain %u: a domain spans %.0f sigma, more than 2^15 at a grid "
                  "of 2^-8: lower domain_size", k, span);
    }
    lc.grid = ldexpf(1.0f, -kexp);
    lc.wall_q = (int64_t)floor(0.5 * c.l0 * ldexp(1.0, kexp));
    h->host_chains.push_back(lc);
    const int pc = c.potential == JMM_POT_LJCUT ? 0 : (c.potential == JMM_POT_SOFTSPHERE ? 1 : 2);
    h->pots[pc] = true;
    h->need[pc] = std::max(h->need[pc], c.potential == JMM_POT_GAUSS ? 1.5 * c.n / c.l0 * c.cutoff
                                                                   : c.cutoff / (0.85 * c.sigma));
    h->win[pc] = window_for(h->need[pc]);
    rec += lc.n_dom;
    max_dom = std::max(max_dom, lc.n_dom);
    h->max_n = std::max(h->max_n, c.n);
    off += (uint64_t)c.n + 2 * kGhost;
  }
  if (rec + n_chains > 0x7fffffffull) {
    large_free(h);
    return fail(JMM_ERR_INVALID, "jmm_large_create: too many domains");
  }
  h->records = (uint32_t)rec;
  h->doms_per_chain = (max_dom + 1) / 2;
  h->total = off;

  const uint64_t n_rec = rec + n_chains;
  cudaError_t e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
  cudaStream_t hs = h->stream;
  if (e == cudaSuccess) e = pool_alloc((void **)&h->d_chains, n_chains * sizeof(LargeChain), hs);
  if (e == cudaSuccess) e = pool_alloc((void **)&h->d_states, n_chains * sizeof(LargeState), hs);
  if (e == cudaSuccess) e = pool_alloc((void **)&h->d_rec, n_rec * sizeof(jmm_chain_result), hs);
  if (e == cudaSuccess) e = pool_alloc((void **)&h->d_q, off * sizeof(int64_t), hs);
  if (e == cudaSuccess) e = pool_alloc((void **)&h->d_e, n_chains * sizeof(double), hs);
  if (e == cudaSuccess)
    e = pool_alloc((void **)&h->d_part,
                   (size_t)n_chains * ((h->max_n + kEnergySeg - 1) / kEnergySeg) * sizeof(double), hs);
  if (e == cudaSuccess) e = pool_alloc((void **)&h->d_bad, sizeof(uint32_t), hs);
  // the copies below run on the legacy stream: the allocations first
  if (e == cudaSuccess) e = cudaStreamSynchronize(hs);
  if (e != cudaSuccess) {
    const int rc = cuda_status(e, "jmm_large_create allocation", __FILE__, __LINE__);
    large_free(h);
    return rc;
  }
  std::vector<jmm_chain_result> recs(n_rec);
  memset(recs.data(), 0, recs.size() * sizeof(jmm_chain_result));
  std::vector<LargeState> st(n_chains);
  memset(st.data(), 0, st.size() * sizeof(LargeState));
  e = cudaMemcpy(h->d_chains, h->host_chains.data(), n_chains * sizeof(LargeChain),
                 cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(h->d_rec, recs.data(), n_rec * sizeof(jmm_chain_result), cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(h->d_states, st.data(), n_chains * sizeof(LargeState), cudaMemcpyHostToDevice);
  const size_t smem = (size_t)kWarpsPerBlock * warp_words(domain_size) * sizeof(float);
  if (e == cudaSuccess && smem > 48 * 1024) {
    e = cudaFuncSetAttribute(domain_kernel_for<JMM_POT_LJCUT>(h->win[0]),
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(domain_kernel_for<JMM_POT_SOFTSPHERE>(h->win[1]),
                               cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(domain_kernel_for<JMM_POT_GAUSS>(h->win[2]),
                               cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  }
  if (e != cudaSuccess) {
    const int rc = cuda_status(e, "jmm_large_create upload", __FILE__, __LINE__);
    large_free(h);
    return rc;
  }
  // lattice (plus jitter, the batched chains' draw) on the grid, far
  // sentinels in the padding
  int rc = JMM_OK;
  lattice_kernel<<<chain_grid(h, 0, n_chains, 2 * kGhost), 256, 0, h->stream>>>(
      h->d_chains, h->d_q, 0, cfg->seed, cfg->init, cfg->jitter);
  e = cudaMemsetAsync(h->d_bad, 0, sizeof(uint32_t), h->stream);
  if (e != cudaSuccess) rc = cuda_status(e, "jmm_large_create lattice", __FILE__, __LINE__);
  if (rc == JMM_OK)
    rc = x_in ? upload_positions(h, x_in, 0, n_chains, "jmm_large_run_host")
              : check_positions(h, 0, n_chains, "jmm_large_create (initial jitter)");
  if (rc == JMM_OK) rc = resum(h, h->stream, false);  // initial energies
  if (rc == JMM_OK) {
    e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) rc = cuda_status(e, "jmm_large_create energies", __FILE__, __LINE__);
  }
  if (rc) {
    large_free(h);
    return rc;
  }
  *out = h;
  return JMM_OK;
}

extern "C" int jmm_large_create(const jmm_batch_config *cfg, const jmm_chain_desc *chains,
                                uint32_t n_chains, uint32_t domain_size, jmm_large **out) {
  return large_create(cfg, chains, n_chains, domain_size, out, nullptr);
}

extern "C" int jmm_large_destroy(jmm_large *h) {
  large_free(h);
  return JMM_OK;
}

extern "C" int jmm_large_run_async(jmm_large *h, uint64_t n_sweeps, int32_t mode, void *stream) {
  clear_error();
  JMM_CHECK_ARG(h, "null handle");
  JMM_CHECK_ARG(mode == JMM_LARGE_DOMAINS || mode == JMM_LARGE_SEQUENTIAL, "unknown sweep mode");
  return enqueue(h, n_sweeps, mode == JMM_LARGE_DOMAINS ? 0 : 1,
                 stream ? (cudaStream_t)stream : h->stream);
}

extern "C" int jmm_large_run(jmm_large *h, uint64_t n_sweeps, int32_t mode) {
  clear_error();
  JMM_CHECK_ARG(h, "null handle");
  JMM_CHECK_ARG(mode == JMM_LARGE_DOMAINS || mode == JMM_LARGE_SEQUENTIAL, "unknown sweep mode");
  const int rc = enqueue(h, n_sweeps, mode == JMM_LARGE_DOMAINS ? 0 : 1, h->stream);
  if (rc) return rc;
  JMM_CUDA(cudaStreamSynchronize(h->stream));
  return JMM_OK;
}

extern "C" int jmm_large_results(jmm_large *h, jmm_large_result *out, uint32_t n_chains) {
  clear_error();
  JMM_CHECK_ARG(h && out, "null argument");
  JMM_CHECK_ARG(n_chains == h->n_chains, "n_chains does not match");
  JMM_CUDA(cudaDeviceSynchronize());
  const uint64_t n_rec = (uint64_t)h->records + n_chains;
  std::vector<LargeState> st(n_chains);
  std::vector<jmm_chain_result> rec(n_rec);
  JMM_CUDA(cudaMemcpy(st.data(), h->d_states, n_chains * sizeof(LargeState), cudaMemcpyDeviceToHost));
  JMM_CUDA(cudaMemcpy(rec.data(), h->d_rec, n_rec * sizeof(jmm_chain_result), cudaMemcpyDeviceToHost));
  for (uint32_t k = 0; k < n_chains; ++k) {
    jmm_large_result &r = out[k];
    memset(&r, 0, sizeof(r));
    const LargeChain &lc = h->host_chains[k];
    double open = 0.0;
    for (uint32_t d = 0; d <= lc.n_dom; ++d) {
      const jmm_chain_result &x = rec[d < lc.n_dom ? lc.rec0 + d : h->records + k];
      open += x.e;
      r.moves += x.disp_att;
      r.accepted += x.disp_acc;
      r.pair_evals += x.pair_evals;
      r.window_overflows += x.window_overflows;
      r.error |= x.error;
    }
    r.e = st[k].e_base + open;
    r.l = lc.l;
    r.sweeps = st[k].sweeps;
    r.samples = st[k].samples;
    r.sum_e = st[k].sum_e;
    r.sum_e2 = st[k].sum_e2;
    r.max_drift = st[k].max_drift;
    r.grid = (double)lc.grid;
  }
  return JMM_OK;
}

extern "C" int jmm_large_reset_stats(jmm_large *h) {
  clear_error();
  JMM_CHECK_ARG(h, "null handle");
  JMM_CUDA(cudaDeviceSynchronize());
  std::vector<LargeState> st(h->n_chains);
  JMM_CUDA(cudaMemcpy(st.data(), h->d_states, h->n_chains * sizeof(LargeState),
                      cudaMemcpyDeviceToHost));
  for (auto &s : st) {
    s.sum_e = s.sum_e2 = 0.0;
    s.samples = 0;
    s.max_drift = 0.0;
  }
  JMM_CUDA(cudaMemcpy(h->d_states, st.data(), h->n_chains * sizeof(LargeState),
                      cudaMemcpyHostToDevice));
  return JMM_OK;
}

extern "C" int jmm_large_energies(jmm_large *h, double *e, uint32_t n_chains) {
  clear_error();
  JMM_CHECK_ARG(h && e, "null argument");
  JMM_CHECK_ARG(n_chains == h->n_chains, "n_chains does not match");
  JMM_CUDA(cudaDeviceSynchronize());
  const int rc = energy_sums(h, h->stream);
  if (rc) return rc;
  JMM_CUDA(cudaStreamSynchronize(h->stream));
  JMM_CUDA(cudaMemcpy(e, h->d_e, n_chains * sizeof(double), cudaMemcpyDeviceToHost));
  return JMM_OK;
}

extern "C" int jmm_large_get_positions(jmm_large *h, uint32_t chain, double *x, uint64_t n) {
  clear_error();
  JMM_CHECK_ARG(h && x, "null argument");
  JMM_CHECK_ARG(chain < h->n_chains, "chain index out of range");
  JMM_CHECK_ARG(n == h->host_chains[chain].n, "N does not match the chain");
  JMM_CUDA(cudaDeviceSynchronize());
  return download_positions(h, x, chain, chain + 1);
}

extern "C" int jmm_large_set_positions(jmm_large *h, uint32_t chain, const double *x, uint64_t n) {
  clear_error();
  JMM_CHECK_ARG(h && x, "null argument");
  JMM_CHECK_ARG(chain < h->n_chains, "chain index out of range");
  JMM_CHECK_ARG(n == h->host_chains[chain].n, "N does not match the chain");
  JMM_CUDA(cudaDeviceSynchronize());
  std::vector<int64_t> keep(n);  // the chain's positions, restored if the new ones are refused
  const LargeChain &lc = h->host_chains[chain];
  JMM_CUDA(cudaMemcpy(keep.data(), h->d_q + lc.x_base, n * sizeof(int64_t), cudaMemcpyDeviceToHost));
  int rc = upload_positions(h, x, chain, chain + 1, "jmm_large_set_positions");
  if (rc) {
    JMM_CUDA(cudaMemcpy(h->d_q + lc.x_base, keep.data(), n * sizeof(int64_t), cudaMemcpyHostToDevice));
    return rc;
  }
  // fresh base energies for every chain; open changes folded
  rc = resum(h, h->stream, false);
  if (rc) return rc;
  JMM_CUDA(cudaStreamSynchronize(h->stream));
  return JMM_OK;
}

extern "C" int jmm_large_run_host(const jmm_batch_config *cfg, const jmm_chain_desc *chains,
                                  uint32_t n_chains, uint32_t domain_size, int32_t mode,
                                  const double *x_in, uint64_t n_sweeps, jmm_large_result *results,
                                  double *x_out) {
  jmm_large *h = nullptr;
  // x_in gives the starting positions (no lattice, one FP64 energy sum)
  int rc = large_create(cfg, chains, n_chains, domain_size, &h, x_in);
  if (rc) return rc;
  if (rc == JMM_OK) rc = jmm_large_run(h, n_sweeps, mode);
  if (rc == JMM_OK && results) rc = jmm_large_results(h, results, n_chains);
  if (rc == JMM_OK && x_out) rc = download_positions(h, x_out, 0, n_chains);
  large_free(h);
  return rc;
}
