// plain.cu -- the plain one-chain FP64 form of jmmOneDMC's move loop on one
// GB300, behind the jmm_plain_* entry points of include/jmm_gpu.h.
//
// This is the reference's algorithm step for step, so that, fed the same
// uniforms, it reproduces the reference's accept/reject sequence and its
// FP64 totals bit for bit:
//   phiLJcut / phiLJinfcutoff / phiHarmoniccut   src/pot.cpp:19-141
//   fad                                          src/jmmMCState.cpp:853-1003
//   qad2 (incremental separations, two partial   src/jmmMCState.cpp:1160-1464
//         sums i<nm then i>nm, in index order)
//   qavLJ                                        src/jmmMCState.cpp:1648-1730
//   Step / incrementStep                         src/jmmMCState.cpp:1734-1811
//   updateThermo                                 src/jmmMCState.cpp:1941-1961
//   ECheck                                       src/jmmMCState.cpp:1965-2095
//   fav                                          src/jmmMCState.cpp:2161-2293
//   fgrho / ugrho / qagrho (rho(x), g(x))        src/jmmMCState.cpp:1069-1149, :2297-2384
//   relaxVolume, calculateEnergyOfTrialVolumeChange, moveVolume
//                                                src/jmmMCState.cpp:2396-2643, :2756-2905
//
// GB300 mapping: one persistent 1024-thread block runs many steps per launch.
// Pair terms of a step are evaluated in parallel; the FP64 sums that decide
// acceptance are formed by nine lanes of warp 0 (one per quantity) in the
// reference's index order, because a reordered FP64 sum would not round the
// same.  Per-pair state (separations and nine quantities) stays in HBM,
// (i<j) at i*N+j; a step touches N-1 pairs, a volume move or energy check
// all N(N-1)/2.  This TU is compiled with -fmad=false: no FP64 expression is
// contracted into a fused multiply-add, matching the reference's x86-64 build.
//
// The in-order sums leave out the pairs whose terms are all +0.0 (pairs
// beyond the cut-off or NBN): no term of any pair is ever -0.0 (each is a
// positive product, a difference x - y of such numbers, or a copy of one), so
// a partial sum that starts at +0.0 is never -0.0, and s - (+0.0) + (+0.0)
// is s bit for bit; every sum is therefore the reference's own, add for add.
// A step's partners are picked by warp ballots; a full sum's pairs are
// marked in a bitmask as their terms are formed and compacted in pair order
// by a block-wide scan.
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <new>

#include "common.cuh"
#include "philox.cuh"

namespace jmm {
namespace plain {

constexpr int kThreads = 1024;
constexpr uint64_t kMaxN = 2900;  // partner terms of one step must fit in shared memory

struct Scalars {
  uint64_t sn;
  uint64_t rng_block;
  uint32_t rng_slot;
  uint32_t error;
  uint32_t words[4];
  double l, max_step, max_dl;
  double bf, ran;  // persist between steps like mcs->bf and the file-static ran
  double tot[9];
  uint64_t d_acc[2], v_acc[2];
  double thermo[12];
  uint64_t echeck_count, echeck_resets;
  double echeck_e, echeck_e_before;
  uint64_t hist_ticks;  // histogram accumulations (ugrho calls) since set-up
  uint64_t rho_l_bits;  // update_thermo's N / L, kept for the box length with these bits
  double rho;
};

struct Args {
  Scalars *s;
  double *r;        // N positions
  double *r_trial;  // N trial positions (volume move, fad)
  double *rij;      // N*N, stored separation r_j - r_i at i*N+j (i<j)
  double *q;        // 9*N*N stored pair quantities
  double *scratch;  // 9*P pair terms of a full sum, packed row-major over (i<j)
  uint32_t *mask;   // bit p: pair p of scratch has a term other than +0.0
  double *comp;     // the marked pairs' terms in pair order (9 per pair)
  uint64_t nwords;  // words of mask
  uint64_t n, nn, npairs, num_trial_types;
  int32_t potential, nbn;
  int32_t use_qavlj;
  int32_t stage_old;  // qad2 stages the stored pair terms in shared memory (where they fit)
  double cutoff, t, p;
  uint64_t seed, eci;
  // rho(x) and g(x) histograms, bins [0, rhonb) density, then gns x gnb
  // separation bins slice after slice.  The reference adds the current counts
  // to the sums at every accumulation (ugrho); here each bin keeps its sum up
  // to the accumulation at which its count last changed (h_acc, h_last), so
  // that an accumulation costs O(1) instead of O(bins).
  int32_t *h_val;               // current counts (rhol, gl)
  long long *h_acc;             // sums up to accumulation h_last
  unsigned long long *h_last;
  uint64_t rhonb, gnb;
  int32_t gns, hist_on;
  double rbw, gsw, gbw;
};

struct Ctl {
  uint64_t nm;
  double rn, md, rt;
  double dl, lnew, lrat1;
  double ran, bf;
  double sum[9];
  double part[2][9];  // qad2: the partner sums over i < nm and over i > nm
  uint64_t ncomp;     // pairs compacted for a full sum
  uint32_t wsum[32];  // per-warp counts of the compaction scan
  // qad2 with its old terms staged: bit p of the partner slots, set where any
  // of the partner's eighteen terms (new and stored) is not +0.0
  uint32_t nz[48];
  int32_t wall, accept, kind, outcome, reset, pad;
};
constexpr uint64_t kNzSlots = 32 * 48;

// ---- pair potentials (FP64, the reference's operand order) --------------

// The reference forms r^-6 and r^-12 for every pair and uses them only within
// the cut-off; here they are formed there only (same values where used).
__device__ __forceinline__ void phi_lj(double d, double cut, bool virial, double *phi) {
  double phitot = 0, phi6 = 0, phi12 = 0, vir6 = 0, vir12 = 0, virtot = 0;
  double hv6 = 0, hv12 = 0, hvtot = 0;
  if (d <= cut) {
    const double d3 = __dmul_rn(__dmul_rn(d, d), d);
    const double r6 = __ddiv_rn(1.0, __dmul_rn(d3, d3));
    const double r12 = __dmul_rn(r6, r6);
    phi6 = __dmul_rn(4.0, r6);
    phi12 = __dmul_rn(4.0, r12);
    phitot = __dsub_rn(phi12, phi6);
    if (virial) {
      vir6 = __dmul_rn(24.0, r6);
      vir12 = __dmul_rn(48.0, r12);
      virtot = __dsub_rn(vir12, vir6);
      hv6 = __dmul_rn(144.0, r6);
      hv12 = __dmul_rn(576.0, r12);
      hvtot = __dsub_rn(hv12, hv6);
    }
  }
  phi[0] = phitot;
  phi[1] = virtot;
  phi[2] = phi12;
  phi[3] = vir12;
  phi[4] = phi6;
  phi[5] = vir6;
  phi[6] = hvtot;
  phi[7] = hv12;
  phi[8] = hv6;
}

// phiHarmoniccut leaves phi[2..8] unwritten (and phi[1] undefined without the
// virial flag); they are 0 here.
__device__ __forceinline__ void phi_harmonic(double d, double cut, bool virial, double l,
                                             double *phi) {
#pragma unroll
  for (int k = 0; k < 9; ++k) phi[k] = 0.0;
  if (d <= 0) {
    phi[0] = 10E10;
    phi[1] = 10E10;
  } else if (d < cut) {
    double rijm = __dsub_rn(d, 1.0);
    phi[0] = __dmul_rn(rijm, rijm);
    phi[1] = virial ? __dmul_rn(__dmul_rn(__ddiv_rn(2.0, l), d), rijm) : 0.0;
  }
}

__device__ __forceinline__ void phi_eval(const Args &a, double d, bool virial, double l,
                                         double *phi) {
  if (a.potential == JMM_POT_HARMONIC)
    phi_harmonic(d, a.cutoff, virial, l, phi);
  else
    phi_lj(d, a.potential == JMM_POT_LJ ? (double)INFINITY : a.cutoff, virial, phi);
}

__device__ __forceinline__ bool pair_cut(const Args &a, uint64_t i, uint64_t j) {
  return a.nbn >= 0 && (j - i) > (uint64_t)a.nbn;
}

__device__ __forceinline__ uint64_t packed_index(uint64_t i, uint64_t j, uint64_t n) {
  return i * (n - 1) - (i * (i + 1)) / 2 + j - 1;
}

// ---- the stream the reference consumes (thread 0 only) ----------------

__device__ void open_block(Scalars *S, uint64_t seed) {
  S->rng_block += 1;
  Words4 w = step_words(seed, S->rng_block, 0u);
#pragma unroll
  for (int k = 0; k < 4; ++k) S->words[k] = w.w[k];
  S->rng_slot = 0;
}

__device__ uint64_t draw_int(Scalars *S, uint64_t seed, uint64_t n) {
  open_block(S, seed);
  S->rng_slot = 1;
  return word_to_index(S->words[0], n);
}

__device__ double draw_uniform(Scalars *S, uint64_t seed) {
  if (S->rng_slot >= 4) {
    open_block(S, seed);
    S->rng_slot = 1;
  }
  uint32_t w = S->words[S->rng_slot];
  S->rng_slot += 1;
  return word_to_unit(w);
}

// ---- block-wide pieces ----------------------------------------------------

__device__ __forceinline__ bool any_term(const double *phi) {
  unsigned long long bits = 0;
#pragma unroll
  for (int k = 0; k < 9; ++k) bits |= (unsigned long long)__double_as_longlong(phi[k]);
  return bits != 0;  // some term other than +0.0
}

// Clears the pair mask before a full pass over the pairs (all threads).
__device__ void clear_mask(const Args &a) {
  for (uint64_t w = threadIdx.x; w < a.nwords; w += blockDim.x) a.mask[w] = 0u;
  __syncthreads();
}

// Marks pair q (packed index) when nz.  Called in a row loop where the lanes
// of one iteration hold consecutive pair indices from lane 0 on, and
// `left` pairs of the row remain from lane 0's: the lanes of the iteration
// are 0 .. min(left, 32) - 1.
__device__ __forceinline__ void mark_pairs(const Args &a, uint64_t q, bool nz, uint64_t left) {
  const unsigned act = left >= 32 ? 0xffffffffu : ((1u << left) - 1u);
  const unsigned bits = __ballot_sync(act, nz);
  if ((threadIdx.x & 31) == 0 && bits) {  // lane 0 holds the lowest index q
    const uint64_t w = q >> 5;
    const unsigned sh = (unsigned)(q & 31);
    atomicOr(a.mask + w, bits << sh);
    if (sh && (bits >> (32 - sh))) atomicOr(a.mask + w + 1, bits >> (32 - sh));
  }
}

// Pair terms of every pair at positions `x` (box length `l` for HARMONIC's
// virial) into scratch[k*9 + q]; pairs beyond NBN get zeros.  Marks the
// pairs with a term other than +0.0.
__device__ void full_terms(const Args &a, const double *x, bool virial, double l) {
  const uint64_t n = a.n;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
  clear_mask(a);
  for (uint64_t i = warp; i < n; i += nwarps) {
    const uint64_t row = packed_index(i, i + 1, n);
    for (uint64_t j = i + 1 + lane; j < n; j += 32) {
      double phi[9];
      if (pair_cut(a, i, j)) {
#pragma unroll
        for (int k = 0; k < 9; ++k) phi[k] = 0.0;
      } else {
        phi_eval(a, __dsub_rn(x[j], x[i]), virial, l, phi);
      }
      const uint64_t q = row + (j - i - 1);
      double *dst = a.scratch + q * 9;
#pragma unroll
      for (int k = 0; k < 9; ++k) dst[k] = phi[k];
      mark_pairs(a, q, any_term(phi), n - (j - lane));
    }
  }
}

// The marked pairs' terms, in pair order, into comp (pair of rank r at
// comp[9r ..]); their number into ctl.ncomp.  A block-wide exclusive scan of
// the mask words' bit counts gives each word its first rank.  All threads.
__device__ void compact_terms(const Args &a, Ctl &ctl) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  uint64_t base = 0;
  for (uint64_t w0 = 0; w0 < a.nwords; w0 += blockDim.x) {
    const uint64_t w = w0 + threadIdx.x;
    const uint32_t m = w < a.nwords ? a.mask[w] : 0u;
    const uint32_t c = (uint32_t)__popc(m);
    uint32_t x = c;  // inclusive scan within the warp
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) ctl.wsum[warp] = x;
    __syncthreads();
    if (warp == 0) {
      uint32_t t = lane < nwarps ? ctl.wsum[lane] : 0u;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, t, o);
        if (lane >= o) t += y;
      }
      if (lane < nwarps) ctl.wsum[lane] = t;
    }
    __syncthreads();
    uint64_t r = base + (warp ? ctl.wsum[warp - 1] : 0u) + (x - c);
    for (uint32_t mm = m; mm; mm &= mm - 1u, ++r) {
      const uint64_t p = w * 32 + (uint64_t)(__ffs(mm) - 1);
      const double *src = a.scratch + p * 9;
      double *dst = a.comp + r * 9;
#pragma unroll
      for (int k = 0; k < 9; ++k) dst[k] = src[k];
    }
    base += ctl.wsum[nwarps - 1];
    __syncthreads();
  }
  if (threadIdx.x == 0) ctl.ncomp = base;
  __syncthreads();
}

// The nine full sums of the scratch terms in pair order, by lanes 0..8 of
// warp 0 over the compacted terms (unrolled so that many of the independent
// loads are in flight ahead of the dependent adds).  All threads.
__device__ void full_sums(const Args &a, Ctl &ctl) {
  compact_terms(a, ctl);
  if (threadIdx.x < 9) {
    const int k = threadIdx.x;
    const uint64_t nc = ctl.ncomp;
    double s = 0.0;
#pragma unroll 32
    for (uint64_t p = 0; p < nc; ++p) s = __dadd_rn(s, a.comp[p * 9 + k]);
    ctl.sum[k] = s;
  }
}

// Scratch terms into the stored pair arrays, with separations from `x`.
__device__ void commit_all(const Args &a, const double *x) {
  const uint64_t n = a.n;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
  for (uint64_t i = warp; i < n; i += nwarps) {
    const uint64_t row = packed_index(i, i + 1, n);
    for (uint64_t j = i + 1 + lane; j < n; j += 32) {
      const uint64_t ind = i * n + j;
      const double *src = a.scratch + (row + (j - i - 1)) * 9;
      a.rij[ind] = __dsub_rn(x[j], x[i]);
#pragma unroll
      for (int k = 0; k < 9; ++k) a.q[k * a.nn + ind] = src[k];
    }
  }
}

__device__ void update_thermo(Scalars *S, uint64_t n) {
  double *acc = S->thermo;
  const double l = S->l, e = S->tot[JMM_Q_E], vir = S->tot[JMM_Q_VIR], hv = S->tot[JMM_Q_HV];
  const double rho = __ddiv_rn((double)n, l);
  acc[0] = __dadd_rn(acc[0], rho);
  acc[1] = __dadd_rn(acc[1], __dmul_rn(rho, rho));
  acc[2] = __dadd_rn(acc[2], l);
  acc[3] = __dadd_rn(acc[3], __dmul_rn(l, l));
  acc[4] = __dadd_rn(acc[4], e);
  acc[5] = __dadd_rn(acc[5], __dmul_rn(e, e));
  acc[6] = __dadd_rn(acc[6], __dmul_rn(l, e));
  acc[7] = __dadd_rn(acc[7], vir);
  acc[8] = __dadd_rn(acc[8], __dmul_rn(vir, vir));
  acc[9] = __dadd_rn(acc[9], __dmul_rn(e, vir));
  acc[10] = __dadd_rn(acc[10], hv);
  acc[11] = __dadd_rn(acc[11], __dmul_rn(hv, hv));
}

// Accumulator k < 12 of update_thermo, for lane k: the same add of the same
// term, with the term written as x * y (y = 1 for the plain sums, and x * 1 is
// exact), so that the twelve adds are one FP64 instruction and no branch.
// N / L is divided afresh only when L has changed (the same quotient).
__device__ __forceinline__ void update_thermo_lane(Scalars *S, uint64_t n, int k) {
  const double l = S->l, e = S->tot[JMM_Q_E], vir = S->tot[JMM_Q_VIR], hv = S->tot[JMM_Q_HV];
  const uint64_t lbits = (uint64_t)__double_as_longlong(l);
  const double rho = lbits == S->rho_l_bits ? S->rho : __ddiv_rn((double)n, l);
  __syncwarp(0xfffu);
  if (k == 0) {
    S->rho_l_bits = lbits;
    S->rho = rho;
  }
  const double x = k < 2 ? rho : k < 4 ? l : k < 6 ? e : k == 6 ? l : k < 9 ? vir : k == 9 ? e : hv;
  const double y = k == 1                 ? rho
                   : k == 3               ? l
                   : (k == 5 || k == 6)   ? e
                   : (k == 8 || k == 9)   ? vir
                   : k == 11              ? hv
                                          : 1.0;
  S->thermo[k] = __dadd_rn(S->thermo[k], __dmul_rn(x, y));
}

// ---- rho(x) and g(x) histograms ---------------------------------------------

// Bin indices as the reference forms them: (long) floor(x/w + nb/2.0).
__device__ __forceinline__ long long rho_bin(const Args &a, double x) {
  return (long long)floor(__dadd_rn(__ddiv_rn(x, a.rbw), __ddiv_rn((double)a.rhonb, 2.0)));
}
__device__ __forceinline__ long long slice_of(const Args &a, double x) {
  return (long long)floor(__dadd_rn(__ddiv_rn(x, a.gsw), __ddiv_rn((double)a.gns, 2.0)));
}
// Separation bin of qagrho: (unsigned long) floor(|d| / gbw).
__device__ __forceinline__ long long sep_bin(const Args &a, double d) {
  return (long long)(unsigned long long)floor(__ddiv_rn(fabs(d), a.gbw));
}

// Brings bin b's sum up to accumulation T before its count changes; the
// first caller of a step for a bin does it (the count is not yet changed:
// changes are applied after a barrier).
__device__ __forceinline__ void hist_flush(const Args &a, uint64_t b, uint64_t T) {
  const unsigned long long old = atomicExch(&a.h_last[b], (unsigned long long)T);
  if (old != T) a.h_acc[b] += (long long)a.h_val[b] * (long long)(T - old);
}

__device__ __forceinline__ void hist_touch(const Args &a, uint64_t b, uint64_t T, int phase,
                                           int delta) {
  if (phase == 0)
    hist_flush(a, b, T);
  else
    atomicAdd(&a.h_val[b], delta);
}

// qagrho: particle ctl.nm moved by ctl.md, a.r[nm] already holds the new
// position (the old one is formed as r[nm] - md, as the reference does).
// Phase 0 flushes every bin the move touches, phase 1 changes the counts.
__device__ void qagrho(const Args &a, Scalars *S, const Ctl &ctl) {
  const uint64_t n = a.n, nm = ctl.nm, nm1 = n - 1;
  const uint64_t T = S->hist_ticks;
  const double xn = a.r[nm];
  const double xo = __dsub_rn(xn, ctl.md);
  const long long rb1 = rho_bin(a, xo), rb2 = rho_bin(a, xn);
  const long long gs11 = slice_of(a, xo), gs12 = slice_of(a, xn);
  const bool v11 = gs11 >= 0 && gs11 < a.gns, v12 = gs12 >= 0 && gs12 < a.gns;
  const long long nb = (long long)a.gnb;
  for (int phase = 0; phase < 2; ++phase) {
    if (threadIdx.x == 0) {
      if (rb1 >= 0 && rb1 < (long long)a.rhonb) hist_touch(a, rb1, T, phase, -1);
      if (rb2 >= 0 && rb2 < (long long)a.rhonb) hist_touch(a, rb2, T, phase, +1);
    }
    for (uint64_t p = threadIdx.x; p < nm1; p += blockDim.x) {
      const uint64_t ii = p < nm ? p : p + 1;
      const double xi = a.r[ii];
      const long long gs2 = slice_of(a, xi);
      const bool v2 = gs2 >= 0 && gs2 < a.gns;
      const long long gb1 = sep_bin(a, __dsub_rn(xo, xi));
      const long long gb2 = sep_bin(a, __dsub_rn(xn, xi));
      const bool vb1 = gb1 >= 0 && gb1 < nb, vb2 = gb2 >= 0 && gb2 < nb;
      const uint64_t g0 = a.rhonb;
      if (v11 && vb1) hist_touch(a, g0 + gs11 * nb + gb1, T, phase, -1);
      if (v12 && vb2) hist_touch(a, g0 + gs12 * nb + gb2, T, phase, +1);
      if (v2 && vb1) hist_touch(a, g0 + gs2 * nb + gb1, T, phase, -1);
      if (v2 && vb2) hist_touch(a, g0 + gs2 * nb + gb2, T, phase, +1);
    }
    __syncthreads();
  }
}

// fgrho: counts of the current positions and stored separations, after every
// bin's sum has been brought up to the current accumulation.  A negative
// separation (particles that passed each other) gives a negative bin, which
// the reference writes out of bounds; here it is not counted.
__device__ void fgrho(const Args &a, Scalars *S) {
  const uint64_t n = a.n, T = S->hist_ticks;
  const uint64_t total = a.rhonb + (uint64_t)a.gns * a.gnb;
  for (uint64_t b = threadIdx.x; b < total; b += blockDim.x) {
    a.h_acc[b] += (long long)a.h_val[b] * (long long)(T - a.h_last[b]);
    a.h_last[b] = T;
    a.h_val[b] = 0;
  }
  __syncthreads();
  for (uint64_t i = threadIdx.x; i < n; i += blockDim.x) {
    const long long rb = rho_bin(a, a.r[i]);
    if (rb >= 0 && rb < (long long)a.rhonb) atomicAdd(&a.h_val[rb], 1);
  }
  const long long nb = (long long)a.gnb;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
  for (uint64_t i = warp; i < n; i += nwarps) {
    const long long gs1 = slice_of(a, a.r[i]);
    for (uint64_t j = i + 1 + lane; j < n; j += 32) {
      const long long gb = (long long)floor(__ddiv_rn(a.rij[i * n + j], a.gbw));
      if (gb < 0 || gb >= nb) continue;
      const long long gs2 = slice_of(a, a.r[j]);
      if (gs1 >= 0 && gs1 < a.gns) atomicAdd(&a.h_val[a.rhonb + gs1 * nb + gb], 1);
      if (gs2 >= 0 && gs2 < a.gns) atomicAdd(&a.h_val[a.rhonb + gs2 * nb + gb], 1);
    }
  }
  __syncthreads();
}

// ugrho: one accumulation.
__device__ __forceinline__ void ugrho(const Args &a, Scalars *S) {
  if (threadIdx.x == 0) S->hist_ticks += 1;
}

// ---- the moves --------------------------------------------------------------

// qad2: displacement of particle ctl.nm by (rn - 0.5) * 2 * maxStep.
__device__ void qad2(const Args &a, Scalars *S, Ctl &ctl, double *s_new, double *s_rij,
                     const jmm_draw *rp) {
  const uint64_t n = a.n, nm = ctl.nm, nm1 = n - 1;
  if (threadIdx.x == 0) {
    const double md = __dmul_rn(__dmul_rn(__dsub_rn(ctl.rn, 0.5), 2.0), S->max_step);
    const double rt = __dadd_rn(a.r[nm], md);
    ctl.md = md;
    ctl.rt = rt;
    ctl.kind = JMM_KIND_DISPLACEMENT;
    ctl.ran = NAN;
    ctl.bf = NAN;
    ctl.wall = fabs(rt) > __dmul_rn(S->l, 0.5);  // L * 0.5 is L / 2.0 bit for bit
    if (ctl.wall) {
      S->d_acc[1] += 1;
      ctl.outcome = JMM_OUT_REJECT_WALL;
    }
  }
  __syncthreads();
  if (ctl.wall) return;
  const double md = ctl.md, l = S->l;
  double *s_old = s_rij + nm1;  // 9 * nm1 when a.stage_old
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  // with the old terms staged, each warp marks its 32 partner slots whose
  // eighteen terms are not all +0.0 as it forms them
  const bool use_nz = a.stage_old && nm1 <= kNzSlots;
  for (uint64_t base = threadIdx.x - lane; base < nm1; base += blockDim.x) {
    const uint64_t p = base + lane;
    unsigned long long bits = 0;
    if (p < nm1) {
      const uint64_t i = p < nm ? p : p + 1;
      const uint64_t lo = i < nm ? i : nm, hi = i < nm ? nm : i;
      const uint64_t ind = lo * n + hi;
      const double rt = (i < nm) ? __dadd_rn(a.rij[ind], md) : __dsub_rn(a.rij[ind], md);
      double phi[9];
      if (pair_cut(a, lo, hi)) {
#pragma unroll
        for (int k = 0; k < 9; ++k) phi[k] = 0.0;
      } else {
        phi_eval(a, rt, true, l, phi);
      }
      s_rij[p] = rt;
#pragma unroll
      for (int k = 0; k < 9; ++k) {
        s_new[k * nm1 + p] = phi[k];
        bits |= (unsigned long long)__double_as_longlong(phi[k]);
      }
      if (a.stage_old) {
#pragma unroll
        for (int k = 0; k < 9; ++k) {
          const double v = a.q[k * a.nn + ind];
          s_old[k * nm1 + p] = v;
          bits |= (unsigned long long)__double_as_longlong(v);
        }
      }
    }
    if (use_nz) {
      const unsigned m = __ballot_sync(0xffffffffu, bits != 0);
      if (lane == 0) ctl.nz[base / 32] = m;
    }
  }
  __syncthreads();
  // the reference's order: (sum - old) + new over the partners i < nm (lanes
  // 0-8 of warp 0) and, as a separate sum, over i > nm (lanes 0-8 of warp 1):
  // two dependent FP64 chains, which overlap only in different warps.  The
  // nine summing lanes add the partners marked above (any of the eighteen
  // terms other than +0.0) in index order; the others would add +0.0 twice.
  // Without the marks the 32 lanes of the warp test 32 partners at a time.
  if (warp < 2 && use_nz) {
    const uint64_t p0 = warp == 0 ? 0 : nm, p1 = warp == 0 ? nm : nm1;
    double sp = 0.0;
    if (lane < 9) {
      for (uint64_t w = p0 / 32; w * 32 < p1; ++w) {
        unsigned m = ctl.nz[w];
        if (w * 32 < p0) m &= ~0u << (unsigned)(p0 - w * 32);
        if (p1 - w * 32 < 32) m &= (1u << (unsigned)(p1 - w * 32)) - 1u;
        for (; m; m &= m - 1u) {
          const uint64_t pp = w * 32 + (uint64_t)(__ffs(m) - 1);
          sp = __dadd_rn(__dsub_rn(sp, s_old[(uint64_t)lane * nm1 + pp]),
                         s_new[(uint64_t)lane * nm1 + pp]);
        }
      }
      ctl.part[warp][lane] = sp;
    }
  } else if (warp < 2) {
    const uint64_t p0 = warp == 0 ? 0 : nm, p1 = warp == 0 ? nm : nm1;
    // stored term k of partner slot p
    auto old_term = [&](int k, uint64_t p) -> double {
      if (a.stage_old) return s_old[(uint64_t)k * nm1 + p];
      const double *old = a.q + (uint64_t)k * a.nn;
      return warp == 0 ? old[p * n + nm] : old[nm * n + p + 1];
    };
    double sp = 0.0;
    for (uint64_t c0 = p0; c0 < p1; c0 += 32) {
      const uint64_t p = c0 + lane;
      unsigned long long bits = 0;
      if (p < p1) {
#pragma unroll
        for (int k = 0; k < 9; ++k)
          bits |= (unsigned long long)__double_as_longlong(s_new[(uint64_t)k * nm1 + p]) |
                  (unsigned long long)__double_as_longlong(old_term(k, p));
      }
      unsigned m = __ballot_sync(0xffffffffu, bits != 0);
      if (lane < 9) {
        for (; m; m &= m - 1u) {
          const uint64_t pp = c0 + (uint64_t)(__ffs(m) - 1);
          sp = __dadd_rn(__dsub_rn(sp, old_term(lane, pp)), s_new[(uint64_t)lane * nm1 + pp]);
        }
      }
    }
    if (lane < 9) ctl.part[warp][lane] = sp;
  }
  __syncthreads();
  if (threadIdx.x < 9)
    ctl.sum[threadIdx.x] = __dadd_rn(ctl.part[0][threadIdx.x], ctl.part[1][threadIdx.x]);
  __syncthreads();
  if (threadIdx.x == 0) {
    const double de = ctl.sum[JMM_Q_E];
    if (de > 0) {
      S->ran = rp ? rp->ran : draw_uniform(S, a.seed);
      S->bf = exp(__ddiv_rn(-de, a.t));
      ctl.ran = S->ran;
      ctl.bf = S->bf;
    }
    const bool acc = (de <= 0) || (S->bf > S->ran);
    if (acc) {
      S->d_acc[0] += 1;
      a.r[nm] = ctl.rt;
      ctl.outcome = JMM_OUT_ACCEPT;
    } else {
      S->d_acc[1] += 1;
      ctl.outcome = JMM_OUT_REJECT;
    }
    ctl.accept = acc;
  }
  __syncthreads();
  if (ctl.accept) {
    // E += dE and the other eight totals, one per lane (one FP64 add each).
    if (threadIdx.x < 9)
      S->tot[threadIdx.x] = __dadd_rn(S->tot[threadIdx.x], ctl.sum[threadIdx.x]);
    for (uint64_t p = threadIdx.x; p < nm1; p += blockDim.x) {
      const uint64_t i = p < nm ? p : p + 1;
      const uint64_t ind = i < nm ? i * n + nm : nm * n + i;
      a.rij[ind] = s_rij[p];
#pragma unroll
      for (int k = 0; k < 9; ++k) a.q[k * a.nn + ind] = s_new[k * nm1 + p];
    }
  }
  __syncthreads();
  if (ctl.accept && a.hist_on) qagrho(a, S, ctl);  // src/jmmMCState.cpp:1431
}

// qad2 with its histogram accumulation, which the reference makes whatever
// the outcome, the wall rejection included (src/jmmMCState.cpp:1453).
__device__ void qad2_step(const Args &a, Scalars *S, Ctl &ctl, double *s_new, double *s_rij,
                          const jmm_draw *rp) {
  qad2(a, S, ctl, s_new, s_rij, rp);
  if (a.hist_on) ugrho(a, S);
}

// fav: full-energy volume move, linear dl uniform in +-maxdl.
__device__ void fav(const Args &a, Scalars *S, Ctl &ctl, const jmm_draw *rp) {
  const uint64_t n = a.n;
  if (threadIdx.x == 0) {
    const double dl = __dmul_rn(__dmul_rn(__dsub_rn(ctl.rn, 0.5), 2.0), S->max_dl);
    const double lnew = __dadd_rn(S->l, dl);
    ctl.dl = dl;
    ctl.lnew = lnew;
    ctl.lrat1 = __ddiv_rn(lnew, S->l);
    ctl.kind = JMM_KIND_VOLUME;
    ctl.ran = NAN;
  }
  __syncthreads();
  for (uint64_t i = threadIdx.x; i < n; i += blockDim.x) a.r_trial[i] = __dmul_rn(a.r[i], ctl.lrat1);
  __syncthreads();
  full_terms(a, a.r_trial, true, ctl.lnew);
  __syncthreads();
  full_sums(a, ctl);
  __syncthreads();
  if (threadIdx.x == 0) {
    const double arg = __dadd_rn(
        __ddiv_rn(-__dadd_rn(__dsub_rn(ctl.sum[JMM_Q_E], S->tot[JMM_Q_E]), __dmul_rn(a.p, ctl.dl)),
                  a.t),
        __dmul_rn((double)n, log(ctl.lrat1)));
    S->bf = exp(arg);
    ctl.bf = S->bf;
    if (S->bf < 1.0) {
      S->ran = rp ? rp->ran : draw_uniform(S, a.seed);
      ctl.ran = S->ran;
    }
    const bool acc = (S->bf >= 1.0) || (S->bf > S->ran);
    if (acc) {
      S->v_acc[0] += 1;
      S->l = __dadd_rn(S->l, ctl.dl);
#pragma unroll
      for (int k = 0; k < 9; ++k) S->tot[k] = ctl.sum[k];
      ctl.outcome = JMM_OUT_ACCEPT;
    } else {
      S->v_acc[1] += 1;
      ctl.outcome = JMM_OUT_REJECT;
    }
    ctl.accept = acc;
  }
  __syncthreads();
  if (ctl.accept) {
    for (uint64_t i = threadIdx.x; i < n; i += blockDim.x) a.r[i] = a.r_trial[i];
    commit_all(a, a.r_trial);
  }
  __syncthreads();
}

// qavLJ with a nine-entry phi buffer.  The reference's six-entry buffer
// (src/jmmMCState.cpp:1651) overflows and aborts there; nothing here is
// pinned to it.
__device__ void qav_lj(const Args &a, Scalars *S, Ctl &ctl, const jmm_draw *rp) {
  const uint64_t n = a.n;
  __shared__ double lrat1_s;
  if (threadIdx.x == 0) {
    const double dl = __dmul_rn(__dmul_rn(__dsub_rn(ctl.rn, 0.5), 2.0), S->max_dl);
    const double lrat1 = __ddiv_rn(__dadd_rn(S->l, dl), S->l);
    const double lrat3 = __dmul_rn(__dmul_rn(lrat1, lrat1), lrat1);
    const double lrat6 = __ddiv_rn(1.0, __dmul_rn(lrat3, lrat3));
    const double lrat12 = __dmul_rn(lrat6, lrat6);
    const double e12t = __dmul_rn(lrat12, S->tot[JMM_Q_E12]);
    const double e6t = __dmul_rn(lrat6, S->tot[JMM_Q_E6]);
    const double de = __dsub_rn(__dsub_rn(e12t, e6t), S->tot[JMM_Q_E]);
    const double arg =
        __dadd_rn(__ddiv_rn(-__dadd_rn(de, __dmul_rn(a.p, dl)), a.t), __dmul_rn((double)n, log(lrat1)));
    S->bf = exp(arg);
    ctl.kind = JMM_KIND_VOLUME;
    ctl.bf = S->bf;
    ctl.ran = NAN;
    if (S->bf < 1.0) {
      S->ran = rp ? rp->ran : draw_uniform(S, a.seed);
      ctl.ran = S->ran;
    }
    const bool acc = (S->bf >= 1.0) || (S->bf > S->ran);
    if (acc) {
      S->v_acc[0] += 1;
      S->tot[JMM_Q_E] = __dadd_rn(S->tot[JMM_Q_E], de);
      S->tot[JMM_Q_E12] = e12t;
      S->tot[JMM_Q_E6] = e6t;
      S->l = __dadd_rn(S->l, dl);
      const double lrat7 = __ddiv_rn(lrat6, lrat1);
      const double lrat13 = __ddiv_rn(lrat12, lrat1);
      S->tot[JMM_Q_VIR6] = __dmul_rn(lrat7, S->tot[JMM_Q_VIR6]);
      S->tot[JMM_Q_VIR12] = __dmul_rn(lrat13, S->tot[JMM_Q_VIR12]);
      S->tot[JMM_Q_VIR] = __dsub_rn(
          __dadd_rn(__ddiv_rn(__dmul_rn((double)n, a.t), S->l), S->tot[JMM_Q_VIR12]),
          S->tot[JMM_Q_VIR6]);
      ctl.outcome = JMM_OUT_ACCEPT;
    } else {
      S->v_acc[1] += 1;
      ctl.outcome = JMM_OUT_REJECT;
    }
    ctl.accept = acc;
    lrat1_s = lrat1;
  }
  __syncthreads();
  if (ctl.accept) {
    const double lrat1 = lrat1_s, l = S->l;
    for (uint64_t i = threadIdx.x; i < n; i += blockDim.x) a.r[i] = __dmul_rn(lrat1, a.r[i]);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
    for (uint64_t i = warp; i < n; i += nwarps) {
      for (uint64_t j = i + 1 + lane; j < n; j += 32) {
        const uint64_t ind = i * n + j;
        const double rij = __dmul_rn(lrat1, a.rij[ind]);
        a.rij[ind] = rij;
        double phi[9];
        phi_eval(a, rij, true, l, phi);
#pragma unroll
        for (int k = 0; k < 9; ++k) a.q[k * a.nn + ind] = phi[k];
      }
    }
  }
  __syncthreads();
  if (a.hist_on) {  // fgrho on acceptance, ugrho always (src/jmmMCState.cpp:1717, :1726)
    if (ctl.accept) fgrho(a, S);
    ugrho(a, S);
  }
}

// ECheck: full FP64 re-sum of E from the positions; on |dE| > 1e-4 rebuild
// every pair and total.
__device__ void echeck(const Args &a, Scalars *S, Ctl &ctl) {
  const uint64_t n = a.n;
  full_terms(a, a.r, false, S->l);
  __syncthreads();
  compact_terms(a, ctl);
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (uint64_t p = 0; p < ctl.ncomp; ++p) s = __dadd_rn(s, a.comp[p * 9]);
    S->echeck_count += 1;
    S->echeck_e = s;
    S->echeck_e_before = S->tot[JMM_Q_E];
    ctl.reset = fabs(__dsub_rn(s, S->tot[JMM_Q_E])) > 0.0001;
    if (ctl.reset) S->echeck_resets += 1;
  }
  __syncthreads();
  if (!ctl.reset) return;
  const double l = S->l;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
  clear_mask(a);
  for (uint64_t i = warp; i < n; i += nwarps) {
    const uint64_t row = packed_index(i, i + 1, n);
    for (uint64_t j = i + 1 + lane; j < n; j += 32) {
      const uint64_t ind = i * n + j;
      double phi[9];
      if (pair_cut(a, i, j)) {
#pragma unroll
        for (int k = 0; k < 9; ++k) phi[k] = 0.0;
      } else {
        const double rij = __dsub_rn(a.r[j], a.r[i]);
        a.rij[ind] = rij;
        phi_eval(a, rij, true, l, phi);
      }
      const uint64_t q = row + (j - i - 1);
      double *dst = a.scratch + q * 9;
#pragma unroll
      for (int k = 0; k < 9; ++k) {
        a.q[k * a.nn + ind] = phi[k];
        dst[k] = phi[k];
      }
      mark_pairs(a, q, any_term(phi), n - (j - lane));
    }
  }
  __syncthreads();
  full_sums(a, ctl);
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < 9; ++k) S->tot[k] = ctl.sum[k];
  }
  __syncthreads();
}

// ---- kernels ------------------------------------------------------------------

static_assert(sizeof(Scalars) % 8 == 0, "Scalars copies as 8-byte words");

// The chain's scalars live in shared memory for the launch (copied in at the
// start, back at the end), so that thread 0's serial part of a step (draws,
// the decision, counters, totals) waits on no global-memory round trip.
__global__ void __launch_bounds__(kThreads, 1)
    steps_kernel(Args a, uint64_t n_steps, const jmm_draw *replay, jmm_step_record *log) {
  extern __shared__ double smem[];
  __shared__ Ctl ctl;
  __shared__ Scalars s_sh;
  for (uint32_t k = threadIdx.x; k < sizeof(Scalars) / 8; k += blockDim.x)
    reinterpret_cast<uint64_t *>(&s_sh)[k] = reinterpret_cast<const uint64_t *>(a.s)[k];
  __syncthreads();
  Scalars *S = &s_sh;
  const uint64_t nm1 = a.n - 1;
  double *s_new = smem;
  double *s_rij = smem + 9 * nm1;
  for (uint64_t step = 0; step < n_steps; ++step) {
    const jmm_draw *rp = replay ? replay + step : nullptr;
    if (threadIdx.x == 0) {
      S->sn += 1;
      if (rp) {
        ctl.nm = rp->nm;
        ctl.rn = rp->rn;
      } else {
        ctl.nm = draw_int(S, a.seed, a.num_trial_types);
        ctl.rn = draw_uniform(S, a.seed);
      }
      ctl.outcome = JMM_OUT_REJECT;
      ctl.kind = JMM_KIND_DISPLACEMENT;
      ctl.ran = NAN;
      ctl.bf = NAN;
    }
    __syncthreads();
    if (ctl.nm < a.n) {
      qad2_step(a, S, ctl, s_new, s_rij, rp);
    } else if (ctl.nm == a.n) {
      if (a.use_qavlj)
        qav_lj(a, S, ctl, rp);
      else
        fav(a, S, ctl, rp);
    } else if (threadIdx.x == 0) {
      S->error = JMM_ERR_INVALID;  // trial type beyond N: "unknown trial type"
    }
    __syncthreads();
    if (a.eci && (S->sn % a.eci) == 0) echeck(a, S, ctl);
    if (threadIdx.x < 12) update_thermo_lane(S, a.n, threadIdx.x);
    if (threadIdx.x == 0) {
      if (log) {
        jmm_step_record rec;
        rec.sn = S->sn;
        rec.nm = ctl.nm;
        rec.rn = ctl.rn;
        rec.ran = ctl.ran;
        rec.bf = ctl.bf;
        rec.e = S->tot[JMM_Q_E];
        rec.vir = S->tot[JMM_Q_VIR];
        rec.hv = S->tot[JMM_Q_HV];
        rec.l = S->l;
        rec.kind = ctl.kind;
        rec.outcome = ctl.outcome;
        log[step] = rec;
      }
    }
    __syncthreads();
  }
  for (uint32_t k = threadIdx.x; k < sizeof(Scalars) / 8; k += blockDim.x)
    reinterpret_cast<uint64_t *>(a.s)[k] = reinterpret_cast<const uint64_t *>(&s_sh)[k];
}

__global__ void __launch_bounds__(kThreads, 1) fad_kernel(Args a, uint64_t nm, double d) {
  __shared__ Ctl ctl;
  Scalars *S = a.s;
  const uint64_t n = a.n;
  if (threadIdx.x == 0) {
    const double md = __dmul_rn(__dmul_rn(__dsub_rn(d, 0.5), 2.0), S->max_step);
    ctl.rt = __dadd_rn(a.r[nm], md);
    ctl.wall = fabs(ctl.rt) > __ddiv_rn(S->l, 2.0);
    if (ctl.wall) S->d_acc[1] += 1;
  }
  __syncthreads();
  if (ctl.wall) return;
  for (uint64_t i = threadIdx.x; i < n; i += blockDim.x) a.r_trial[i] = (i == nm) ? ctl.rt : a.r[i];
  __syncthreads();
  full_terms(a, a.r_trial, true, S->l);
  __syncthreads();
  full_sums(a, ctl);
  __syncthreads();
  if (threadIdx.x == 0) {
    const double et = ctl.sum[JMM_Q_E], e = S->tot[JMM_Q_E];
    if (et > e) {
      S->ran = draw_uniform(S, a.seed);
      S->bf = exp(__ddiv_rn(__dsub_rn(e, et), a.t));
    }
    const bool acc = (et < e) || (S->bf > S->ran);
    if (acc) {
      S->d_acc[0] += 1;
#pragma unroll
      for (int k = 0; k < 9; ++k) S->tot[k] = ctl.sum[k];
      a.r[nm] = ctl.rt;
    } else {
      S->d_acc[1] += 1;
    }
    ctl.accept = acc;
  }
  __syncthreads();
  if (ctl.accept) commit_all(a, a.r_trial);
}

__global__ void __launch_bounds__(kThreads, 1) echeck_kernel(Args a) {
  __shared__ Ctl ctl;
  echeck(a, a.s, ctl);
}

// One trial of a given kind outside Step: qad2 of particle nm with trial
// uniform rn, or the volume move (fav / qavLJ) with rn; no step increment,
// energy check or thermo update (those belong to Step).
__global__ void __launch_bounds__(kThreads, 1)
    move_kernel(Args a, int32_t kind, uint64_t nm, double rn, jmm_step_record *rec) {
  extern __shared__ double smem[];
  __shared__ Ctl ctl;
  const uint64_t nm1 = a.n - 1;
  if (threadIdx.x == 0) {
    ctl.nm = kind == JMM_KIND_VOLUME ? a.n : nm;
    ctl.rn = rn;
    ctl.outcome = JMM_OUT_REJECT;
    ctl.ran = NAN;
    ctl.bf = NAN;
  }
  __syncthreads();
  if (kind == JMM_KIND_DISPLACEMENT)
    qad2_step(a, a.s, ctl, smem, smem + 9 * nm1, nullptr);
  else if (a.use_qavlj)
    qav_lj(a, a.s, ctl, nullptr);
  else
    fav(a, a.s, ctl, nullptr);
  if (threadIdx.x == 0 && rec) {
    Scalars *S = a.s;
    rec->sn = S->sn;
    rec->nm = ctl.nm;
    rec->rn = ctl.rn;
    rec->ran = ctl.ran;
    rec->bf = ctl.bf;
    rec->e = S->tot[JMM_Q_E];
    rec->vir = S->tot[JMM_Q_VIR];
    rec->hv = S->tot[JMM_Q_HV];
    rec->l = S->l;
    rec->kind = kind;
    rec->outcome = ctl.outcome;
  }
}

__global__ void separations_kernel(Args a) {
  const uint64_t n = a.n;
  for (uint64_t ind = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; ind < a.nn;
       ind += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t i = ind / n, j = ind % n;
    if (j > i) a.rij[ind] = __dsub_rn(a.r[j], a.r[i]);
  }
}

__global__ void update_thermo_kernel(Args a) { update_thermo(a.s, a.n); }

// ---- volume relaxation ----------------------------------------------------

// calculateEnergyOfTrialVolumeChange: E of the positions scaled to L + dl,
// pair terms in parallel, summed in pair order (pairs beyond NBN add zero).
__device__ double trial_volume_energy(const Args &a, Ctl &ctl, double dl) {
  Scalars *S = a.s;
  if (threadIdx.x == 0) ctl.lrat1 = __ddiv_rn(__dadd_rn(S->l, dl), S->l);
  __syncthreads();
  const double lrat1 = ctl.lrat1;
  for (uint64_t i = threadIdx.x; i < a.n; i += blockDim.x) a.r_trial[i] = __dmul_rn(a.r[i], lrat1);
  __syncthreads();
  full_terms(a, a.r_trial, false, S->l);
  __syncthreads();
  full_sums(a, ctl);
  __syncthreads();
  return ctl.sum[JMM_Q_E];
}

// moveVolume: positions scaled to box length l, every pair recomputed
// (separations of pairs beyond NBN stay as they were), totals re-summed.
__device__ void move_volume(const Args &a, Ctl &ctl, double l) {
  Scalars *S = a.s;
  const uint64_t n = a.n;
  if (threadIdx.x == 0) ctl.lrat1 = __ddiv_rn(l, S->l);
  __syncthreads();
  const double lrat1 = ctl.lrat1;
  for (uint64_t i = threadIdx.x; i < n; i += blockDim.x) a.r[i] = __dmul_rn(a.r[i], lrat1);
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
  clear_mask(a);
  for (uint64_t i = warp; i < n; i += nwarps) {
    const uint64_t row = packed_index(i, i + 1, n);
    for (uint64_t j = i + 1 + lane; j < n; j += 32) {
      const uint64_t ind = i * n + j;
      double phi[9];
      if (pair_cut(a, i, j)) {
#pragma unroll
        for (int k = 0; k < 9; ++k) phi[k] = 0.0;
      } else {
        const double rij = __dsub_rn(a.r[j], a.r[i]);
        a.rij[ind] = rij;
        phi_eval(a, rij, true, l, phi);
      }
      const uint64_t q = row + (j - i - 1);
      double *dst = a.scratch + q * 9;
#pragma unroll
      for (int k = 0; k < 9; ++k) {
        a.q[k * a.nn + ind] = phi[k];
        dst[k] = phi[k];
      }
      mark_pairs(a, q, any_term(phi), n - (j - lane));
    }
  }
  __syncthreads();
  full_sums(a, ctl);
  __syncthreads();
  if (threadIdx.x == 0) {
    S->l = l;
#pragma unroll
    for (int k = 0; k < 9; ++k) S->tot[k] = ctl.sum[k];
  }
  __syncthreads();
}

__global__ void __launch_bounds__(kThreads, 1) trial_volume_energy_kernel(Args a, double dl,
                                                                          double *out) {
  __shared__ Ctl ctl;
  const double e = trial_volume_energy(a, ctl, dl);
  if (threadIdx.x == 0) *out = e;
}

__global__ void __launch_bounds__(kThreads, 1) move_volume_kernel(Args a, double l) {
  __shared__ Ctl ctl;
  move_volume(a, ctl, l);
}

// relaxVolume: up to 20 Newton steps, the scalar arithmetic by thread 0 in
// the reference's operand order; out[0] = steps taken, out[1] = converged.
__global__ void __launch_bounds__(kThreads, 1) relax_kernel(Args a, jmm_relax_step *log,
                                                             int32_t *out) {
  __shared__ Ctl ctl;
  __shared__ double ltrymin, ltrymax, dle;
  __shared__ int done;
  Scalars *S = a.s;
  const double hh = 0.1;
  if (threadIdx.x == 0) {
    ltrymin = 0.0;
    ltrymax = 1E10;
    done = 0;
    out[0] = 0;
    out[1] = 0;
  }
  __syncthreads();
  for (int count = 0; count < 20; ++count) {
    const double eup = trial_volume_energy(a, ctl, hh);
    const double edown = trial_volume_energy(a, ctl, -hh);
    if (threadIdx.x == 0) {
      const double e = S->tot[JMM_Q_E], l = S->l, nd = (double)a.n;
      const double first = __ddiv_rn(__dsub_rn(eup, edown), __dmul_rn(2.0, hh));
      const double second =
          __ddiv_rn(__dadd_rn(__dsub_rn(eup, __dmul_rn(2.0, e)), edown), __dmul_rn(hh, hh));
      double d = __ddiv_rn(-__dadd_rn(__dsub_rn(a.p, __dmul_rn(__ddiv_rn(nd, l), a.t)), first),
                           second);
      const double relax_max = __dmul_rn(0.10, nd);
      if (fabs(d) > relax_max) d = d < 0 ? -relax_max : relax_max;
      if (__dadd_rn(l, d) > ltrymax)
        d = __dmul_rn(0.5, __dsub_rn(ltrymax, l));
      else if (__dadd_rn(l, d) < ltrymin)
        d = __dmul_rn(0.5, __dsub_rn(ltrymin, l));
      if (d > 0.0)
        ltrymin = l;
      else
        ltrymax = l;
      done = fabs(d) < __dmul_rn(0.0025, nd);
      dle = d;
      log[count].e_up = eup;
      log[count].e_down = edown;
      log[count].dl = d;
    }
    __syncthreads();
    move_volume(a, ctl, __dadd_rn(S->l, dle));
    if (threadIdx.x == 0) {
      log[count].l = S->l;
      log[count].e = S->tot[JMM_Q_E];
      out[0] = count + 1;
      out[1] = done;
    }
    __syncthreads();
    if (done) break;
  }
}

// Set-up of the histograms: counts of the current configuration, accumulated
// once (setupMCS, src/jmmMCState.cpp:773-776).
__global__ void __launch_bounds__(kThreads, 1) hist_init_kernel(Args a) {
  const uint64_t total = a.rhonb + (uint64_t)a.gns * a.gnb;
  for (uint64_t b = threadIdx.x; b < total; b += blockDim.x) {
    a.h_val[b] = 0;
    a.h_acc[b] = 0;
    a.h_last[b] = 0;
  }
  if (threadIdx.x == 0) a.s->hist_ticks = 0;
  __syncthreads();
  fgrho(a, a.s);
  ugrho(a, a.s);
}

// Sums of bins [b0, b0 + nb) since the last take, as the reference's int
// accumulators hold them (wrapped to 32 bits), then zeroed (printRho /
// printG, src/jmmMCState.cpp:1021-1061).
__global__ void hist_take_kernel(Args a, uint64_t b0, uint64_t nb, int32_t *out) {
  const uint64_t T = a.s->hist_ticks;
  for (uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; k < nb;
       k += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t b = b0 + k;
    const long long total = a.h_acc[b] + (long long)a.h_val[b] * (long long)(T - a.h_last[b]);
    out[k] = (int32_t)(uint32_t)(unsigned long long)total;
    a.h_acc[b] = 0;
    a.h_last[b] = T;
  }
}

}  // namespace plain
}  // namespace jmm

using namespace jmm;
using namespace jmm::plain;

struct jmm_plain {
  jmm_params prm;
  Args a;
  size_t smem_bytes;
  jmm_draw *d_replay;
  uint64_t replay_cap;
  jmm_step_record *d_log;
  uint64_t log_cap;
  int32_t *d_hist_out;  // staging of a histogram take
  bool initialised;  // fad has run since set-up
};

static void plain_free(jmm_plain *h) {
  if (!h) return;
  cudaFree(h->a.s);
  cudaFree(h->a.r);
  cudaFree(h->a.r_trial);
  cudaFree(h->a.rij);
  cudaFree(h->a.q);
  cudaFree(h->a.scratch);
  cudaFree(h->a.mask);
  cudaFree(h->a.comp);
  cudaFree(h->a.h_val);
  cudaFree(h->a.h_acc);
  cudaFree(h->a.h_last);
  cudaFree(h->d_hist_out);
  cudaFree(h->d_replay);
  cudaFree(h->d_log);
  delete h;
}

static int plain_sync(const char *what) {
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e != cudaSuccess) return cuda_status(e, what, __FILE__, __LINE__);
  return JMM_OK;
}

static int plain_reset_separations(jmm_plain *h) {
  const uint64_t nn = h->a.nn;
  int blocks = (int)((nn + 255) / 256);
  if (blocks > 4096) blocks = 4096;
  separations_kernel<<<blocks, 256>>>(h->a);
  return plain_sync("separations_kernel");
}

extern "C" int jmm_plain_create(const jmm_params *prm, jmm_plain **out) {
  clear_error();
  JMM_CHECK_ARG(prm && out, "null argument");
  *out = nullptr;
  JMM_CHECK_ARG(prm->n >= 2 && prm->n <= kMaxN, "N must be in [2, 2900] for the plain form");
  JMM_CHECK_ARG(prm->ensemble == JMM_NLT || prm->ensemble == JMM_NPT, "unknown ensemble");
  JMM_CHECK_ARG(prm->potential == JMM_POT_LJCUT || prm->potential == JMM_POT_LJ ||
                    prm->potential == JMM_POT_HARMONIC,
                "the plain form runs the reference's potentials LJcut, LJ and HARMONIC");
  JMM_CHECK_ARG(prm->t > 0, "T must be positive");
  JMM_CHECK_ARG(prm->ensemble == JMM_NPT || prm->l > 0, "L must be positive");
  if (!jmm_device_available()) return fail(JMM_ERR_CUDA, "jmm_plain_create: no CUDA device");

  jmm_plain *h = new (std::nothrow) jmm_plain();
  if (!h) return fail(JMM_ERR_NOMEM, "jmm_plain_create: host allocation failed");
  h->prm = *prm;
  const uint64_t n = prm->n;
  Args &a = h->a;
  a.n = n;
  a.nn = n * n;
  a.npairs = n * (n - 1) / 2;
  a.num_trial_types = prm->ensemble == JMM_NPT ? n + 1 : n;
  a.potential = prm->potential;
  a.nbn = prm->nbn;
  a.use_qavlj = (prm->potential == JMM_POT_LJ && prm->nbn < 0) ? 1 : 0;
  a.cutoff = prm->potential == JMM_POT_LJ ? INFINITY : prm->cutoff;
  a.t = prm->t;
  a.p = prm->p;
  a.seed = prm->seed;
  a.eci = prm->eci;
  // s_new (9 quantities) and s_rij per partner; and, where it fits beside
  // the kernels' own static shared memory, the stored old terms too, so that
  // qad2's in-order sums read shared memory instead of one strided load per
  // term
  size_t static_smem = 0;
  {
    cudaFuncAttributes fa;
    if (cudaFuncGetAttributes(&fa, steps_kernel) == cudaSuccess && fa.sharedSizeBytes > static_smem)
      static_smem = fa.sharedSizeBytes;
    if (cudaFuncGetAttributes(&fa, move_kernel) == cudaSuccess && fa.sharedSizeBytes > static_smem)
      static_smem = fa.sharedSizeBytes;
    cudaGetLastError();
  }
  const size_t room = 227 * 1024 - static_smem;
  a.stage_old = 19 * (n - 1) * sizeof(double) <= room ? 1 : 0;
  h->smem_bytes = (a.stage_old ? 19 : 10) * (n - 1) * sizeof(double);

  int rc = JMM_OK;
#define ALLOC(ptr, bytes)                                               \
  do {                                                                  \
    cudaError_t e_ = cudaMalloc((void **)&(ptr), (bytes));              \
    if (e_ != cudaSuccess) {                                            \
      rc = cuda_status(e_, "cudaMalloc " #ptr, __FILE__, __LINE__);     \
      plain_free(h);                                                    \
      return rc;                                                        \
    }                                                                   \
  } while (0)
  ALLOC(a.s, sizeof(Scalars));
  ALLOC(a.r, n * sizeof(double));
  ALLOC(a.r_trial, n * sizeof(double));
  ALLOC(a.rij, a.nn * sizeof(double));
  ALLOC(a.q, 9 * a.nn * sizeof(double));
  ALLOC(a.scratch, 9 * a.npairs * sizeof(double));
  a.nwords = (a.npairs + 31) / 32;
  ALLOC(a.mask, a.nwords * sizeof(uint32_t));
  ALLOC(a.comp, 9 * a.npairs * sizeof(double));
#undef ALLOC

  Scalars s;
  memset(&s, 0, sizeof(s));
  s.rng_slot = 4;
  s.l = prm->ensemble == JMM_NPT ? (double)n : prm->l;
  s.max_step = prm->max_step;
  s.max_dl = prm->max_dl;
  s.tot[JMM_Q_E] = 10E10;
  s.tot[JMM_Q_VIR] = 10E10;
  s.tot[JMM_Q_HV] = 10E10;
  s.tot[JMM_Q_E6] = -5E10;
  s.tot[JMM_Q_E12] = 5E10;
  s.tot[JMM_Q_VIR6] = -5E10;
  s.tot[JMM_Q_VIR12] = 5E10;
  s.tot[JMM_Q_HV6] = -5E10;
  s.tot[JMM_Q_HV12] = 5E10;
  double *r = (double *)malloc(n * sizeof(double));
  if (!r) {
    plain_free(h);
    return fail(JMM_ERR_NOMEM, "jmm_plain_create: host allocation failed");
  }
  for (uint64_t i = 0; i < n; ++i) r[i] = ((i + 0.5) / n - 0.5) * s.l;
  cudaError_t e = cudaMemcpy(a.r, r, n * sizeof(double), cudaMemcpyHostToDevice);
  free(r);
  if (e == cudaSuccess) e = cudaMemcpy(a.s, &s, sizeof(s), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(a.q, 0, 9 * a.nn * sizeof(double));
  if (e == cudaSuccess) e = cudaMemset(a.rij, 0, a.nn * sizeof(double));
  if (e == cudaSuccess && h->smem_bytes > 48 * 1024)
    e = cudaFuncSetAttribute(steps_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)h->smem_bytes);
  if (e == cudaSuccess && h->smem_bytes > 48 * 1024)
    e = cudaFuncSetAttribute(move_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)h->smem_bytes);
  if (e != cudaSuccess) {
    rc = cuda_status(e, "jmm_plain_create set-up", __FILE__, __LINE__);
    plain_free(h);
    return rc;
  }
  rc = plain_reset_separations(h);
  if (rc != JMM_OK) {
    plain_free(h);
    return rc;
  }
  *out = h;
  return JMM_OK;
}

extern "C" int jmm_plain_destroy(jmm_plain *h) {
  plain_free(h);
  return JMM_OK;
}

static int get_scalars(jmm_plain *h, Scalars *s) {
  JMM_CUDA(cudaMemcpy(s, h->a.s, sizeof(Scalars), cudaMemcpyDeviceToHost));
  return JMM_OK;
}

static int put_scalars(jmm_plain *h, const Scalars *s) {
  JMM_CUDA(cudaMemcpy(h->a.s, s, sizeof(Scalars), cudaMemcpyHostToDevice));
  return JMM_OK;
}

extern "C" int jmm_plain_set_config(jmm_plain *h, const double *r, uint64_t n, double l,
                                    uint64_t sn) {
  clear_error();
  JMM_CHECK_ARG(h && r, "null argument");
  JMM_CHECK_ARG(n == h->a.n, "N does not match the chain");
  JMM_CHECK_ARG(l > 0, "box length must be positive");
  Scalars s;
  int rc = get_scalars(h, &s);
  if (rc) return rc;
  s.l = l;
  s.sn = sn;
  s.tot[JMM_Q_E] = 10.0E10;
  s.tot[JMM_Q_VIR] = 10.0E10;
  s.tot[JMM_Q_HV] = 10.0E10;
  JMM_CUDA(cudaMemcpy(h->a.r, r, n * sizeof(double), cudaMemcpyHostToDevice));
  rc = put_scalars(h, &s);
  if (rc) return rc;
  h->initialised = false;
  return plain_reset_separations(h);
}

extern "C" int jmm_plain_fad(jmm_plain *h, uint64_t nm, double d) {
  clear_error();
  JMM_CHECK_ARG(h, "null handle");
  JMM_CHECK_ARG(nm < h->a.n, "particle index out of range");
  fad_kernel<<<1, kThreads>>>(h->a, nm, d);
  int rc = plain_sync("fad_kernel");
  if (rc == JMM_OK) h->initialised = true;
  return rc;
}

extern "C" int jmm_plain_steps(jmm_plain *h, uint64_t n_steps, const jmm_draw *replay,
                               jmm_step_record *log) {
  clear_error();
  JMM_CHECK_ARG(h, "null handle");
  if (!h->initialised)
    return fail(JMM_ERR_STATE, "jmm_plain_steps: run jmm_plain_fad first (the driver's step 0)");
  const uint64_t chunk_max = (replay || log) ? (1u << 16) : (1u << 20);
  for (uint64_t done = 0; done < n_steps;) {
    const uint64_t chunk = (n_steps - done) < chunk_max ? (n_steps - done) : chunk_max;
    if (replay) {
      if (h->replay_cap < chunk) {
        cudaFree(h->d_replay);
        h->d_replay = nullptr;
        JMM_CUDA(cudaMalloc((void **)&h->d_replay, chunk * sizeof(jmm_draw)));
        h->replay_cap = chunk;
      }
      for (uint64_t k = 0; k < chunk; ++k) {
        if (replay[done + k].nm > h->a.n)
          return fail(JMM_ERR_INVALID, "jmm_plain_steps: replay draw %llu has trial type %llu > N",
                      (unsigned long long)(done + k), (unsigned long long)replay[done + k].nm);
      }
      JMM_CUDA(cudaMemcpy(h->d_replay, replay + done, chunk * sizeof(jmm_draw),
                          cudaMemcpyHostToDevice));
    }
    if (log && h->log_cap < chunk) {
      cudaFree(h->d_log);
      h->d_log = nullptr;
      JMM_CUDA(cudaMalloc((void **)&h->d_log, chunk * sizeof(jmm_step_record)));
      h->log_cap = chunk;
    }
    steps_kernel<<<1, kThreads, h->smem_bytes>>>(h->a, chunk, replay ? h->d_replay : nullptr,
                                                  log ? h->d_log : nullptr);
    int rc = plain_sync("steps_kernel");
    if (rc) return rc;
    if (log)
      JMM_CUDA(cudaMemcpy(log + done, h->d_log, chunk * sizeof(jmm_step_record),
                          cudaMemcpyDeviceToHost));
    done += chunk;
  }
  Scalars s;
  int rc = get_scalars(h, &s);
  if (rc) return rc;
  if (s.error) return fail((int)s.error, "jmm_plain_steps: kernel reported error %u", s.error);
  return JMM_OK;
}

extern "C" int jmm_plain_move(jmm_plain *h, int32_t kind, uint64_t nm, double rn,
                              jmm_step_record *rec) {
  clear_error();
  JMM_CHECK_ARG(h, "null handle");
  JMM_CHECK_ARG(kind == JMM_KIND_DISPLACEMENT || kind == JMM_KIND_VOLUME, "unknown move kind");
  JMM_CHECK_ARG(kind == JMM_KIND_VOLUME || nm < h->a.n, "particle index out of range");
  JMM_CHECK_ARG(kind == JMM_KIND_DISPLACEMENT || h->prm.ensemble == JMM_NPT,
                "volume moves need the NPT ensemble");
  if (!h->initialised) return fail(JMM_ERR_STATE, "jmm_plain_move: run jmm_plain_fad first");
  if (rec && h->log_cap < 1) {
    cudaFree(h->d_log);
    h->d_log = nullptr;
    JMM_CUDA(cudaMalloc((void **)&h->d_log, sizeof(jmm_step_record)));
    h->log_cap = 1;
  }
  move_kernel<<<1, kThreads, h->smem_bytes>>>(h->a, kind, nm, rn, rec ? h->d_log : nullptr);
  int rc = plain_sync("move_kernel");
  if (rc) return rc;
  if (rec) JMM_CUDA(cudaMemcpy(rec, h->d_log, sizeof(jmm_step_record), cudaMemcpyDeviceToHost));
  return JMM_OK;
}

extern "C" int jmm_plain_update_thermo(jmm_plain *h) {
  clear_error();
  JMM_CHECK_ARG(h, "null handle");
  update_thermo_kernel<<<1, 1>>>(h->a);
  return plain_sync("update_thermo_kernel");
}

extern "C" int jmm_plain_reset_thermo(jmm_plain *h) {
  clear_error();
  JMM_CHECK_ARG(h, "null handle");
  Scalars s;
  int rc = get_scalars(h, &s);
  if (rc) return rc;
  memset(s.thermo, 0, sizeof(s.thermo));
  return put_scalars(h, &s);
}

extern "C" int jmm_plain_echeck(jmm_plain *h, double *e_test, int32_t *reset) {
  clear_error();
  JMM_CHECK_ARG(h, "null handle");
  Scalars before;
  int rc = get_scalars(h, &before);
  if (rc) return rc;
  echeck_kernel<<<1, kThreads>>>(h->a);
  rc = plain_sync("echeck_kernel");
  if (rc) return rc;
  Scalars s;
  rc = get_scalars(h, &s);
  if (rc) return rc;
  if (e_test) *e_test = s.echeck_e;
  if (reset) *reset = s.echeck_resets > before.echeck_resets ? 1 : 0;
  return JMM_OK;
}

extern "C" int jmm_plain_set_step_sizes(jmm_plain *h, double max_step, double max_dl) {
  clear_error();
  JMM_CHECK_ARG(h, "null handle");
  Scalars s;
  int rc = get_scalars(h, &s);
  if (rc) return rc;
  s.max_step = max_step;
  s.max_dl = max_dl;
  return put_scalars(h, &s);
}

extern "C" int jmm_plain_get_state(jmm_plain *h, jmm_state *out) {
  clear_error();
  JMM_CHECK_ARG(h && out, "null argument");
  Scalars s;
  int rc = get_scalars(h, &s);
  if (rc) return rc;
  memset(out, 0, sizeof(*out));
  out->sn = s.sn;
  out->rng_block = s.rng_block;
  out->rng_slot = s.rng_slot;
  out->error = s.error;
  out->l = s.l;
  memcpy(out->tot, s.tot, sizeof(s.tot));
  out->d_acc[0] = s.d_acc[0];
  out->d_acc[1] = s.d_acc[1];
  out->v_acc[0] = s.v_acc[0];
  out->v_acc[1] = s.v_acc[1];
  out->max_step = s.max_step;
  out->max_dl = s.max_dl;
  memcpy(out->thermo, s.thermo, sizeof(s.thermo));
  out->echeck_count = s.echeck_count;
  out->echeck_resets = s.echeck_resets;
  out->echeck_e = s.echeck_e;
  out->echeck_e_before = s.echeck_e_before;
  return JMM_OK;
}

extern "C" int jmm_plain_get_positions(jmm_plain *h, double *r, uint64_t n) {
  clear_error();
  JMM_CHECK_ARG(h && r, "null argument");
  JMM_CHECK_ARG(n == h->a.n, "N does not match the chain");
  JMM_CUDA(cudaMemcpy(r, h->a.r, n * sizeof(double), cudaMemcpyDeviceToHost));
  return JMM_OK;
}

extern "C" int jmm_plain_get_separations(jmm_plain *h, double *rij, uint64_t n_pairs) {
  clear_error();
  JMM_CHECK_ARG(h && rij, "null argument");
  const uint64_t n = h->a.n;
  JMM_CHECK_ARG(n_pairs == n * (n - 1) / 2, "n_pairs must be N(N-1)/2");
  double *dense = (double *)malloc(h->a.nn * sizeof(double));
  if (!dense) return fail(JMM_ERR_NOMEM, "jmm_plain_get_separations: host allocation failed");
  cudaError_t e = cudaMemcpy(dense, h->a.rij, h->a.nn * sizeof(double), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) {
    free(dense);
    return cuda_status(e, "cudaMemcpy separations", __FILE__, __LINE__);
  }
  uint64_t k = 0;
  for (uint64_t i = 0; i < n; ++i)
    for (uint64_t j = i + 1; j < n; ++j) rij[k++] = dense[i * n + j];
  free(dense);
  return JMM_OK;
}

// ---- rho(x) and g(x) histograms --------------------------------------------

extern "C" int jmm_plain_histograms(jmm_plain *h, uint64_t rhonb, double rbw, int32_t gns,
                                    double gsw, uint64_t gnb, double gbw) {
  clear_error();
  JMM_CHECK_ARG(h, "null handle");
  JMM_CHECK_ARG(rhonb >= 1 && gns >= 1 && gnb >= 1, "bin counts must be positive");
  JMM_CHECK_ARG(rbw > 0 && gsw > 0 && gbw > 0, "bin widths must be positive");
  const uint64_t total = rhonb + (uint64_t)gns * gnb;
  JMM_CHECK_ARG(total <= (1ull << 26), "at most 2^26 histogram bins");
  Args &a = h->a;
  cudaFree(a.h_val);
  cudaFree(a.h_acc);
  cudaFree(a.h_last);
  cudaFree(h->d_hist_out);
  a.h_val = nullptr;
  a.h_acc = nullptr;
  a.h_last = nullptr;
  h->d_hist_out = nullptr;
  a.hist_on = 0;
  JMM_CUDA(cudaMalloc((void **)&a.h_val, total * sizeof(int32_t)));
  JMM_CUDA(cudaMalloc((void **)&a.h_acc, total * sizeof(long long)));
  JMM_CUDA(cudaMalloc((void **)&a.h_last, total * sizeof(unsigned long long)));
  JMM_CUDA(cudaMalloc((void **)&h->d_hist_out, total * sizeof(int32_t)));
  a.rhonb = rhonb;
  a.rbw = rbw;
  a.gns = gns;
  a.gsw = gsw;
  a.gnb = gnb;
  a.gbw = gbw;
  a.hist_on = 1;
  hist_init_kernel<<<1, kThreads>>>(a);
  return plain_sync("hist_init_kernel");
}

static int hist_take(jmm_plain *h, uint64_t b0, uint64_t nb, int32_t *out) {
  hist_take_kernel<<<(unsigned)((nb + 255) / 256 < 1024 ? (nb + 255) / 256 : 1024), 256>>>(
      h->a, b0, nb, h->d_hist_out);
  int rc = plain_sync("hist_take_kernel");
  if (rc) return rc;
  JMM_CUDA(cudaMemcpy(out, h->d_hist_out, nb * sizeof(int32_t), cudaMemcpyDeviceToHost));
  return JMM_OK;
}

extern "C" int jmm_plain_take_rho(jmm_plain *h, int32_t *counts, uint64_t rhonb) {
  clear_error();
  JMM_CHECK_ARG(h && counts, "null argument");
  if (!h->a.hist_on) return fail(JMM_ERR_STATE, "jmm_plain_take_rho: histograms are not set up");
  JMM_CHECK_ARG(rhonb == h->a.rhonb, "rhonb does not match the set-up");
  return hist_take(h, 0, rhonb, counts);
}

extern "C" int jmm_plain_take_g(jmm_plain *h, int32_t *counts, uint64_t n) {
  clear_error();
  JMM_CHECK_ARG(h && counts, "null argument");
  if (!h->a.hist_on) return fail(JMM_ERR_STATE, "jmm_plain_take_g: histograms are not set up");
  JMM_CHECK_ARG(n == (uint64_t)h->a.gns * h->a.gnb, "n must be gns * gnb");
  return hist_take(h, h->a.rhonb, n, counts);
}

extern "C" int jmm_plain_hist_counts(jmm_plain *h, int32_t *rho, uint64_t rhonb, int32_t *g,
                                     uint64_t ng) {
  clear_error();
  JMM_CHECK_ARG(h && rho && g, "null argument");
  if (!h->a.hist_on)
    return fail(JMM_ERR_STATE, "jmm_plain_hist_counts: histograms are not set up");
  JMM_CHECK_ARG(rhonb == h->a.rhonb && ng == (uint64_t)h->a.gns * h->a.gnb,
                "sizes do not match the set-up");
  JMM_CUDA(cudaDeviceSynchronize());
  JMM_CUDA(cudaMemcpy(rho, h->a.h_val, rhonb * sizeof(int32_t), cudaMemcpyDeviceToHost));
  JMM_CUDA(cudaMemcpy(g, h->a.h_val + rhonb, ng * sizeof(int32_t), cudaMemcpyDeviceToHost));
  return JMM_OK;
}

// ---- volume relaxation --------------------------------------------------------

extern "C" int jmm_plain_relax_volume(jmm_plain *h, jmm_relax_step *log, int32_t *n_steps,
                                      int32_t *converged) {
  clear_error();
  JMM_CHECK_ARG(h, "null handle");
  jmm_relax_step *d_log = nullptr;
  int32_t *d_out = nullptr;
  JMM_CUDA(cudaMalloc((void **)&d_log, 20 * sizeof(jmm_relax_step)));
  cudaError_t e = cudaMalloc((void **)&d_out, 2 * sizeof(int32_t));
  if (e != cudaSuccess) {
    cudaFree(d_log);
    return cuda_status(e, "cudaMalloc relax", __FILE__, __LINE__);
  }
  relax_kernel<<<1, kThreads>>>(h->a, d_log, d_out);
  int rc = plain_sync("relax_kernel");
  int32_t out[2] = {0, 0};
  if (rc == JMM_OK) {
    e = cudaMemcpy(out, d_out, sizeof(out), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && log)
      e = cudaMemcpy(log, d_log, out[0] * sizeof(jmm_relax_step), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) rc = cuda_status(e, "cudaMemcpy relax", __FILE__, __LINE__);
  }
  cudaFree(d_log);
  cudaFree(d_out);
  if (rc) return rc;
  if (n_steps) *n_steps = out[0];
  if (converged) *converged = out[1];
  return JMM_OK;
}

extern "C" int jmm_plain_trial_volume_energy(jmm_plain *h, double dl, double *e_out) {
  clear_error();
  JMM_CHECK_ARG(h && e_out, "null argument");
  double *d = nullptr;
  JMM_CUDA(cudaMalloc((void **)&d, sizeof(double)));
  trial_volume_energy_kernel<<<1, kThreads>>>(h->a, dl, d);
  int rc = plain_sync("trial_volume_energy_kernel");
  if (rc == JMM_OK) {
    cudaError_t e = cudaMemcpy(e_out, d, sizeof(double), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) rc = cuda_status(e, "cudaMemcpy trial energy", __FILE__, __LINE__);
  }
  cudaFree(d);
  return rc;
}

extern "C" int jmm_plain_move_volume(jmm_plain *h, double l) {
  clear_error();
  JMM_CHECK_ARG(h, "null handle");
  JMM_CHECK_ARG(l > 0, "box length must be positive");
  move_volume_kernel<<<1, kThreads>>>(h->a, l);
  return plain_sync("move_volume_kernel");
}
