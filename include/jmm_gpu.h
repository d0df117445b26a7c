/*
 * include/jmm_gpu.h -- the C ABI of libjmmgpu.so, the GB300 (sm_103a)
 * implementation of jmmOneDMC's Monte Carlo move loop.
 *
 * Plain C: plain pointers and sizes, no CUDA or C++ types in any signature.
 * Every entry point returns a status (JMM_OK = 0); jmm_last_error() gives the
 * message of the last failure on the calling thread.  There is no CPU
 * fallback: without a usable CUDA device every compute call fails with
 * JMM_ERR_CUDA.
 *
 * Two forms of the same Metropolis chain:
 *
 *  - jmm_plain_*  : one chain, FP64, the reference's algorithm step for step
 *                   (pair-state arrays, incremental separations, summation
 *                   order, random-draw conditions).  It is the drop-in behind
 *                   the reference's C++ API (src/jmmMCState.h:6-48) and, fed
 *                   the same uniforms, reproduces its accept/reject sequence.
 *  - jmm_batch_*  : thousands of independent chains in one persistent kernel
 *                   (declared further down).
 *
 * Quantity order of every 9-vector (the reference's phi[] layout,
 * src/pot.cpp:90-100): E, Vir, E12, Vir12, E6, Vir6, HV, HV12, HV6.
 * Thermo accumulator order (src/jmmMCState.cpp:1941-1961): rhoSysA,
 * rhoSysSA, lA, lSA, EA, ESA, lEA, VirA, VirSA, EVirA, HVA, HVSA.
 */
#ifndef JMM_GPU_H
#define JMM_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define JMM_OK 0
#define JMM_ERR_INVALID 1     /* bad argument or unsupported combination     */
#define JMM_ERR_CUDA 2        /* no device, launch failure, driver error     */
#define JMM_ERR_NOMEM 3       /* device or host allocation failed            */
#define JMM_ERR_TIMEOUT 4     /* a bounded device wait ran out               */
#define JMM_ERR_NUMERIC 5     /* NaN/Inf energy or position seen by a kernel */
#define JMM_ERR_STATE 6       /* call out of order (e.g. steps before fad)   */

/* ---- enums ------------------------------------------------------------- */
#define JMM_NLT 0             /* ENSEMBLE NLT (src/jmmMCState.cpp:412-421)   */
#define JMM_NPT 1             /* ENSEMBLE NPT (src/jmmMCState.cpp:402-411)   */

#define JMM_POT_LJCUT 0       /* POT LJcut <rc>: phiLJcut, src/pot.cpp:19-101 */
#define JMM_POT_LJ 1          /* POT LJ: phiLJinfcutoff, src/pot.cpp:104-108  */
#define JMM_POT_HARMONIC 2    /* POT HARMONIC [rc]: src/pot.cpp:110-141       */
#define JMM_POT_SOFTSPHERE 3  /* eps (sigma/r)^12, batched form only          */
#define JMM_POT_GAUSS 4       /* eps exp(-(r/sigma)^2), batched form only     */

/* Quantity indices of the 9-vectors. */
#define JMM_Q_E 0
#define JMM_Q_VIR 1
#define JMM_Q_E12 2
#define JMM_Q_VIR12 3
#define JMM_Q_E6 4
#define JMM_Q_VIR6 5
#define JMM_Q_HV 6
#define JMM_Q_HV12 7
#define JMM_Q_HV6 8

/* ---- plain form: one FP64 chain ---------------------------------------- */

/* The INPUT keywords that reach the move loop (src/jmmMCState.h:50-85). */
typedef struct jmm_params {
  uint64_t n;          /* N                                                   */
  int32_t ensemble;    /* JMM_NLT | JMM_NPT                                   */
  int32_t potential;   /* JMM_POT_LJCUT | JMM_POT_LJ | JMM_POT_HARMONIC       */
  double p;            /* P (NPT)                                             */
  double l;            /* L (NLT); NPT starts from L = N                      */
  double t;            /* T                                                   */
  double cutoff;       /* POT cut-off; INFINITY for POT LJ                    */
  int32_t nbn;         /* NBN, -1 = no neighbour-number limit                 */
  int32_t reserved0;
  double max_step;     /* MAXSTEP                                             */
  double max_dl;       /* MAXDV                                               */
  uint64_t seed;       /* SEED                                                */
  uint64_t eci;        /* ENGCHECK interval, 0 = never                        */
} jmm_params;

typedef struct jmm_state {
  uint64_t sn;             /* step number                                     */
  uint64_t rng_block;      /* Philox blocks opened since set-up               */
  uint32_t rng_slot;       /* next word of the open block (4 = exhausted)     */
  uint32_t error;          /* sticky JMM_ERR_* seen by a kernel, 0 = none     */
  double l;                /* box length                                      */
  double tot[9];           /* E, Vir, E12, Vir12, E6, Vir6, HV, HV12, HV6     */
  uint64_t d_acc[2];       /* displacements accepted / rejected               */
  uint64_t v_acc[2];       /* volume changes accepted / rejected              */
  double max_step;
  double max_dl;
  double thermo[12];       /* block accumulators, order in the file header    */
  uint64_t echeck_count;   /* energy checks run                               */
  uint64_t echeck_resets;  /* energy checks that found |dE| > 1e-4            */
  double echeck_e;         /* ETest of the last energy check                  */
  double echeck_e_before;  /* running E just before the last energy check     */
} jmm_state;

/* Replay input: the values the reference consumed at one step. */
typedef struct jmm_draw {
  uint64_t nm;   /* trial type: particle index, or N for a volume move        */
  double rn;     /* trial magnitude uniform                                   */
  double ran;    /* Metropolis uniform, read only when the step draws one     */
} jmm_draw;

#define JMM_KIND_DISPLACEMENT 0
#define JMM_KIND_VOLUME 1
#define JMM_OUT_REJECT_WALL 0     /* |r_trial| > L/2: no energy work          */
#define JMM_OUT_REJECT 1          /* Metropolis rejection                      */
#define JMM_OUT_ACCEPT 2

typedef struct jmm_step_record {
  uint64_t sn;
  uint64_t nm;
  double rn;
  double ran;      /* NaN when the step drew no Metropolis uniform            */
  double bf;       /* Boltzmann factor when one was formed, else NaN          */
  double e;
  double vir;
  double hv;
  double l;
  int32_t kind;    /* JMM_KIND_*                                               */
  int32_t outcome; /* JMM_OUT_*                                                */
} jmm_step_record;

typedef struct jmm_plain jmm_plain;

/* setupMCS (src/jmmMCState.cpp:261-790), fresh start: lattice
 * r_i = ((i+0.5)/N - 0.5) L, separations, E = Vir = HV = 1e11 until fad. */
int jmm_plain_create(const jmm_params *params, jmm_plain **out);
/* Restart branch of setupMCS (src/jmmMCState.cpp:572-769): positions, box
 * length and step number from a saved frame; energies back to 1e11. */
int jmm_plain_set_config(jmm_plain *h, const double *r, uint64_t n, double l,
                         uint64_t sn);
/* fad (src/jmmMCState.cpp:853-1003) with explicit particle and uniform;
 * the driver's step 0 is jmm_plain_fad(h, 0, 0.5) (src/Main.cpp:66-68). */
int jmm_plain_fad(jmm_plain *h, uint64_t nm, double d);
/* n_steps x (incrementStep + Step) (src/jmmMCState.cpp:1734-1811): draw,
 * qad2 / fav / qavLJ, ECheck when sn % ENGCHECK == 0, updateThermo.
 * replay: NULL to draw from the Philox stream, else n_steps draws.
 * log: NULL, or room for n_steps records. */
int jmm_plain_steps(jmm_plain *h, uint64_t n_steps, const jmm_draw *replay,
                    jmm_step_record *log);
/* One trial outside Step (qad2 of particle nm with trial uniform rn, or the
 * volume move fav / qavLJ with rn), as the reference's qad/qad2/fav/qav when
 * called directly (src/jmmMCState.cpp:1154-1464, :1642-1730, :2161-2293):
 * no step increment, energy check or thermo update.  rec: NULL or one record. */
int jmm_plain_move(jmm_plain *h, int32_t kind, uint64_t nm, double rn, jmm_step_record *rec);
/* updateThermo on its own (the driver's step-0 call, src/Main.cpp:95). */
int jmm_plain_update_thermo(jmm_plain *h);
/* Zero the 12 thermo accumulators (what printThermo does after printing,
 * src/jmmMCState.cpp:1922-1934). */
int jmm_plain_reset_thermo(jmm_plain *h);
/* ECheck on its own (src/jmmMCState.cpp:1965-2095). */
int jmm_plain_echeck(jmm_plain *h, double *e_test, int32_t *reset);
/* maxDisAdjust / maxDVAdjust results written back (src/jmmMCState.cpp:2100-2139). */
int jmm_plain_set_step_sizes(jmm_plain *h, double max_step, double max_dl);
int jmm_plain_get_state(jmm_plain *h, jmm_state *out);
int jmm_plain_get_positions(jmm_plain *h, double *r, uint64_t n);
/* Stored pair separations r_j - r_i (i < j), row-major over i, N*(N-1)/2. */
int jmm_plain_get_separations(jmm_plain *h, double *rij, uint64_t n_pairs);
int jmm_plain_destroy(jmm_plain *h);

/* rho(x) and g(x) histograms (fgrho / ugrho / qagrho, src/jmmMCState.cpp:
 * 1069-1149, :2297-2384): rhonb density bins of width rbw (bin of x =
 * floor(x/rbw + rhonb/2)); gns slices of width gsw (slice of x = floor(x/gsw
 * + gns/2)), each with gnb separation bins of width gbw, a pair counted in
 * the slices of both its particles.  Set-up takes the counts of the current
 * configuration and accumulates them once, as setupMCS does (:773-776):
 * call it after jmm_plain_set_config.  Then, as in the reference, every
 * displacement step accumulates the counts once whatever its outcome (qad2
 * calls ugrho), an accepted displacement updates them (qagrho), a qavLJ
 * volume step recounts on acceptance and accumulates, and a fav volume step
 * does neither (the reference's counts stay those of the old box).  A
 * negative stored separation gives no g count (the reference writes out of
 * bounds there). */
int jmm_plain_histograms(jmm_plain *h, uint64_t rhonb, double rbw, int32_t gns, double gsw,
                         uint64_t gnb, double gbw);
/* Sums of the counts since the last take (the reference's int rhoA / gA,
 * 32-bit wrapping), then zeroed, as printRho / printG do (:1021-1061);
 * g is slice after slice (gns * gnb). */
int jmm_plain_take_rho(jmm_plain *h, int32_t *counts, uint64_t rhonb);
int jmm_plain_take_g(jmm_plain *h, int32_t *counts, uint64_t n);
/* The current counts (rhol, gl). */
int jmm_plain_hist_counts(jmm_plain *h, int32_t *rho, uint64_t rhonb, int32_t *g, uint64_t ng);

/* Volume relaxation (relaxVolume, src/jmmMCState.cpp:2396-2643; the RELAX
 * keyword): up to 20 Newton steps toward -dE/dL + N T / L = P, from central
 * differences of E at L +- 0.1 (calculateEnergyOfTrialVolumeChange), each
 * step clamped to 0.1 N and to the bracket of lengths tried, applied with
 * moveVolume (positions scaled, every pair and total recomputed), until a
 * step is shorter than 0.0025 N.  One launch for the whole relaxation. */
typedef struct jmm_relax_step {
  double e_up, e_down;  /* E at L + 0.1 and L - 0.1                           */
  double dl;            /* the step taken                                     */
  double l, e;          /* box length and E after it                          */
} jmm_relax_step;
/* log: room for 20 records; *n_steps records written; *converged 1 when the
 * last step was below the criterion, 0 after 20 steps. */
int jmm_plain_relax_volume(jmm_plain *h, jmm_relax_step *log, int32_t *n_steps,
                           int32_t *converged);
/* E of the positions scaled to L + dl (calculateEnergyOfTrialVolumeChange,
 * :2756-2800); the state is not changed. */
int jmm_plain_trial_volume_energy(jmm_plain *h, double dl, double *e);
/* Positions scaled to box length l, every pair and total recomputed
 * (moveVolume, :2803-2905). */
int jmm_plain_move_volume(jmm_plain *h, double l);

/* ---- batched form: many independent chains ------------------------------
 *
 * Each chain is the reference's sequential single-particle Metropolis chain
 * (random particle, uniform displacement, hard walls at +-L/2 by default),
 * run with FP32 pair energies and FP64 totals and accumulators.  Thousands of
 * chains of uneven N, temperature, pressure and potential share one
 * persistent kernel: a group of lanes per chain, positions staged in shared
 * memory, the energy change reduced with warp shuffles.  Particles keep
 * their order along the line (a move that would pass a neighbour is
 * rejected), so a move needs only the index neighbours within the cut-off.
 * Chain k draws from Philox block (step, k) of the batch seed.
 */
#define JMM_BOUNDARY_WALLS 0     /* hard walls at +-L/2 (src/jmmMCState.cpp:1188-1193) */
#define JMM_BOUNDARY_PERIODIC 1  /* ring of length L                                   */
#define JMM_VOLMOVE_LINEAR 0     /* dL uniform in +-vol_step, weight N ln(L'/L) (fav)  */
#define JMM_VOLMOVE_LNL 1        /* ln L uniform in +-vol_step, weight (N+1) ln(L'/L)  */
#define JMM_VOLSCHED_RANDOM 0    /* trial type uniform over N+1 each step (Step)       */
#define JMM_VOLSCHED_SWEEP 1     /* N displacements then one volume move per sweep     */
#define JMM_PREC_FAST 0          /* hardware reciprocal and exp: production            */
#define JMM_PREC_EXACT 1         /* IEEE reciprocal, portable exp: replayable on a CPU */
#define JMM_INIT_LATTICE 0       /* r_i = ((i+0.5)/N - 0.5) L  (jmmMCState.cpp:559-562) */
#define JMM_INIT_JITTER 1        /* lattice plus U(-jitter, jitter) per particle        */

typedef struct jmm_chain_desc {
  uint32_t n;          /* particles                                          */
  int32_t potential;   /* JMM_POT_LJCUT | JMM_POT_SOFTSPHERE | JMM_POT_GAUSS */
  int32_t ensemble;    /* JMM_NLT (constant L) | JMM_NPT                     */
  int32_t reserved0;
  double eps;
  double sigma;
  double cutoff;
  double t;            /* temperature                                        */
  double p;            /* pressure (NPT)                                     */
  double l0;           /* initial box length                                 */
  double max_step;     /* displacement half-width                            */
  double vol_step;     /* ln L half-width (LNL) or max dL (LINEAR)           */
} jmm_chain_desc;

typedef struct jmm_batch_config {
  uint64_t seed;
  int32_t boundary;          /* JMM_BOUNDARY_*                                  */
  int32_t vol_move;          /* JMM_VOLMOVE_*                                   */
  int32_t vol_schedule;      /* JMM_VOLSCHED_*                                  */
  int32_t precision;         /* JMM_PREC_*                                      */
  uint32_t resum_sweeps;     /* constant-L chains: FP64 re-sum of E every this
                                many sweeps (0 = only at the end of a run)      */
  uint32_t lanes_per_chain;  /* lanes G of one trial move: 2, 4, 8, 16 or 32;
                                0 = 4 in EXACT precision, and in FAST a default
                                shape per potential class from its densest and
                                its longest chain (4x8, or 2x16 with a chain
                                of 1024 or more; window 8 where more than 4
                                neighbours per side fall within the cut-off;
                                32x1 beyond 8)                                  */
  uint32_t steps_per_round;  /* S steps evaluated at once per chain: G x S is
                                2x16, 4x8, 4x4, 4x2, 8x4, 8x2, 16x2, 16x1 or
                                32x1; 0 = 32/G                                  */
  uint32_t chains_per_block; /* 0 = 128 / (G*S)                                 */
  int32_t init;              /* JMM_INIT_*                                      */
  double jitter;             /* half-width of the initial jitter               */
  uint32_t window;           /* neighbours W per side a trial move looks at
                                before it extends its window: 0 = max(4, G/2);
                                8 with the shapes 2x16, 4x8 and 8x4, 3 with
                                2x16                                           */
  uint32_t split_n;          /* 0, or at least 64: constant-L chains between
                                walls with split_n or more particles run
                                split, one block of up to 8 warps per chain:
                                per sweep the chain is cut into domains of
                                B = max(32, 32 ceil(N / 480)) particles from a
                                random offset, and the domains of one colour
                                make their steps at once, one warp each, then
                                the other colour (detailed balance as the
                                large chains' alternating-domain sweep); each
                                domain runs 4 lanes x 8 steps per round with a
                                window of 4, or 8 / 16 where the class's
                                window is wider.  A split chain's statistics
                                sample once per sweep (samples count sweeps).
                                NPT chains and rings always run whole.         */
} jmm_batch_config;

/* Per-chain state and statistics, FP64 (also the device-side record). */
typedef struct jmm_chain_result {
  double e;              /* running total energy                               */
  double l;              /* box length                                         */
  uint64_t steps;        /* attempted moves since creation                     */
  uint64_t samples;      /* steps accumulated since the last reset             */
  double sum_e, sum_e2, sum_l, sum_l2, sum_le, sum_rho, sum_rho2;
  uint64_t disp_acc, disp_att, vol_acc, vol_att;
  uint64_t pair_evals;   /* pair slots evaluated: 4 x window per displacement
                          * and per window extension; 2 per pair within the
                          * cut-off at the old or new length of a volume move,
                          * 1 per in-cut-off pair of a re-sum                */
  double max_drift;      /* largest |running E - fresh FP64 sum| at a re-sum   */
  uint32_t error;        /* JMM_ERR_* seen by the kernel, 0 = none             */
  uint32_t window_overflows; /* moves whose neighbour window was extended      */
} jmm_chain_result;

typedef struct jmm_batch jmm_batch;

int jmm_batch_create(const jmm_batch_config *cfg, const jmm_chain_desc *chains,
                     uint32_t n_chains, jmm_batch **out);
/* As jmm_batch_create, starting from the caller's positions instead of the
 * configured lattice: x holds the chains' positions back to back (FP32,
 * sum of N floats, each chain strictly increasing, within +-l0/2 between
 * walls), the box lengths are the chains' l0. */
int jmm_batch_create_at(const jmm_batch_config *cfg, const jmm_chain_desc *chains,
                        uint32_t n_chains, const float *x, jmm_batch **out);
/* n_sweeps sweeps of every chain (N steps, N+1 with volume moves), then wait. */
int jmm_batch_run(jmm_batch *b, uint64_t n_sweeps);
/* Same, enqueued on a CUDA stream (cudaStream_t passed as void*), no wait. */
int jmm_batch_run_async(jmm_batch *b, uint64_t n_sweeps, void *stream);
int jmm_batch_results(jmm_batch *b, jmm_chain_result *out, uint32_t n_chains);
/* Replaces every chain's record (state and sums: energy, box length, step
 * count, accumulators, counters), e.g. from a checkpoint taken with
 * jmm_batch_results together with the positions: the chains then continue
 * exactly as the checkpointed ones (the step count selects the Philox
 * blocks).  Box lengths must be positive; with walls every chain's positions
 * must lie within +-l/2 of the record's box length. */
int jmm_batch_set_results(jmm_batch *b, const jmm_chain_result *in, uint32_t n_chains);
/* Zero the statistics (sums, samples, counters) but keep the state. */
int jmm_batch_reset_stats(jmm_batch *b);
int jmm_batch_get_positions(jmm_batch *b, uint32_t chain, float *x, uint32_t n);
int jmm_batch_set_positions(jmm_batch *b, uint32_t chain, const float *x, uint32_t n,
                            double l);
/* FP64 sums of the FP32 pair energies of every chain's current positions. */
int jmm_batch_energies(jmm_batch *b, double *e, uint32_t n_chains);
/* The two energies a volume move of every chain compares (fav's ETrial and
 * E, src/jmmMCState.cpp:2193-2249), formed as the chain kernel's volume move
 * forms them (same lanes, order and precision): out[3k .. 3k+2] = U_old of
 * the current positions, U_new of the positions and box scaled by scale[k]
 * (FP32 products x_i * s, box length l * s), and U_new - U_old (FP64; in
 * FAST precision an FP64 sum of per-pair differences, and U_new = U_old +
 * that).  The state is not changed.  NaN where the chain's window would
 * reach half a periodic ring. */
int jmm_batch_volume_energies(jmm_batch *b, const float *scale, double *out, uint32_t n_chains);
/* Device addresses of the positions (float, chain k at offsets[k]) and of the
 * jmm_chain_result array, for zero-copy tooling (torch, benchmarks). */
int jmm_batch_device_views(jmm_batch *b, void **positions, void **results,
                           uint64_t *offsets, uint32_t n_chains);
/* Time candidate launch shapes on a copy of the state and keep the fastest:
 * in FAST precision one per potential class (each class timed alone), in
 * EXACT one for the whole batch; writes the lanes_per_chain,
 * steps_per_round and chains_per_block of the largest class. */
int jmm_batch_autotune(jmm_batch *b, uint32_t trial_sweeps, uint32_t *lanes_per_chain,
                       uint32_t *steps_per_round, uint32_t *chains_per_block);
/* The launch shape of each potential class (LJcut, soft sphere, Gaussian
 * core): shapes[4k .. 4k+3] = lanes, steps per round, chains per block,
 * neighbours per side; 0 for a class without chains (n = 12). */
int jmm_batch_shapes(jmm_batch *b, uint32_t *shapes, uint32_t n);
/* Step-size adjustment on the device, enqueued on the batch's stream
 * (maxDisAdjust / maxDVAdjust, src/jmmMCState.cpp:2100-2139, per chain from
 * its counts since creation or the last reset): what = 1 displacement,
 * 2 volume, 3 both; the next run uses the new sizes.  A linear volume step
 * keeps the reference's clamps in units of N, an ln L step stays in
 * [1e-4, 1]. */
int jmm_batch_adjust_steps(jmm_batch *b, double ideal_ratio, int32_t what);
/* The current maximum displacement and volume step of every chain. */
int jmm_batch_step_sizes(jmm_batch *b, double *max_step, double *vol_step, uint32_t n_chains);
int jmm_batch_destroy(jmm_batch *b);

/* ---- energy gradients (the backward of U) ------------------------------ */

/* One chain configuration for jmm_energy_grad. */
typedef struct jmm_grad_chain {
  uint64_t x_off;      /* float offset of the chain's positions                */
  uint32_t n;
  int32_t potential;   /* JMM_POT_LJCUT | JMM_POT_SOFTSPHERE | JMM_POT_GAUSS   */
  double eps;
  double sigma;
  double cutoff;
  double l;            /* box length                                          */
} jmm_grad_chain;

/* Per-chain gradient statistics of a sampled run (FP64): the moments the
 * fluctuation formulas d<A>/dtheta = -beta(<A dU/dtheta> - <A><dU/dtheta>)
 * need, for theta = eps, sigma, L (g[0], g[1], g[2]). */
typedef struct jmm_grad_stats {
  uint64_t samples;
  double sum_u, sum_u2, sum_rho, sum_rho2, sum_l;
  double sum_g[3];
  double sum_u_g[3];
  double sum_rho_g[3];
  double sum_l_g[3];
} jmm_grad_stats;

/* U, dU/deps, dU/dsigma and dU/dL (positions scaled with the box) of every
 * configuration, as out[4k .. 4k+3] (FP64), with FP32 pair terms and FP64
 * sums; forces: NULL, or -dU/dx per particle at the chains' offsets.
 * chains, x, out and forces are device pointers; enqueued on stream (a
 * cudaStream_t as void*, NULL = the default stream), no wait.  The call
 * cannot see their sizes: the caller guarantees n_chains records in chains,
 * x_off + n positions of x for every record (forces likewise) and 4 n_chains
 * doubles of out. */
int jmm_energy_grad(const jmm_grad_chain *chains, uint32_t n_chains, const float *x,
                    int32_t boundary, double *out, float *forces, void *stream);
/* The same for a batch's current configurations, into host memory. */
int jmm_batch_energy_grad(jmm_batch *b, double *out, uint32_t n_chains);
/* n_sweeps sweeps; after every sample_every sweeps the configuration of every
 * chain and its energy gradient are added to the chain's jmm_grad_stats (one
 * CUDA graph: chain kernel, gradient kernel, chain kernel, ...). */
int jmm_batch_run_sampled(jmm_batch *b, uint64_t n_sweeps, uint32_t sample_every);
/* Same, enqueued on a CUDA stream (cudaStream_t as void*, NULL = the batch's
 * own), no wait. */
int jmm_batch_run_sampled_async(jmm_batch *b, uint64_t n_sweeps, uint32_t sample_every,
                                void *stream);
int jmm_batch_grad_stats(jmm_batch *b, jmm_grad_stats *out, uint32_t n_chains);

/* Sampled rho(x) and g(x) histograms of every chain, the layout of the
 * reference's printRho / printG (src/jmmMCState.cpp:1021-1061) and its bin
 * rules (fgrho / qagrho, :1069-1127, :2297-2384): rhonb position bins
 * floor(x / rbw + rhonb/2); gns slices floor(x / gsw + gns/2) x gnb
 * separation bins floor(|x_j - x_i| / gbw), each pair counted in the slice
 * of both particles (FP32 arithmetic on the chains' positions).  Unlike the
 * reference, which adds the counts of every step, a batch adds a sample
 * when asked: jmm_batch_sample_histograms, and after every sample_every
 * sweeps of jmm_batch_run_sampled once histograms are configured.
 * Configuring (again) clears them. */
int jmm_batch_histograms(jmm_batch *b, uint32_t rhonb, double rbw, uint32_t gns, double gsw,
                         uint32_t gnb, double gbw);
/* Adds the current configuration of every chain, enqueued on stream
 * (cudaStream_t as void*, NULL = the batch's own), no wait. */
int jmm_batch_sample_histograms(jmm_batch *b, void *stream);
/* Per chain (user order) one row of 1 + rhonb + gns*gnb counts: samples,
 * rho bins, then g bins slice by slice; n = n_chains * row length. */
int jmm_batch_take_histograms(jmm_batch *b, uint64_t *out, uint64_t n);

/* Host-buffer convenience: create, upload positions (NULL = the configured
 * initial lattice), run n_sweeps, copy results and positions back, destroy. */
int jmm_batch_run_host(const jmm_batch_config *cfg, const jmm_chain_desc *chains,
                       uint32_t n_chains, const float *x_in, uint64_t n_sweeps,
                       jmm_chain_result *results, float *x_out);

/* ---- large chains (N up to 2^24): the alternating-domain sweep ---------- */
/* No counterpart in the reference, which holds O(N^2) pair arrays per chain
 * (src/jmmMCState.cpp:308-328,439-455) and cannot run N = 2^20.  Constant-L
 * chains with hard walls; positions are int64 multiples of a grid step 2^-k
 * per chain (chosen so that a domain spans < 2^23 steps), exact in the FP32
 * step arithmetic; trial displacements are snapped to the grid. */

#define JMM_LARGE_DOMAINS 0     /* alternating-domain sweep: domains of B
                                   particles from a random offset, two colours
                                   in random order, one warp per domain       */
#define JMM_LARGE_SEQUENTIAL 1  /* plain sweep: one warp per chain, N steps in
                                   order on the HBM positions                 */

typedef struct jmm_large_result {
  double e;              /* running total energy                               */
  double l;              /* box length                                         */
  uint64_t sweeps;       /* sweeps since creation                              */
  uint64_t samples;      /* sweeps accumulated since the last reset            */
  double sum_e, sum_e2;  /* one sample of E per sweep                          */
  uint64_t moves, accepted, pair_evals, window_overflows;
  double max_drift;      /* largest |running E - fresh FP64 sum| at a re-sum   */
  double grid;           /* positions are multiples of this step (2^-k)        */
  uint32_t error;        /* JMM_ERR_* seen by a kernel (JMM_ERR_INVALID: a
                            domain's 16-particle halo did not reach beyond the
                            cut-off, or the domain spanned more than 2^24 grid
                            steps; the domain was skipped that sweep)         */
  uint32_t reserved;
} jmm_large_result;

typedef struct jmm_large jmm_large;

/* Chains as jmm_chain_desc (ensemble JMM_NLT, potential LJCUT, SOFTSPHERE or
 * GAUSS, domain_size <= N <= 2^24); cfg gives seed, init/jitter and
 * resum_sweeps (boundary JMM_BOUNDARY_WALLS, precision JMM_PREC_FAST);
 * domain_size B in [32, 8192]. */
int jmm_large_create(const jmm_batch_config *cfg, const jmm_chain_desc *chains,
                     uint32_t n_chains, uint32_t domain_size, jmm_large **out);
/* n_sweeps sweeps (N steps each) in mode JMM_LARGE_*, then wait. */
int jmm_large_run(jmm_large *h, uint64_t n_sweeps, int32_t mode);
/* Same, enqueued on stream (cudaStream_t as void*, NULL = the handle's), no wait. */
int jmm_large_run_async(jmm_large *h, uint64_t n_sweeps, int32_t mode, void *stream);
int jmm_large_results(jmm_large *h, jmm_large_result *out, uint32_t n_chains);
int jmm_large_reset_stats(jmm_large *h);
/* Fresh energies of the current positions (FP32 pair terms, FP64 sums). */
int jmm_large_energies(jmm_large *h, double *e, uint32_t n_chains);
int jmm_large_get_positions(jmm_large *h, uint32_t chain, double *x, uint64_t n);
/* Positions are snapped to the grid, must then increase and lie within
 * +-L/2; energies are re-summed. */
int jmm_large_set_positions(jmm_large *h, uint32_t chain, const double *x, uint64_t n);
int jmm_large_destroy(jmm_large *h);
/* Host-buffer convenience: create, upload positions (NULL = the configured
 * initial lattice; chain after chain, snapped to the grid), run n_sweeps in
 * mode JMM_LARGE_*, copy results and positions (NULL = skip) back, destroy. */
int jmm_large_run_host(const jmm_batch_config *cfg, const jmm_chain_desc *chains,
                       uint32_t n_chains, uint32_t domain_size, int32_t mode,
                       const double *x_in, uint64_t n_sweeps, jmm_large_result *results,
                       double *x_out);

/* The Philox words of steps [block0, block0 + count) of one chain, computed
 * on the device (4 words per step), for RNG verification tooling. */
int jmm_rng_words(uint64_t seed, uint64_t block0, uint32_t chain, uint64_t count,
                  uint32_t *out);

/* Full FP64 pair sums (the nine totals that fad and ECheck form) of N
 * positions held in device memory by the caller, written as nine doubles to
 * the caller's device buffer `out`, enqueued on `stream` (cudaStream_t as
 * void*, NULL = the default stream); no device memory is allocated or freed.
 * It has no counterpart in the reference: it is for callers that cannot
 * allocate -- code capturing a CUDA graph, hosts that reserve all device
 * memory up front, per-step loops that cannot afford allocation latency.
 * The pair terms go through one fixed device array shared by all calls,
 * sized for N <= 256 (2.35 MB per GPU, held until exit): larger N fails with
 * JMM_ERR_INVALID, and calls that overlap on the GPU race on that array.
 * The first call on a device looks the array's address up; make it before
 * any stream capture.  JMM_ERR_INVALID also for a box length that is not
 * finite and positive, and for r or out that are not device (or managed)
 * memory of the current device. */
int jmm_plain_full_energy_noalloc(const jmm_params *params, const double *r, uint64_t n,
                                  double l, double *out, void *stream);

/* Roofline denominators measured live on the current device: FP32 FMA
 * throughput (TFLOP/s, 2 FLOP per FMA) and MUFU reciprocal throughput
 * (T ops/s), each the best of several event-timed launches. */
int jmm_measure_peaks(double *fp32_tflops, double *rcp_tops);

const char *jmm_last_error(void);
/* 1 when a CUDA device can be used by this library, else 0. */
int jmm_device_available(void);

#ifdef __cplusplus
}
#endif

#endif /* JMM_GPU_H */
