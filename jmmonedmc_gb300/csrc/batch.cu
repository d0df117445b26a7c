// batch.cu -- host side of the batched chain kernel (jmm_batch_* in
// include/jmm_gpu.h): validation, HBM layout, launch shapes, the CUDA graph
// that holds a run, the launch-shape autotuner and the host-buffer entry.
//
// Layout: positions are FP32, chain k at a 16-byte aligned offset (user
// order); per-chain parameters live in launch order (chains sorted by N,
// largest first, so that a block holds chains of similar length); each block
// stages its chains' positions in shared memory for the whole run.
#include <string.h>

#include <algorithm>
#include <cmath>
#include <map>
#include <new>
#include <numeric>
#include <vector>

#include "batch_core.cuh"
#include "common.cuh"
#include "grad_core.cuh"

using namespace jmm;
using namespace jmm::batch;

namespace {

constexpr size_t kMaxSmem = 227 * 1024;

typedef void (*ChainsKernel)(const ChainParams *, jmm_chain_result *, float *, KernelCfg);

template <int G, int S, bool E, int WIN = window_of(G)>
ChainsKernel pick_pot(int pot, bool per) {
  switch (pot * 2 + (per ? 1 : 0)) {
    case JMM_POT_LJCUT * 2: return chains_kernel<G, S, JMM_POT_LJCUT, false, E, WIN>;
    case JMM_POT_LJCUT * 2 + 1: return chains_kernel<G, S, JMM_POT_LJCUT, true, E, WIN>;
    case JMM_POT_SOFTSPHERE * 2: return chains_kernel<G, S, JMM_POT_SOFTSPHERE, false, E, WIN>;
    case JMM_POT_SOFTSPHERE * 2 + 1: return chains_kernel<G, S, JMM_POT_SOFTSPHERE, true, E, WIN>;
    case JMM_POT_GAUSS * 2: return chains_kernel<G, S, JMM_POT_GAUSS, false, E, WIN>;
    case JMM_POT_GAUSS * 2 + 1: return chains_kernel<G, S, JMM_POT_GAUSS, true, E, WIN>;
    default: return nullptr;
  }
}

// Launch shapes: G window lanes x S steps per round (G*S = 16 or 32 lanes),
// W neighbours per side (0 = the default of G); `wide`: the 128-register
// instantiation of a single-warp FAST shape (a batch with at most 16 such
// chains per SM).
ChainsKernel pick_kernel(uint32_t g, uint32_t s, uint32_t w, bool exact, int pot, bool per,
                         bool wide = false) {
  if (w == 0) w = (uint32_t)window_of((int)g);
  if (wide && !exact && g * s == 32) {
    ChainsKernel k = pick_kernel_wide(g, s, w, pot, per);
    if (k) return k;
  }
#define JMM_SHAPE(G_, S_, W_)                                                        \
  if (g == G_ && s == S_ && w == W_)                                                \
    return exact ? pick_pot<G_, S_, true, W_>(pot, per) : pick_pot<G_, S_, false, W_>(pot, per);
  JMM_SHAPE(4, 8, 4)
  JMM_SHAPE(2, 16, 4)
  JMM_SHAPE(2, 16, 3)
  JMM_SHAPE(4, 4, 4)
  JMM_SHAPE(4, 2, 4)
  JMM_SHAPE(8, 4, 4)
  JMM_SHAPE(8, 2, 4)
  JMM_SHAPE(16, 2, 8)
  JMM_SHAPE(16, 1, 8)
  JMM_SHAPE(32, 1, 16)
  JMM_SHAPE(4, 8, 8)
  JMM_SHAPE(2, 16, 8)
  JMM_SHAPE(8, 4, 8)
#undef JMM_SHAPE
  return nullptr;
}

constexpr int kPots[3] = {JMM_POT_LJCUT, JMM_POT_SOFTSPHERE, JMM_POT_GAUSS};

// Split chains (split_kernel): 4 lanes x 8 steps per round per domain, a
// window of 4, 8 or 16 neighbours per side.
template <bool E, int WIN>
ChainsKernel pick_split_pot(int pot) {
  switch (pot) {
    case JMM_POT_LJCUT: return split_kernel<4, 8, JMM_POT_LJCUT, E, WIN>;
    case JMM_POT_SOFTSPHERE: return split_kernel<4, 8, JMM_POT_SOFTSPHERE, E, WIN>;
    case JMM_POT_GAUSS: return split_kernel<4, 8, JMM_POT_GAUSS, E, WIN>;
    default: return nullptr;
  }
}

ChainsKernel pick_split(uint32_t w, bool exact, int pot) {
  switch (w) {
    case 4: return exact ? pick_split_pot<true, 4>(pot) : pick_split_pot<false, 4>(pot);
    case 8: return exact ? pick_split_pot<true, 8>(pot) : pick_split_pot<false, 8>(pot);
    case 16: return exact ? pick_split_pot<true, 16>(pot) : pick_split_pot<false, 16>(pot);
    default: return nullptr;
  }
}

// A chain that runs split: the batch asks for it (split_n) and the chain has
// constant L between walls and at least split_n particles.
bool is_split(const jmm_batch_config &cfg, const jmm_chain_desc &c) {
  return cfg.split_n > 0 && c.n >= cfg.split_n && c.ensemble == JMM_NLT &&
         cfg.boundary == JMM_BOUNDARY_WALLS;
}

// The window of a potential class's split chains from the class's window:
// 8 or 16 where the class needs more than 4 neighbours per side, else 4.
uint32_t split_window(uint32_t w) { return w > 8 ? 16u : (w > 4 ? 8u : 4u); }

// The chains of one potential: a contiguous range of launch slots with its
// own blocks and shared-memory size.
// A launch shape: G window lanes x S steps per round, chains per block, W
// neighbours per side.
struct Shape {
  uint32_t g, spr, cpb, w;
};

struct PotClass {
  int pot;
  Shape shape;
  uint32_t first, count;
  uint32_t n_blocks;
  size_t smem;
  bool split = false;   // split chains: one block of `warps` warps per chain
  uint32_t warps = 0;
  bool wide = false;    // the 128-register kernel (pick_kernel)
};

constexpr int kMaxClasses = 6;  // three potentials, each whole and split

uint64_t pad4(uint64_t n) { return (n + 3) & ~uint64_t(3); }

}  // namespace

struct jmm_batch {
  jmm_batch_config cfg;
  uint32_t n_chains = 0;
  std::vector<jmm_chain_desc> chains;
  std::vector<uint64_t> x_off;  // by user index
  std::vector<uint32_t> order;  // launch order -> user index
  uint64_t total_floats = 0;
  std::vector<ChainParams> params;  // launch order
  char *d_block = nullptr;  // the one device allocation behind the arrays below
  ChainParams *d_params = nullptr;
  jmm_chain_result *d_res = nullptr;
  float *d_x = nullptr;
  double *d_e = nullptr;
  uint32_t g = 8, spr = 4, cpb = 4, win = 4, n_blocks = 0;  // the shape of the largest class
  uint32_t n_sm = 0;  // SMs of the batch's device
  Shape shapes[3] = {{8, 4, 4, 4}, {8, 4, 4, 4}, {8, 4, 4, 4}};  // per potential class (kPots order)
  size_t smem = 0;
  cudaStream_t stream = nullptr;
  std::map<uint64_t, cudaGraphExec_t> graphs;  // n_sweeps -> instantiated run
  std::vector<PotClass> classes;
  cudaStream_t side[kMaxClasses] = {};  // concurrent classes in a graph
  cudaEvent_t fork = nullptr, join[kMaxClasses] = {};
  // energy gradients and their sampled statistics
  jmm_chain_desc *d_desc = nullptr;     // user order
  uint64_t *d_xoff = nullptr;           // user order
  uint64_t *d_poff = nullptr;           // user order: offsets in the packed layout
  float *d_pack = nullptr;              // positions back to back (host-buffer copies)
  uint64_t n_packed = 0;
  double *d_gout = nullptr;             // 4 per chain
  jmm_grad_stats *d_gstats = nullptr;   // user order
  std::map<std::pair<uint64_t, uint32_t>, cudaGraphExec_t> sampled;  // (sweeps, every)
  // sampled rho(x) / g(x) histograms (jmm_batch_histograms): one row per chain
  uint64_t *d_hist = nullptr;
  uint32_t h_rhonb = 0, h_gns = 0, h_gnb = 0;
  float h_rbw = 0.0f, h_gsw = 0.0f, h_gbw = 0.0f;
};

static void drop_graphs(jmm_batch *b) {
  for (auto &kv : b->graphs) cudaGraphExecDestroy(kv.second);
  b->graphs.clear();
  for (auto &kv : b->sampled) cudaGraphExecDestroy(kv.second);
  b->sampled.clear();
}

static void batch_free(jmm_batch *b) {
  if (!b) return;
  drop_graphs(b);
  cudaFree(b->d_block);  // every device array of the batch
  cudaFree(b->d_hist);
  for (int k = 0; k < kMaxClasses; ++k) {
    if (b->side[k]) cudaStreamDestroy(b->side[k]);
    if (b->join[k]) cudaEventDestroy(b->join[k]);
  }
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
}

// Step sizes changed on the device (jmm_batch_adjust_steps) back into the
// chain descriptions, so that a new layout keeps them.
static int sync_step_sizes(jmm_batch *b) {
  if (b->params.empty() || !b->d_params) return JMM_OK;
  std::vector<ChainParams> cur(b->params.size());
  JMM_CUDA(cudaStreamSynchronize(b->stream));
  JMM_CUDA(cudaMemcpy(cur.data(), b->d_params, cur.size() * sizeof(ChainParams),
                      cudaMemcpyDeviceToHost));
  for (const ChainParams &P : cur) {
    jmm_chain_desc &c = b->chains[P.id];
    c.max_step = 0.5 * (double)P.two_max_step;
    c.vol_step = (double)P.vol_step;
  }
  return JMM_OK;
}

// Per-chain kernel parameters for one launch shape per potential class
// (kPots order); uploads them.
static int apply_layout(jmm_batch *b, const Shape shapes[3]) {
  const bool per = b->cfg.boundary == JMM_BOUNDARY_PERIODIC;
  {
    const int rc = sync_step_sizes(b);
    if (rc) return rc;
  }
  const bool exact = b->cfg.precision == JMM_PREC_EXACT;
  std::vector<ChainParams> prm(b->n_chains);
  std::vector<PotClass> classes;
  uint32_t slot0 = 0;
  // the chain parameters every launch takes
  auto fill = [&](uint32_t slot, uint32_t s_off) {
    const uint32_t id = b->order[slot];
    const jmm_chain_desc &c = b->chains[id];
    ChainParams &P = prm[slot];
    memset(&P, 0, sizeof(P));
    P.id = id;
    P.n = c.n;
    P.pot = (uint32_t)c.potential;
    P.ensemble = (uint32_t)c.ensemble;
    P.steps_per_sweep = c.ensemble == JMM_NPT ? c.n + 1 : c.n;
    P.s_off = s_off;
    P.x_off = b->x_off[id];
    P.eps4 = c.potential == JMM_POT_LJCUT ? (float)(4.0 * c.eps) : (float)c.eps;
    P.sigma2 = (float)(c.sigma * c.sigma);
    P.inv_sigma2 = (float)(1.0 / (c.sigma * c.sigma));
    P.rc2 = (float)(c.cutoff * c.cutoff);
    P.rc = (float)c.cutoff;
    P.beta = (float)(1.0 / c.t);
    P.beta_d = 1.0 / c.t;
    P.p = c.p;
    P.two_max_step = (float)(2.0 * c.max_step);
    P.vol_step = (float)c.vol_step;
  };
  // Single-warp FAST classes take the 128-register kernel when the batch's
  // chains that run whole come to at most 16 warps per SM (a full wave at
  // 72 registers holds 27).
  double whole_warps = 0.0;
  for (const jmm_chain_desc &c : b->chains) {
    if (is_split(b->cfg, c)) continue;
    for (int pi = 0; pi < 3; ++pi)
      if (c.potential == kPots[pi]) whole_warps += shapes[pi].g * shapes[pi].spr / 32.0;
  }
  const bool wide = !exact && b->n_sm > 0 && whole_warps <= 16.0 * b->n_sm;
  for (int pi = 0; pi < 3; ++pi) {
    const int pot = kPots[pi];
    // split chains of this potential: the leading ones in launch order, one
    // block each, as many warps as the largest one's colour has domains
    {
      PotClass sc;
      sc.pot = pot;
      sc.shape = Shape{4, 8, 1, split_window(shapes[pi].w ? shapes[pi].w
                                                            : (uint32_t)window_of((int)shapes[pi].g))};
      sc.first = slot0;
      sc.count = 0;
      sc.split = true;
      sc.warps = 1;
      sc.smem = 0;
      while (slot0 + sc.count < b->n_chains) {
        const jmm_chain_desc &c = b->chains[b->order[slot0 + sc.count]];
        if (c.potential != pot || !is_split(b->cfg, c)) break;
        const uint32_t dom = split_domain_size(c.n);
        const uint32_t per_colour = (c.n / dom + 2u + 1u) / 2u;
        sc.warps = std::max(sc.warps, std::min(kSplitWarps, per_colour));
        fill(slot0 + sc.count, 0);
        prm[slot0 + sc.count].dom = dom;
        sc.count++;
      }
      if (sc.count) {
        for (uint32_t k = 0; k < sc.count; ++k)
          sc.smem = std::max(sc.smem,
                             (size_t)split_smem_bytes(prm[sc.first + k].n, sc.warps));
        // the kernel's own static shared memory (per-warp tallies) comes on top
        if (sc.smem + 1024 > kMaxSmem)
          return fail(JMM_ERR_INVALID, "a split chain needs %zu bytes of shared memory (max %zu)",
                      sc.smem, kMaxSmem - 1024);
        sc.n_blocks = sc.count;
        ChainsKernel kf = pick_split(sc.shape.w, exact, pot);
        if (sc.smem > 48 * 1024)
          JMM_CUDA(cudaFuncSetAttribute(kf, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)sc.smem));
        classes.push_back(sc);
        slot0 += sc.count;
      }
    }
    const uint32_t g = shapes[pi].g, spr = shapes[pi].spr, cpb = shapes[pi].cpb;
    const uint32_t win = shapes[pi].w ? shapes[pi].w : (uint32_t)window_of((int)g);
    if (!pick_kernel(g, spr, win, false, JMM_POT_LJCUT, false))
      return fail(JMM_ERR_INVALID, "unsupported launch shape: lanes_per_chain x steps_per_round "
                  "must be 2x16, 4x8, 4x4, 4x2, 8x4, 8x2, 16x2, 16x1 or 32x1, with a window "
                  "of 0 (the default), 8 for 2x16, 4x8 and 8x4, or 3 for 2x16");
    if (cpb == 0 || cpb * g * spr > 256)
      return fail(JMM_ERR_INVALID, "chains_per_block * lanes per chain must be <= 256");
    const uint64_t ring_floats = (uint64_t)cpb * kRingWords;
    PotClass pc;
    pc.pot = pot;
    pc.shape = shapes[pi];
    pc.shape.w = win;
    pc.first = slot0;
    pc.count = 0;
    pc.wide = wide && g * spr == 32;
    while (slot0 + pc.count < b->n_chains && b->chains[b->order[slot0 + pc.count]].potential == pot)
      pc.count++;
    if (per) {
      for (uint32_t k = 0; k < pc.count; ++k)
        if (b->chains[b->order[pc.first + k]].n < 2 * win + 1)
          return fail(JMM_ERR_INVALID, "periodic chains need N > twice the neighbour window");
    }
    pc.n_blocks = (pc.count + cpb - 1) / cpb;
    pc.smem = 0;
    for (uint32_t blk = 0; blk < pc.n_blocks; ++blk) {
      uint64_t s_off = ring_floats;
      for (uint32_t k = 0; k < cpb; ++k) {
        const uint32_t local = blk * cpb + k;
        if (local >= pc.count) break;
        fill(pc.first + local, (uint32_t)s_off);
        s_off += pad4(b->chains[b->order[pc.first + local]].n + 2 * kGhost);
      }
      pc.smem = std::max(pc.smem, (size_t)s_off * sizeof(float));
    }
    if (pc.smem > kMaxSmem)
      return fail(JMM_ERR_INVALID, "a block's chains need %zu bytes of shared memory (max %zu): "
                  "lower chains_per_block", pc.smem, kMaxSmem);
    if (pc.count) {
      ChainsKernel kf = pick_kernel(g, spr, win, exact, pot, per, pc.wide);
      JMM_CUDA(cudaFuncSetAttribute(kf, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMaxSmem));
      classes.push_back(pc);
    }
    slot0 += pc.count;
  }
  JMM_CUDA(cudaMemcpy(b->d_params, prm.data(), prm.size() * sizeof(ChainParams),
                      cudaMemcpyHostToDevice));
  b->params.swap(prm);
  b->classes.swap(classes);
  uint32_t most = 0;
  for (int pi = 0; pi < 3; ++pi) {
    b->shapes[pi] = shapes[pi];
    if (!b->shapes[pi].w) b->shapes[pi].w = (uint32_t)window_of((int)shapes[pi].g);
  }
  for (const PotClass &pc : b->classes) {
    if (!pc.split && pc.count > most) {
      most = pc.count;
      b->g = pc.shape.g;
      b->spr = pc.shape.spr;
      b->cpb = pc.shape.cpb;
      b->win = pc.shape.w;
    }
  }
  drop_graphs(b);
  return JMM_OK;
}

// The FAST default launch shape of each potential class (kPots order).
static void default_shapes(const jmm_batch *b, Shape sh[3]) {
  // From the densest chain's neighbours within the cut-off and the longest
  // chain.  A 12-power core keeps LJ and soft-sphere neighbours at least
  // ~0.85 sigma apart, a Gaussian core lets them overlap (about 1.5 rho rc
  // per side at the densest).  Windows of 4 or 8 per side take 8 steps per
  // round, or 16 where the class holds a chain of 1024 or more particles (a
  // class lasts as long as its longest chain, whose rounds rarely conflict).
  // The window comes from every chain of the class (split chains take the
  // class's window too), the round shape from the chains that run whole.
  for (int pi = 0; pi < 3; ++pi) {
    double need = 0.0;
    uint32_t n_max = 0;
    for (const auto &c : b->chains) {
      if (c.potential != kPots[pi]) continue;
      const double side = c.potential == JMM_POT_GAUSS ? 1.5 * c.n / c.l0 * c.cutoff
                                                       : c.cutoff / (0.85 * c.sigma);
      need = std::max(need, side);
      if (!is_split(b->cfg, c)) n_max = std::max(n_max, c.n);
    }
    const uint32_t gg = need > 8.0 ? 32u : (n_max >= 1024 ? 2u : 4u);
    const uint32_t ss = 32 / gg;
    // two lanes a step may look at 3 neighbours per side where 3 suffice
    const uint32_t ww = need > 8.0 ? 16u : (need > 4.0 ? 8u : (need > 3.0 || gg != 2 ? 4u : 3u));
    sh[pi] = Shape{gg, ss, 128 / (gg * ss), ww};
  }
}

// The same launch shape for every class.
static int apply_layout(jmm_batch *b, uint32_t g, uint32_t spr, uint32_t cpb, uint32_t w) {
  const Shape sh[3] = {{g, spr, cpb, w}, {g, spr, cpb, w}, {g, spr, cpb, w}};
  return apply_layout(b, sh);
}

// One launch per potential class; with several classes they run on forked
// streams that rejoin `s`, so that a graph holds them as parallel nodes.
// Class k's kernel on stream st.
static int launch_class(jmm_batch *b, size_t k, uint64_t n_sweeps, cudaStream_t st) {
  const PotClass &pc = b->classes[k];
  KernelCfg kc;
  kc.seed = b->cfg.seed;
  kc.n_sweeps = n_sweeps;
  kc.boundary = b->cfg.boundary;
  kc.vol_move = b->cfg.vol_move;
  kc.vol_schedule = b->cfg.vol_schedule;
  kc.resum_sweeps = (int32_t)b->cfg.resum_sweeps;
  kc.chains_per_block = pc.shape.cpb;
  kc.n_chains = pc.count;
  const bool per = b->cfg.boundary == JMM_BOUNDARY_PERIODIC;
  const bool exact = b->cfg.precision == JMM_PREC_EXACT;
  if (pc.split) {
    ChainsKernel kf = pick_split(pc.shape.w, exact, pc.pot);
    kf<<<pc.n_blocks, 32 * pc.warps, pc.smem, st>>>(b->d_params + pc.first, b->d_res, b->d_x, kc);
    JMM_CUDA(cudaGetLastError());
    return JMM_OK;
  }
  const uint32_t threads = pc.shape.g * pc.shape.spr * pc.shape.cpb;
  ChainsKernel kf = pick_kernel(pc.shape.g, pc.shape.spr, pc.shape.w, exact, pc.pot, per, pc.wide);
  kf<<<pc.n_blocks, threads, pc.smem, st>>>(b->d_params + pc.first, b->d_res, b->d_x, kc);
  JMM_CUDA(cudaGetLastError());
  return JMM_OK;
}

static int launch(jmm_batch *b, uint64_t n_sweeps, cudaStream_t s) {
  const bool fork = b->classes.size() > 1;
  if (fork) JMM_CUDA(cudaEventRecord(b->fork, s));
  for (size_t k = 0; k < b->classes.size(); ++k) {
    cudaStream_t st = fork ? b->side[k] : s;
    if (fork) JMM_CUDA(cudaStreamWaitEvent(st, b->fork, 0));
    const int rc = launch_class(b, k, n_sweeps, st);
    if (rc) return rc;
    if (fork) {
      JMM_CUDA(cudaEventRecord(b->join[k], st));
      JMM_CUDA(cudaStreamWaitEvent(s, b->join[k], 0));
    }
  }
  return JMM_OK;
}

static int energies(jmm_batch *b, cudaStream_t s) {
  const uint32_t per_block = 8;
  const uint32_t blocks = (b->n_chains + per_block - 1) / per_block;
  if (b->cfg.precision == JMM_PREC_EXACT)
    energies_kernel<true><<<blocks, 32 * per_block, 0, s>>>(b->d_params, b->d_x, b->d_res, b->d_e,
                                                           b->n_chains, b->cfg.boundary);
  else
    energies_kernel<false><<<blocks, 32 * per_block, 0, s>>>(b->d_params, b->d_x, b->d_res, b->d_e,
                                                            b->n_chains, b->cfg.boundary);
  JMM_CUDA(cudaGetLastError());
  return JMM_OK;
}

__global__ void set_energies_kernel(jmm_chain_result *res, const double *e, uint32_t n) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) res[i].e = e[i];
}

static int validate(const jmm_batch_config *cfg, const jmm_chain_desc *chains, uint32_t n_chains) {
  JMM_CHECK_ARG(cfg && chains && n_chains > 0, "null argument or no chains");
  JMM_CHECK_ARG(cfg->boundary == JMM_BOUNDARY_WALLS || cfg->boundary == JMM_BOUNDARY_PERIODIC,
                "unknown boundary");
  JMM_CHECK_ARG(cfg->vol_move == JMM_VOLMOVE_LINEAR || cfg->vol_move == JMM_VOLMOVE_LNL,
                "unknown volume move");
  JMM_CHECK_ARG(cfg->vol_schedule == JMM_VOLSCHED_RANDOM || cfg->vol_schedule == JMM_VOLSCHED_SWEEP,
                "unknown volume schedule");
  JMM_CHECK_ARG(cfg->precision == JMM_PREC_FAST || cfg->precision == JMM_PREC_EXACT,
                "unknown precision");
  JMM_CHECK_ARG(cfg->split_n == 0 || cfg->split_n >= 64,
                "split_n must be 0 (no split chains) or at least 64");
  if (cfg->lanes_per_chain) {
    const uint32_t g = cfg->lanes_per_chain;
    const uint32_t spr = cfg->steps_per_round ? cfg->steps_per_round : (g <= 32 ? 32 / g : 1);
    if (!pick_kernel(g, spr, cfg->window, false, JMM_POT_LJCUT, false))
      return fail(JMM_ERR_INVALID, "unsupported launch shape: lanes_per_chain x steps_per_round "
                  "must be 2x16, 4x8, 4x4, 4x2, 8x4, 8x2, 16x2, 16x1 or 32x1, with a window "
                  "of 0 (the default), 8 for 2x16, 4x8 and 8x4, or 3 for 2x16");
  }
  for (uint32_t k = 0; k < n_chains; ++k) {
    const jmm_chain_desc &c = chains[k];
    if (c.n < 2 || c.n > 16384)
      return fail(JMM_ERR_INVALID, "chain %u: N must be in [2, 16384]", k);
    if (c.potential != JMM_POT_LJCUT && c.potential != JMM_POT_SOFTSPHERE &&
        c.potential != JMM_POT_GAUSS)
      return fail(JMM_ERR_INVALID, "chain %u: potential must be LJcut, soft sphere or Gaussian", k);
    if (c.ensemble != JMM_NLT && c.ensemble != JMM_NPT)
      return fail(JMM_ERR_INVALID, "chain %u: unknown ensemble", k);
    if (!(c.t > 0) || !(c.l0 > 0) || !(c.sigma > 0) || !(c.cutoff > 0) || !(c.max_step > 0))
      return fail(JMM_ERR_INVALID, "chain %u: T, L, sigma, cut-off and step must be positive", k);
    if (!std::isfinite(c.t) || !std::isfinite(c.l0) || !std::isfinite(c.sigma) ||
        !std::isfinite(c.cutoff) || !std::isfinite(c.max_step) || !std::isfinite(c.eps) ||
        !std::isfinite(c.p) || !std::isfinite(c.vol_step) || !(c.vol_step >= 0))
      return fail(JMM_ERR_INVALID, "chain %u: parameters must be finite (volume step >= 0)", k);
    if (cfg->boundary == JMM_BOUNDARY_PERIODIC && !(c.l0 > 2 * c.cutoff))
      return fail(JMM_ERR_INVALID, "chain %u: a periodic ring needs L > 2 cut-off", k);
    const double spacing = c.l0 / c.n;
    if (cfg->init == JMM_INIT_JITTER && !(cfg->jitter >= 0 && cfg->jitter < 0.5 * spacing))
      return fail(JMM_ERR_INVALID, "chain %u: jitter must be below half the lattice spacing", k);
  }
  return JMM_OK;
}

// Lattice r_i = ((i+0.5)/N - 0.5) L (src/jmmMCState.cpp:559-562), plus the
// optional jitter from Philox blocks (2^63 + i) of the chain's stream.
static void initial_positions(const jmm_batch_config *cfg, const jmm_chain_desc &c, uint32_t id,
                              float *x) {
  for (uint32_t i = 0; i < c.n; ++i) {
    double r = ((i + 0.5) / c.n - 0.5) * c.l0;
    if (cfg->init == JMM_INIT_JITTER) {
      const Words4 w = step_words(cfg->seed, (1ull << 63) | i, id);
      r += cfg->jitter * (2.0 * word_to_unit(w.w[0]) - 1.0);
    }
    x[i] = (float)r;
  }
}

// Positions between the packed layout (chains back to back) and the padded
// one; one warp per chain.
__global__ void unpack_positions_kernel(const float *__restrict__ pack, float *__restrict__ x,
                                        const uint64_t *__restrict__ poff,
                                        const uint64_t *__restrict__ xoff,
                                        const jmm_chain_desc *__restrict__ desc, uint32_t n_chains) {
  const uint32_t c = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
  if (c >= n_chains) return;
  const uint32_t n = desc[c].n;
  for (uint32_t i = threadIdx.x & 31; i < n; i += 32) x[xoff[c] + i] = pack[poff[c] + i];
}

__global__ void pack_positions_kernel(const float *__restrict__ x, float *__restrict__ pack,
                                      const uint64_t *__restrict__ poff,
                                      const uint64_t *__restrict__ xoff,
                                      const jmm_chain_desc *__restrict__ desc, uint32_t n_chains) {
  const uint32_t c = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
  if (c >= n_chains) return;
  const uint32_t n = desc[c].n;
  for (uint32_t i = threadIdx.x & 31; i < n; i += 32) pack[poff[c] + i] = x[xoff[c] + i];
}

// A fresh result record per chain: zero sums, the box length l0.
__global__ void init_results_kernel(jmm_chain_result *__restrict__ res,
                                    const jmm_chain_desc *__restrict__ desc, uint32_t n_chains) {
  const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n_chains) return;
  jmm_chain_result r;
  memset(&r, 0, sizeof(r));
  r.l = desc[c].l0;
  res[c] = r;
}

// Positions a caller gives for one chain (index `chain`): finite, strictly
// increasing, within the walls at +-L/2 (the kernel's own wall test, |x| <=
// L/2 rounded to FP32, with room for the rounding of positions that a volume
// move scaled in FP32), or spanning less than L on a ring.
static int check_host_positions(const float *x, uint32_t n, double l, bool periodic,
                                uint32_t chain) {
  if (!(l > 0)) return fail(JMM_ERR_INVALID, "chain %u: box length must be positive", chain);
  const float half = (float)(0.5 * l) * (1.0f + 1e-6f);
  // branch-free passes first (comparisons with NaN are false, so NaN counts
  // as bad); the element loop below only names the first bad position
  uint32_t bad = n > 0 && !(x[0] == x[0]);
  for (uint32_t i = 1; i < n; ++i) bad |= (uint32_t)!(x[i] > x[i - 1]);
  if (!periodic)
    for (uint32_t i = 0; i < n; ++i) bad |= (uint32_t)!(fabsf(x[i]) <= half);
  else
    bad |= (uint32_t)(n > 0 && !(x[n - 1] < x[0] + l));
  if (!bad) return JMM_OK;
  for (uint32_t i = 0; i < n; ++i) {
    if (!(x[i] == x[i]) || (i > 0 && !(x[i] > x[i - 1])))
      return fail(JMM_ERR_INVALID, "chain %u: positions must be finite and strictly increasing",
                  chain);
    if (!periodic && !(fabsf(x[i]) <= half))
      return fail(JMM_ERR_INVALID, "chain %u: position %u lies beyond the walls at +-L/2", chain,
                  i);
  }
  if (periodic && n > 0 && !(x[n - 1] < x[0] + l))
    return fail(JMM_ERR_INVALID, "chain %u: periodic positions must span less than L", chain);
  return JMM_OK;
}

// Creates a batch; with x_packed (the chains' positions back to back, host
// memory, box lengths l0) the positions start there instead of the
// configured lattice.
static int batch_create(const jmm_batch_config *cfg, const jmm_chain_desc *chains,
                        uint32_t n_chains, jmm_batch **out, const float *x_packed) {
  clear_error();
  JMM_CHECK_ARG(out, "null output");
  *out = nullptr;
  int rc = validate(cfg, chains, n_chains);
  if (rc) return rc;
  if (x_packed) {
    uint64_t src = 0;
    for (uint32_t k = 0; k < n_chains; ++k) {
      rc = check_host_positions(x_packed + src, chains[k].n, chains[k].l0,
                                cfg->boundary == JMM_BOUNDARY_PERIODIC, k);
      if (rc) return rc;
      src += chains[k].n;
    }
  }
  if (!jmm_device_available()) return fail(JMM_ERR_CUDA, "jmm_batch_create: no CUDA device");
  jmm_batch *b = new (std::nothrow) jmm_batch();
  if (!b) return fail(JMM_ERR_NOMEM, "jmm_batch_create: host allocation failed");
  b->cfg = *cfg;
  b->n_chains = n_chains;
  b->chains.assign(chains, chains + n_chains);
  b->x_off.resize(n_chains);
  uint64_t off = 0;
  for (uint32_t k = 0; k < n_chains; ++k) {
    b->x_off[k] = off;
    off += pad4(chains[k].n);
  }
  b->total_floats = off;
  b->order.resize(n_chains);
  std::iota(b->order.begin(), b->order.end(), 0u);
  std::stable_sort(b->order.begin(), b->order.end(), [&](uint32_t a, uint32_t c) {
    if (chains[a].potential != chains[c].potential) return chains[a].potential < chains[c].potential;
    const bool sa = is_split(*cfg, chains[a]), sc = is_split(*cfg, chains[c]);
    if (sa != sc) return sa;
    return chains[a].n > chains[c].n;
  });

  cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) {
    int dev = 0, n_sm = 0;
    e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev);
    b->n_sm = (uint32_t)n_sm;
  }
  for (int k = 0; k < kMaxClasses && e == cudaSuccess; ++k) {
    e = cudaStreamCreateWithFlags(&b->side[k], cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->join[k], cudaEventDisableTiming);
  }
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming);
  // one allocation, carved into the batch's arrays at 256-byte boundaries
  std::vector<uint64_t> p_off(n_chains);
  b->n_packed = 0;
  for (uint32_t k = 0; k < n_chains; ++k) {
    p_off[k] = b->n_packed;
    b->n_packed += chains[k].n;
  }
  const size_t sizes[10] = {n_chains * sizeof(ChainParams), n_chains * sizeof(jmm_chain_result),
                            b->total_floats * sizeof(float), n_chains * sizeof(double),
                            n_chains * sizeof(jmm_chain_desc), n_chains * sizeof(uint64_t),
                            4 * n_chains * sizeof(double), n_chains * sizeof(jmm_grad_stats),
                            n_chains * sizeof(uint64_t), b->n_packed * sizeof(float)};
  size_t offs[10], bytes = 0;
  for (int k = 0; k < 10; ++k) {
    offs[k] = bytes;
    bytes += (sizes[k] + 255) & ~(size_t)255;
  }
  if (e == cudaSuccess) e = cudaMalloc((void **)&b->d_block, bytes);
  if (e == cudaSuccess) {
    b->d_params = reinterpret_cast<ChainParams *>(b->d_block + offs[0]);
    b->d_res = reinterpret_cast<jmm_chain_result *>(b->d_block + offs[1]);
    b->d_x = reinterpret_cast<float *>(b->d_block + offs[2]);
    b->d_e = reinterpret_cast<double *>(b->d_block + offs[3]);
    b->d_desc = reinterpret_cast<jmm_chain_desc *>(b->d_block + offs[4]);
    b->d_xoff = reinterpret_cast<uint64_t *>(b->d_block + offs[5]);
    b->d_gout = reinterpret_cast<double *>(b->d_block + offs[6]);
    b->d_gstats = reinterpret_cast<jmm_grad_stats *>(b->d_block + offs[7]);
    b->d_poff = reinterpret_cast<uint64_t *>(b->d_block + offs[8]);
    b->d_pack = reinterpret_cast<float *>(b->d_block + offs[9]);
  }
  if (e == cudaSuccess)
    e = cudaMemcpy(b->d_desc, chains, n_chains * sizeof(jmm_chain_desc), cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(b->d_xoff, b->x_off.data(), n_chains * sizeof(uint64_t), cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(b->d_poff, p_off.data(), n_chains * sizeof(uint64_t), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(b->d_gstats, 0, n_chains * sizeof(jmm_grad_stats));
  if (e != cudaSuccess) {
    rc = cuda_status(e, "jmm_batch_create allocation", __FILE__, __LINE__);
    batch_free(b);
    return rc;
  }
  if (x_packed) {
    // the caller's positions in one copy, spread into the padded layout on
    // the device
    e = cudaMemcpyAsync(b->d_pack, x_packed, b->n_packed * sizeof(float), cudaMemcpyHostToDevice,
                        b->stream);
    if (e == cudaSuccess) {
      unpack_positions_kernel<<<(n_chains + 7) / 8, 256, 0, b->stream>>>(
          b->d_pack, b->d_x, b->d_poff, b->d_xoff, b->d_desc, n_chains);
      e = cudaGetLastError();
    }
  } else {
    std::vector<float> x(b->total_floats, 0.0f);
    for (uint32_t k = 0; k < n_chains; ++k)
      initial_positions(cfg, chains[k], k, x.data() + b->x_off[k]);
    e = cudaMemcpy(b->d_x, x.data(), x.size() * sizeof(float), cudaMemcpyHostToDevice);
  }
  if (e == cudaSuccess) {
    init_results_kernel<<<(n_chains + 255) / 256, 256, 0, b->stream>>>(b->d_res, b->d_desc,
                                                                       n_chains);
    e = cudaGetLastError();
  }
  if (e != cudaSuccess) {
    rc = cuda_status(e, "jmm_batch_create upload", __FILE__, __LINE__);
    batch_free(b);
    return rc;
  }
  const uint32_t g = cfg->lanes_per_chain ? cfg->lanes_per_chain : 4;
  const uint32_t spr = cfg->steps_per_round ? cfg->steps_per_round : (g <= 32 ? 32 / g : 1);
  const uint32_t cpb = cfg->chains_per_block ? cfg->chains_per_block : 128 / (g * spr ? g * spr : 1);
  if (cfg->lanes_per_chain == 0 && cfg->precision != JMM_PREC_EXACT) {
    // no shape given, FAST precision: a default per potential class
    Shape sh[3];
    default_shapes(b, sh);
    rc = apply_layout(b, sh);
  } else {
    rc = apply_layout(b, g, spr, cpb, cfg->window);
  }
  if (rc == JMM_OK) rc = energies(b, b->stream);
  if (rc == JMM_OK) {
    set_energies_kernel<<<(n_chains + 255) / 256, 256, 0, b->stream>>>(b->d_res, b->d_e, n_chains);
    e = cudaStreamSynchronize(b->stream);
    if (e != cudaSuccess) rc = cuda_status(e, "jmm_batch_create energies", __FILE__, __LINE__);
  }
  if (rc) {
    batch_free(b);
    return rc;
  }
  *out = b;
  return JMM_OK;
}

extern "C" int jmm_batch_create(const jmm_batch_config *cfg, const jmm_chain_desc *chains,
                                uint32_t n_chains, jmm_batch **out) {
  return batch_create(cfg, chains, n_chains, out, nullptr);
}

extern "C" int jmm_batch_create_at(const jmm_batch_config *cfg, const jmm_chain_desc *chains,
                                   uint32_t n_chains, const float *x, jmm_batch **out) {
  clear_error();
  JMM_CHECK_ARG(x, "null positions");
  return batch_create(cfg, chains, n_chains, out, x);
}

extern "C" int jmm_batch_destroy(jmm_batch *b) {
  batch_free(b);
  return JMM_OK;
}

static int graph_for(jmm_batch *b, uint64_t n_sweeps, cudaGraphExec_t *exec) {
  auto it = b->graphs.find(n_sweeps);
  if (it != b->graphs.end()) {
    *exec = it->second;
    return JMM_OK;
  }
  cudaGraph_t graph;
  JMM_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
  int rc = launch(b, n_sweeps, b->stream);
  cudaError_t e = cudaStreamEndCapture(b->stream, &graph);
  if (rc) return rc;
  if (e != cudaSuccess) return cuda_status(e, "cudaStreamEndCapture", __FILE__, __LINE__);
  e = cudaGraphInstantiate(exec, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) return cuda_status(e, "cudaGraphInstantiate", __FILE__, __LINE__);
  b->graphs[n_sweeps] = *exec;
  return JMM_OK;
}

extern "C" int jmm_batch_run_async(jmm_batch *b, uint64_t n_sweeps, void *stream) {
  clear_error();
  JMM_CHECK_ARG(b, "null handle");
  if (n_sweeps == 0) return JMM_OK;
  for (const auto &c : b->chains)
    if (n_sweeps * (uint64_t)(c.n + 1) >= (1ull << 31))
      return fail(JMM_ERR_INVALID, "one run may hold at most 2^31 steps per chain: split it");
  cudaGraphExec_t exec;
  int rc = graph_for(b, n_sweeps, &exec);
  if (rc) return rc;
  JMM_CUDA(cudaGraphLaunch(exec, stream ? (cudaStream_t)stream : b->stream));
  return JMM_OK;
}

static int check_errors(jmm_batch *b) {
  std::vector<jmm_chain_result> res(b->n_chains);
  JMM_CUDA(cudaMemcpy(res.data(), b->d_res, res.size() * sizeof(jmm_chain_result),
                      cudaMemcpyDeviceToHost));
  for (uint32_t k = 0; k < b->n_chains; ++k)
    if (res[k].error)
      return fail((int)res[k].error, "chain %u reported error %u (energy %g)", k, res[k].error,
                  res[k].e);
  return JMM_OK;
}

extern "C" int jmm_batch_run(jmm_batch *b, uint64_t n_sweeps) {
  int rc = jmm_batch_run_async(b, n_sweeps, nullptr);
  if (rc) return rc;
  JMM_CUDA(cudaStreamSynchronize(b->stream));
  return check_errors(b);
}

extern "C" int jmm_batch_results(jmm_batch *b, jmm_chain_result *out, uint32_t n_chains) {
  clear_error();
  JMM_CHECK_ARG(b && out, "null argument");
  JMM_CHECK_ARG(n_chains == b->n_chains, "n_chains does not match the batch");
  JMM_CUDA(cudaStreamSynchronize(b->stream));
  JMM_CUDA(cudaMemcpy(out, b->d_res, n_chains * sizeof(jmm_chain_result), cudaMemcpyDeviceToHost));
  return JMM_OK;
}

extern "C" int jmm_batch_set_results(jmm_batch *b, const jmm_chain_result *in, uint32_t n_chains) {
  clear_error();
  JMM_CHECK_ARG(b && in, "null argument");
  JMM_CHECK_ARG(n_chains == b->n_chains, "n_chains does not match the batch");
  const bool walls = b->cfg.boundary != JMM_BOUNDARY_PERIODIC;
  std::vector<float> x;
  JMM_CUDA(cudaStreamSynchronize(b->stream));
  if (walls) {
    x.resize(b->total_floats);
    JMM_CUDA(cudaMemcpy(x.data(), b->d_x, x.size() * sizeof(float), cudaMemcpyDeviceToHost));
  }
  for (uint32_t k = 0; k < n_chains; ++k) {
    if (!(in[k].l > 0) || !std::isfinite(in[k].l) || !std::isfinite(in[k].e))
      return fail(JMM_ERR_INVALID, "chain %u: box length and energy must be finite, L > 0", k);
    if (walls) {  // ordered positions: the end particles decide
      const float *xc = x.data() + b->x_off[k];
      const float half = (float)(0.5 * in[k].l) * (1.0f + 1e-6f);
      if (!(fabsf(xc[0]) <= half) || !(fabsf(xc[b->chains[k].n - 1]) <= half))
        return fail(JMM_ERR_INVALID, "chain %u: positions lie beyond the walls of the record's L", k);
    }
  }
  JMM_CUDA(cudaMemcpy(b->d_res, in, n_chains * sizeof(jmm_chain_result), cudaMemcpyHostToDevice));
  return JMM_OK;
}

__global__ void reset_stats_kernel(jmm_chain_result *res, uint32_t n) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  jmm_chain_result r = res[i];
  r.samples = 0;
  r.sum_e = r.sum_e2 = r.sum_l = r.sum_l2 = r.sum_le = r.sum_rho = r.sum_rho2 = 0.0;
  r.disp_acc = r.disp_att = r.vol_acc = r.vol_att = 0;
  r.pair_evals = 0;
  r.max_drift = 0.0;
  r.window_overflows = 0;
  res[i] = r;
}

extern "C" int jmm_batch_reset_stats(jmm_batch *b) {
  clear_error();
  JMM_CHECK_ARG(b, "null handle");
  reset_stats_kernel<<<(b->n_chains + 255) / 256, 256, 0, b->stream>>>(b->d_res, b->n_chains);
  JMM_CUDA(cudaGetLastError());
  JMM_CUDA(cudaMemsetAsync(b->d_gstats, 0, b->n_chains * sizeof(jmm_grad_stats), b->stream));
  JMM_CUDA(cudaStreamSynchronize(b->stream));
  return JMM_OK;
}

// maxDisAdjust / maxDVAdjust (src/jmmMCState.cpp:2100-2139) per chain, from
// the chain's counts since creation or the last reset: the step is scaled by
// ln(0.672924 ideal + 0.0644284) / ln(0.672924 (actual + 0.0644284)), the
// displacement clamped to [0.002, 0.5]; a linear volume step (max dL) to
// [0.002 N, 0.1 N] with values above 0.1 N set to 0.5 N as the reference
// does; an ln L step to [1e-4, 1].
__global__ void adjust_steps_kernel(ChainParams *prm, const jmm_chain_result *res, uint32_t n_chains,
                                    double ideal, int32_t what, int32_t vol_move) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n_chains) return;
  ChainParams P = prm[k];
  const jmm_chain_result &r = res[P.id];
  const double num = log(__dadd_rn(__dmul_rn(0.672924, ideal), 0.0644284));
  if ((what & 1) && r.disp_att > 0) {
    const double actual = __ddiv_rn((double)r.disp_acc, (double)r.disp_att);
    double ms = __ddiv_rn(__dmul_rn(__dmul_rn(0.5, (double)P.two_max_step), num),
                          log(__dmul_rn(0.672924, __dadd_rn(actual, 0.0644284))));
    ms = ms < 0.002 ? 0.002 : (ms > 0.5 ? 0.5 : ms);
    P.two_max_step = (float)__dmul_rn(2.0, ms);
  }
  if ((what & 2) && P.ensemble == JMM_NPT && r.vol_att > 0) {
    const double actual = __ddiv_rn((double)r.vol_acc, (double)r.vol_att);
    double vs = __ddiv_rn(__dmul_rn((double)P.vol_step, num),
                          log(__dmul_rn(0.672924, __dadd_rn(actual, 0.0644284))));
    if (vol_move == JMM_VOLMOVE_LINEAR) {
      const double nd = (double)P.n;
      if (vs < __dmul_rn(0.002, nd))
        vs = __dmul_rn(0.002, nd);
      else if (vs > __dmul_rn(0.10, nd))
        vs = __dmul_rn(0.50, nd);
    } else {
      vs = vs < 1e-4 ? 1e-4 : (vs > 1.0 ? 1.0 : vs);
    }
    P.vol_step = (float)vs;
  }
  prm[k] = P;
}

extern "C" int jmm_batch_adjust_steps(jmm_batch *b, double ideal_ratio, int32_t what) {
  clear_error();
  JMM_CHECK_ARG(b, "null handle");
  JMM_CHECK_ARG(ideal_ratio > 0 && ideal_ratio < 1, "ideal_ratio must be in (0, 1)");
  JMM_CHECK_ARG(what >= 1 && what <= 3, "what: 1 displacement, 2 volume, 3 both");
  adjust_steps_kernel<<<(b->n_chains + 255) / 256, 256, 0, b->stream>>>(
      b->d_params, b->d_res, b->n_chains, ideal_ratio, what, b->cfg.vol_move);
  JMM_CUDA(cudaGetLastError());
  return JMM_OK;
}

extern "C" int jmm_batch_step_sizes(jmm_batch *b, double *max_step, double *vol_step,
                                    uint32_t n_chains) {
  clear_error();
  JMM_CHECK_ARG(b && max_step && vol_step, "null argument");
  JMM_CHECK_ARG(n_chains == b->n_chains, "n_chains does not match the batch");
  const int rc = sync_step_sizes(b);
  if (rc) return rc;
  for (uint32_t k = 0; k < n_chains; ++k) {
    max_step[k] = b->chains[k].max_step;
    vol_step[k] = b->chains[k].vol_step;
  }
  return JMM_OK;
}

extern "C" int jmm_batch_get_positions(jmm_batch *b, uint32_t chain, float *x, uint32_t n) {
  clear_error();
  JMM_CHECK_ARG(b && x, "null argument");
  JMM_CHECK_ARG(chain < b->n_chains, "chain index out of range");
  JMM_CHECK_ARG(n == b->chains[chain].n, "N does not match the chain");
  JMM_CUDA(cudaStreamSynchronize(b->stream));
  JMM_CUDA(cudaMemcpy(x, b->d_x + b->x_off[chain], n * sizeof(float), cudaMemcpyDeviceToHost));
  return JMM_OK;
}

extern "C" int jmm_batch_set_positions(jmm_batch *b, uint32_t chain, const float *x, uint32_t n,
                                       double l) {
  clear_error();
  JMM_CHECK_ARG(b && x, "null argument");
  JMM_CHECK_ARG(chain < b->n_chains, "chain index out of range");
  JMM_CHECK_ARG(n == b->chains[chain].n, "N does not match the chain");
  int rc = check_host_positions(x, n, l, b->cfg.boundary == JMM_BOUNDARY_PERIODIC, chain);
  if (rc) return rc;
  JMM_CUDA(cudaStreamSynchronize(b->stream));
  JMM_CUDA(cudaMemcpy(b->d_x + b->x_off[chain], x, n * sizeof(float), cudaMemcpyHostToDevice));
  jmm_chain_result r;
  JMM_CUDA(cudaMemcpy(&r, b->d_res + chain, sizeof(r), cudaMemcpyDeviceToHost));
  r.l = l;
  JMM_CUDA(cudaMemcpy(b->d_res + chain, &r, sizeof(r), cudaMemcpyHostToDevice));
  rc = energies(b, b->stream);
  if (rc) return rc;
  double e;
  JMM_CUDA(cudaMemcpyAsync(&e, b->d_e + chain, sizeof(double), cudaMemcpyDeviceToHost, b->stream));
  JMM_CUDA(cudaStreamSynchronize(b->stream));
  r.e = e;
  JMM_CUDA(cudaMemcpy(b->d_res + chain, &r, sizeof(r), cudaMemcpyHostToDevice));
  return JMM_OK;
}

extern "C" int jmm_batch_energies(jmm_batch *b, double *e, uint32_t n_chains) {
  clear_error();
  JMM_CHECK_ARG(b && e, "null argument");
  JMM_CHECK_ARG(n_chains == b->n_chains, "n_chains does not match the batch");
  int rc = energies(b, b->stream);
  if (rc) return rc;
  JMM_CUDA(cudaStreamSynchronize(b->stream));
  JMM_CUDA(cudaMemcpy(e, b->d_e, n_chains * sizeof(double), cudaMemcpyDeviceToHost));
  return JMM_OK;
}

// Trial energies of a volume move of every chain: one group of L = G*S lanes
// per chain (its class's shape), through the chain_energies call that the
// chain kernel's volume move makes, so lanes, summation order and precision
// are the move's own.
template <int L, int POT, bool PER, bool kExact>
__global__ void volume_energies_kernel(const ChainParams *__restrict__ prm,
                                       const jmm_chain_result *__restrict__ res,
                                       const float *__restrict__ xg, const float *__restrict__ scale,
                                       double *__restrict__ out, uint32_t n_chains) {
  const uint32_t c = (blockIdx.x * blockDim.x + threadIdx.x) / L;
  if (c >= n_chains) return;  // whole groups leave together
  const int cl = threadIdx.x % L;
  const unsigned gmask =
      (L == 32) ? 0xffffffffu : (((1u << L) - 1u) << (((threadIdx.x & 31) / L) * L));
  const ChainParams P = prm[c];
  Hot H;
  H.eps4 = P.eps4;
  H.sigma2 = P.sigma2;
  H.inv_sigma2 = P.inv_sigma2;
  H.rc2 = P.rc2;
  H.beta = P.beta;
  H.two_max_step = P.two_max_step;
  const double l = res[P.id].l;
  const float s = scale[P.id];
  const double lnew = __dmul_rn(l, (double)s);
  double uo, un;
  uint64_t pairs = 0;
  uint32_t err = 0;
  chain_energies<L, POT, PER, kExact, true>(xg + P.x_off, H, (int)P.n, cl, gmask, (float)l, s,
                                            (float)lnew, uo, un, pairs, err);
  const double du = __dsub_rn(un, uo);  // as the volume move forms it
  if (cl == 0) {
    double *o = out + 3 * (uint64_t)P.id;
    o[0] = err ? (double)NAN : uo;
    o[1] = err ? (double)NAN : un;
    o[2] = err ? (double)NAN : du;
  }
}

typedef void (*VolKernel)(const ChainParams *, const jmm_chain_result *, const float *,
                          const float *, double *, uint32_t);

template <int L, bool E>
static VolKernel pick_vol_pot(int pot, bool per) {
  switch (pot * 2 + (per ? 1 : 0)) {
    case JMM_POT_LJCUT * 2: return volume_energies_kernel<L, JMM_POT_LJCUT, false, E>;
    case JMM_POT_LJCUT * 2 + 1: return volume_energies_kernel<L, JMM_POT_LJCUT, true, E>;
    case JMM_POT_SOFTSPHERE * 2: return volume_energies_kernel<L, JMM_POT_SOFTSPHERE, false, E>;
    case JMM_POT_SOFTSPHERE * 2 + 1: return volume_energies_kernel<L, JMM_POT_SOFTSPHERE, true, E>;
    case JMM_POT_GAUSS * 2: return volume_energies_kernel<L, JMM_POT_GAUSS, false, E>;
    case JMM_POT_GAUSS * 2 + 1: return volume_energies_kernel<L, JMM_POT_GAUSS, true, E>;
    default: return nullptr;
  }
}

static VolKernel pick_vol(uint32_t lanes, bool exact, int pot, bool per) {
  switch (lanes) {
    case 32: return exact ? pick_vol_pot<32, true>(pot, per) : pick_vol_pot<32, false>(pot, per);
    case 16: return exact ? pick_vol_pot<16, true>(pot, per) : pick_vol_pot<16, false>(pot, per);
    case 8: return exact ? pick_vol_pot<8, true>(pot, per) : pick_vol_pot<8, false>(pot, per);
    default: return nullptr;
  }
}

extern "C" int jmm_batch_volume_energies(jmm_batch *b, const float *scale, double *out,
                                         uint32_t n_chains) {
  clear_error();
  JMM_CHECK_ARG(b && scale && out, "null argument");
  JMM_CHECK_ARG(n_chains == b->n_chains, "n_chains does not match the batch");
  for (uint32_t k = 0; k < n_chains; ++k)
    JMM_CHECK_ARG(std::isfinite(scale[k]) && scale[k] > 0.0f,
                  "scale factors must be finite and positive");
  float *d_scale = nullptr;
  double *d_out = nullptr;
  JMM_CUDA(cudaStreamSynchronize(b->stream));
  cudaError_t e = cudaMalloc((void **)&d_scale, n_chains * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc((void **)&d_out, 3 * (size_t)n_chains * sizeof(double));
  int rc = JMM_OK;
  if (e != cudaSuccess) rc = cuda_status(e, "cudaMalloc", __FILE__, __LINE__);
  if (rc == JMM_OK) {
    e = cudaMemcpyAsync(d_scale, scale, n_chains * sizeof(float), cudaMemcpyHostToDevice,
                        b->stream);
    if (e != cudaSuccess) rc = cuda_status(e, "cudaMemcpyAsync", __FILE__, __LINE__);
  }
  const bool per = b->cfg.boundary == JMM_BOUNDARY_PERIODIC;
  const bool exact = b->cfg.precision == JMM_PREC_EXACT;
  for (size_t k = 0; rc == JMM_OK && k < b->classes.size(); ++k) {
    const PotClass &pc = b->classes[k];
    const uint32_t lanes = pc.shape.g * pc.shape.spr;
    VolKernel kf = pick_vol(lanes, exact, pc.pot, per);
    if (!kf) {
      rc = fail(JMM_ERR_INVALID, "no volume-energy kernel for this launch shape");
      break;
    }
    const uint32_t threads = 128;
    const uint32_t blocks = (uint32_t)(((uint64_t)pc.count * lanes + threads - 1) / threads);
    kf<<<blocks, threads, 0, b->stream>>>(b->d_params + pc.first, b->d_res, b->d_x, d_scale, d_out,
                                          pc.count);
    e = cudaGetLastError();
    if (e != cudaSuccess) rc = cuda_status(e, "volume_energies_kernel", __FILE__, __LINE__);
  }
  if (rc == JMM_OK) {
    e = cudaMemcpyAsync(out, d_out, 3 * (size_t)n_chains * sizeof(double), cudaMemcpyDeviceToHost,
                        b->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    if (e != cudaSuccess) rc = cuda_status(e, "volume energies read-back", __FILE__, __LINE__);
  }
  cudaFree(d_scale);
  cudaFree(d_out);
  return rc;
}

extern "C" int jmm_batch_device_views(jmm_batch *b, void **positions, void **results,
                                      uint64_t *offsets, uint32_t n_chains) {
  clear_error();
  JMM_CHECK_ARG(b, "null handle");
  if (positions) *positions = b->d_x;
  if (results) *results = b->d_res;
  if (offsets) {
    JMM_CHECK_ARG(n_chains == b->n_chains, "n_chains does not match the batch");
    memcpy(offsets, b->x_off.data(), n_chains * sizeof(uint64_t));
  }
  return JMM_OK;
}

// Launch shapes tried by the autotuner: G x S, and threads per block.
static const uint32_t kTuneShapes[][3] = {{4, 8, 4}, {2, 16, 4}, {2, 16, 3}, {4, 4, 4}, {4, 2, 4},
                                          {8, 4, 4}, {8, 2, 4}, {16, 2, 8}, {16, 1, 8},
                                          {32, 1, 16}, {4, 8, 8}, {2, 16, 8}, {8, 4, 8}};
static const uint32_t kTuneThreads[] = {32u, 64u, 128u, 256u};

extern "C" int jmm_batch_autotune(jmm_batch *b, uint32_t trial_sweeps, uint32_t *lanes_out,
                                  uint32_t *spr_out, uint32_t *cpb_out) {
  clear_error();
  JMM_CHECK_ARG(b, "null handle");
  if (trial_sweeps == 0) trial_sweeps = 4;
  JMM_CUDA(cudaStreamSynchronize(b->stream));
  float *x_save = nullptr;
  jmm_chain_result *r_save = nullptr;
  JMM_CUDA(cudaMalloc((void **)&x_save, b->total_floats * sizeof(float)));
  cudaError_t e = cudaMalloc((void **)&r_save, b->n_chains * sizeof(jmm_chain_result));
  if (e != cudaSuccess) {
    cudaFree(x_save);
    return cuda_status(e, "autotune cudaMalloc", __FILE__, __LINE__);
  }
  cudaMemcpy(x_save, b->d_x, b->total_floats * sizeof(float), cudaMemcpyDeviceToDevice);
  cudaMemcpy(r_save, b->d_res, b->n_chains * sizeof(jmm_chain_result), cudaMemcpyDeviceToDevice);
  cudaEvent_t t0, t1;
  cudaEventCreate(&t0);
  cudaEventCreate(&t1);
  // Time of a trial: the whole batch (cls < 0), or class cls alone; the
  // state is restored before each run, the first run warms the code path and
  // the best of the next three counts (a single short run can land on a
  // clock ramp).
  auto trial = [&](int cls, float *ms_out, uint32_t sweeps) -> int {
    float best_run = 1e30f;
    for (int rep = 0; rep < 4; ++rep) {
      float ms = 0.0f;
      cudaMemcpyAsync(b->d_x, x_save, b->total_floats * sizeof(float), cudaMemcpyDeviceToDevice,
                      b->stream);
      cudaMemcpyAsync(b->d_res, r_save, b->n_chains * sizeof(jmm_chain_result),
                      cudaMemcpyDeviceToDevice, b->stream);
      cudaEventRecord(t0, b->stream);
      int rc = JMM_OK;
      if (cls < 0) {
        rc = launch(b, sweeps, b->stream);
      } else {
        for (size_t k = 0; k < b->classes.size(); ++k)
          if (b->classes[k].pot == kPots[cls]) rc = launch_class(b, k, sweeps, b->stream);
      }
      cudaEventRecord(t1, b->stream);
      if (rc) return rc;
      cudaEventSynchronize(t1);
      cudaEventElapsedTime(&ms, t0, t1);
      if (rep > 0 && ms < best_run) best_run = ms;
    }
    *ms_out = best_run;
    return JMM_OK;
  };
  Shape best[3];
  for (int pi = 0; pi < 3; ++pi) best[pi] = b->shapes[pi];
  int rc = JMM_OK;
  // EXACT runs keep one shape for the whole batch (the oracle replays one G);
  // FAST runs tune every potential class on its own
  const bool per_class = b->cfg.precision != JMM_PREC_EXACT;
  const int rounds = per_class ? 3 : 1;
  for (int pi = 0; pi < rounds && rc == JMM_OK; ++pi) {
    if (per_class) {
      bool present = false;
      for (const PotClass &pc : b->classes) present = present || pc.pot == kPots[pi];
      if (!present) continue;
    }
    // every candidate once, then the three fastest again, so that a drift
    // of the clocks over the scan cannot decide
    std::vector<std::pair<float, std::vector<Shape>>> timed;
    for (const auto &shape : kTuneShapes) {
      for (uint32_t threads : kTuneThreads) {
        const uint32_t cpb = threads / (shape[0] * shape[1]);
        if (cpb == 0) continue;
        std::vector<Shape> sh(3);
        for (int q = 0; q < 3; ++q)
          sh[q] = per_class ? best[q] : Shape{shape[0], shape[1], cpb, shape[2]};
        if (per_class) sh[pi] = Shape{shape[0], shape[1], cpb, shape[2]};
        if (apply_layout(b, sh.data()) != JMM_OK) {
          clear_error();
          continue;
        }
        float ms = 0.0f;
        rc = trial(per_class ? pi : -1, &ms, trial_sweeps);
        if (rc) break;
        timed.emplace_back(ms, sh);
      }
      if (rc) break;
    }
    if (rc) break;
    std::sort(timed.begin(), timed.end(),
              [](const auto &x, const auto &y) { return x.first < y.first; });
    float best_ms = 1e30f;
    for (size_t c = 0; c < timed.size() && c < 3 && rc == JMM_OK; ++c) {
      if (apply_layout(b, timed[c].second.data()) != JMM_OK) {
        clear_error();
        continue;
      }
      float ms = 0.0f;
      rc = trial(per_class ? pi : -1, &ms, trial_sweeps);
      if (rc == JMM_OK && ms < best_ms) {
        best_ms = ms;
        for (int q = 0; q < 3; ++q) best[q] = timed[c].second[q];
      }
    }
  }
  if (per_class && rc == JMM_OK && b->classes.size() > 1) {
    // the classes were timed alone but run side by side: keep the per-class
    // defaults unless the tuned shapes run the whole batch at least 3 %
    // faster, timed over ten times the trial sweeps (short side-by-side runs
    // of several class kernels did not rank the two sets as long runs do)
    Shape dflt[3];
    default_shapes(b, dflt);
    float t_best = 1e30f, t_dflt = 1e30f;
    if (apply_layout(b, best) == JMM_OK) rc = trial(-1, &t_best, 10 * trial_sweeps);
    if (rc == JMM_OK && apply_layout(b, dflt) == JMM_OK) rc = trial(-1, &t_dflt, 10 * trial_sweeps);
    clear_error();
    if (rc == JMM_OK && t_dflt < 1.03f * t_best)
      for (int q = 0; q < 3; ++q) best[q] = dflt[q];
  }
  cudaMemcpy(b->d_x, x_save, b->total_floats * sizeof(float), cudaMemcpyDeviceToDevice);
  cudaMemcpy(b->d_res, r_save, b->n_chains * sizeof(jmm_chain_result), cudaMemcpyDeviceToDevice);
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  cudaFree(x_save);
  cudaFree(r_save);
  if (rc) return rc;
  rc = apply_layout(b, best);
  if (rc) return rc;
  b->cfg.lanes_per_chain = b->g;
  b->cfg.steps_per_round = b->spr;
  b->cfg.chains_per_block = b->cpb;
  b->cfg.window = b->win;
  if (lanes_out) *lanes_out = b->g;
  if (spr_out) *spr_out = b->spr;
  if (cpb_out) *cpb_out = b->cpb;
  JMM_CUDA(cudaDeviceSynchronize());
  return JMM_OK;
}

extern "C" int jmm_batch_shapes(jmm_batch *b, uint32_t *shapes, uint32_t n) {
  clear_error();
  JMM_CHECK_ARG(b && shapes, "null argument");
  JMM_CHECK_ARG(n == 12, "shapes holds 3 x (lanes, steps per round, chains per block, window)");
  for (int pi = 0; pi < 3; ++pi) {
    bool present = false;
    for (const PotClass &pc : b->classes) present = present || pc.pot == kPots[pi];
    shapes[4 * pi + 0] = present ? b->shapes[pi].g : 0;
    shapes[4 * pi + 1] = present ? b->shapes[pi].spr : 0;
    shapes[4 * pi + 2] = present ? b->shapes[pi].cpb : 0;
    shapes[4 * pi + 3] = present ? b->shapes[pi].w : 0;
  }
  return JMM_OK;
}

extern "C" int jmm_batch_run_host(const jmm_batch_config *cfg, const jmm_chain_desc *chains,
                                  uint32_t n_chains, const float *x_in, uint64_t n_sweeps,
                                  jmm_chain_result *results, float *x_out) {
  jmm_batch *b = nullptr;
  // the positions in x_in are the batch's starting positions (no lattice)
  int rc = batch_create(cfg, chains, n_chains, &b, x_in);
  if (rc) return rc;
  // one run: launched directly, without building a graph to replay
  if (n_sweeps > 0) {
    for (const auto &c : b->chains)
      if (n_sweeps * (uint64_t)(c.n + 1) >= (1ull << 31)) {
        batch_free(b);
        return fail(JMM_ERR_INVALID, "one run may hold at most 2^31 steps per chain: split it");
      }
    rc = launch(b, n_sweeps, b->stream);
  }
  std::vector<jmm_chain_result> own;
  jmm_chain_result *res = results;
  if (!res) {
    own.resize(n_chains);
    res = own.data();
  }
  cudaError_t e = cudaSuccess;
  if (rc == JMM_OK) {
    e = cudaMemcpyAsync(res, b->d_res, n_chains * sizeof(jmm_chain_result),
                        cudaMemcpyDeviceToHost, b->stream);
    if (e == cudaSuccess && x_out) {
      pack_positions_kernel<<<(n_chains + 7) / 8, 256, 0, b->stream>>>(
          b->d_x, b->d_pack, b->d_poff, b->d_xoff, b->d_desc, n_chains);
      e = cudaGetLastError();
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(x_out, b->d_pack, b->n_packed * sizeof(float),
                            cudaMemcpyDeviceToHost, b->stream);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    if (e != cudaSuccess) rc = cuda_status(e, "jmm_batch_run_host", __FILE__, __LINE__);
  }
  if (rc == JMM_OK)
    for (uint32_t k = 0; k < n_chains; ++k)
      if (res[k].error) {
        rc = fail((int)res[k].error, "chain %u reported error %u (energy %g)", k, res[k].error,
                  res[k].e);
        break;
      }
  batch_free(b);
  return rc;
}

__global__ void rng_words_kernel(uint64_t seed, uint64_t block0, uint32_t chain, uint64_t count,
                                 uint32_t *out) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < count;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const Words4 w = step_words(seed, block0 + i, chain);
    out[4 * i + 0] = w.w[0];
    out[4 * i + 1] = w.w[1];
    out[4 * i + 2] = w.w[2];
    out[4 * i + 3] = w.w[3];
  }
}

extern "C" int jmm_rng_words(uint64_t seed, uint64_t block0, uint32_t chain, uint64_t count,
                             uint32_t *out) {
  clear_error();
  JMM_CHECK_ARG(out || count == 0, "null output");
  if (count == 0) return JMM_OK;
  if (!jmm_device_available()) return fail(JMM_ERR_CUDA, "jmm_rng_words: no CUDA device");
  uint32_t *d = nullptr;
  JMM_CUDA(cudaMalloc((void **)&d, count * 4 * sizeof(uint32_t)));
  const uint64_t blocks64 = (count + 255) / 256;
  const int blocks = (int)(blocks64 < 4096 ? blocks64 : 4096);
  rng_words_kernel<<<blocks, 256>>>(seed, block0, chain, count, d);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpy(out, d, count * 4 * sizeof(uint32_t), cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess) return cuda_status(e, "jmm_rng_words", __FILE__, __LINE__);
  return JMM_OK;
}

// ---- energy gradients of the batch's configurations -------------------------

// One warp per chain (user order): U and its derivatives into out (mode 0),
// or added with the fluctuation moments to the chain's jmm_grad_stats.
template <bool kAccumulate>
__global__ void batch_grad_kernel(const jmm_chain_desc *__restrict__ desc,
                                  const uint64_t *__restrict__ xoff, const float *__restrict__ x,
                                  const jmm_chain_result *__restrict__ res, uint32_t n_chains,
                                  int32_t boundary, double *__restrict__ out,
                                  jmm_grad_stats *__restrict__ stats) {
  const uint32_t c = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
  if (c >= n_chains) return;
  const jmm_chain_desc d = desc[c];
  const double l = res[c].l;
  const grad::PotParams p = grad::make_pot(d.potential, d.eps, d.sigma, d.cutoff);
  __shared__ double tmp[8][4];
  double *o = kAccumulate ? tmp[(threadIdx.x / 32) % 8] : out + 4 * c;
  grad::chain_grad(x + xoff[c], (int)d.n, p, l, boundary == JMM_BOUNDARY_PERIODIC, o, nullptr);
  if (kAccumulate && (threadIdx.x & 31) == 0) {
    jmm_grad_stats st = stats[c];
    const double u = o[0];
    const double rho = __ddiv_rn((double)d.n, l);
    const double g[3] = {o[1], o[2], o[3]};
    st.samples += 1;
    st.sum_u = __dadd_rn(st.sum_u, u);
    st.sum_u2 = __dadd_rn(st.sum_u2, __dmul_rn(u, u));
    st.sum_rho = __dadd_rn(st.sum_rho, rho);
    st.sum_rho2 = __dadd_rn(st.sum_rho2, __dmul_rn(rho, rho));
    st.sum_l = __dadd_rn(st.sum_l, l);
    for (int k = 0; k < 3; ++k) {
      st.sum_g[k] = __dadd_rn(st.sum_g[k], g[k]);
      st.sum_u_g[k] = __dadd_rn(st.sum_u_g[k], __dmul_rn(u, g[k]));
      st.sum_rho_g[k] = __dadd_rn(st.sum_rho_g[k], __dmul_rn(rho, g[k]));
      st.sum_l_g[k] = __dadd_rn(st.sum_l_g[k], __dmul_rn(l, g[k]));
    }
    stats[c] = st;
  }
}

static int launch_grad(jmm_batch *b, bool accumulate, cudaStream_t s) {
  const uint32_t per_block = 8;
  const uint32_t blocks = (b->n_chains + per_block - 1) / per_block;
  if (accumulate)
    batch_grad_kernel<true><<<blocks, 32 * per_block, 0, s>>>(
        b->d_desc, b->d_xoff, b->d_x, b->d_res, b->n_chains, b->cfg.boundary, nullptr, b->d_gstats);
  else
    batch_grad_kernel<false><<<blocks, 32 * per_block, 0, s>>>(
        b->d_desc, b->d_xoff, b->d_x, b->d_res, b->n_chains, b->cfg.boundary, b->d_gout, nullptr);
  JMM_CUDA(cudaGetLastError());
  return JMM_OK;
}

extern "C" int jmm_batch_energy_grad(jmm_batch *b, double *out, uint32_t n_chains) {
  clear_error();
  JMM_CHECK_ARG(b && out, "null argument");
  JMM_CHECK_ARG(n_chains == b->n_chains, "n_chains does not match the batch");
  int rc = launch_grad(b, false, b->stream);
  if (rc) return rc;
  JMM_CUDA(cudaStreamSynchronize(b->stream));
  JMM_CUDA(cudaMemcpy(out, b->d_gout, 4 * n_chains * sizeof(double), cudaMemcpyDeviceToHost));
  return JMM_OK;
}

// ---- sampled rho(x) and g(x) histograms ------------------------------------

// Bin floor(x / w + nb / 2) of a position (rho) or a slice (g), in FP32 as
// the oracle restates it; -1 outside [0, nb).
__device__ __forceinline__ int hist_bin(float x, float w, uint32_t nb) {
  const float f = floorf(__fadd_rn(__fdiv_rn(x, w), __fmul_rn(0.5f, (float)nb)));
  return (f >= 0.0f && f < (float)nb) ? (int)f : -1;
}

// One warp per chain (user order): adds the current configuration to the
// chain's row [samples, rho bins, g bins].  Pairs are taken in index order
// from each particle to the right (on a ring, through the wrap, at most half
// way round) until the separation reaches gnb * gbw.
__global__ void batch_hist_kernel(const jmm_chain_desc *__restrict__ desc,
                                  const uint64_t *__restrict__ xoff, const float *__restrict__ x,
                                  const jmm_chain_result *__restrict__ res, uint32_t n_chains,
                                  int32_t boundary, uint32_t rhonb, float rbw, uint32_t gns,
                                  float gsw, uint32_t gnb, float gbw, uint64_t *__restrict__ hist) {
  const uint32_t c = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
  if (c >= n_chains) return;
  const int lane = threadIdx.x & 31;
  const int n = (int)desc[c].n;
  const float *xc = x + xoff[c];
  const bool periodic = boundary == JMM_BOUNDARY_PERIODIC;
  const float lf = (float)res[c].l;
  const float range = __fmul_rn((float)gnb, gbw);
  uint64_t *row = hist + (uint64_t)c * (1u + rhonb + gns * gnb);
  uint64_t *g = row + 1 + rhonb;
  if (lane == 0) row[0] += 1;
  for (int i = lane; i < n; i += 32) {
    const float xi = xc[i];
    const int rb = hist_bin(xi, rbw, rhonb);
    if (rb >= 0) atomicAdd((unsigned long long *)&row[1 + rb], 1ull);
    const int si = hist_bin(xi, gsw, gns);
    for (int k = 1; k < n; ++k) {
      if (periodic && 2 * k > n) break;  // the other way round is shorter
      int j = i + k;
      float shift = 0.0f;
      if (j >= n) {
        if (!periodic) break;
        j -= n;
        shift = lf;
      }
      const float xj = xc[j];
      const float d = __fsub_rn(__fadd_rn(xj, shift), xi);
      if (!(d < range)) break;
      const float gf = floorf(__fdiv_rn(d, gbw));
      if (!(gf < (float)gnb)) continue;
      const int gb = (int)gf;
      if (si >= 0) atomicAdd((unsigned long long *)&g[(uint64_t)si * gnb + gb], 1ull);
      const int sj = hist_bin(xj, gsw, gns);  // the partner's own slice
      if (sj >= 0) atomicAdd((unsigned long long *)&g[(uint64_t)sj * gnb + gb], 1ull);
    }
  }
}

static int launch_hist(jmm_batch *b, cudaStream_t s) {
  const uint32_t per_block = 8;
  const uint32_t blocks = (b->n_chains + per_block - 1) / per_block;
  batch_hist_kernel<<<blocks, 32 * per_block, 0, s>>>(
      b->d_desc, b->d_xoff, b->d_x, b->d_res, b->n_chains, b->cfg.boundary, b->h_rhonb, b->h_rbw,
      b->h_gns, b->h_gsw, b->h_gnb, b->h_gbw, b->d_hist);
  JMM_CUDA(cudaGetLastError());
  return JMM_OK;
}

extern "C" int jmm_batch_histograms(jmm_batch *b, uint32_t rhonb, double rbw, uint32_t gns,
                                    double gsw, uint32_t gnb, double gbw) {
  clear_error();
  JMM_CHECK_ARG(b, "null handle");
  JMM_CHECK_ARG(rhonb > 0 && gns > 0 && gnb > 0, "bin counts must be positive");
  JMM_CHECK_ARG(rbw > 0 && gsw > 0 && gbw > 0, "bin widths must be positive");
  JMM_CHECK_ARG((uint64_t)rhonb + (uint64_t)gns * gnb <= (1u << 20), "at most 2^20 bins per chain");
  JMM_CUDA(cudaStreamSynchronize(b->stream));
  cudaFree(b->d_hist);
  b->d_hist = nullptr;
  const uint64_t words = (uint64_t)b->n_chains * (1u + rhonb + gns * gnb);
  JMM_CUDA(cudaMalloc((void **)&b->d_hist, words * sizeof(uint64_t)));
  JMM_CUDA(cudaMemset(b->d_hist, 0, words * sizeof(uint64_t)));
  b->h_rhonb = rhonb;
  b->h_gns = gns;
  b->h_gnb = gnb;
  b->h_rbw = (float)rbw;
  b->h_gsw = (float)gsw;
  b->h_gbw = (float)gbw;
  drop_graphs(b);  // sampled runs now take histograms too
  return JMM_OK;
}

extern "C" int jmm_batch_sample_histograms(jmm_batch *b, void *stream) {
  clear_error();
  JMM_CHECK_ARG(b, "null handle");
  JMM_CHECK_ARG(b->d_hist, "no histograms configured (jmm_batch_histograms)");
  return launch_hist(b, stream ? (cudaStream_t)stream : b->stream);
}

extern "C" int jmm_batch_take_histograms(jmm_batch *b, uint64_t *out, uint64_t n) {
  clear_error();
  JMM_CHECK_ARG(b && out, "null argument");
  JMM_CHECK_ARG(b->d_hist, "no histograms configured (jmm_batch_histograms)");
  const uint64_t words = (uint64_t)b->n_chains * (1u + b->h_rhonb + b->h_gns * b->h_gnb);
  JMM_CHECK_ARG(n == words, "out must hold n_chains * (1 + rhonb + gns * gnb) counts");
  JMM_CUDA(cudaStreamSynchronize(b->stream));
  JMM_CUDA(cudaMemcpy(out, b->d_hist, words * sizeof(uint64_t), cudaMemcpyDeviceToHost));
  return JMM_OK;
}

extern "C" int jmm_batch_run_sampled(jmm_batch *b, uint64_t n_sweeps, uint32_t sample_every) {
  int rc = jmm_batch_run_sampled_async(b, n_sweeps, sample_every, nullptr);
  if (rc) return rc;
  JMM_CUDA(cudaStreamSynchronize(b->stream));
  return check_errors(b);
}

extern "C" int jmm_batch_run_sampled_async(jmm_batch *b, uint64_t n_sweeps, uint32_t sample_every,
                                           void *stream) {
  clear_error();
  JMM_CHECK_ARG(b, "null handle");
  JMM_CHECK_ARG(sample_every > 0, "sample_every must be positive");
  if (n_sweeps == 0) return JMM_OK;
  for (const auto &c : b->chains)
    if (n_sweeps * (uint64_t)(c.n + 1) >= (1ull << 31))
      return fail(JMM_ERR_INVALID, "one run may hold at most 2^31 steps per chain: split it");
  const auto key = std::make_pair(n_sweeps, sample_every);
  auto it = b->sampled.find(key);
  cudaGraphExec_t exec;
  if (it != b->sampled.end()) {
    exec = it->second;
  } else {
    cudaGraph_t graph;
    JMM_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    int rc = JMM_OK;
    uint64_t done = 0;
    while (rc == JMM_OK && done + sample_every <= n_sweeps) {
      rc = launch(b, sample_every, b->stream);
      if (rc == JMM_OK) rc = launch_grad(b, true, b->stream);
      if (rc == JMM_OK && b->d_hist) rc = launch_hist(b, b->stream);
      done += sample_every;
    }
    if (rc == JMM_OK && done < n_sweeps) rc = launch(b, n_sweeps - done, b->stream);
    cudaError_t e = cudaStreamEndCapture(b->stream, &graph);
    if (rc) return rc;
    if (e != cudaSuccess) return cuda_status(e, "cudaStreamEndCapture", __FILE__, __LINE__);
    e = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return cuda_status(e, "cudaGraphInstantiate", __FILE__, __LINE__);
    b->sampled[key] = exec;
  }
  JMM_CUDA(cudaGraphLaunch(exec, stream ? (cudaStream_t)stream : b->stream));
  return JMM_OK;
}

extern "C" int jmm_batch_grad_stats(jmm_batch *b, jmm_grad_stats *out, uint32_t n_chains) {
  clear_error();
  JMM_CHECK_ARG(b && out, "null argument");
  JMM_CHECK_ARG(n_chains == b->n_chains, "n_chains does not match the batch");
  JMM_CUDA(cudaStreamSynchronize(b->stream));
  JMM_CUDA(cudaMemcpy(out, b->d_gstats, n_chains * sizeof(jmm_grad_stats), cudaMemcpyDeviceToHost));
  return JMM_OK;
}
