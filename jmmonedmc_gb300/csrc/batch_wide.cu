// batch_wide.cu -- the chain kernel's 128-register instantiations.
//
// The single-warp shapes (G x S = 32) of the batched chain kernel are held
// to 72 registers so that a full wave of 27 chains per SM fits; a batch
// with at most 16 single-warp chains per SM takes these instantiations
// instead, which keep every value in registers.  FAST precision only (the
// EXACT kernels exist for the oracle's replay, whose results do not depend
// on the register budget).  A translation unit of its own so that it
// compiles beside batch.cu.
#include "batch_core.cuh"

namespace jmm {
namespace batch {

namespace {

template <int G, int S, int WIN>
ChainsKernelFn wide_pot(int pot, bool per) {
  switch (pot * 2 + (per ? 1 : 0)) {
    case JMM_POT_LJCUT * 2: return chains_kernel<G, S, JMM_POT_LJCUT, false, false, WIN, 128>;
    case JMM_POT_LJCUT * 2 + 1: return chains_kernel<G, S, JMM_POT_LJCUT, true, false, WIN, 128>;
    case JMM_POT_SOFTSPHERE * 2:
      return chains_kernel<G, S, JMM_POT_SOFTSPHERE, false, false, WIN, 128>;
    case JMM_POT_SOFTSPHERE * 2 + 1:
      return chains_kernel<G, S, JMM_POT_SOFTSPHERE, true, false, WIN, 128>;
    case JMM_POT_GAUSS * 2: return chains_kernel<G, S, JMM_POT_GAUSS, false, false, WIN, 128>;
    case JMM_POT_GAUSS * 2 + 1: return chains_kernel<G, S, JMM_POT_GAUSS, true, false, WIN, 128>;
    default: return nullptr;
  }
}

}  // namespace

ChainsKernelFn pick_kernel_wide(uint32_t g, uint32_t s, uint32_t w, int pot, bool per) {
  if (w == 0) w = (uint32_t)window_of((int)g);
#define JMM_WIDE(G_, S_, W_) \
  if (g == G_ && s == S_ && w == W_) return wide_pot<G_, S_, W_>(pot, per);
  JMM_WIDE(4, 8, 4)
  JMM_WIDE(2, 16, 4)
  JMM_WIDE(2, 16, 3)
  JMM_WIDE(8, 4, 4)
  JMM_WIDE(16, 2, 8)
  JMM_WIDE(32, 1, 16)
  JMM_WIDE(4, 8, 8)
  JMM_WIDE(2, 16, 8)
  JMM_WIDE(8, 4, 8)
#undef JMM_WIDE
  return nullptr;
}

}  // namespace batch
}  // namespace jmm
