// grad.cu -- jmm_energy_grad: the backward of the total energy of many
// chain configurations held in device memory (the gradient tooling behind
// jmmonedmc_gb300.grad's torch.autograd.Function).  One warp per chain.
#include "common.cuh"
#include "grad_core.cuh"

using namespace jmm;
using namespace jmm::grad;

namespace {

__global__ void energy_grad_kernel(const jmm_grad_chain *__restrict__ chains, uint32_t n_chains,
                                   const float *__restrict__ x, int32_t boundary,
                                   double *__restrict__ out, float *__restrict__ forces) {
  const uint32_t c = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
  if (c >= n_chains) return;
  const jmm_grad_chain ch = chains[c];
  const PotParams p = make_pot(ch.potential, ch.eps, ch.sigma, ch.cutoff);
  chain_grad(x + ch.x_off, (int)ch.n, p, ch.l, boundary == JMM_BOUNDARY_PERIODIC, out + 4 * c,
             forces ? forces + ch.x_off : nullptr);
}

}  // namespace

extern "C" int jmm_energy_grad(const jmm_grad_chain *chains, uint32_t n_chains, const float *x,
                               int32_t boundary, double *out, float *forces, void *stream) {
  clear_error();
  JMM_CHECK_ARG(chains && x && out, "null argument");
  JMM_CHECK_ARG(boundary == JMM_BOUNDARY_WALLS || boundary == JMM_BOUNDARY_PERIODIC,
                "unknown boundary");
  if (n_chains == 0) return JMM_OK;
  const uint32_t per_block = 8;
  const uint32_t blocks = (n_chains + per_block - 1) / per_block;
  energy_grad_kernel<<<blocks, 32 * per_block, 0, (cudaStream_t)stream>>>(chains, n_chains, x,
                                                                         boundary, out, forces);
  JMM_CUDA(cudaGetLastError());
  return JMM_OK;
}
