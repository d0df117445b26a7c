// grad_core.cuh -- the backward of a chain's total energy.
//
// For a configuration (positions x, box length L) of a chain with pair
// potential phi(r; eps, sigma), truncated at rc:
//   U        = sum_pairs phi
//   dU/deps  = sum_pairs phi / eps
//   dU/dsigma = sum_pairs dphi/dsigma      (rc fixed: no boundary term)
//   dU/dL    = sum_pairs r phi'(r) / L     (positions scaled with the box;
//                                           -Vir/L in the reference's terms,
//                                           src/pot.cpp:59-67)
// and, on request, the forces f_i = -dU/dx_i.  Pair terms are FP32, the
// per-particle partial sums FP32, lane and chain sums FP64.  A pair exactly
// at the cut-off makes U jump under a change of L (truncated, not shifted);
// the derivative here is that of the smooth part, which is what a central
// difference sees when no pair crosses rc within the step.
#pragma once
#include <math.h>
#include <stdint.h>

#include "../../include/jmm_gpu.h"

namespace jmm {
namespace grad {

struct PairDerivs {
  float e;      // phi
  float g_eps;  // dphi/deps
  float g_sig;  // dphi/dsigma
  float r_dphi; // r dphi/dr
};

struct PotParams {
  int pot;
  float eps, sigma, inv_sigma, sigma2, inv_sigma2, rc2;
};

__device__ __forceinline__ PotParams make_pot(int pot, double eps, double sigma, double rc) {
  PotParams p;
  p.pot = pot;
  p.eps = (float)eps;
  p.sigma = (float)sigma;
  p.inv_sigma = (float)(1.0 / sigma);
  p.sigma2 = (float)(sigma * sigma);
  p.inv_sigma2 = (float)(1.0 / (sigma * sigma));
  p.rc2 = (float)(rc * rc);
  return p;
}

__device__ __forceinline__ PairDerivs pair_derivs(float r2, const PotParams &p) {
  PairDerivs d;
  if (p.pot == JMM_POT_GAUSS) {
    const float a = __fmul_rn(r2, p.inv_sigma2);   // (r/sigma)^2
    const float ex = expf(-a);
    d.g_eps = ex;
    d.e = __fmul_rn(p.eps, ex);
    d.g_sig = __fmul_rn(__fmul_rn(__fmul_rn(2.0f, d.e), a), p.inv_sigma);
    d.r_dphi = -__fmul_rn(__fmul_rn(2.0f, d.e), a);
  } else {
    const float inv2 = __fdiv_rn(p.sigma2, r2);     // (sigma/r)^2
    const float inv6 = __fmul_rn(__fmul_rn(inv2, inv2), inv2);
    const float inv12 = __fmul_rn(inv6, inv6);
    if (p.pot == JMM_POT_SOFTSPHERE) {
      d.g_eps = inv12;
      d.e = __fmul_rn(p.eps, inv12);
      d.r_dphi = -__fmul_rn(12.0f, d.e);
    } else {  // LJ 12-6: phi = 4 eps (inv12 - inv6)
      d.g_eps = __fmul_rn(4.0f, __fsub_rn(inv12, inv6));
      d.e = __fmul_rn(p.eps, d.g_eps);
      d.r_dphi = -__fmul_rn(__fmul_rn(24.0f, p.eps), __fsub_rn(__fmul_rn(2.0f, inv12), inv6));
    }
    d.g_sig = -__fmul_rn(d.r_dphi, p.inv_sigma);  // phi depends on sigma/r only
  }
  if (!(r2 <= p.rc2)) {
    d.e = 0.0f;
    d.g_eps = 0.0f;
    d.g_sig = 0.0f;
    d.r_dphi = 0.0f;
  }
  return d;
}

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int m = 1; m < 32; m <<= 1) v = __dadd_rn(v, __shfl_xor_sync(0xffffffffu, v, m));
  return v;
}

// One warp: U, dU/deps, dU/dsigma, dU/dL of one chain into out[0..3], and
// the forces when `forces` is not null.
static __device__ void chain_grad(const float *x, int n, const PotParams &p, double l, bool periodic,
                           double *out, float *forces) {
  const int lane = threadIdx.x & 31;
  const float lf = (float)l;
  double su = 0.0, se = 0.0, ss = 0.0, sl = 0.0;
  for (int i = lane; i < n; i += 32) {
    const float xi = x[i];
    float pu = 0.0f, pe = 0.0f, ps = 0.0f, pl = 0.0f;
    for (int k = 1; periodic ? (2 * k <= n - 1) : (i + k < n); ++k) {
      int j = i + k;
      float shift = 0.0f;
      if (j >= n) {
        j -= n;
        shift = lf;
      }
      const float d = __fsub_rn(__fadd_rn(x[j], shift), xi);
      const float r2 = __fmul_rn(d, d);
      if (r2 > p.rc2) break;
      const PairDerivs q = pair_derivs(r2, p);
      pu = __fadd_rn(pu, q.e);
      pe = __fadd_rn(pe, q.g_eps);
      ps = __fadd_rn(ps, q.g_sig);
      pl = __fadd_rn(pl, q.r_dphi);
    }
    su = __dadd_rn(su, (double)pu);
    se = __dadd_rn(se, (double)pe);
    ss = __dadd_rn(ss, (double)ps);
    sl = __dadd_rn(sl, (double)pl);
    if (forces) {
      // f_i = sum over partners of -dphi/dx_i: phi'(d) d/|d| with d = x_j - x_i
      float f = 0.0f;
      for (int side = -1; side <= 1; side += 2) {
        for (int k = 1; periodic ? (2 * k <= n - 1) : true; ++k) {
          int j = i + side * k;
          float sh = 0.0f;
          if (!periodic && (j < 0 || j >= n)) break;
          if (j < 0) {
            j += n;
            sh = -lf;
          } else if (j >= n) {
            j -= n;
            sh = lf;
          }
          const float d = __fsub_rn(__fadd_rn(x[j], sh), xi);
          const float r2 = __fmul_rn(d, d);
          if (r2 > p.rc2) break;
          const PairDerivs q = pair_derivs(r2, p);
          // dphi/dx_i = phi'(|d|) * (-sign d); r phi'(r) / d = phi'(r) sign(d)
          f = __fadd_rn(f, __fdiv_rn(q.r_dphi, d));
        }
      }
      forces[i] = f;
    }
  }
  su = warp_sum_d(su);
  se = warp_sum_d(se);
  ss = warp_sum_d(ss);
  sl = warp_sum_d(sl);
  if (lane == 0) {
    out[0] = su;
    out[1] = se;
    out[2] = ss;
    out[3] = __ddiv_rn(sl, l);
  }
}

}  // namespace grad
}  // namespace jmm
