// Portable FP32 exp and log for the batched chain kernel.
//
// Both are built only from IEEE-754 single-precision +, *, / and fused
// multiply-add with round-to-nearest, so a C compiler on any host that
// provides a correct fmaf() gets the same bits; the oracle's FP32 mode relies
// on that to replay the kernel exactly.
//
//  log: x = 2^e * m with m in [sqrt(1/2), sqrt(2)); ln m = 2 atanh(z),
//       z = (m - 1) / (m + 1), from the series
//       atanh z = z + z^3/3 + z^5/5 + ... (|z| <= 0.1716, five terms).
//  exp: Cody-Waite reduction x = k ln2 + r with |r| <= ln2/2 (ln2 split in
//       a high part exact in 16 bits and a low part), Taylor polynomial of
//       e^r to degree 7, scaling by 2^k through the exponent field.
// Relative error of both is a few ulp over the ranges used (Metropolis
// thresholds -ln u with u in (0, 1), Gaussian-core energies and volume
// scale factors).
#pragma once
#include <math.h>
#include <stdint.h>

namespace jmm {

#if defined(__CUDA_ARCH__)
#define JMM_FMA(a, b, c) __fmaf_rn((a), (b), (c))
#define JMM_MUL(a, b) __fmul_rn((a), (b))
#define JMM_ADD(a, b) __fadd_rn((a), (b))
#define JMM_SUB(a, b) __fsub_rn((a), (b))
#define JMM_DIV(a, b) __fdiv_rn((a), (b))
#else
#define JMM_FMA(a, b, c) fmaf((a), (b), (c))
#define JMM_MUL(a, b) ((a) * (b))
#define JMM_ADD(a, b) ((a) + (b))
#define JMM_SUB(a, b) ((a) - (b))
#define JMM_DIV(a, b) ((a) / (b))
#endif

__host__ __device__ __forceinline__ uint32_t f2u(float f) {
#if defined(__CUDA_ARCH__)
  return __float_as_uint(f);
#else
  union { float f; uint32_t u; } v;
  v.f = f;
  return v.u;
#endif
}

__host__ __device__ __forceinline__ float u2f(uint32_t u) {
#if defined(__CUDA_ARCH__)
  return __uint_as_float(u);
#else
  union { float f; uint32_t u; } v;
  v.u = u;
  return v.f;
#endif
}

// Natural log of a positive, normal x.
__host__ __device__ __forceinline__ float portable_logf(float x) {
  uint32_t b = f2u(x);
  int e = (int)((b >> 23) & 0xffu) - 127;
  float m = u2f((b & 0x007fffffu) | 0x3f800000u);  // [1, 2)
  if (m > 1.41421356f) {
    m = JMM_MUL(m, 0.5f);
    e += 1;
  }
  const float z = JMM_DIV(JMM_SUB(m, 1.0f), JMM_ADD(m, 1.0f));
  const float z2 = JMM_MUL(z, z);
  float p = 0.11111111f;                 // 1/9
  p = JMM_FMA(p, z2, 0.14285715f);       // 1/7
  p = JMM_FMA(p, z2, 0.2f);              // 1/5
  p = JMM_FMA(p, z2, 0.33333334f);       // 1/3
  p = JMM_FMA(p, z2, 1.0f);
  const float lnm = JMM_MUL(JMM_MUL(2.0f, z), p);
  return JMM_FMA((float)e, 0.69314718f, lnm);
}

// e^x for x in [-87, 88]; 0 below, +inf above.
__host__ __device__ __forceinline__ float portable_expf(float x) {
  if (x < -87.0f) return 0.0f;
  if (x > 88.0f) return u2f(0x7f800000u);
  const float kf = (float)(int)JMM_FMA(x, 1.44269504f, x >= 0.0f ? 0.5f : -0.5f);
  const float ln2_hi = 0.693145751953125f;   // 16 significant bits: k*ln2_hi exact
  const float ln2_lo = 1.42860677e-06f;
  float r = JMM_FMA(-kf, ln2_hi, x);
  r = JMM_FMA(-kf, ln2_lo, r);
  float p = 1.98412701e-04f;             // 1/5040
  p = JMM_FMA(p, r, 1.38888892e-03f);    // 1/720
  p = JMM_FMA(p, r, 8.33333377e-03f);    // 1/120
  p = JMM_FMA(p, r, 4.16666679e-02f);    // 1/24
  p = JMM_FMA(p, r, 1.66666672e-01f);    // 1/6
  p = JMM_FMA(p, r, 0.5f);
  p = JMM_FMA(p, r, 1.0f);
  p = JMM_FMA(p, r, 1.0f);
  int k = (int)kf;
  // 2^k in two factors so that k down to -126-ish stays representable
  int k1 = k / 2, k2 = k - k1;
  const float s1 = u2f((uint32_t)(k1 + 127) << 23);
  const float s2 = u2f((uint32_t)(k2 + 127) << 23);
  return JMM_MUL(JMM_MUL(p, s1), s2);
}

}  // namespace jmm
