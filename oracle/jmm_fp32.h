/*
 * oracle/jmm_fp32.h -- TEST INFRASTRUCTURE (the oracle), never shipped.
 *
 * The FP32 exp and log of the batched kernel's EXACT mode, restated from
 * their mathematical definitions so that the oracle produces the same bits
 * on any IEEE-754 host with a correct fmaf():
 *   log: x = 2^e m, m in [sqrt(1/2), sqrt(2)), ln m = 2 atanh((m-1)/(m+1)),
 *        atanh z = z + z^3/3 + z^5/5 + z^7/7 + z^9/9 (Horner in z^2);
 *   exp: Cody-Waite x = k ln2 + r, ln2 in a 16-bit high and a low part,
 *        e^r by its Taylor series to degree 7 (Horner), times 2^k split in
 *        two exponent-field factors.
 * Compiled with -ffp-contract=off: every operation rounds on its own.
 */
#ifndef JMM_ORACLE_FP32_H
#define JMM_ORACLE_FP32_H

#include <math.h>
#include <stdint.h>
#include <string.h>

static inline uint32_t jmmo_f2u(float f) {
  uint32_t u;
  memcpy(&u, &f, 4);
  return u;
}

static inline float jmmo_u2f(uint32_t u) {
  float f;
  memcpy(&f, &u, 4);
  return f;
}

static inline float jmmo_logf(float x) {
  uint32_t b = jmmo_f2u(x);
  int e = (int)((b >> 23) & 0xffu) - 127;
  float m = jmmo_u2f((b & 0x007fffffu) | 0x3f800000u);
  if (m > 1.41421356f) {
    m = m * 0.5f;
    e += 1;
  }
  float z = (m - 1.0f) / (m + 1.0f);
  float z2 = z * z;
  float p = 0.11111111f;
  p = fmaf(p, z2, 0.14285715f);
  p = fmaf(p, z2, 0.2f);
  p = fmaf(p, z2, 0.33333334f);
  p = fmaf(p, z2, 1.0f);
  float lnm = (2.0f * z) * p;
  return fmaf((float)e, 0.69314718f, lnm);
}

static inline float jmmo_expf(float x) {
  if (x < -87.0f) return 0.0f;
  if (x > 88.0f) return jmmo_u2f(0x7f800000u);
  float kf = (float)(int)fmaf(x, 1.44269504f, x >= 0.0f ? 0.5f : -0.5f);
  float r = fmaf(-kf, 0.693145751953125f, x);
  r = fmaf(-kf, 1.42860677e-06f, r);
  float p = 1.98412701e-04f;
  p = fmaf(p, r, 1.38888892e-03f);
  p = fmaf(p, r, 8.33333377e-03f);
  p = fmaf(p, r, 4.16666679e-02f);
  p = fmaf(p, r, 1.66666672e-01f);
  p = fmaf(p, r, 0.5f);
  p = fmaf(p, r, 1.0f);
  p = fmaf(p, r, 1.0f);
  int k = (int)kf;
  int k1 = k / 2, k2 = k - k1;
  float s1 = jmmo_u2f((uint32_t)(k1 + 127) << 23);
  float s2 = jmmo_u2f((uint32_t)(k2 + 127) << 23);
  return (p * s1) * s2;
}

#endif
