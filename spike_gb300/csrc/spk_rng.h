// spk_rng.h - counter-based random numbers and the logarithm used by the
// Poisson inputs, shared bit-for-bit between host and device code.
//
// The reference draws Poisson uniforms from one cuRAND XORWOW state per
// thread (Spike/Backend/CUDA/Neurons/PoissonInputSpikingNeurons.cu:107,
// states seeded in Spike/Backend/CUDA/Helpers/RandomStateManager.cu:39-50).
// Here every draw is a pure function of (seed, neuron, step, domain):
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy
// as 1, 2, 3", SC'11), so there is no generator state to store, reset or
// checkpoint and a draw does not depend on which thread makes it.
//
// All arithmetic here is written as individual IEEE-754 single operations;
// translation units that include this header are compiled without
// multiply-add contraction (-fmad=false for nvcc, -ffp-contract=off for gcc)
// so the host and the device produce identical bits.
#pragma once

#include <stdint.h>

#if defined(__CUDACC__)
#define SPK_HD __host__ __device__ __forceinline__
#else
#define SPK_HD inline
#endif

namespace spk {

// Domains separate the independent streams that share one seed.
enum : uint32_t {
  DOMAIN_POISSON = 0x504f4953u,  // Poisson inter-spike intervals
  DOMAIN_VINIT = 0x56494e49u,    // initial membrane potentials
  DOMAIN_CONNECT = 0x434f4e4eu,  // generated networks: Bernoulli connection draws
  DOMAIN_SYNAPSE = 0x53594e41u,  // generated networks: weight and delay draws
};

struct u32x4 {
  uint32_t x, y, z, w;
};

SPK_HD uint32_t mulhi32(uint32_t a, uint32_t b) {
  return (uint32_t)(((uint64_t)a * (uint64_t)b) >> 32);
}

// One Philox4x32 round: two 32x32->64 multiplies, the high halves xored with
// the other two counter words and the round key (SC'11, section 3.3).
SPK_HD u32x4 philox_round(u32x4 c, uint32_t k0, uint32_t k1) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
  uint32_t hi0 = mulhi32(M0, c.x), lo0 = M0 * c.x;
  uint32_t hi1 = mulhi32(M1, c.z), lo1 = M1 * c.z;
  u32x4 r;
  r.x = hi1 ^ c.y ^ k0;
  r.y = lo1;
  r.z = hi0 ^ c.w ^ k1;
  r.w = lo0;
  return r;
}

// Philox4x32 with 10 rounds; the key is bumped by the Weyl constants between
// rounds.
SPK_HD u32x4 philox4x32_10(u32x4 ctr, uint32_t k0, uint32_t k1) {
  const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#ifdef __CUDACC__
#pragma unroll
#endif
  for (int r = 0; r < 10; ++r) {
    ctr = philox_round(ctr, k0, k1);
    k0 += W0;
    k1 += W1;
  }
  return ctr;
}

// Uniform in (0, 1] from the top 24 bits of a word, exactly representable in
// float (same half-open interval as curand_uniform).
SPK_HD float uniform_open0(uint32_t x) {
  return (float)((x >> 8) + 1u) * 5.9604644775390625e-08f;  // 2^-24
}

// Draw for (seed, neuron, step) in a domain: first Philox output word.
SPK_HD uint32_t draw_u32(uint64_t seed, uint32_t neuron, uint32_t step, uint32_t domain) {
  u32x4 c;
  c.x = neuron;
  c.y = step;
  c.z = 0u;
  c.w = domain;
  return philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32)).x;
}

// All four words of one Philox block keyed by seed with counter (a, b, 0, domain).
SPK_HD u32x4 draw4(uint64_t seed, uint32_t a, uint32_t b, uint32_t domain) {
  u32x4 c;
  c.x = a;
  c.y = b;
  c.z = 0u;
  c.w = domain;
  return philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
}

SPK_HD float draw_uniform(uint64_t seed, uint32_t neuron, uint32_t step, uint32_t domain) {
  return uniform_open0(draw_u32(seed, neuron, step, domain));
}

SPK_HD uint32_t f2u(float f) {
  union {
    float f;
    uint32_t u;
  } v;
  v.f = f;
  return v.u;
}
SPK_HD float u2f(uint32_t u) {
  union {
    float f;
    uint32_t u;
  } v;
  v.u = u;
  return v.f;
}

// Natural logarithm of a positive, normal float.
//
// Method: x = m * 2^e with m in [sqrt(1/2), sqrt(2)); with f = m - 1 and
// s = f / (2 + f), log(m) = 2 atanh(s) = 2s + 2s^3/3 + 2s^5/5 + ... .  The
// series is evaluated to the s^9 term (|s| <= 0.1716, truncation < 1e-9
// relative) in the arrangement log(1+f) = f - (h - s (h + R)), h = f^2/2,
// R = 2z/3 + 2z^2/5 + 2z^3/7 + 2z^4/9, z = s^2, which keeps the leading term f
// exact; e*ln2 is added as a two-part constant (ln2_hi has 17 significant bits
// so e*ln2_hi is exact for |e| < 128, i.e. for every x <= 1 used here).  This is the classical argument-reduction scheme of
// Cody & Waite ("Software Manual for the Elementary Functions", 1980) with the
// plain Taylor coefficients of atanh.
SPK_HD float logf_spk(float x) {
  uint32_t ix = f2u(x);
  int e = (int)(ix >> 23) - 127;
  uint32_t mb = (ix & 0x007fffffu) | 0x3f800000u;
  if (mb > 0x3fb504f3u) {  // m > sqrt(2): halve it
    mb -= 0x00800000u;
    e += 1;
  }
  const float m = u2f(mb);
  const float f = m - 1.0f;
  const float s = f / (2.0f + f);
  const float z = s * s;
  const float c1 = u2f(0x3f2aaaabu);  // 2/3
  const float c2 = u2f(0x3ecccccdu);  // 2/5
  const float c3 = u2f(0x3e924925u);  // 2/7
  const float c4 = u2f(0x3e638e39u);  // 2/9
  float R = c4;
  R = R * z;
  R = c3 + R;
  R = R * z;
  R = c2 + R;
  R = R * z;
  R = c1 + R;
  R = R * z;
  const float h = 0.5f * f;
  const float hf = h * f;
  const float fe = (float)e;
  const float ln2_hi = u2f(0x3f317180u);  // 0.693138122558594 (17 significant bits)
  const float ln2_lo = u2f(0x3717f7d2u);  // ln2 - ln2_hi
  float t = hf + R;
  t = s * t;
  t = t + fe * ln2_lo;
  t = hf - t;
  t = f - t;
  return fe * ln2_hi + t;
}

}  // namespace spk
