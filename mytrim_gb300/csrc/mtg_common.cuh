// Shared host/device building blocks of the cascade engine:
//   * counter-based random streams (Philox4x32-10) and cascade-member keys
//   * project-owned FP64 exp / log / pow
//
// Everything here compiles both for the GPU and, unchanged, for the host replay
// build that checks GPU trajectories bit for bit.  The FP64 math therefore uses
// only correctly rounded IEEE operations (+ - * / sqrt fma, rint) so that the two
// builds produce identical bits; the FP64 engine translation unit is compiled
// with -fmad=false and the host build with -ffp-contract=off for the same reason.
#pragma once

#include <stdint.h>
#include <math.h>
#include <string.h>

#if defined(__CUDACC__)
#define MTG_HD __host__ __device__ __forceinline__
#else
#define MTG_HD inline
#endif

namespace mtg
{

// ------------------------------------------------------------------ Philox
// Philox4x32-10: Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy
// as 1, 2, 3", SC'11.  Multipliers and Weyl increments are the published ones.
struct U4
{
  uint32_t x, y, z, w;
};

MTG_HD uint32_t
mulhi32(uint32_t a, uint32_t b)
{
#if defined(__CUDA_ARCH__)
  return __umulhi(a, b);
#else
  return uint32_t((uint64_t(a) * uint64_t(b)) >> 32);
#endif
}

MTG_HD U4
philox(U4 c, uint32_t k0, uint32_t k1)
{
#pragma unroll
  for (int r = 0; r < 10; ++r)
  {
    const uint32_t h0 = mulhi32(0xD2511F53u, c.x), l0 = 0xD2511F53u * c.x;
    const uint32_t h1 = mulhi32(0xCD9E8D57u, c.z), l1 = 0xCD9E8D57u * c.z;
    c = U4{h1 ^ c.y ^ k0, l1, h0 ^ c.w ^ k1, l0};
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  return c;
}

// splitmix64 finaliser (Steele, Lea, Flood, OOPSLA 2014): a bijective 64-bit mixer
MTG_HD uint64_t
mix64(uint64_t z)
{
  z ^= z >> 30;
  z *= 0xBF58476D1CE4E5B9ull;
  z ^= z >> 27;
  z *= 0x94D049BB133111EBull;
  z ^= z >> 31;
  return z;
}

// Cascade-member keys are derived from the path through the cascade tree, not
// from processing order, so every trajectory replays identically whatever the
// GPU schedule: the primary n of simulation s has key mix64((s << 40) ^ (n + 1)),
// and the recoil created in collision ic of a member with key k has key
// mix64(k + 0x9E3779B97F4A7C15 * ic).
MTG_HD uint64_t
root_key(uint64_t sim, uint64_t primary)
{
  return mix64((sim << 40) ^ (primary + 1));
}

MTG_HD uint64_t
child_key(uint64_t parent, uint32_t collision)
{
  return mix64(parent + 0x9E3779B97F4A7C15ull * uint64_t(collision));
}

// Counter layout: (key lo, key hi, collision index, block).  Collision index 0
// block 0 holds the member's first-flight draw; collision ic >= 1 block 0 holds
// the impact-parameter and target-atom draws, blocks 1.. the perpendicular-vector
// rejection passes.
MTG_HD U4
draw_block(uint64_t member, uint32_t ic, uint32_t block, uint32_t k0, uint32_t k1)
{
  return philox(U4{uint32_t(member), uint32_t(member >> 32), ic, block}, k0, k1);
}

// uniform in (0, 1] with 53 random bits
MTG_HD double
u53(uint32_t hi, uint32_t lo)
{
  const uint64_t v = (uint64_t(hi) << 21) ^ uint64_t(lo >> 11);
  return double(v + 1) * (1.0 / 9007199254740992.0);
}

// uniform in (0, 1] with 32 random bits
MTG_HD double
u32d(uint32_t x)
{
  return (double(x) + 1.0) * (1.0 / 4294967296.0);
}

// uniform in (0, 1] with 24 random bits (single precision)
MTG_HD float
u24f(uint32_t x)
{
  return float((x >> 8) + 1u) * (1.0f / 16777216.0f);
}

// The uniform r1 of a member's first free flight (trim.C:71, 93-94), taken from
// the bits of its path key.  A key is the output of a 64-bit mixing function of
// (parent key, collision) or (simulation, primary), so its bits are as random as a
// generator draw and independent of the Philox draws keyed by it; a member start
// then needs no generator call.  FP64 takes 53 bits, FP32 the leading 24 of them.
MTG_HD double
key_u53(uint64_t key)
{
  return u53(uint32_t(key >> 32), uint32_t(key));
}

MTG_HD float
key_u24f(uint64_t key)
{
  return u24f(uint32_t(key >> 32));
}

// ------------------------------------------------------------------ FP64 math
MTG_HD double
bits_to_double(uint64_t b)
{
#if defined(__CUDA_ARCH__)
  return __longlong_as_double((long long)b);
#else
  double d;
  memcpy(&d, &b, sizeof d);
  return d;
#endif
}

MTG_HD uint64_t
double_to_bits(double d)
{
#if defined(__CUDA_ARCH__)
  return (uint64_t)__double_as_longlong(d);
#else
  uint64_t b;
  memcpy(&b, &d, sizeof b);
  return b;
#endif
}

// 2^k for -1022 <= k <= 1023
MTG_HD double
pow2i(int k)
{
  return bits_to_double(uint64_t(k + 1023) << 52);
}

// e^x.  Cody-Waite reduction x = k ln2 + r with ln2 split into a 42-bit head
// (k * head is exact for |k| < 2^11) and a tail, |r| <= ln2/2, then the Taylor
// series of e^r to degree 13 (truncation below 5e-18 relative), scaled by 2^k.
MTG_HD double
exp64(double x)
{
  if (x < -745.2)
    return 0.0;
  if (x > 709.7)
    return HUGE_VAL;
  const double k = rint(x * 0x1.71547652b82fep+0);
  double r = fma(-k, 0x1.62e42fefa3800p-1, x);
  r = fma(-k, 0x1.ef35793c76730p-45, r);
  double p = 0x1.6124613a86d09p-33; // 1/13!
  p = fma(p, r, 0x1.1eed8eff8d898p-29); // 1/12!
  p = fma(p, r, 0x1.ae64567f544e4p-26); // 1/11!
  p = fma(p, r, 0x1.27e4fb7789f5cp-22); // 1/10!
  p = fma(p, r, 0x1.71de3a556c734p-19); // 1/9!
  p = fma(p, r, 0x1.a01a01a01a01ap-16); // 1/8!
  p = fma(p, r, 0x1.a01a01a01a01ap-13); // 1/7!
  p = fma(p, r, 0x1.6c16c16c16c17p-10); // 1/6!
  p = fma(p, r, 0x1.1111111111111p-7);  // 1/5!
  p = fma(p, r, 0x1.5555555555555p-5);  // 1/4!
  p = fma(p, r, 0x1.5555555555555p-3);  // 1/3!
  p = fma(p, r, 0.5);
  p = fma(p, r, 1.0);
  p = fma(p, r, 1.0);
  const int ki = int(k);
  if (ki >= -1022)
    return p * pow2i(ki);
  // subnormal results: scale in two steps
  return (p * pow2i(ki + 600)) * pow2i(-600);
}

// natural logarithm for finite x > 0.  x = m 2^e with m in (sqrt(1/2), sqrt(2)],
// f = m - 1, s = f / (2 + f); log(1 + f) = 2 atanh(s) is summed as
// f - hf + s (hf + R) with hf = f^2/2 and R = sum_{k=1..12} 2 s^{2k} / (2k + 1)
// (the series tail is below 1e-19 relative for |s| <= 0.1716).
MTG_HD double
log64(double x)
{
  if (!(x > 0.0))
    return x == 0.0 ? -HUGE_VAL : NAN;
  int eadj = 0;
  if (x < 0x1p-1022)
  {
    x *= 0x1p54;
    eadj = -54;
  }
  const uint64_t bits = double_to_bits(x);
  int e = int((bits >> 52) & 0x7ff) - 1023 + eadj;
  double m = bits_to_double((bits & 0x000fffffffffffffull) | 0x3ff0000000000000ull);
  if (m > 0x1.6a09e667f3bcdp+0)
  {
    m *= 0.5;
    e += 1;
  }
  const double f = m - 1.0;
  const double s = f / (2.0 + f);
  const double z = s * s;
  double R = 0x1.47ae147ae147bp-4;      // 2/25
  R = fma(R, z, 0x1.642c8590b2164p-4);  // 2/23
  R = fma(R, z, 0x1.8618618618618p-4);  // 2/21
  R = fma(R, z, 0x1.af286bca1af28p-4);  // 2/19
  R = fma(R, z, 0x1.e1e1e1e1e1e1ep-4);  // 2/17
  R = fma(R, z, 0x1.1111111111111p-3);  // 2/15
  R = fma(R, z, 0x1.3b13b13b13b14p-3);  // 2/13
  R = fma(R, z, 0x1.745d1745d1746p-3);  // 2/11
  R = fma(R, z, 0x1.c71c71c71c71cp-3);  // 2/9
  R = fma(R, z, 0x1.2492492492492p-2);  // 2/7
  R = fma(R, z, 0x1.999999999999ap-2);  // 2/5
  R = fma(R, z, 0x1.5555555555555p-1);  // 2/3
  R = R * z;
  const double hf = 0.5 * f * f;
  const double de = double(e);
  return fma(de, 0x1.62e42fefa3800p-1,
             f - (hf - fma(s, hf + R, de * 0x1.ef35793c76730p-45)));
}

// x^y for x >= 0 (every use in the engine has a positive base)
MTG_HD double
pow64(double x, double y)
{
  if (x == 0.0)
    return y > 0.0 ? 0.0 : (y == 0.0 ? 1.0 : HUGE_VAL);
  return exp64(y * log64(x));
}

} // namespace mtg
