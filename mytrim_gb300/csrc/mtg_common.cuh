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

#include "mtg_fp64_tables.h"

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

struct U2
{
  uint32_t x, y;
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

// Philox2x32-10 (same paper): 64-bit counter, 32-bit key, multiplier 0xD256D193
MTG_HD U2
philox2(U2 c, uint32_t k)
{
#pragma unroll
  for (int r = 0; r < 10; ++r)
  {
    const uint32_t h = mulhi32(0xD256D193u, c.x), l = 0xD256D193u * c.x;
    c = U2{h ^ k ^ c.y, l};
    k += 0x9E3779B9u;
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

// Two 32-bit draws of collision ic of a member (the FP32 engine): Philox2x32-10
// with the member key as counter and the collision index, through a bijection, in
// the key.  A separate stream family from draw_block's.
MTG_HD U2
draw_pair(uint64_t member, uint32_t ic, uint32_t k0, uint32_t k1)
{
  return philox2(U2{uint32_t(member), uint32_t(member >> 32)}, (k0 ^ k1) + ic * 0x85EBCA6Bu);
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

// ---- table-driven FP64 exp and log (P. T. P. Tang, ACM TOMS 15 (1989) 144; 16
// (1990) 378).  Tables from gen_fp64_tables.py (mtg_fp64_tables.h); the device
// reads its own copies in global memory, the host build (replay) the same values.
namespace fp64tab
{
#if defined(__CUDACC__)
static __device__ const double d_exp_hi[64] = {MTG_EXP_TABLE_HI};
static __device__ const double d_exp_lo[64] = {MTG_EXP_TABLE_LO};
static __device__ const double d_log_invc[92] = {MTG_LOG_INVC};
static __device__ const double d_log_hi[92] = {MTG_LOG_TABLE_HI};
static __device__ const double d_log_lo[92] = {MTG_LOG_TABLE_LO};
#endif
static const double h_exp_hi[64] = {MTG_EXP_TABLE_HI};
static const double h_exp_lo[64] = {MTG_EXP_TABLE_LO};
static const double h_log_invc[92] = {MTG_LOG_INVC};
static const double h_log_hi[92] = {MTG_LOG_TABLE_HI};
static const double h_log_lo[92] = {MTG_LOG_TABLE_LO};
} // namespace fp64tab

#if defined(__CUDA_ARCH__)
#define MTG_TAB(name) fp64tab::d_##name
#else
#define MTG_TAB(name) fp64tab::h_##name
#endif

// e^x.  x = (64 m + j) ln2/64 + r with n = 64 m + j = rint(64 x / ln2), |r| <= ln2/128
// (ln2/64 in two parts, the first with 29 significant bits so that n times it is
// exact); e^x = 2^m (S_j + S_j p(r)), S_j = 2^(j/64) as a double pair and p the
// Taylor polynomial of e^r - 1 to degree 6 (truncation below 3e-20 relative).
// This is the full-range form; exp64 below takes a shorter route for |x| < 704.
MTG_HD double
exp64_wide(double x)
{
  if (x < -745.2)
    return 0.0;
  if (x > 709.7)
    return HUGE_VAL;
  const double k = rint(x * MTG_EXP_INV_L);
  double r = fma(-k, MTG_EXP_L1, x);
  r = fma(-k, MTG_EXP_L2, r);
  const int n = int(k);
  const int j = n & 63;
  const int m = (n - j) / 64;
  double p = 0x1.6c16c16c16c17p-10;   // 1/720
  p = fma(p, r, 0x1.1111111111111p-7); // 1/120
  p = fma(p, r, 0x1.5555555555555p-5); // 1/24
  p = fma(p, r, 0x1.5555555555555p-3); // 1/6
  p = fma(p, r, 0.5);
  p = fma(p, r * r, r);
  const double sh = MTG_TAB(exp_hi)[j];
  const double y = sh + fma(sh, p, MTG_TAB(exp_lo)[j]);
  if (m >= -1022)
    return y * pow2i(m);
  // subnormal results: scale in two steps
  return (y * pow2i(m + 600)) * pow2i(-600);
}

// e^x with the same arithmetic as exp64_wide, hence the same result for every x.
// For |x| < 704 (judged on the high word, no FP64 compare) the result is a normal
// number 2^m y with -1017 <= m <= 1016: n = rint(64 x / ln2) comes from adding and
// subtracting 1.5 * 2^52 (the sum's low word is n), and the scaling by 2^m is an
// integer add to the exponent field.  The FP64 unit is the narrow one on GB300, so
// this keeps the compares, conversions and the scaling multiply off it.
MTG_HD double
exp64(double x)
{
  const uint64_t bx = double_to_bits(x);
  if ((uint32_t(bx >> 32) & 0x7fffffffu) >= 0x40860000u) // |x| >= 704, inf, NaN
    return exp64_wide(x);
  // rint(x * 64/ln2) + 1.5 * 2^52, the product rounded first as in exp64_wide
  // (never contracted to an fma, whatever the translation unit's flags)
#if defined(__CUDA_ARCH__)
  const double t = __dadd_rn(__dmul_rn(x, MTG_EXP_INV_L), 0x1.8p52);
#else
  const double t = x * MTG_EXP_INV_L + 0x1.8p52; // host builds use -ffp-contract=off
#endif
  const double k = t - 0x1.8p52;
  const int n = int(uint32_t(double_to_bits(t)));
  double r = fma(-k, MTG_EXP_L1, x);
  r = fma(-k, MTG_EXP_L2, r);
  const int j = n & 63;
  const int m = n >> 6; // floor(n / 64)
  double p = 0x1.6c16c16c16c17p-10;   // 1/720
  p = fma(p, r, 0x1.1111111111111p-7); // 1/120
  p = fma(p, r, 0x1.5555555555555p-5); // 1/24
  p = fma(p, r, 0x1.5555555555555p-3); // 1/6
  p = fma(p, r, 0.5);
  p = fma(p, r * r, r);
  const double sh = MTG_TAB(exp_hi)[j];
  const double y = sh + fma(sh, p, MTG_TAB(exp_lo)[j]);
  return bits_to_double(double_to_bits(y) + (uint64_t(int64_t(m)) << 52));
}

// natural logarithm for finite x > 0.  x = 2^e m with m in (sqrt(1/2), sqrt(2)];
// m falls in interval j of 0.703125 + j/128, whose approximate reciprocal inv_c has
// at most 10 significant bits, so u = m inv_c - 1 is a single rounding (|u| < 1/128,
// u = m - 1 exactly around 1); log x = e ln2 - log(inv_c) + log1p(u) with the
// first two summed exactly (both multiples of 2^-42) and log1p(u) its Taylor
// polynomial to degree 9 (truncation below 1e-20 relative).
MTG_HD double
log64_wide(double x)
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
  int j = int((m - 0.703125) * 128.0);
  j = j < 0 ? 0 : (j > 91 ? 91 : j);
  const double u = fma(m, MTG_TAB(log_invc)[j], -1.0);
  // log1p(u) - u = u^2 (-1/2 + u/3 - u^2/4 + ... + u^7/9), Horner from the top
  double q = 0x1.c71c71c71c71cp-4;      // 1/9
  q = fma(q, u, -0x1.0000000000000p-3); // -1/8
  q = fma(q, u, 0x1.2492492492492p-3);  // 1/7
  q = fma(q, u, -0x1.5555555555555p-3); // -1/6
  q = fma(q, u, 0x1.999999999999ap-3);  // 1/5
  q = fma(q, u, -0x1.0000000000000p-2); // -1/4
  q = fma(q, u, 0x1.5555555555555p-2);  // 1/3
  q = fma(q, u, -0.5);                  // -1/2
  q = q * (u * u);
  const double de = double(e);
  const double hi = fma(de, MTG_LOG_LN2_HI, MTG_TAB(log_hi)[j]);
  const double lo = fma(de, MTG_LOG_LN2_LO, MTG_TAB(log_lo)[j]);
  return hi + (u + (lo + q));
}

// log x with the same arithmetic as log64_wide, hence the same result for every x.
// For positive normal finite x (judged on the bit pattern) the exponent, the halving
// of m above sqrt(2) and the interval index come from integer operations on the
// bits: j = 38 + (f >> 45) for m = 1 + f / 2^52 <= sqrt(2), j = (f >> 46) - 26 for
// m / 2, the same integer parts of (m - 0.703125) 128 that log64_wide computes in
// FP64 (exactly: m - 0.703125 is representable).  e becomes a double through the
// 1.5 * 2^52 trick.
MTG_HD double
log64(double x)
{
  const uint64_t bits = double_to_bits(x);
  if (bits - 0x0010000000000000ull >= 0x7fe0000000000000ull) // zero, subnormal, negative, inf, NaN
    return log64_wide(x);
  const uint64_t f = bits & 0x000fffffffffffffull;
  int e = int(bits >> 52) - 1023;
  double m;
  int j;
  if (f > 0x6a09e667f3bcdull) // m = 1 + f / 2^52 > sqrt(2): use m / 2
  {
    m = bits_to_double(f | 0x3fe0000000000000ull);
    e += 1;
    j = int(f >> 46) - 26;
  }
  else
  {
    m = bits_to_double(f | 0x3ff0000000000000ull);
    j = 38 + int(f >> 45);
  }
  const double u = fma(m, MTG_TAB(log_invc)[j], -1.0);
  double q = 0x1.c71c71c71c71cp-4;      // 1/9
  q = fma(q, u, -0x1.0000000000000p-3); // -1/8
  q = fma(q, u, 0x1.2492492492492p-3);  // 1/7
  q = fma(q, u, -0x1.5555555555555p-3); // -1/6
  q = fma(q, u, 0x1.999999999999ap-3);  // 1/5
  q = fma(q, u, -0x1.0000000000000p-2); // -1/4
  q = fma(q, u, 0x1.5555555555555p-2);  // 1/3
  q = fma(q, u, -0.5);                  // -1/2
  q = q * (u * u);
  const double de = bits_to_double(0x4338000000000000ull + uint64_t(int64_t(e))) - 0x1.8p52;
  const double hi = fma(de, MTG_LOG_LN2_HI, MTG_TAB(log_hi)[j]);
  const double lo = fma(de, MTG_LOG_LN2_LO, MTG_TAB(log_lo)[j]);
  return hi + (u + (lo + q));
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
