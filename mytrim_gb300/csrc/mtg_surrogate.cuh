// Learned scattering surrogate: MLP 2 -> 64 -> 64 -> 64 -> 2 with SiLU, inputs
// (log10 reduced energy, reduced impact parameter), outputs sin^2(theta/2) and
// the reduced time integral.  Weights live in BF16, accumulation in FP32.
#pragma once

#include <stdint.h>

namespace mtg
{

constexpr int SG_H = 64;            // hidden width
constexpr float SG_LOGEPS_MIN = -4.0f, SG_LOGEPS_MAX = 4.0f;
constexpr float SG_B_MAX = 12.0f;

struct SurrogateNet;

__device__ __forceinline__ bool
surrogate_in_domain(float eps, float b)
{
  return false;
}

__device__ __forceinline__ void
surrogate_s2(const SurrogateNet * net, float eps, float b, float & s2, float & c2)
{
  s2 = 0.0f;
  c2 = 1.0f;
}

} // namespace mtg
