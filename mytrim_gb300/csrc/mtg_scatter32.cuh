// Screened-potential scattering in FP32, shared by the FP32 engine and the
// scattering service.  The same Newton steps as trim.C:192-233, iterated on
// d = r - b (no cancellation for distant collisions), and sin^2(theta/2) formed as
// (1 - co)(1 + co) with 1 - co = d (1 - A F / (F + 1)) / (r + roc), algebraically
// equal to 1 - co^2 of trim.C:266-269.
//
// Each potential is phi(r) = sum_i w_i exp(-k_i r) with v = phi / r and
// v1 = -(v + sum_i c_i exp(-k_i r)) / r (trim.C:197-222), so that
// f'(r) = -b^2/r^2 - (sum_i c_i exp(-k_i r)) / eps - 1.  c_i = k_i w_i for the
// universal and Moliere potentials; for C-Kr the reference writes c_i that are
// not the derivative's, and they are kept as written.  The Moliere terms
// exp(-0.3 r)^4 and exp(-0.3 r)^20 are evaluated as exp(-1.2 r) and exp(-6 r).
// v and v1 are formed once, after the loop, from the last iterate's values.
//
// The Newton solve starts from a tabulated first guess (mtg_newton_guess.h):
// inside the table's range one step nearly always meets the stopping test, where
// the reference's guess needs 2 to 5, so a warp no longer waits on its slowest
// lane's extra iterations.  The converged root differs from the one reached from
// the reference's guess by less than the stopping test's tolerance.
#pragma once

#include <cuda_runtime.h>

#include "mtg_newton_guess.h"

namespace mtg
{

// log2(r0 - b) per potential, row-major over (log2 eps, b); one copy per
// translation unit that scatters in FP32, filled by upload_newton_guess32_here
static __device__ float g_newton_guess32[NG_CELLS];

static inline cudaError_t
upload_newton_guess32_here(const float * table)
{
  return cudaMemcpyToSymbol(g_newton_guess32, table, sizeof(float) * NG_CELLS);
}

// first guess at d = r0 - b: bilinear in the table inside its range (universal
// and Moliere potentials), else the reference's guess (trim.C:183-190)
template <int POT>
__device__ __forceinline__ float
newton_start32(float eps, float b)
{
  const float fu = (__log2f(eps) - float(NG_U0)) * float(1.0 / NG_DU);
  const float fb = b * float(1.0 / NG_DB);
  if (POT < NG_POT && fu >= 0.0f && fb < float(NG_B - 1))
  {
    const int i = min(int(fu), NG_U - 2);
    const int j = int(fb);
    const float a = fu - float(i), c = fb - float(j);
    const float * t = g_newton_guess32 + (POT * NG_U + i) * NG_B + j;
    const float t00 = __ldg(t), t01 = __ldg(t + 1);
    const float t10 = __ldg(t + NG_B), t11 = __ldg(t + NG_B + 1);
    const float lo = fmaf(c, t01 - t00, t00);
    const float hi = fmaf(c, t11 - t10, t10);
    return exp2f(fmaf(a, hi - lo, lo));
  }
  float r = b;
  float rr = -2.7f * __logf(eps * b);
  if (rr >= b)
  {
    rr = -2.7f * __logf(eps * rr);
    if (rr >= b)
      r = rr;
  }
  return r - b;
}

// phi(r) and sum_i c_i exp(-k_i r) with each weighted exponential as one 2^x:
// w_i exp(-k_i r) = 2^(r (-k_i log2 e) + log2 w_i), and the derivative sum written on
// the weighted terms (coefficient c_i / w_i).  Constants from the coefficients of
// trim.C:197-222 in double precision.
template <int POT>
__device__ __forceinline__ void
screening32(float r, float & phi, float & tk)
{
  if constexpr (POT == 1)
  {
    // Moliere (trim.C:206-213): w = 0.35, 0.55, 0.1; k = 0.3, 1.2, 6; c / w = k
    const float e1 = exp2f(fmaf(r, -0.432808512f, -1.51457317f));
    const float e2 = exp2f(fmaf(r, -1.73123405f, -0.862496476f));
    const float e3 = exp2f(fmaf(r, -8.65617025f, -3.32192809f));
    phi = e1 + e2 + e3;
    tk = 0.3f * e1 + 1.2f * e2 + 6.0f * e3;
  }
  else if constexpr (POT == 2)
  {
    // C-Kr (trim.C:215-222): w = 0.191, 0.474, 0.335; k = 0.279, 0.637, 1.1919; the
    // reference's c = 0.531865, 0.30181, 0.6437 give c / w = 2.7846335, 0.63672996,
    // 1.9214925
    const float e1 = exp2f(fmaf(r, -0.402511916f, -2.38835546f));
    const float e2 = exp2f(fmaf(r, -0.918996741f, -1.07704104f));
    const float e3 = exp2f(fmaf(r, -1.71954822f, -1.57776700f));
    phi = e1 + e2 + e3;
    tk = 2.7846335f * e1 + 0.63672996f * e2 + 1.9214925f * e3;
  }
  else
  {
    // universal (trim.C:197-204)
    const float e1 = exp2f(fmaf(r, -4.61633559f, -2.45997273f));
    const float e2 = exp2f(fmaf(r, -1.35943711f, -0.971826936f));
    const float e3 = exp2f(fmaf(r, -0.581261832f, -1.83536817f));
    const float e4 = exp2f(fmaf(r, -0.290876174f, -5.14964541f));
    phi = e1 + e2 + e3 + e4;
    tk = 3.1998f * e1 + 0.94229f * e2 + 0.4029f * e3 + 0.20162f * e4;
  }
}

// magic-formula constants (trim.C:236-258): beta = (m0 + sqe) / (m1 + sqe),
// A = 2 eps (1 + m2 / sqe) b^beta, F = (sqrt(A^2 + 1) - A) (m3 + eps) / (m4 + eps)
template <int POT>
struct Magic32;
template <>
struct Magic32<0>
{
  static constexpr float m0 = 0.011615f, m1 = 0.0071222f, m2 = 0.99229f, m3 = 9.3066f, m4 = 14.813f;
};
template <>
struct Magic32<1>
{
  static constexpr float m0 = 0.009611f, m1 = 0.005175f, m2 = 0.6743f, m3 = 6.314f, m4 = 10.0f;
};
template <>
struct Magic32<2>
{
  static constexpr float m0 = 0.235809f, m1 = 0.126000f, m2 = 1.0144f, m3 = 6935.0f, m4 = 83550.0f;
};

// Returns s2 = sin^2(theta/2) and c2 = cos^2(theta/2).
template <int POT>
__device__ __forceinline__ void
scatter32_pot(float eps, float b, float & s2, float & c2, int & niter)
{
  niter = 0;
  if (eps > 10.0f)
  {
    const float w = 2.0f * eps * b;
    s2 = 1.0f / (1.0f + (1.0f + b * (1.0f + b)) * (w * w));
    c2 = 1.0f - s2;
    return;
  }
  float d = newton_start32<POT>(eps, b);
  const float inv_eps = 1.0f / eps;
  float r, phi, tk, ir, q;
  do
  {
    r = b + d;
    screening32<POT>(r, phi, tk);
    ir = 1.0f / r;
    // f(r) = b^2/r + v r/eps - r and f'(r), written in d = r - b
    const float fr = -d * (2.0f * b + d) * ir + phi * inv_eps;
    const float br = b * ir;
    const float fr1 = -br * br - tk * inv_eps - 1.0f;
    q = fr / fr1;
    d -= q;
    ++niter;
  } while (fabsf(q) > 0.001f * fabsf(b + d) && niter < 100);
  // v and v1 at the last iterate's r, as the reference uses them (trim.C:235)
  const float v = phi * ir;
  const float v1 = -(v + tk) * ir;
  r = b + d;
  using M = Magic32<POT>;
  const float roc = -2.0f * (eps - v) / v1;
  const float sqe = sqrtf(eps);
  const float cc = (M::m0 + sqe) / (M::m1 + sqe);
  const float aa = 2.0f * eps * (1.0f + (M::m2 / sqe)) * __expf(cc * __logf(b));
  const float ff = (1.0f / (sqrtf(aa * aa + 1.0f) + aa)) * ((M::m3 + eps) / (M::m4 + eps));
  const float omc = d * (1.0f - aa * ff / (ff + 1.0f)) / (r + roc);
  s2 = omc * (2.0f - omc);
  c2 = 1.0f - s2;
}

// universal potential (the default)
__device__ __forceinline__ void
scatter32(float eps, float b, float & s2, float & c2, int & niter)
{
  scatter32_pot<0>(eps, b, s2, c2, niter);
}

// potential chosen at run time (TrimBase::Potential: 0 universal, 1 Moliere, 2 C-Kr)
__device__ __forceinline__ void
scatter32(float eps, float b, float & s2, float & c2, int & niter, int pot)
{
  if (pot == 1)
    scatter32_pot<1>(eps, b, s2, c2, niter);
  else if (pot == 2)
    scatter32_pot<2>(eps, b, s2, c2, niter);
  else
    scatter32_pot<0>(eps, b, s2, c2, niter);
}

} // namespace mtg
