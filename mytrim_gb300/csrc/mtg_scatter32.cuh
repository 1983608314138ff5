// Universal-potential scattering in FP32, shared by the FP32 engine and the
// scattering service.  The same Newton steps as trim.C:192-233, iterated on
// d = r - b (no cancellation for distant collisions), and sin^2(theta/2) formed as
// (1 - co)(1 + co) with 1 - co = d (1 - A F / (F + 1)) / (r + roc), algebraically
// equal to 1 - co^2 of trim.C:266-269.
#pragma once

namespace mtg
{

// Returns s2 = sin^2(theta/2) and c2 = cos^2(theta/2).
__device__ __forceinline__ void
scatter32(float eps, float b, float & s2, float & c2, int & niter)
{
  niter = 0;
  if (eps > 10.0f)
  {
    const float w = 2.0f * eps * b;
    s2 = 1.0f / (1.0f + (1.0f + b * (1.0f + b)) * (w * w));
    c2 = 1.0f - s2;
    return;
  }
  // first guess at the distance of closest approach (trim.C:183-190)
  float r = b;
  float rr = -2.7f * __logf(eps * b);
  if (rr >= b)
  {
    rr = -2.7f * __logf(eps * rr);
    if (rr >= b)
      r = rr;
  }
  float d = r - b;
  const float inv_eps = 1.0f / eps;
  float v, v1, q;
  do
  {
    r = b + d;
    const float ex1 = 0.18175f * __expf(-3.1998f * r);
    const float ex2 = 0.50986f * __expf(-0.94229f * r);
    const float ex3 = 0.28022f * __expf(-0.4029f * r);
    const float ex4 = 0.028171f * __expf(-0.20162f * r);
    const float phi = ex1 + ex2 + ex3 + ex4;
    const float tk = 3.1998f * ex1 + 0.94229f * ex2 + 0.4029f * ex3 + 0.20162f * ex4;
    const float ir = 1.0f / r;
    v = phi * ir;
    v1 = -(v + tk) * ir;
    // f(r) = b^2/r + v r/eps - r and f'(r), written in d = r - b
    const float fr = -d * (2.0f * b + d) * ir + phi * inv_eps;
    const float br = b * ir;
    const float fr1 = -br * br - tk * inv_eps - 1.0f;
    q = fr / fr1;
    d -= q;
    ++niter;
  } while (fabsf(q) > 0.001f * fabsf(b + d) && niter < 100);
  r = b + d;
  const float roc = -2.0f * (eps - v) / v1;
  const float sqe = sqrtf(eps);
  const float cc = (0.011615f + sqe) / (0.0071222f + sqe);
  const float aa = 2.0f * eps * (1.0f + (0.99229f / sqe)) * __expf(cc * __logf(b));
  const float ff = (1.0f / (sqrtf(aa * aa + 1.0f) + aa)) * ((9.3066f + eps) / (14.813f + eps));
  const float omc = d * (1.0f - aa * ff / (ff + 1.0f)) / (r + roc);
  s2 = omc * (2.0f - omc);
  c2 = 1.0f - s2;
}

} // namespace mtg
