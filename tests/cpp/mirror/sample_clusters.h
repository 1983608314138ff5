// Test stand-in for the reference's sample_clusters.h (see trim.h in this folder).
#pragma once
#include "trim.h"

namespace MyTRIM_NS
{
class sampleClusters : public SampleBase
{
public:
  sampleClusters(Real x, Real y, Real z) : SampleBase(x, y, z), kn{1, 1, 1}, cn(0), c{nullptr, nullptr, nullptr, nullptr}
  {
  }
  int kn[3];
  int cn;
  Real * c[4];
};
} // namespace MyTRIM_NS
