// Test stand-in for the reference's sample_layers.h (see trim.h in this folder).
#pragma once
#include "trim.h"

namespace MyTRIM_NS
{
class SampleLayers : public SampleBase
{
public:
  SampleLayers(Real x, Real y, Real z) : SampleBase(x, y, z) {}
  std::vector<Real> layerThickness;
};
} // namespace MyTRIM_NS
