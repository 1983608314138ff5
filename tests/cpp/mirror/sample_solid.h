// Test stand-in for the reference's sample_solid.h (see trim.h in this folder).
#pragma once
#include "trim.h"

namespace MyTRIM_NS
{
class SampleSolid : public SampleBase
{
public:
  SampleSolid(Real x, Real y, Real z) : SampleBase(x, y, z) {}
};
} // namespace MyTRIM_NS
