// Test stand-in for the reference's class declarations (trim.h, simconf.h,
// material.h, element.h, sample.h, ion.h, shim/point.h): the class names and the
// public fields that mytrim_gb300/cpp/trim_gpu.h reads, and nothing else, so that
// the C++ drop-in (TrimGPU) compiles and runs on a machine without the reference
// checkout.  Written for the tests; it holds no physics.
#pragma once
#define MYTRIM_TRIM_H

#include <vector>

namespace MyTRIM_NS
{
typedef double Real;

// shim/point.h: a 3-vector read through operator()
class Point
{
public:
  Point(Real x = 0, Real y = 0, Real z = 0) : _v{x, y, z} {}
  Real & operator()(unsigned int i) { return _v[i]; }
  const Real & operator()(unsigned int i) const { return _v[i]; }

private:
  Real _v[3];
};

// simconf.h: run settings, the SCOEF.95A / SLFCTR rows and the global tallies
class SimconfType
{
public:
  struct ScoefLine
  {
    Real mm1 = 0, m1 = 0, mnat = 0, rho = 0, atrho = 0, vfermi = 0, heat = 0, lfctr = 0;
    std::vector<Real> pcoef = std::vector<Real>(8, 0.0);
  };
  Real lengthScale() { return _length_scale; }
  void setLengthScale(Real l) { _length_scale = l; }
  Real tmin = 0.2, tau = 0.0, cw = 0.001;
  std::vector<ScoefLine> scoef = std::vector<ScoefLine>(92);
  Real EelTotal = 0.0, EnucTotal = 0.0;
  int vacancies_created = 0;

private:
  Real _length_scale = 1.0;
};

// element.h
class Element
{
public:
  int _Z = 1;
  Real _m = 1.0, _t = 1.0;
  Real _Edisp = 25.0, _Elbind = 3.0;
};

// material.h
class MaterialBase
{
public:
  MaterialBase(SimconfType *, Real rho) : _rho(rho) {}
  Real _rho;
  std::vector<Element> _element;
};

// sample.h
class SampleBase
{
public:
  SampleBase(Real x, Real y, Real z) : w{x, y, z}, bc{PBC, PBC, PBC} {}
  virtual ~SampleBase() {}
  std::vector<MaterialBase *> material;
  Real w[3];
  enum sampleBoundary
  {
    PBC,
    INF,
    CUT
  };
  sampleBoundary bc[3];
};

// ion.h
class IonBase
{
public:
  int _Z = 1;
  Real _m = 1.0, _E = 0.0;
  Point _dir, _pos;
  Real _Ef = 3.0;
};

// trim.h: the constructor, the public _potential and the state the hooks see
class TrimBase
{
public:
  TrimBase(SimconfType * simconf, SampleBase * sample)
    : _potential(UNIVERSAL), _simconf(simconf), _sample(sample)
  {
  }
  virtual ~TrimBase() {}
  enum Potential
  {
    UNIVERSAL,
    MOLIERE,
    CKR
  };
  Potential _potential;

protected:
  SimconfType * _simconf;
  SampleBase * _sample;
};
} // namespace MyTRIM_NS
