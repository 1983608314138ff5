// runmytrim with the reference's own output plugins, built from the reference's
// sources by oracle/Makefile (test infrastructure: it makes the golden output
// files the restated writers are checked against; never part of the product).
//
// apps/runmytrim.C itself cannot be built here (jsoncpp is absent), so this
// program takes the run spec of oracle/runspec.h instead of JSON and otherwise
// follows runmytrim.C:185-331 with one thread: the plugin class chosen by the
// output type (TrimVacCount, TrimVacEnergyCount or TrimRange from apps/src), the
// master seed -> 16-bit per-primary seeds, per primary a reseed and the FIFO
// cascade loop of computeThread (runmytrim.C:71-93), then writeOutput() and the
// two summary lines on stderr.
//
// Usage: ref_runmytrim < spec   (the spec must carry "output <type> <base>")

#include "runspec.h"

#include "simconf.h"
#include "element.h"
#include "material.h"
#include "sample_layers.h"
#include "ion.h"
#include "trim.h"
#include "apps/include/TrimVacCount.h"
#include "apps/include/TrimVacEnergyCount.h"
#include "apps/include/TrimRange.h"

#include <queue>

using namespace MyTRIM_NS;

int
main()
{
  runspec::Spec spec;
  std::string err;
  if (!runspec::parse(std::cin, spec, err))
  {
    fprintf(stderr, "ref_runmytrim: %s\n", err.c_str());
    return 2;
  }
  if (spec.philox || spec.out_type.empty())
  {
    fprintf(stderr, "ref_runmytrim: needs compat seeding and an output key\n");
    return 2;
  }

  SimconfType simconf;
  simconf.fullTraj = false;
  simconf.tmin = 0.2;
  simconf.setLengthScale(spec.scale);

  SampleLayers sample(spec.size[0], spec.size[1], spec.size[2]);
  for (int i = 0; i < 3; ++i)
    sample.bc[i] = SampleBase::sampleBoundary(spec.bc[i]);

  ThreadedTrimBase * trim = nullptr;
  if (spec.out_type == "vaccount")
    trim = new TrimVacCount(&simconf, &sample);
  else if (spec.out_type == "vacenergycount")
    trim = new TrimVacEnergyCount(&simconf, &sample);
  else
    trim = new TrimRange(&simconf, &sample);
  trim->setBaseName(spec.out_base);
  trim->_primaries_only = spec.primaries_only;

  for (auto & l : spec.layers)
  {
    MaterialBase * material = new MaterialBase(&simconf, l.rho);
    for (auto & e : l.el)
    {
      Element el;
      el._Z = e.Z;
      el._m = e.m;
      el._t = e.t;
      el._Edisp = e.Edisp;
      el._Elbind = e.Elbind;
      material->_element.push_back(el);
    }
    material->prepare();
    sample.material.push_back(material);
    sample.layerThickness.push_back(l.thickness);
  }

  simconf.seed(spec.seed);
  std::vector<unsigned int> seeds(spec.count);
  for (long long i = 0; i < spec.count; ++i)
    seeds[i] = simconf.irand();

  std::queue<IonBase *> recoils;
  for (long long n = spec.first; n < spec.first + spec.n; ++n)
  {
    IonBase * pka = new IonBase;
    pka->_Z = spec.Z;
    pka->_m = spec.m;
    pka->_E = spec.E;
    pka->_Ef = spec.Ef;
    pka->_gen = 0;
    pka->_dir = Point(spec.dir[0], spec.dir[1], spec.dir[2]);
    pka->_pos = Point(spec.pos[0], spec.pos[1], spec.pos[2]);
    simconf.seed(seeds[n]);
    recoils.push(pka);
    while (!recoils.empty())
    {
      IonBase * ion = recoils.front();
      recoils.pop();
      sample.averages(ion);
      trim->trim(ion, recoils);
      delete ion;
    }
  }
  trim->writeOutput();
  std::cerr << "Vacancies/ion: " << Real(simconf.vacancies_created) / Real(spec.n) << '\n'
            << "Electronic energy loss/ion: " << simconf.EelTotal / Real(spec.n) << '\n';
  return 0;
}
