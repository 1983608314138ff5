// Runs the C++ drop-in on the GPU the way a reference user would: SimconfType,
// MaterialBase/Element, SampleLayers/SampleSolid and IonBase built in code, then
// TrimGPU::runPrimaries and TrimGPU::runBatch (mytrim_gb300/cpp/trim_gpu.h).
// Compiled against tests/cpp/mirror, which declares the reference's class and field
// names, so that it runs where the reference's headers are absent.
//
//   trim_gpu_run <stopping_tables.tsv>
// prints one line per result: "tot <label> <integer totals> <Eel> <Enuc>" (hex
// floats), then the SimconfType tallies the runs added to.
#include "trim.h"
#include "sample_layers.h"
#include "sample_solid.h"
#include "trim_gpu.h"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <sstream>
#include <string>

using namespace MyTRIM_NS;

// SCOEF.95A / SLFCTR columns of the engine's table file into SimconfType::scoef
static bool
read_tables(const char * path, SimconfType & simconf)
{
  std::ifstream in(path);
  std::string line;
  int rows = 0;
  while (std::getline(in, line))
  {
    if (line.empty() || line[0] == '#')
      continue;
    std::istringstream ls(line);
    int Z;
    std::string sym;
    ls >> Z >> sym;
    if (Z < 1 || Z > 92)
      return false;
    SimconfType::ScoefLine & s = simconf.scoef[Z - 1];
    ls >> s.mm1 >> s.m1 >> s.mnat >> s.rho >> s.atrho >> s.vfermi >> s.heat >> s.lfctr;
    for (int j = 0; j < 8; ++j)
      ls >> s.pcoef[j];
    if (!ls)
      return false;
    ++rows;
  }
  return rows == 92;
}

static Element
element(int Z, double m, double t, double Edisp, double Elbind)
{
  Element e;
  e._Z = Z;
  e._m = m;
  e._t = t;
  e._Edisp = Edisp;
  e._Elbind = Elbind;
  return e;
}

static void
print(const char * label, const mtg_totals & t)
{
  std::printf("tot %s %lld %lld %lld %lld %lld %lld %lld %lld %a %a\n", label, t.primaries, t.members, t.collisions,
              t.vacancies, t.replacements, t.interstitials, t.substitutionals, t.lost, t.Eel, t.Enuc);
}

int
main(int argc, char ** argv)
{
  SimconfType simconf;
  if (argc < 2 || !read_tables(argv[1], simconf))
  {
    std::fprintf(stderr, "usage: trim_gpu_run <stopping_tables.tsv>\n");
    return 2;
  }
  // 10 nm SiO2 on bulk Si, CUT entrance surface (apps/runmytrim.C:121-283 builds the same objects)
  MaterialBase sio2(&simconf, 2.2), si(&simconf, 2.33), cu(&simconf, 8.96);
  sio2._element = {element(14, 28.086, 1.0, 15.0, 3.0), element(8, 15.999, 2.0, 28.0, 3.0)};
  si._element = {element(14, 28.086, 1.0, 15.0, 3.0)};
  cu._element = {element(29, 63.546, 1.0, 25.0, 3.0)};
  SampleLayers layers(1e9, 1e9, 1e9);
  layers.material = {&sio2, &si};
  layers.layerThickness = {100.0, 1e7};
  layers.bc[0] = SampleBase::CUT;
  layers.bc[1] = layers.bc[2] = SampleBase::INF;
  SampleSolid solid(1e7, 100.0, 100.0);
  solid.material = {&cu};

  IonBase boron;
  boron._Z = 5;
  boron._m = 11.009;
  boron._E = 10e3;
  boron._dir = Point(std::cos(7.0 * M_PI / 180.0), std::sin(7.0 * M_PI / 180.0), 0.0);
  boron._pos = Point(0.0, 0.0, 0.0);
  IonBase copper;
  copper._Z = 29;
  copper._m = 63.546;
  copper._E = 5e3;
  copper._Ef = 5.0;
  copper._dir = Point(1.0, 0.0, 0.0);
  copper._pos = Point(0.0, 50.0, 50.0);

  try
  {
    TrimGPU trim(&simconf, &layers, MTG_PREC_FP64);
    print("boron_primaries", trim.runPrimaries(&boron, 3000, 17));
    std::vector<TrimGPU::Job> jobs(2);
    jobs[0].sample = &layers;
    jobs[0].pka = &boron;
    jobs[0].n = 3000;
    jobs[1].sample = &solid;
    jobs[1].pka = &copper;
    jobs[1].n = 500;
    trim._potential = TrimBase::MOLIERE; // honoured per run, as the reference's TrimBase does
    std::vector<mtg_totals> t = trim.runBatch(jobs, 18);
    print("batch_boron_moliere", t[0]);
    print("batch_copper_moliere", t[1]);
  }
  catch (const std::exception & e)
  {
    std::fprintf(stderr, "trim_gpu_run: %s\n", e.what());
    return 1;
  }
  std::printf("simconf %d %a %a\n", simconf.vacancies_created, simconf.EelTotal, simconf.EnucTotal);
  return 0;
}
