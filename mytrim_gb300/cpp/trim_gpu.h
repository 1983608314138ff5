// trim_gpu.h -- C++ drop-in for MyTRIM's cascade engine on a GB300 GPU.
//
// Header-only; link with -lmytrim_gpu (mytrim_gb300/_lib/libmytrim_gpu.so).
//
// A reference user keeps building SimconfType, MaterialBase/Element,
// SampleSolid/SampleLayers and an IonBase template exactly as runmytrim does
// (apps/runmytrim.C:121-304) and replaces the per-primary loop
//     for each primary: seed; push; while queue: averages(); trim(ion, queue)
// (apps/runmytrim.C:71-93) by one call:
//     MyTRIM_NS::TrimGPU trim(&simconf, &sample);
//     mtg_totals t = trim.runPrimaries(&pka, n);
// which runs every primary's full cascade on the GPU and adds the totals to
// simconf.vacancies_created / EelTotal / EnucTotal like the reference's hooks do.
//
// The generic part (mtg::flatten_*, mtg::Context) only needs the reference's field
// names, so it works on the reference's classes and on any type that mirrors them.
// The TrimBase subclass is defined when the reference's trim.h is included first.
#pragma once

#include <cmath>
#include <stdexcept>
#include <string>
#include <vector>

#include "mytrim_gpu.h"

namespace mtg
{

// SimconfType::scoef (simconf.h:71-94) -> 92 mtg_scoef_row
template <class Simconf>
std::vector<mtg_scoef_row>
flatten_tables(const Simconf & simconf)
{
  std::vector<mtg_scoef_row> rows(MTG_SCOEF_ROWS);
  for (int i = 0; i < MTG_SCOEF_ROWS; ++i)
  {
    const auto & s = simconf.scoef[i];
    mtg_scoef_row & r = rows[i];
    r.mm1 = s.mm1;
    r.m1 = s.m1;
    r.mnat = s.mnat;
    r.rho = s.rho;
    r.atrho = s.atrho;
    r.vfermi = s.vfermi;
    r.heat = s.heat;
    r.lfctr = s.lfctr;
    for (int j = 0; j < 8; ++j)
      r.pcoef[j] = s.pcoef[j];
  }
  return rows;
}

// MaterialBase (material.h:34-75) before or after prepare(): rho and elements
template <class Material>
mtg_material
flatten_material(const Material & m)
{
  mtg_material o{};
  if (m._element.size() < 1 || m._element.size() > MTG_MAX_ELEMENTS)
    throw std::invalid_argument("TrimGPU: a material needs 1 to 4 elements");
  o.rho = m._rho;
  o.n_elements = int(m._element.size());
  for (int j = 0; j < o.n_elements; ++j)
  {
    const auto & e = m._element[j];
    o.elements[j] = mtg_element{e._Z, e._m, e._t, e._Edisp, e._Elbind};
  }
  return o;
}

// A sample with `material` (and, for SampleLayers, `layerThickness`), `w`, `bc`;
// thickness == nullptr means one material everywhere (SampleSolid).
template <class Sample>
mtg_sample
flatten_sample(const Sample & sample, const std::vector<double> * thickness)
{
  mtg_sample o{};
  const size_t n = sample.material.size();
  if (n < 1 || n > MTG_MAX_LAYERS)
    throw std::invalid_argument("TrimGPU: a sample needs 1 to 8 materials");
  if (thickness && thickness->size() < n)
    throw std::invalid_argument("TrimGPU: every layer needs a thickness");
  o.n_layers = thickness ? int(n) : 1;
  for (int k = 0; k < o.n_layers; ++k)
  {
    o.thickness[k] = thickness ? (*thickness)[k] : sample.w[0];
    o.material[k] = flatten_material(*sample.material[k]);
  }
  for (int i = 0; i < 3; ++i)
  {
    o.w[i] = sample.w[i];
    o.bc[i] = int(sample.bc[i]);
  }
  return o;
}

// IonBase template (ion.h:30-85)
template <class Ion>
mtg_ion
flatten_ion(const Ion & pka)
{
  mtg_ion o{};
  o.Z = pka._Z;
  o.m = pka._m;
  o.E = pka._E;
  o.Ef = pka._Ef;
  for (int i = 0; i < 3; ++i)
  {
    o.dir[i] = pka._dir(i);
    o.pos[i] = pka._pos(i);
  }
  return o;
}

// RAII owner of one engine context.
class Context
{
public:
  explicit Context(int device = 0)
  {
    mtg_status st = mtg_create(device, &_ctx);
    if (st != MTG_OK)
      throw std::runtime_error("mtg_create failed with status " + std::to_string(int(st)));
  }
  ~Context() { mtg_destroy(_ctx); }
  Context(const Context &) = delete;
  Context & operator=(const Context &) = delete;

  void check(mtg_status st) const
  {
    if (st != MTG_OK)
      throw std::runtime_error(std::string("mytrim_gpu: ") + mtg_last_error(_ctx));
  }
  mtg_ctx * get() const { return _ctx; }

private:
  mtg_ctx * _ctx = nullptr;
};

} // namespace mtg

#ifdef MYTRIM_TRIM_H
#include "sample_layers.h"
#include "sample_solid.h"
#include "sample_clusters.h"

namespace mtg
{

// sampleClusters (sample_clusters.h:30-57): material[0] the matrix, material[1] the
// clusters, the cluster centres and radii c[0..3][0..cn) interleaved into
// `storage` (which must outlive the call that reads the sample), the hash cells kn.
inline mtg_sample
flatten_clusters(const MyTRIM_NS::sampleClusters & sample, std::vector<double> & storage)
{
  if (sample.material.size() != 2)
    throw std::invalid_argument("TrimGPU: a cluster sample needs two materials (matrix, cluster)");
  mtg_sample o{};
  o.n_layers = 2;
  for (int k = 0; k < 2; ++k)
  {
    o.thickness[k] = sample.w[0];
    o.material[k] = flatten_material(*sample.material[k]);
  }
  for (int i = 0; i < 3; ++i)
  {
    o.w[i] = sample.w[i];
    o.bc[i] = int(sample.bc[i]);
    o.cluster_hash[i] = sample.kn[i];
  }
  storage.resize(4 * size_t(sample.cn));
  for (int l = 0; l < sample.cn; ++l)
    for (int i = 0; i < 4; ++i)
      storage[4 * size_t(l) + i] = sample.c[i][l];
  o.geometry = MTG_GEOM_CLUSTERS;
  o.n_clusters = sample.cn;
  o.clusters = storage.data();
  return o;
}

} // namespace mtg

namespace MyTRIM_NS
{

// TrimBase subclass that runs whole batches of primaries on the GPU.
// trim(ion, queue) stays the reference's host implementation (it is not
// virtual, trim.h:53); runPrimaries is the batched entry point.
class TrimGPU : public TrimBase
{
public:
  TrimGPU(SimconfType * simconf, SampleBase * sample, int precision = MTG_PREC_FP64, int device = 0)
    : TrimBase(simconf, sample), _ctx(device), _precision(precision)
  {
    std::vector<mtg_scoef_row> rows = mtg::flatten_tables(*simconf);
    _ctx.check(mtg_set_tables(_ctx.get(), rows.data(), int(rows.size())));
  }

  // Full cascades of n primaries cloned from `pka` (direction and position as
  // set on the template), tallied like TrimVacCount (or TrimRange with mode
  // MTG_TALLY_RANGE, TrimPrimaries / TrimRecoils with MTG_TALLY_PRIMARIES and
  // max_generation 1 / 2) with TrimPhononOut energy accounting, scattering in the
  // potential set in _potential.
  mtg_totals runPrimaries(IonBase * pka, long long n, unsigned long long seed = 1,
                          int mode = MTG_TALLY_VACCOUNT, bool primaries_only = false,
                          long long first_primary = 0, int max_generation = 1)
  {
    Job job{_sample, pka, n, mode, primaries_only, first_primary, max_generation};
    return runBatch(std::vector<Job>{job}, seed)[0];
  }

  // One simulation of a batch: its own sample, ion template and primaries.
  struct Job
  {
    SampleBase * sample;
    IonBase * pka;
    long long n;
    int mode = MTG_TALLY_VACCOUNT;
    bool primaries_only = false;
    long long first_primary = 0;
    int max_generation = 1;
  };

  // Several independent simulations in one launch (a parameter scan, many small
  // targets); totals in job order, each added to the SimconfType counters.
  std::vector<mtg_totals> runBatch(const std::vector<Job> & jobs, unsigned long long seed = 1)
  {
    mtg_config cfg{};
    cfg.tmin = _simconf->tmin;
    cfg.tau = _simconf->tau;
    cfg.cw = _simconf->cw;
    cfg.length_scale = _simconf->lengthScale();
    cfg.precision = _precision;
    cfg.seed = seed;
    _ctx.check(mtg_configure(_ctx.get(), &cfg));
    std::vector<mtg_sim> sims(jobs.size());
    std::vector<std::vector<double>> cluster_storage(jobs.size()); // read by mtg_run
    for (size_t i = 0; i < jobs.size(); ++i)
    {
      const Job & j = jobs[i];
      mtg_sim & sim = sims[i];
      sim = mtg_sim{};
      if (auto * layers = dynamic_cast<SampleLayers *>(j.sample))
        sim.sample = mtg::flatten_sample(*layers, &layers->layerThickness);
      else if (dynamic_cast<SampleSolid *>(j.sample))
        sim.sample = mtg::flatten_sample(*j.sample, nullptr);
      else if (auto * clusters = dynamic_cast<sampleClusters *>(j.sample))
        sim.sample = mtg::flatten_clusters(*clusters, cluster_storage[i]);
      else
        throw std::invalid_argument("TrimGPU supports SampleSolid, SampleLayers and sampleClusters");
      sim.ion = mtg::flatten_ion(*j.pka);
      sim.n_primaries = j.n;
      sim.first_primary = j.first_primary;
      sim.tally_mode = j.mode;
      sim.primaries_only = j.primaries_only ? 1 : 0;
      sim.max_generation = j.max_generation;
      sim.potential = int(_potential); // TrimBase's public member (trim.h:63-69)
    }
    std::vector<mtg_totals> t(jobs.size());
    _ctx.check(mtg_run(_ctx.get(), sims.data(), int(sims.size()), t.data(), nullptr));
    for (const mtg_totals & x : t)
    {
      _simconf->vacancies_created += int(x.vacancies);
      _simconf->EelTotal += x.Eel;
      _simconf->EnucTotal += x.Enuc;
    }
    return t;
  }

private:
  mtg::Context _ctx;
  int _precision;
};

} // namespace MyTRIM_NS
#endif
