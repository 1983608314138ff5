// Driver for the reference MyTRIM library, built from the reference's own sources
// by oracle/Makefile (test infrastructure: a checker and the timed CPU baseline,
// never part of the product).
//
// It replaces runmytrim (apps/runmytrim.C), which cannot be built here because
// jsoncpp is absent.  It keeps runmytrim's loop semantics exactly:
//   * master seed -> thread-0 stream -> 16-bit per-primary seed (runmytrim.C:288-302)
//   * per primary: reseed, FIFO queue, averages() then trim() per member
//     (runmytrim.C:71-93)
// Tallies are taken only through the reference's public virtual hooks
// (trim.h:72-84), with TrimVacCount / TrimRange / TrimPhononOut semantics
// (apps/src/TrimVacCount.C:32-54, apps/src/TrimRange.C:32-47, trim.C:504-527).
//
// Usage: ref_driver < spec      (spec format: oracle/runspec.h)

#include "runspec.h"

#include "simconf.h"
#include "element.h"
#include "material.h"
#include "sample_layers.h"
#include "sample_clusters.h"
#include "ion.h"
#include "trim.h"

#include <cmath>
#include <queue>
#include <chrono>

using namespace MyTRIM_NS;

// The tally hooks over a reference trim class: TrimBase, or TrimPrimaries /
// TrimRecoils (trim.h:113-133), whose own followRecoil and vacancyCreation then
// decide and count.
template <class Base>
class OracleTrimT : public Base
{
public:
  OracleTrimT(SimconfType * simconf, SampleBase * sample, const runspec::Spec & spec)
    : Base(simconf, sample), _spec(spec)
  {
    t.hist_range.assign(spec.hist_range_n, 0);
    t.hist_vac.assign(spec.hist_vac_n, 0);
    t.hist_repl.assign(spec.hist_vac_n, 0);
    t.spec = &spec;
    t.vox_depth.assign(spec.vox_n[0] > 0 ? spec.vox_n[0] : 0, 0.0);
  }

  runspec::Tally t;
  // per-primary accumulators
  long long p_vac = 0, p_coll = 0;
  double p_enuc = 0.0, p_eel = 0.0;
  double last_x = 0, last_y = 0, last_z = 0;
  int last_state = 0;

protected:
  using Base::_dee;
  using Base::_element;
  using Base::_pka;
  using Base::_recoil;
  using Base::_simconf;
  const runspec::Spec & _spec;

  bool followRecoil() override
  {
    // TrimPhononOut: the binding energy stays behind where a recoil branches off
    t.Enuc += _element->_Elbind;
    p_enuc += _element->_Elbind;
    t.deposit(_recoil->_pos(0), _recoil->_pos(1), _recoil->_pos(2), _element->_Elbind);
    bool follow = _spec.primaries_mode ? Base::followRecoil()
                  : _spec.range_mode   ? (_recoil->_gen < 1)
                                       : !_spec.primaries_only;
    if (!follow)
      t.Eunfollowed += _recoil->_E;
    return follow;
  }

  void vacancyCreation() override
  {
    if (_spec.primaries_mode)
    {
      // the reference class counts into vacancies_created (an int)
      const int before = _simconf->vacancies_created;
      Base::vacancyCreation();
      const long long add = (long long)_simconf->vacancies_created - before;
      t.vacancies += add;
      p_vac += add;
      return;
    }
    if (_spec.range_mode)
    {
      // TrimRange::vacancyCreation (apps/src/TrimRange.C:32-47); the reference adds
      // the double to an int, which truncates each increment
      const Real Ed = _element->_Edisp;
      const Real ed = 0.0115 * std::pow(_recoil->_Z, -7.0 / 3.0) * _recoil->_E;
      const Real kd = 0.1337 * std::pow(_recoil->_Z, 2.0 / 3.0) / std::sqrt(_recoil->_m);
      const Real g = 3.4008 * std::pow(ed, 1.0 / 6.0) + 0.40244 * std::pow(ed, 3.0 / 4.0) + ed;
      const Real Ev = _recoil->_E / (1.0 + kd * g);
      long long add = 0;
      if (Ev < Ed)
        add = 0;
      else if (Ev >= Ed / 0.4)
        add = (long long)(Ev * 0.4 / Ed);
      else
        add = 1;
      t.vacancies += add;
      p_vac += add;
      return;
    }
    t.vacancies++;
    p_vac++;
    int b = runspec::bin_of(_recoil->_pos(0), _spec.hist_vac_bin, _spec.hist_vac_n);
    if (b >= 0)
      t.hist_vac[b]++;
  }

  void replacementCollision() override
  {
    t.replacements++;
    int b = runspec::bin_of(_recoil->_pos(0), _spec.hist_vac_bin, _spec.hist_vac_n);
    if (b >= 0)
      t.hist_repl[b]++;
  }

  void dissipateRecoilEnergy() override
  {
    const double e = _recoil->_E + _element->_Elbind;
    t.Enuc += e;
    p_enuc += e;
    t.deposit(_recoil->_pos(0), _recoil->_pos(1), _recoil->_pos(2), e);
  }

  void checkPKAState() override
  {
    t.collisions++;
    p_coll++;
    p_eel += _dee; // electronic loss of this collision, after the clamp (trim.C:277-289)
    // deposited where the flight path started: the recoil's position (trim.C:306)
    t.deposit(_recoil->_pos(0), _recoil->_pos(1), _recoil->_pos(2), _dee);
    const int st = _pka->_state;
    if (st == IonBase::MOVING)
      return;
    last_state = st;
    if (st == IonBase::LOST)
    {
      t.lost++;
      // the projectile's energy and the recoil dropped with it (trim.C:357) leave the sample
      t.Elost += _pka->_E + (_recoil->_E + _element->_Elbind);
      t.exit_surface(_pka->_pos(0), _pka->_gen, _pka->_E, _pka->_dir(0));
      return;
    }
    t.Enuc += _pka->_E;
    p_enuc += _pka->_E;
    t.deposit(_pka->_pos(0), _pka->_pos(1), _pka->_pos(2), _pka->_E);
    if (st == IonBase::INTERSTITIAL)
      t.interstitials++;
    else if (st == IonBase::SUBSTITUTIONAL)
      t.substitutionals++;
    if (_pka->_gen == 0)
    {
      const double x = _pka->_pos(0), y = _pka->_pos(1), z = _pka->_pos(2);
      last_x = x;
      last_y = y;
      last_z = z;
      t.range_n++;
      t.sx += x;
      t.sxx += x * x;
      t.sy += y;
      t.syy += y * y;
      t.sz += z;
      t.szz += z * z;
      int b = runspec::bin_of(x, _spec.hist_range_bin, _spec.hist_range_n);
      if (b >= 0)
        t.hist_range[b]++;
    }
  }
};

// runmytrim's loop (runmytrim.C:71-93, 288-302) over one trim class
template <class Trim>
int
run_with(SimconfType & simconf, SampleBase & sample, const runspec::Spec & spec)
{
  Trim trim(&simconf, &sample, spec);
  trim._potential = typename Trim::Potential(spec.potential); // the public member (trim.h:63-69)

  // per-primary seeds from the master stream, as runmytrim.C:288-302 does
  simconf.seed(spec.seed);
  std::vector<unsigned int> seeds(spec.count);
  for (long long i = 0; i < spec.count; ++i)
    seeds[i] = simconf.irand();

  auto t0 = std::chrono::steady_clock::now();
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

    trim.p_vac = 0;
    trim.p_eel = 0.0;
    trim.p_coll = 0;
    trim.p_enuc = 0.0;
    long long members = 0;

    recoils.push(pka);
    while (!recoils.empty())
    {
      IonBase * ion = recoils.front();
      recoils.pop();
      sample.averages(ion);
      trim.trim(ion, recoils);
      ++members;
      delete ion;
    }
    const double p_eel = trim.p_eel;
    trim.t.primaries++;
    trim.t.members += members;
    trim.t.vac_s2 += double(trim.p_vac) * double(trim.p_vac);
    trim.t.eel_s2 += p_eel * p_eel;
    trim.t.enuc_s2 += trim.p_enuc * trim.p_enuc;
    trim.t.coll_s2 += double(trim.p_coll) * double(trim.p_coll);
    if (n - spec.first < spec.records)
    {
      runspec::Record r{n,           members,     trim.p_coll, trim.p_vac, p_eel, trim.p_enuc,
                        trim.last_x, trim.last_y, trim.last_z, trim.last_state};
      runspec::print_record(stdout, r);
    }
  }
  auto t1 = std::chrono::steady_clock::now();
  trim.t.Eel = simconf.EelTotal;
  trim.t.print(stdout);
  printf("wall_s %.6f\n", std::chrono::duration<double>(t1 - t0).count());
  return 0;
}

int
main()
{
  runspec::Spec spec;
  std::string err;
  if (!runspec::parse(std::cin, spec, err))
  {
    fprintf(stderr, "ref_driver: %s\n", err.c_str());
    return 2;
  }
  if (spec.philox)
  {
    fprintf(stderr, "ref_driver: the reference library only has mt19937 streams\n");
    return 2;
  }

  SimconfType simconf;
  simconf.fullTraj = false;
  simconf.tmin = 0.2;
  simconf.setLengthScale(spec.scale);

  // SampleLayers, or sampleClusters with the spec's clusters (material 0 the
  // matrix, material 1 the clusters)
  SampleLayers layers(spec.size[0], spec.size[1], spec.size[2]);
  sampleClusters clusters(spec.size[0], spec.size[1], spec.size[2]);
  SampleBase & sample = spec.clusters ? static_cast<SampleBase &>(clusters) : static_cast<SampleBase &>(layers);
  for (int i = 0; i < 3; ++i)
    sample.bc[i] = SampleBase::sampleBoundary(spec.bc[i]);
  if (spec.clusters)
  {
    clusters.initSpatialhash(spec.kn[0], spec.kn[1], spec.kn[2]);
    for (size_t l = 0; l + 3 < spec.cl.size(); l += 4)
      clusters.addCluster(spec.cl[l], spec.cl[l + 1], spec.cl[l + 2], spec.cl[l + 3]);
  }
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
    layers.layerThickness.push_back(l.thickness);
  }

  if (!spec.primaries_mode)
    return run_with<OracleTrimT<TrimBase>>(simconf, sample, spec);
  if (spec.max_gen == 1)
    return run_with<OracleTrimT<TrimPrimaries>>(simconf, sample, spec);
  if (spec.max_gen == 2)
    return run_with<OracleTrimT<TrimRecoils>>(simconf, sample, spec);
  fprintf(stderr, "ref_driver: the reference has TrimPrimaries (1) and TrimRecoils (2) only\n");
  return 2;
}
