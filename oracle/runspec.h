// Run description shared by the two CPU oracles (test infrastructure only).
//
// A run spec is a small line-oriented text format written by the Python test
// harness; it carries exactly what the reference's runmytrim JSON carries
// (apps/runmytrim.C:103-285) plus the extensions the workloads need (tilted
// incidence, CUT boundaries, generation cut, histogram binning, primary subsets).
//
//   seed <uint>                 master seed (runmytrim "options.seed")
//   seeding compat|philox       compat: per-primary 16-bit mt19937 seeds drawn from
//                               the master stream (runmytrim.C:288-302);
//                               philox: counter-based streams keyed like the GPU
//   ion <Z> <mass> <E_eV> <count> [<Ef_eV>]
//   dir <x> <y> <z>             initial direction (runmytrim hard-codes 1 0 0)
//   pos <x> <y> <z>             start position (default 0, w1/2, w2/2)
//   size <wx> <wy> <wz>         sample box (runmytrim: total thickness, 100, 100)
//   bc <b0> <b1> <b2>           0 = PBC, 1 = INF, 2 = CUT (sample.h:49-54)
//   scale <l>                   length scale (simconf.C:75-80)
//   layer <thickness> <rho>     appends a layer
//   element <Z> <mass> <fraction> [<Edisp> <Elbind>]   appends to the last layer
//   mode vaccount|range|primaries [<maxgen>]
//                               vaccount: TrimVacCount; range: TrimRange (KP, gen cut);
//                               primaries: TrimPrimaries (maxgen 1) / TrimRecoils (2)
//   primaries_only 0|1          ThreadedTrimBase::_primaries_only
//   potential 0|1|2             TrimBase::_potential: universal, Moliere, C-Kr (trim.h:63-69)
//   hist_range <bin_A> <nbins>  histogram of primary stopping depth
//   hist_vac <bin_A> <nbins>    histogram of vacancy depth (TrimVacCount bins are 1 A)
//   subset <first> <count>      run primaries [first, first+count)
//   events <mask>               print an "ev" line per event of the kinds whose bit
//                               (1 << kind) is set, with the fields of the GPU event
//                               log (mtg_event): 1 vacancy, 2 replacement, 3 followRecoil
//                               branch, 4 dissipated recoil, 5 rest, 6 lost, 7 history
//   mdtag <Z> <Emin> <Emax>     IonMDTag::_md as the demo programs set it: a member of
//                               atomic number Z starting with Emin < E < Emax has _md 1
//                               (apps/mytrim_solid.C:156-159), reported in the "ev" lines
//   sim <index>                 simulation index of the member keys (philox seeding):
//                               the keys the GPU gives simulation <index> of a batch
//   records <n>                 emit per-primary records for the first n primaries
//   sputter <Esurf>             count recoils leaving through x < 0 with E cos^2 > Esurf
//   voxels nx ny nz ox oy oz sx sy sz   energy-deposition voxel box (depth profile reported)
//   clusters <kx> <ky> <kz>     sampleClusters geometry (sample_clusters.C): the first
//                               layer is the matrix, the second the cluster material;
//                               kx ky kz spatial-hash cells (initSpatialhash)
//   cluster <x> <y> <z> <r>     appends a spherical cluster (addCluster)
//   output <type> <base>        write runmytrim's output file for type vaccount,
//                               vacenergycount or range as <base>_vac.dat, _evac.dat
//                               or _ranges.dat (runmytrim.C:185-206, 309)
#pragma once

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cmath>
#include <algorithm>
#include <string>
#include <vector>
#include <sstream>
#include <fstream>
#include <iostream>

namespace runspec
{

struct ElementSpec
{
  int Z;
  double m, t, Edisp, Elbind;
};

struct LayerSpec
{
  double thickness, rho;
  std::vector<ElementSpec> el;
};

struct Spec
{
  unsigned int seed = 1;
  bool philox = false;
  int Z = 29;
  double m = 63.546, E = 1000.0, Ef = 3.0;
  long long count = 1;
  double dir[3] = {1.0, 0.0, 0.0};
  bool have_pos = false;
  double pos[3] = {0.0, 0.0, 0.0};
  bool have_size = false;
  double size[3] = {0.0, 100.0, 100.0};
  int bc[3] = {0, 0, 0};
  double scale = 1.0;
  std::vector<LayerSpec> layers;
  bool range_mode = false;
  bool primaries_mode = false; // TrimPrimaries / TrimRecoils
  int max_gen = 1;
  bool primaries_only = false;
  int potential = 0;
  double hist_range_bin = 10.0;
  int hist_range_n = 0;
  double hist_vac_bin = 1.0;
  int hist_vac_n = 0;
  long long first = 0, n = -1;
  unsigned long long sim_index = 0;
  unsigned int event_mask = 0;
  int md_Z = 0;
  double md_Emin = 0.0, md_Emax = 0.0;
  int records = 0;
  double esurf = 0.0;
  int vox_n[3] = {0, 0, 0};
  double vox_o[3] = {0, 0, 0}, vox_s[3] = {0, 0, 0};
  std::string out_type, out_base;
  bool clusters = false;
  int kn[3] = {1, 1, 1};
  std::vector<double> cl; // x, y, z, r per cluster

  double total_thickness() const
  {
    double t = 0.0;
    for (auto & l : layers)
      t += l.thickness;
    return t;
  }
  void finalize()
  {
    if (!have_size)
    {
      size[0] = total_thickness();
      size[1] = 100.0;
      size[2] = 100.0;
    }
    if (!have_pos)
    {
      pos[0] = 0.0;
      pos[1] = size[1] / 2.0;
      pos[2] = size[2] / 2.0;
    }
    if (n < 0)
      n = count - first;
  }
};

inline bool
parse(std::istream & in, Spec & s, std::string & err)
{
  std::string line;
  int lineno = 0;
  while (std::getline(in, line))
  {
    ++lineno;
    auto hash = line.find('#');
    if (hash != std::string::npos)
      line.resize(hash);
    std::istringstream ls(line);
    std::string key;
    if (!(ls >> key))
      continue;
    bool ok = true;
    if (key == "seed")
      ok = bool(ls >> s.seed);
    else if (key == "seeding")
    {
      std::string v;
      ok = bool(ls >> v);
      s.philox = (v == "philox");
    }
    else if (key == "ion")
    {
      ok = bool(ls >> s.Z >> s.m >> s.E >> s.count);
      double ef;
      if (ok && (ls >> ef))
        s.Ef = ef;
    }
    else if (key == "dir")
      ok = bool(ls >> s.dir[0] >> s.dir[1] >> s.dir[2]);
    else if (key == "pos")
    {
      ok = bool(ls >> s.pos[0] >> s.pos[1] >> s.pos[2]);
      s.have_pos = true;
    }
    else if (key == "size")
    {
      ok = bool(ls >> s.size[0] >> s.size[1] >> s.size[2]);
      s.have_size = true;
    }
    else if (key == "bc")
      ok = bool(ls >> s.bc[0] >> s.bc[1] >> s.bc[2]);
    else if (key == "scale")
      ok = bool(ls >> s.scale);
    else if (key == "layer")
    {
      LayerSpec l;
      ok = bool(ls >> l.thickness >> l.rho);
      s.layers.push_back(l);
    }
    else if (key == "element")
    {
      ElementSpec e;
      e.Edisp = 25.0;
      e.Elbind = 3.0;
      ok = bool(ls >> e.Z >> e.m >> e.t) && !s.layers.empty();
      double ed, eb;
      if (ok && (ls >> ed >> eb))
      {
        e.Edisp = ed;
        e.Elbind = eb;
      }
      if (ok)
        s.layers.back().el.push_back(e);
    }
    else if (key == "mode")
    {
      std::string v;
      ok = bool(ls >> v);
      s.range_mode = (v == "range");
      s.primaries_mode = (v == "primaries");
      int g;
      if (s.primaries_mode && (ls >> g))
        s.max_gen = g;
    }
    else if (key == "primaries_only")
    {
      int v;
      ok = bool(ls >> v);
      s.primaries_only = v != 0;
    }
    else if (key == "potential")
      ok = bool(ls >> s.potential) && s.potential >= 0 && s.potential <= 2;
    else if (key == "hist_range")
      ok = bool(ls >> s.hist_range_bin >> s.hist_range_n);
    else if (key == "hist_vac")
      ok = bool(ls >> s.hist_vac_bin >> s.hist_vac_n);
    else if (key == "subset")
      ok = bool(ls >> s.first >> s.n);
    else if (key == "records")
      ok = bool(ls >> s.records);
    else if (key == "mdtag")
      ok = bool(ls >> s.md_Z >> s.md_Emin >> s.md_Emax);
    else if (key == "events")
      ok = bool(ls >> s.event_mask);
    else if (key == "sim")
      ok = bool(ls >> s.sim_index) && s.sim_index < (1ull << 23);
    else if (key == "sputter")
      ok = bool(ls >> s.esurf);
    else if (key == "clusters")
    {
      ok = bool(ls >> s.kn[0] >> s.kn[1] >> s.kn[2]) && s.kn[0] > 0 && s.kn[1] > 0 && s.kn[2] > 0;
      s.clusters = true;
    }
    else if (key == "cluster")
    {
      double v[4];
      ok = bool(ls >> v[0] >> v[1] >> v[2] >> v[3]);
      s.cl.insert(s.cl.end(), v, v + 4);
    }
    else if (key == "output")
      ok = bool(ls >> s.out_type >> s.out_base) &&
           (s.out_type == "vaccount" || s.out_type == "vacenergycount" || s.out_type == "range");
    else if (key == "voxels")
      ok = bool(ls >> s.vox_n[0] >> s.vox_n[1] >> s.vox_n[2] >> s.vox_o[0] >> s.vox_o[1] >> s.vox_o[2] >>
                s.vox_s[0] >> s.vox_s[1] >> s.vox_s[2]);
    else
    {
      err = "unknown key '" + key + "' on line " + std::to_string(lineno);
      return false;
    }
    if (!ok)
    {
      err = "bad value for '" + key + "' on line " + std::to_string(lineno);
      return false;
    }
  }
  if (s.layers.empty())
  {
    err = "no layers";
    return false;
  }
  for (auto & l : s.layers)
    if (l.el.empty())
    {
      err = "layer without elements";
      return false;
    }
  if (s.clusters && s.layers.size() != 2)
  {
    err = "a cluster sample needs two materials (matrix, cluster)";
    return false;
  }
  s.finalize();
  return true;
}

// The spatial hash of sampleClusters (sample_clusters.C:139-225): per cell the
// head of a linked list of clusters in insertion order.
struct ClusterHash
{
  int kn[3] = {1, 1, 1};
  double w[3] = {1, 1, 1}, kd[3] = {1, 1, 1}, cmr = 0.0;
  int bc[3] = {0, 0, 0};
  std::vector<double> c; // x, y, z, r
  std::vector<int> next, head;

  void build(const Spec & s)
  {
    for (int i = 0; i < 3; ++i)
    {
      kn[i] = s.kn[i];
      w[i] = s.size[i];
      bc[i] = s.bc[i];
      kd[i] = w[i] / double(kn[i]);
    }
    c = s.cl;
    const size_t n = c.size() / 4;
    next.assign(n, -1);
    head.assign(size_t(kn[0]) * kn[1] * kn[2], -1);
    std::vector<int> tail(head.size(), -1);
    cmr = 0.0;
    for (size_t l = 0; l < n; ++l)
    {
      int k[3];
      for (int i = 0; i < 3; ++i)
      {
        k[i] = int(std::floor((c[4 * l + i] * kn[i]) / w[i])) % kn[i];
        k[i] = k[i] < 0 ? k[i] + kn[i] : k[i];
      }
      const int cell = k[0] + kn[0] * (k[1] + kn[1] * k[2]);
      if (head[cell] < 0)
        head[cell] = int(l);
      else
        next[tail[cell]] = int(l);
      tail[cell] = int(l);
      if (c[4 * l + 3] > cmr)
        cmr = c[4 * l + 3];
    }
  }

  // sampleClusters::lookupCluster with dr = 0 (sample_clusters.C:60-130): the
  // cluster containing pos, -1 in the matrix, -2 outside a CUT boundary
  int lookup(const double pos[3]) const
  {
    int k[3], k1[3], k2[3];
    for (int i = 0; i < 3; ++i)
    {
      k[i] = int(std::floor((pos[i] * kn[i]) / w[i]));
      if (pos[i] < 0.0 || pos[i] >= w[i])
      {
        if (bc[i] == 2)
          return -2;
        if (bc[i] == 1)
          return -1;
        k[i] = k[i] % kn[i];
        if (k[i] < 0)
          k[i] += kn[i];
      }
      const int ks = int((cmr + 0.0) / kd[i]) + 1;
      k1[i] = k[i] - ks;
      k2[i] = k[i] + ks;
      if (k1[i] < 0 && bc[i] != 0)
        k1[i] = 0;
      if (k2[i] >= kn[i] && bc[i] != 0)
        k2[i] = kn[i] - 1;
    }
    int j[3];
    for (j[0] = k1[0]; j[0] <= k2[0]; ++j[0])
      for (j[1] = k1[1]; j[1] <= k2[1]; ++j[1])
        for (j[2] = k1[2]; j[2] <= k2[2]; ++j[2])
        {
          int m[3];
          for (int i = 0; i < 3; ++i)
          {
            m[i] = j[i] % kn[i];
            if (m[i] < 0)
              m[i] += kn[i];
          }
          for (int l = head[m[0] + kn[0] * (m[1] + kn[1] * m[2])]; l >= 0; l = next[l])
          {
            double dif[3];
            for (int i = 0; i < 3; ++i)
            {
              dif[i] = pos[i] - c[4 * l + i];
              if (bc[i] == 0)
                dif[i] -= std::round(dif[i] / w[i]) * w[i];
            }
            const double r2 = dif[0] * dif[0] + dif[1] * dif[1] + dif[2] * dif[2];
            const double rr = c[4 * l + 3] + 0.0;
            if (r2 < rr * rr)
              return l;
          }
        }
    return -1;
  }
};

// Tallies reported by both oracles (one line per key on stdout).
struct Tally
{
  long long primaries = 0, members = 0, collisions = 0;
  long long vacancies = 0, replacements = 0, interstitials = 0, substitutionals = 0,
            lost = 0;
  double Eel = 0.0, Enuc = 0.0, Elost = 0.0, Eunfollowed = 0.0;
  // primary end points (generation 0, stopped inside the sample)
  long long range_n = 0;
  double sx = 0, sxx = 0, sy = 0, syy = 0, sz = 0, szz = 0;
  // per-primary moments for Monte Carlo error bars
  double vac_s2 = 0.0, eel_s2 = 0.0, enuc_s2 = 0.0, coll_s2 = 0.0;
  std::vector<long long> hist_range, hist_vac, hist_repl;
  // extensions: sputtering and energy-deposition voxels (depth profile over x cells)
  long long sputtered = 0, backscattered = 0;
  double Esputtered = 0.0, Evoxel = 0.0;
  std::vector<double> vox_depth;
  const Spec * spec = nullptr;

  void deposit(double x, double y, double z, double e)
  {
    if (!spec || spec->vox_n[0] <= 0)
      return;
    const double p[3] = {x, y, z};
    int ix[3];
    for (int i = 0; i < 3; ++i)
    {
      const double q = (p[i] - spec->vox_o[i]) * spec->vox_n[i] / spec->vox_s[i];
      if (!(q >= 0.0) || q >= spec->vox_n[i])
        return;
      ix[i] = int(q);
    }
    Evoxel += e;
    vox_depth[ix[0]] += e;
  }
  // a member lost through x < 0 with energy E and direction cosine dx
  void exit_surface(double x, int gen, double E, double dx)
  {
    if (!spec || !(x < 0.0) || spec->bc[0] != 2)
      return;
    if (gen == 0)
      ++backscattered;
    else if (spec->esurf > 0.0 && E * dx * dx > spec->esurf)
    {
      ++sputtered;
      Esputtered += E;
    }
  }

  void print(FILE * f) const
  {
    fprintf(f, "primaries %lld\nmembers %lld\ncollisions %lld\n", primaries, members, collisions);
    fprintf(f, "vacancies %lld\nreplacements %lld\ninterstitials %lld\n", vacancies,
            replacements, interstitials);
    fprintf(f, "substitutionals %lld\nlost %lld\n", substitutionals, lost);
    fprintf(f, "Eel %.17g\nEnuc %.17g\nElost %.17g\nEunfollowed %.17g\n", Eel, Enuc, Elost,
            Eunfollowed);
    fprintf(f, "range_n %lld\nsx %.17g\nsxx %.17g\nsy %.17g\nsyy %.17g\nsz %.17g\nszz %.17g\n",
            range_n, sx, sxx, sy, syy, sz, szz);
    fprintf(f, "vac_s2 %.17g\neel_s2 %.17g\nenuc_s2 %.17g\ncoll_s2 %.17g\n", vac_s2, eel_s2,
            enuc_s2, coll_s2);
    auto hist = [&](const char * name, const std::vector<long long> & h)
    {
      fprintf(f, "%s", name);
      for (auto v : h)
        fprintf(f, " %lld", v);
      fprintf(f, "\n");
    };
    hist("hist_range", hist_range);
    hist("hist_vac", hist_vac);
    hist("hist_repl", hist_repl);
    fprintf(f, "sputtered %lld\nbackscattered %lld\nEsputtered %.17g\nEvoxel %.17g\n", sputtered,
            backscattered, Esputtered, Evoxel);
    fprintf(f, "vox_depth");
    for (double v : vox_depth)
      fprintf(f, " %.17g", v);
    fprintf(f, "\n");
  }
};

// The tallies of runmytrim's three output plugins, grown on demand as the
// reference grows them, and their file writers: a restatement of
// apps/src/TrimVacCount.C:32-79, apps/src/TrimVacEnergyCount.C:32-81 and
// apps/src/TrimRange.C:49-121 (same bins, same text through std::ostream).
struct PluginOut
{
  std::string type, base;
  std::vector<unsigned int> vac, repl;          // by int(x) of the recoil
  std::vector<std::vector<unsigned int>> evac;  // by int(ln E) of the recoil, then int(x)
  std::vector<std::vector<double>> range = std::vector<std::vector<double>>(112); // x by recoil Z

  static void bump(std::vector<unsigned int> & h, int x)
  {
    if (x >= int(h.size()))
      h.resize(x + 1, 0);
    h[x]++;
  }
  // vacancyCreation of a TrimVacCount / TrimVacEnergyCount run
  void vacancy(double rx, double rE)
  {
    const int x = int(rx);
    if (x < 0)
      return;
    if (type == "vaccount")
      bump(vac, x);
    else if (type == "vacenergycount")
    {
      int e = int(std::log(rE));
      e = e < 0 ? 0 : e;
      if (e >= int(evac.size()))
        evac.resize(e + 1);
      bump(evac[e], x);
    }
  }
  // replacementCollision of a TrimVacCount run
  void replacement(double rx)
  {
    const int x = int(rx);
    if (type == "vaccount" && x >= 0)
      bump(repl, x);
  }
  // dissipateRecoilEnergy of a TrimRange run
  void dissipate(int Z, double rx)
  {
    if (type == "range" && Z >= 0 && Z < int(range.size()))
      range[Z].push_back(rx);
  }

  bool write() const
  {
    if (type == "vaccount")
    {
      const size_t n = std::max(vac.size(), repl.size());
      std::ofstream out(base + "_vac.dat");
      for (size_t x = 0; x < n; ++x)
        out << x << ' ' << (x < vac.size() ? vac[x] : 0u) << ' ' << (x < repl.size() ? repl[x] : 0u) << '\n';
      return bool(out);
    }
    if (type == "vacenergycount")
    {
      std::ofstream out(base + "_evac.dat");
      for (size_t e = 0; e < evac.size(); ++e)
      {
        for (size_t x = 0; x < evac[e].size(); ++x)
          out << e << ' ' << x << ' ' << evac[e][x] << '\n';
        out << '\n';
      }
      return bool(out);
    }
    if (type == "range")
    {
      // histogram extent and bin width as TrimRange::writeOutput chooses them
      unsigned int max_samples = 0;
      double x_min = 0.0, x_max = 0.0;
      for (auto & r : range)
      {
        if (r.size() > max_samples)
          max_samples = (unsigned int)r.size();
        for (double x : r)
        {
          x_min = std::min(x_min, x);
          x_max = std::max(x_max, x);
        }
      }
      std::ofstream out(base + "_ranges.dat");
      out << "#x";
      for (size_t Z = 0; Z < range.size(); ++Z)
        if (!range[Z].empty())
          out << " Z" << Z;
      out << '\n';
      const double xwidth = x_max - x_min;
      if (max_samples == 0 || !(xwidth > 0.0))
        return bool(out); // no extent: header only
      const double bin = std::min(xwidth * 100.0 / max_samples, xwidth / 10.0);
      const unsigned int nbin = (unsigned int)(xwidth / bin + 1);
      std::vector<std::vector<unsigned int>> h;
      for (auto & r : range)
      {
        if (r.empty())
          continue;
        h.emplace_back(nbin, 0u);
        for (double x : r)
          h.back()[(size_t)std::floor((x - x_min) / bin)]++;
      }
      for (unsigned int n = 0; n < nbin; ++n)
      {
        out << (n * bin + x_min);
        for (auto & c : h)
          out << ' ' << c[n];
        out << '\n';
      }
      return bool(out);
    }
    return true;
  }
};

// Per-primary record (emitted for the first `records` primaries).
struct Record
{
  long long index, members, collisions, vacancies;
  double Eel, Enuc, x, y, z;
  int state;
};

inline void
print_record(FILE * f, const Record & r)
{
  fprintf(f, "rec %lld %lld %lld %lld %.17g %.17g %.17g %.17g %.17g %d\n", r.index, r.members,
          r.collisions, r.vacancies, r.Eel, r.Enuc, r.x, r.y, r.z, r.state);
}

inline int
bin_of(double x, double width, int n)
{
  // truncation toward zero like the reference's int(x) (TrimVacCount.C:36-39):
  // depths in (-1 bin, 0) land in bin 0, smaller ones are dropped
  double q = x / width;
  if (n <= 0 || !(q > -1.0) || q >= double(n))
    return -1;
  return int(q);
}

} // namespace runspec
