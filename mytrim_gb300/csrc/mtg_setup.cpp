// Host-side table construction for the cascade engine (see mtg_setup.h).
#include "mtg_setup.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <unordered_map>

namespace mtg
{

void
seed_key(unsigned long long seed, uint32_t & k0, uint32_t & k1)
{
  k0 = uint32_t(seed);
  k1 = uint32_t(seed >> 32) ^ 0x4D795452u;
}

bool
read_table_file(const char * path, mtg_scoef_row * rows, std::string & err)
{
  std::ifstream in(path);
  if (!in)
  {
    err = std::string("cannot open stopping table file ") + path;
    return false;
  }
  std::string line;
  bool seen[MTG_SCOEF_ROWS] = {false};
  int n = 0;
  while (std::getline(in, line))
  {
    if (line.empty() || line[0] == '#')
      continue;
    std::istringstream ls(line);
    int Z;
    std::string sym;
    mtg_scoef_row r;
    ls >> Z >> sym >> r.mm1 >> r.m1 >> r.mnat >> r.rho >> r.atrho >> r.vfermi >> r.heat >> r.lfctr;
    for (int j = 0; j < 8; ++j)
      ls >> r.pcoef[j];
    if (!ls || Z < 1 || Z > MTG_SCOEF_ROWS || seen[Z - 1])
    {
      err = std::string("malformed stopping table row: ") + line;
      return false;
    }
    rows[Z - 1] = r;
    seen[Z - 1] = true;
    ++n;
  }
  if (n != MTG_SCOEF_ROWS)
  {
    err = "stopping table file must hold 92 rows";
    return false;
  }
  return true;
}

// proton stopping with libm (material.C:134-158), used for the constant
// low-velocity matching value
static double
proton_stop_host(const mtg_scoef_row & r, int z2p, double e)
{
  const double pe0 = 25.0;
  const double pe = std::max(pe0, e);
  const double sl = (r.pcoef[0] * std::pow(pe, r.pcoef[1])) + (r.pcoef[2] * std::pow(pe, r.pcoef[3]));
  const double sh = r.pcoef[4] / std::pow(pe, r.pcoef[5]) * std::log(r.pcoef[6] / pe + r.pcoef[7] * pe);
  double sp = sl * sh / (sl + sh);
  if (e <= pe0)
    sp *= std::pow(e / pe0, z2p <= 6 ? 0.25 : 0.45);
  return sp;
}

SpeciesConst
make_species(const mtg_scoef_row * rows, int Z1, double m1)
{
  SpeciesConst s;
  std::memset(&s, 0, sizeof s);
  s.Z1 = Z1;
  s.branch = Z1 == 1 ? STOP_H : (Z1 == 2 ? STOP_HE : STOP_HEAVY);
  s.m1 = m1;
  const double mstop = (m1 == 0.0) ? rows[Z1 - 1].mm1 : m1;
  s.inv_m1k = 0.001 / mstop;
  s.fz1 = double(Z1);
  s.cb = std::cbrt(s.fz1);
  s.cb2 = s.cb * s.cb;
  s.lfctr = rows[Z1 - 1].lfctr;
  s.bq = (std::min(0.43, std::max(0.32, 0.12 + 0.025 * s.fz1))) / s.cb;
  s.l0a = std::min(1.2, 0.6 + s.fz1 / 30.0);
  s.qlo = std::max(0.0, 0.9 - 0.025 * s.fz1);
  s.qden = std::abs(s.qlo - 0.2000001);
  s.qhi = std::max(0.0, 1.0 - 0.025 * std::min(16.0, s.fz1));
  s.qden2 = 0.025 * std::min(16.0, s.fz1);
  s.inv_z1sq = 1.0 / (s.fz1 * s.fz1);
  return s;
}

StopPair
make_stop_pair(const mtg_scoef_row * rows, const SpeciesConst & sc, int Z2)
{
  StopPair p;
  std::memset(&p, 0, sizeof p);
  const mtg_scoef_row & r = rows[Z2 - 1];
  for (int j = 0; j < 8; ++j)
    p.pcoef[j] = r.pcoef[j];
  p.vfermi = r.vfermi;
  p.inv2vf2 = 1.0 / (2.0 * r.vfermi * r.vfermi);
  p.velpwr = Z2 <= 6 ? 0.25 : 0.45;
  // heavy-ion low-velocity branch (material.C:251-268)
  const double yrmin = 0.13, vrmin0 = 1.0;
  p.yrcut = std::max(yrmin, vrmin0 / sc.cb2);
  const double vrmin = std::max(vrmin0, yrmin * sc.cb2);
  const double vmin = 0.5 * (vrmin + std::sqrt(std::max(0.0, vrmin * vrmin - 0.8 * r.vfermi * r.vfermi)));
  p.eee = 25.0 * vmin * vmin;
  p.sp_eee = proton_stop_host(r, Z2, p.eee);
  p.power = (Z2 == 6 || ((Z2 == 14 || Z2 == 32) && sc.Z1 <= 19)) ? 0.375 : 0.5;
  p.zc = 0.18 + 0.0015 * double(Z2);
  p.hez = 0.007 + 0.00005 * double(Z2);
  p.Z2 = Z2;
  return p;
}

int
make_material(const mtg_scoef_row * rows, const SpeciesConst & sc, const mtg_material & m,
              double tmin, MatConst & mc, std::string & err)
{
  std::memset(&mc, 0, sizeof mc);
  if (m.n_elements < 1 || m.n_elements > MAX_EL)
  {
    err = "a material needs 1 to 4 elements";
    return MTG_ERR_BAD_INPUT;
  }
  if (!(m.rho > 0.0))
  {
    err = "material density must be positive";
    return MTG_ERR_BAD_INPUT;
  }
  // MaterialBase::prepare (material.C:37-74)
  double t[MAX_EL];
  double tt = 0.0;
  for (int i = 0; i < m.n_elements; ++i)
  {
    const mtg_element & e = m.elements[i];
    if (e.Z < 1 || e.Z > MTG_SCOEF_ROWS || !(e.m > 0.0))
    {
      err = "element Z must be 1..92 and its mass positive";
      return MTG_ERR_BAD_INPUT;
    }
    t[i] = e.t < 0.0 ? 0.0 : e.t;
    tt += t[i];
  }
  if (!(tt > 0.0))
  {
    err = "stoichiometry invalid, all elements zero";
    return MTG_ERR_BAD_INPUT;
  }
  for (int i = 0; i < m.n_elements; ++i)
    t[i] /= tt;
  double am = 0.0, az = 0.0;
  for (int i = 0; i < m.n_elements; ++i)
  {
    am += m.elements[i].m * t[i];
    az += double(m.elements[i].Z) * t[i];
  }
  mc.am = am;
  mc.az = az;
  mc.arho = m.rho * 0.6022 / am;
  mc.nel = m.n_elements;

  // MaterialBase::average (material.C:78-110)
  const double m1 = sc.m1;
  const double mu = m1 / am;
  const double fZ = sc.fz1;
  const double fZ023 = std::pow(fZ, 0.23);
  mc.a = .5292 * .8853 / (fZ023 + std::pow(az, 0.23));
  mc.f = mc.a * am / (az * fZ * 14.4 * (m1 + am));
  mc.epsdg = tmin * mc.f * ((1.0 + mu) * (1.0 + mu)) / (4.0 * mu);
  for (int i = 0; i < m.n_elements; ++i)
  {
    const mtg_element & e = m.elements[i];
    ElemConst & ec = mc.el[i];
    ec.t = t[i];
    ec.my = m1 / e.m;
    ec.ec = 4.0 * ec.my / ((1.0 + ec.my) * (1.0 + ec.my));
    ec.ai = .5292 * .8853 / (fZ023 + std::pow(e.Z, 0.23));
    ec.fi = ec.ai * e.m / (fZ * double(e.Z) * 14.4 * (m1 + e.m));
    ec.Edisp = e.Edisp;
    ec.Elbind = e.Elbind;
    ec.m2 = e.m;
    ec.maz = az;
    ec.mam = am;
    ec.Z2 = e.Z;
    ec.rspecies = -1;
    mc.sp[i] = make_stop_pair(rows, sc, e.Z);
  }
  return MTG_OK;
}

void
patch_cluster_pointers(std::vector<SimDesc> & sims, const Cl4d * cl, const int * next, const int * head,
                       const uint32_t * mask)
{
  for (SimDesc & d : sims)
  {
    d.cl = d.geometry == 1 && cl ? cl + d.cl_base : nullptr;
    d.cl_next = d.geometry == 1 && next ? next + d.cl_base : nullptr;
    d.cl_head = d.geometry == 1 && head ? head + d.cell_base : nullptr;
    d.cl_mask = d.geometry == 1 && mask ? mask + d.mask_base : nullptr;
  }
}

void
build_fp32_tables(const HostTables & t, std::vector<Species32> & species, std::vector<Mat32> & mats,
                  std::vector<Sim32> & sims)
{
  species.resize(t.species.size());
  for (size_t i = 0; i < t.species.size(); ++i)
  {
    std::memset(&species[i], 0, sizeof(Species32));
    species[i].m1 = float(t.species[i].m1);
    species[i].two_m1 = float(2.0 * t.species[i].m1);
    species[i].Z1 = t.species[i].Z1;
  }
  mats.resize(t.mats.size());
  for (size_t i = 0; i < t.mats.size(); ++i)
  {
    const MatConst & m = t.mats[i];
    Mat32 & o = mats[i];
    std::memset(&o, 0, sizeof o);
    o.a = float(m.a);
    o.f = float(m.f);
    o.epsdg = float(m.epsdg);
    o.inv_pi_arho = float(1.0 / (3.14159265358979323846 * m.arho));
    o.nel = m.nel;
    o.row = m.row;
    for (int j = 0; j < m.nel; ++j)
    {
      const ElemConst & e = m.el[j];
      Elem32 & f = o.el[j];
      f.t = float(e.t);
      f.my = float(e.my);
      f.ec = float(e.ec);
      f.inv_ai = float(1.0 / e.ai);
      f.fi = float(e.fi);
      f.Edisp = float(e.Edisp);
      f.Elbind = float(e.Elbind);
      f.m2 = float(e.m2);
      f.disp_thresh = float(e.Edisp - e.Elbind);
      f.maz = float(e.maz);
      f.mam = float(e.mam);
      f.Z2 = e.Z2;
      f.rspecies = e.rspecies;
    }
  }
  sims.resize(t.sims.size());
  for (size_t i = 0; i < t.sims.size(); ++i)
  {
    const SimDesc & d = t.sims[i];
    Sim32 & o = sims[i];
    std::memset(&o, 0, sizeof o);
    for (int k = 0; k < MAX_LAYERS; ++k)
    {
      o.layer_end[k] = float(d.layer_end[k]);
      o.layer_mat[k] = d.layer_mat[k];
    }
    for (int k = 0; k < 3; ++k)
    {
      o.w[k] = float(d.w[k]);
      o.bc[k] = d.bc[k];
      o.any_cut |= d.bc[k] == 2;
    }
    o.n_layers = d.n_layers;
    o.n_mat = d.n_mat;
    o.mat_base = d.mat_base;
    o.species_base = d.species_base;
    o.Ef = float(d.Ef);
    o.flscale = float(d.invscale);
    o.tau = float(d.tau);
    o.cw = float(d.cw);
    o.range_mode = d.range_mode;
    o.primaries_only = d.primaries_only;
    o.follow_gen = d.follow_gen;
    o.kp_gen = d.kp_gen;
    o.potential = d.potential;
    o.geometry = d.geometry;
    o.n_clusters = d.n_clusters;
    for (int k = 0; k < 3; ++k)
    {
      o.kn[k] = d.kn[k];
      o.kd[k] = float(d.kd[k]);
      o.mn[k] = d.mn[k];
      o.inv_mcell[k] = float(d.inv_mcell[k]);
    }
    o.cmr = float(d.cmr);
    // cluster pointers: set where the device copies are made
  }
}

// Expected cascade members per primary, for the launch heuristics only: one plus
// the Norgett-Robinson-Torrens displacement estimate 0.8 T_dam / (2 E_d), with the
// damage energy T_dam from Lindhard's partition in Robinson's fit (M. J. Norgett,
// M. T. Robinson, I. M. Torrens, Nucl. Eng. Des. 33 (1975) 50), evaluated against
// the first layer's fraction-weighted mean target atom.
static double
expected_members(const mtg_sim & s)
{
  if (s.tally_mode == MTG_TALLY_RANGE || s.primaries_only ||
      (s.tally_mode == MTG_TALLY_PRIMARIES && s.max_generation <= 1))
    return 1.0;
  const mtg_material & m = s.sample.material[0];
  double tt = 0.0, Z2 = 0.0, M2 = 0.0, Ed = 0.0;
  for (int j = 0; j < m.n_elements; ++j)
  {
    const double t = std::max(m.elements[j].t, 0.0);
    tt += t;
    Z2 += t * m.elements[j].Z;
    M2 += t * m.elements[j].m;
    Ed += t * m.elements[j].Edisp;
  }
  if (!(tt > 0.0) || !(Ed > 0.0))
    return 1.0;
  Z2 /= tt;
  M2 /= tt;
  Ed /= tt;
  const double Z1 = s.ion.Z, M1 = s.ion.m, E = s.ion.E;
  const double EL = 30.724 * Z1 * Z2 * std::sqrt(std::pow(Z1, 2.0 / 3.0) + std::pow(Z2, 2.0 / 3.0)) * (M1 + M2) / M2;
  const double eps = E / EL;
  const double k = 0.1337 * std::pow(Z1, 1.0 / 6.0) * std::sqrt(Z1 / M1);
  const double g = 3.4008 * std::pow(eps, 1.0 / 6.0) + 0.40244 * std::pow(eps, 0.75) + eps;
  const double Tdam = E / (1.0 + k * g);
  return 1.0 + std::max(0.0, 0.8 * Tdam / (2.0 * Ed));
}

// Candidate lists of a cluster sample.  A grid of mn cells per axis with edge about
// max(cmr / 2, w / 1024), coarser where it would pass 2^22 cells; for each cell the
// clusters whose sphere, its radius grown by a margin of max(w) / 1024, reaches into
// the cell (periodic images on PBC axes).  The margin covers the rounding of a
// position wrapped into the box and of the distance test in single precision
// (positions within 64 box lengths), so every cluster containing a point of a cell
// is among the cell's candidates.  A cell is marked for the hash search when two of
// its candidates come closer than their radii and two margins (a point could lie in
// both, and which one the search meets first decides the answer; minimum-image
// distances on PBC axes), when it has more than 16 candidates, or when a candidate
// is one the search may not see from every point of its sphere: a cluster centred
// outside the box on a CUT or INF axis (its hash cell is the wrapped one, outside
// the clamped window of the points near it) or one whose sphere and two margins
// span more hash cells than the search window reaches.  Elsewhere at most one
// candidate contains any point, and the search finds it: the cluster it returns.
// Layout from mask_base in the run's words: mn0 mn1 mn2 + 1 cell starts (relative
// to mask_base; bit 31 marks the cell for the search), then the candidates'
// indexes.  Above 2^26 candidates the lists are left out: a cell then holds none and
// is marked when any cluster reaches it (an occupancy mask).
#ifndef MTG_CELL_MAX_ITEMS
#define MTG_CELL_MAX_ITEMS (1LL << 26)
#endif
static void
build_cluster_cells(SimDesc & d, const mtg_sample & smp, std::vector<uint32_t> & words)
{
  constexpr double MAX_CELLS = double(1 << 22);
  constexpr long long MAX_ITEMS = MTG_CELL_MAX_ITEMS; // cells + candidates; lists are left out above
  constexpr uint32_t SEARCH = 0x80000000u;
  constexpr int MAX_CANDIDATES = 16;
  const double wmax = std::max(smp.w[0], std::max(smp.w[1], smp.w[2]));
  double g = std::max(d.cmr * 0.5, wmax / 1024.0);
  g = std::max(g, std::cbrt(smp.w[0] * smp.w[1] * smp.w[2] / MAX_CELLS));
  double cell[3];
  long long ncell = 1;
  for (int i = 0; i < 3; ++i)
  {
    d.mn[i] = int(std::min(512.0, std::max(1.0, std::ceil(smp.w[i] / g))));
    cell[i] = smp.w[i] / d.mn[i];
    d.inv_mcell[i] = double(d.mn[i]) / smp.w[i];
    ncell *= d.mn[i];
  }
  const double margin = wmax / 1024.0;
  // the cells cluster l reaches, in the occupancy test of the grown sphere
  auto for_each_cell = [&](long long l, auto && fn) {
    const double * c = smp.clusters + 4 * l;
    const double R = c[3] + margin;
    long long lo[3], hi[3];
    bool full[3] = {false, false, false};
    for (int i = 0; i < 3; ++i)
    {
      lo[i] = (long long)std::floor((c[i] - R) * d.inv_mcell[i]);
      hi[i] = (long long)std::floor((c[i] + R) * d.inv_mcell[i]);
      if (smp.bc[i] == MTG_BC_PBC)
      {
        if (hi[i] - lo[i] >= d.mn[i]) // the sphere spans the box: some image reaches every cell
        {
          lo[i] = 0;
          hi[i] = d.mn[i] - 1;
          full[i] = true;
        }
      }
      else
      {
        lo[i] = std::max<long long>(lo[i], 0);
        hi[i] = std::min<long long>(hi[i], d.mn[i] - 1);
        if (lo[i] > hi[i])
          return;
      }
    }
    for (long long j2 = lo[2]; j2 <= hi[2]; ++j2)
      for (long long j1 = lo[1]; j1 <= hi[1]; ++j1)
        for (long long j0 = lo[0]; j0 <= hi[0]; ++j0)
        {
          const long long j[3] = {j0, j1, j2};
          double d2 = 0.0;
          long long m[3];
          for (int i = 0; i < 3; ++i)
          {
            const double a = double(j[i]) * cell[i], b = double(j[i] + 1) * cell[i];
            const double e = full[i] ? 0.0 : (c[i] < a ? a - c[i] : (c[i] > b ? c[i] - b : 0.0));
            d2 += e * e;
            m[i] = ((j[i] % d.mn[i]) + d.mn[i]) % d.mn[i];
          }
          if (d2 <= R * R)
            fn(m[0] + (long long)d.mn[0] * (m[1] + (long long)d.mn[1] * m[2]));
        }
  };
  std::vector<uint32_t> count(size_t(ncell), 0u);
  long long items = 0;
  for (long long l = 0; l < smp.n_clusters; ++l)
    for_each_cell(l, [&](long long q) {
      if (count[size_t(q)] < 0x7fffffffu)
        ++count[size_t(q)];
      ++items;
    });
  const bool lists = ncell + 1 + items < MAX_ITEMS;
  d.mask_base = (long long)words.size();
  words.resize(size_t(d.mask_base + ncell + 1 + (lists ? items : 0)), 0u);
  uint32_t * w = words.data() + d.mask_base;
  if (!lists)
  {
    for (long long q = 0; q <= ncell; ++q)
      w[q] = uint32_t(ncell + 1) | (q < ncell && count[size_t(q)] ? SEARCH : 0u);
    return;
  }
  // cell starts, then the candidates in cluster order
  uint32_t at = uint32_t(ncell + 1);
  for (long long q = 0; q < ncell; ++q)
  {
    w[q] = at;
    at += count[size_t(q)];
  }
  w[ncell] = at;
  std::vector<uint32_t> fill(w, w + ncell);
  for (long long l = 0; l < smp.n_clusters; ++l)
    for_each_cell(l, [&](long long q) { w[fill[size_t(q)]++] = uint32_t(l); });
  // clusters the search finds from every point they contain
  std::vector<char> regular(size_t(smp.n_clusters), 1);
  for (long long l = 0; l < smp.n_clusters; ++l)
  {
    const double * c = smp.clusters + 4 * l;
    for (int i = 0; i < 3; ++i)
    {
      const int ks = int(d.cmr / d.kd[i]) + 1; // the window of cluster_lookup
      if ((smp.bc[i] != MTG_BC_PBC && !(c[i] >= 0.0 && c[i] < smp.w[i])) ||
          std::ceil((c[3] + 2.0 * margin) / d.kd[i]) > double(ks))
        regular[size_t(l)] = 0;
    }
  }
  // cells where two candidates could both contain a point, or where the search might
  // miss one, take the search
  auto apart = [&](uint32_t a, uint32_t b) {
    const double * ca = smp.clusters + 4 * size_t(a);
    const double * cb = smp.clusters + 4 * size_t(b);
    double d2 = 0.0;
    for (int i = 0; i < 3; ++i)
    {
      double e = ca[i] - cb[i];
      if (smp.bc[i] == MTG_BC_PBC)
        e -= std::nearbyint(e / smp.w[i]) * smp.w[i];
      d2 += e * e;
    }
    const double reach = ca[3] + cb[3] + 2.0 * margin;
    return d2 >= reach * reach;
  };
  for (long long q = 0; q < ncell; ++q)
  {
    const uint32_t s0 = w[q], s1 = w[q + 1];
    bool search = s1 - s0 > uint32_t(MAX_CANDIDATES);
    for (uint32_t x = s0; x < s1 && !search; ++x)
    {
      search = !regular[w[x]];
      for (uint32_t y = x + 1; y < s1 && !search; ++y)
        search = !apart(w[x], w[y]);
    }
    if (search)
      w[q] |= SEARCH;
  }
}

int
build_tables(const mtg_scoef_row * rows, const mtg_config & cfg, const mtg_sim * sims, int n_sims,
             HostTables & out, std::string & err)
{
  // clear, keeping the vectors' storage for the next batch
  out.sims.clear();
  out.prim_end.clear();
  out.species.clear();
  out.mats.clear();
  out.stop_row_mat.clear();
  out.stop_row_species.clear();
  out.clusters.clear();
  out.cl_next.clear();
  out.cl_head.clear();
  out.cl_mask.clear();
  out.total_primaries = out.hist_total = out.voxel_total = 0;
  out.k0 = out.k1 = 0;
  out.emax = 0.0;
  out.any_evac = 0;
  out.any_mode = 0;
  out.any_extended = 0;
  out.any_clusters = 0;
  out.any_potential = 0;
  out.members_est = 1.0;
  if (n_sims < 1 || !sims)
  {
    err = "need at least one simulation";
    return MTG_ERR_BAD_INPUT;
  }
  if (!(cfg.length_scale > 0.0) || !(cfg.tmin > 0.0) || !(cfg.cw > 0.0))
  {
    err = "length_scale, tmin and cw must be positive";
    return MTG_ERR_BAD_INPUT;
  }
  seed_key(cfg.seed, out.k0, out.k1);
  long long prim = 0, hist = 0;
  {
    // at most (1 + elements) species and layers x species materials per simulation
    size_t nsp = 0, nmat = 0;
    for (int si = 0; si < n_sims; ++si)
    {
      const mtg_sample & smp = sims[si].sample;
      const int nl = std::max(0, std::min(smp.n_layers, int(MAX_LAYERS)));
      size_t ne = 1;
      for (int k = 0; k < nl; ++k)
        ne += size_t(std::max(0, std::min(smp.material[k].n_elements, int(MAX_EL))));
      nsp += ne;
      nmat += ne * size_t(nl);
    }
    out.species.reserve(nsp);
    out.mats.reserve(nmat);
    out.sims.reserve(size_t(n_sims));
    out.prim_end.reserve(size_t(n_sims));
  }
  // (species, material) -> index of its first MatConst: equal pairs across the
  // simulations of a batch share the derived constants and the stopping-table row
  std::unordered_map<std::string, int> mat_cache;
  auto mat_key = [](const SpeciesConst & sc, const mtg_material & m) {
    std::string k;
    auto put = [&k](const void * p, size_t n) { k.append(reinterpret_cast<const char *>(p), n); };
    put(&sc.Z1, sizeof sc.Z1);
    put(&sc.m1, sizeof sc.m1);
    put(&m.rho, sizeof m.rho);
    put(&m.n_elements, sizeof m.n_elements);
    for (int j = 0; j < m.n_elements && j < MAX_EL; ++j)
    {
      const mtg_element & e = m.elements[j];
      put(&e.Z, sizeof e.Z);
      put(&e.m, sizeof e.m);
      put(&e.t, sizeof e.t);
      put(&e.Edisp, sizeof e.Edisp);
      put(&e.Elbind, sizeof e.Elbind);
    }
    return k;
  };
  for (int si = 0; si < n_sims; ++si)
  {
    const mtg_sim & s = sims[si];
    const mtg_sample & smp = s.sample;
    if (smp.n_layers < 1 || smp.n_layers > MAX_LAYERS)
    {
      err = "a sample needs 1 to 8 layers";
      return MTG_ERR_BAD_INPUT;
    }
    if (smp.geometry != MTG_GEOM_LAYERS && smp.geometry != MTG_GEOM_CLUSTERS)
    {
      err = "unknown sample geometry";
      return MTG_ERR_BAD_INPUT;
    }
    if (smp.geometry == MTG_GEOM_CLUSTERS)
    {
      if (smp.n_layers != 2)
      {
        err = "a cluster sample needs two materials (matrix, cluster)";
        return MTG_ERR_BAD_INPUT;
      }
      long long cells = 1;
      for (int i = 0; i < 3; ++i)
      {
        if (smp.cluster_hash[i] < 1 || !(smp.w[i] > 0.0))
        {
          err = "a cluster sample needs a positive box and at least one hash cell per axis";
          return MTG_ERR_BAD_INPUT;
        }
        cells *= smp.cluster_hash[i];
      }
      if (cells > (1LL << 26) || smp.n_clusters < 0 || smp.n_clusters > (1LL << 26) ||
          (smp.n_clusters > 0 && !smp.clusters))
      {
        err = "cluster sample: at most 2^26 hash cells and 2^26 clusters, with a cluster array";
        return MTG_ERR_BAD_INPUT;
      }
      for (long long l = 0; l < smp.n_clusters; ++l)
        if (!(smp.clusters[4 * l + 3] >= 0.0) || !std::isfinite(smp.clusters[4 * l]) ||
            !std::isfinite(smp.clusters[4 * l + 1]) || !std::isfinite(smp.clusters[4 * l + 2]))
        {
          err = "cluster coordinates must be finite and radii non-negative";
          return MTG_ERR_BAD_INPUT;
        }
    }
    if (s.ion.Z < 1 || s.ion.Z > MTG_SCOEF_ROWS || !(s.ion.m > 0.0) || !(s.ion.E > 0.0))
    {
      err = "ion Z must be 1..92 with positive mass and energy";
      return MTG_ERR_BAD_INPUT;
    }
    if (s.n_primaries < 0 || s.first_primary < 0 || s.hist_range_n < 0 || s.hist_vac_n < 0 ||
        (s.hist_range_n > 0 && !(s.hist_range_bin > 0.0)) ||
        (s.hist_vac_n > 0 && !(s.hist_vac_bin > 0.0)))
    {
      err = "invalid primary count or histogram binning";
      return MTG_ERR_BAD_INPUT;
    }
    for (int i = 0; i < 3; ++i)
      if (smp.bc[i] < 0 || smp.bc[i] > 2)
      {
        err = "boundary conditions must be 0 (PBC), 1 (INF) or 2 (CUT)";
        return MTG_ERR_BAD_INPUT;
      }
    const double dn = std::sqrt(s.ion.dir[0] * s.ion.dir[0] + s.ion.dir[1] * s.ion.dir[1] +
                                s.ion.dir[2] * s.ion.dir[2]);
    if (!(dn > 0.0))
    {
      err = "ion direction must be non-zero";
      return MTG_ERR_BAD_INPUT;
    }

    // species: the ion, then every distinct (Z, m) of the target elements
    std::vector<std::pair<int, double>> spc;
    spc.push_back({s.ion.Z, s.ion.m});
    auto species_of = [&](int Z, double m) {
      for (size_t i = 0; i < spc.size(); ++i)
        if (spc[i].first == Z && spc[i].second == m)
          return int(i);
      spc.push_back({Z, m});
      return int(spc.size() - 1);
    };
    for (int k = 0; k < smp.n_layers; ++k)
      for (int j = 0; j < smp.material[k].n_elements && j < MAX_EL; ++j)
        species_of(smp.material[k].elements[j].Z, smp.material[k].elements[j].m);

    SimDesc d;
    std::memset(&d, 0, sizeof d);
    d.species_base = int(out.species.size());
    d.n_species = int(spc.size());
    d.mat_base = int(out.mats.size());
    d.n_mat = smp.n_layers;
    for (auto & sp : spc)
      out.species.push_back(make_species(rows, sp.first, sp.second));
    for (int sidx = 0; sidx < d.n_species; ++sidx)
      for (int k = 0; k < smp.n_layers; ++k)
      {
        const SpeciesConst & sc = out.species[d.species_base + sidx];
        const std::string key = mat_key(sc, smp.material[k]);
        const auto it = mat_cache.find(key);
        MatConst mc;
        if (it != mat_cache.end())
          mc = out.mats[size_t(it->second)];
        else
        {
          int rc = make_material(rows, sc, smp.material[k], cfg.tmin, mc, err);
          if (rc != MTG_OK)
            return rc;
          mc.row = int(out.stop_row_mat.size());
          out.stop_row_mat.push_back(int(out.mats.size()));
          out.stop_row_species.push_back(d.species_base + sidx);
          mat_cache.emplace(key, int(out.mats.size()));
        }
        // the recoil species are numbered within each simulation
        for (int j = 0; j < mc.nel; ++j)
          mc.el[j].rspecies = species_of(mc.el[j].Z2, mc.el[j].m2);
        out.mats.push_back(mc);
      }
    // SampleLayers: cumulative layer ends, summed like lookupLayer does
    d.n_layers = smp.n_layers;
    double dsum = 0.0;
    for (int k = 0; k < smp.n_layers; ++k)
    {
      if (smp.n_layers > 1 && !(smp.thickness[k] >= 0.0))
      {
        err = "layer thickness must be non-negative";
        return MTG_ERR_BAD_INPUT;
      }
      dsum += smp.n_layers > 1 ? smp.thickness[k] : 0.0;
      d.layer_end[k] = dsum;
      d.layer_mat[k] = k;
    }
    for (int i = 0; i < 3; ++i)
    {
      d.bc[i] = smp.bc[i];
      d.w[i] = smp.w[i];
      d.dir[i] = s.ion.dir[i];
      d.pos[i] = s.ion.pos[i];
    }
    d.E0 = s.ion.E;
    d.Ef = s.ion.Ef;
    d.scale = cfg.length_scale;
    d.invscale = 1.0 / cfg.length_scale;
    d.tau = cfg.tau;
    d.cw = cfg.cw;
    if (s.tally_mode < MTG_TALLY_VACCOUNT || s.tally_mode > MTG_TALLY_PRIMARIES ||
        (s.tally_mode == MTG_TALLY_PRIMARIES && s.max_generation < 1))
    {
      err = "unknown tally mode, or a generation cutoff below 1";
      return MTG_ERR_BAD_INPUT;
    }
    d.range_mode = s.tally_mode;
    if (s.tally_mode != MTG_TALLY_VACCOUNT)
      out.any_mode = 1;
    d.primaries_only = s.primaries_only != 0;
    // which displaced recoils are followed (followRecoil): ThreadedTrimBase all, or
    // none with primaries_only; TrimRange none (only generation 0 moves);
    // TrimPrimaries / TrimRecoils those of a generation below maxGen (trim.h:113-133)
    if (s.tally_mode == MTG_TALLY_RANGE)
      d.follow_gen = 1;
    else if (s.tally_mode == MTG_TALLY_PRIMARIES)
      d.follow_gen = s.max_generation;
    else
      d.follow_gen = d.primaries_only ? 1 : 0x7fffffff;
    d.kp_gen = s.tally_mode == MTG_TALLY_PRIMARIES ? s.max_generation : -1;
    if (s.potential < MTG_POT_UNIVERSAL || s.potential > MTG_POT_CKR)
    {
      err = "invalid potential"; // trim.C:224-226 exits on the same condition
      return MTG_ERR_BAD_INPUT;
    }
    d.potential = s.potential;
    if (s.md_tag_Z < 0 || s.md_tag_Z > MTG_SCOEF_ROWS ||
        (s.md_tag_Z > 0 && !(s.md_tag_Emin < s.md_tag_Emax)))
    {
      err = "md_tag_Z must be 0..92 with md_tag_Emin < md_tag_Emax";
      return MTG_ERR_BAD_INPUT;
    }
    d.md_Z = s.md_tag_Z;
    d.md_Emin = s.md_tag_Emin;
    d.md_Emax = s.md_tag_Emax;
    d.md_Emin_f = float(s.md_tag_Emin);
    d.md_Emax_f = float(s.md_tag_Emax);
    if (s.potential != MTG_POT_UNIVERSAL)
      out.any_extended = out.any_potential = 1;
    d.prim_begin = prim;
    d.n_primaries = s.n_primaries;
    d.sim_key = uint64_t(si);
    d.key_offset = s.first_primary;
    d.hist_range_n = s.hist_range_n;
    d.hist_vac_n = s.hist_vac_n;
    d.hist_range_base = hist;
    d.hist_vac_base = hist + s.hist_range_n;
    d.inv_hist_range_bin = s.hist_range_n > 0 ? 1.0 / s.hist_range_bin : 0.0;
    d.inv_hist_vac_bin = s.hist_vac_n > 0 ? 1.0 / s.hist_vac_bin : 0.0;
    d.inv_hist_range_bin_f = float(d.inv_hist_range_bin);
    d.inv_hist_vac_bin_f = float(d.inv_hist_vac_bin);
    if (!(s.surface_binding >= 0.0))
    {
      err = "surface binding energy must be non-negative";
      return MTG_ERR_BAD_INPUT;
    }
    d.surface_binding = float(s.surface_binding);
    const bool vox = s.voxel_n[0] > 0 || s.voxel_n[1] > 0 || s.voxel_n[2] > 0;
    if (vox)
    {
      long long cells = 1;
      for (int i = 0; i < 3; ++i)
      {
        if (s.voxel_n[i] < 1 || s.voxel_n[i] > 4096 || !(s.voxel_size[i] > 0.0))
        {
          err = "voxel tally needs 1..4096 cells and a positive size on every axis";
          return MTG_ERR_BAD_INPUT;
        }
        cells *= s.voxel_n[i];
        d.voxel_n[i] = s.voxel_n[i];
        d.voxel_origin[i] = float(s.voxel_origin[i]);
        d.voxel_inv_cell[i] = float(double(s.voxel_n[i]) / s.voxel_size[i]);
      }
      if (cells > (1LL << 28))
      {
        err = "at most 2^28 voxels per simulation";
        return MTG_ERR_BAD_INPUT;
      }
      d.voxel_base = out.voxel_total;
      out.voxel_total += cells;
    }
    if (s.hist_lateral_n < 0 || s.hist_lateral_n > 4096 || (s.hist_lateral_n > 0 && !(s.hist_lateral_bin > 0.0)))
    {
      err = "invalid lateral histogram binning";
      return MTG_ERR_BAD_INPUT;
    }
    d.hist_lat_n = s.hist_lateral_n;
    if (s.hist_lateral_n > 0)
    {
      d.inv_hist_lat_bin = float(1.0 / s.hist_lateral_bin);
      d.lat_y0 = float(s.ion.pos[1] - 0.5 * s.hist_lateral_n * s.hist_lateral_bin);
      d.lat_z0 = float(s.ion.pos[2] - 0.5 * s.hist_lateral_n * s.hist_lateral_bin);
    }
    d.hist_lat_base = hist + s.hist_range_n + 2LL * s.hist_vac_n;
    hist += s.hist_range_n + 2LL * s.hist_vac_n + (long long)s.hist_lateral_n * s.hist_lateral_n;
    if (s.hist_evac_rows < 0 || s.hist_evac_rows > 64)
    {
      err = "hist_evac_rows must be 0..64";
      return MTG_ERR_BAD_INPUT;
    }
    if (smp.geometry == MTG_GEOM_CLUSTERS)
    {
      // sampleClusters::initSpatialhash + addCluster (sample_clusters.C:139-225): the
      // cell of a cluster is floor(c * kn / w) mod kn; each cell lists its clusters
      // in insertion order
      d.geometry = 1;
      out.any_extended = out.any_clusters = 1;
      d.n_clusters = int(smp.n_clusters);
      d.cl_base = (long long)out.clusters.size();
      d.cell_base = (long long)out.cl_head.size();
      long long cells = 1;
      for (int i = 0; i < 3; ++i)
      {
        d.kn[i] = smp.cluster_hash[i];
        d.kd[i] = smp.w[i] / double(d.kn[i]);
        cells *= d.kn[i];
      }
      out.cl_head.resize(size_t(d.cell_base + cells), -1);
      std::vector<int> tail(size_t(cells), -1);
      d.cmr = 0.0;
      for (long long l = 0; l < smp.n_clusters; ++l)
      {
        const double * c = smp.clusters + 4 * l;
        int k[3];
        for (int i = 0; i < 3; ++i)
        {
          k[i] = int(std::floor((c[i] * d.kn[i]) / smp.w[i])) % d.kn[i];
          k[i] = k[i] < 0 ? k[i] + d.kn[i] : k[i];
        }
        const long long cell = k[0] + (long long)d.kn[0] * (k[1] + (long long)d.kn[1] * k[2]);
        const int idx = int(l); // index within this sample
        if (tail[size_t(cell)] < 0)
          out.cl_head[size_t(d.cell_base + cell)] = idx;
        else
          out.cl_next[size_t(d.cl_base + tail[size_t(cell)])] = idx;
        tail[size_t(cell)] = idx;
        out.clusters.push_back(Cl4d{c[0], c[1], c[2], c[3]});
        out.cl_next.push_back(-1);
        if (c[3] > d.cmr)
          d.cmr = c[3];
      }
      build_cluster_cells(d, smp, out.cl_mask);
    }
    d.hist_evac_rows = s.hist_vac_n > 0 ? s.hist_evac_rows : 0;
    d.hist_evac_base = hist;
    hist += (long long)d.hist_evac_rows * s.hist_vac_n;
    if (d.hist_evac_rows > 0)
      out.any_evac = 1;
    out.members_est += double(s.n_primaries) * expected_members(s);
    prim += s.n_primaries;
    out.prim_end.push_back(prim);
    out.sims.push_back(d);
    out.emax = std::max(out.emax, s.ion.E);
  }
  if (prim > 0xffffffffLL)
  {
    err = "at most 2^32 - 1 primaries per run";
    return MTG_ERR_BAD_INPUT;
  }
  if (hist >= (1LL << 31))
  {
    // bins are addressed with 32-bit indices on the device
    err = "histograms of one run must hold fewer than 2^31 bins";
    return MTG_ERR_BAD_INPUT;
  }
  out.total_primaries = prim;
  out.members_est = prim > 0 ? out.members_est / double(prim) : 1.0;
  out.hist_total = hist;
  return MTG_OK;
}

} // namespace mtg
