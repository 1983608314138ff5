// mtoracle -- CPU restatement of MyTRIM's cascade path.
//
// TEST INFRASTRUCTURE ONLY.  This program is the oracle that the CUDA engine is
// checked against, and the "port" CPU baseline that bench.py times.  Nothing in
// the product links, loads or calls it.
//
// It restates, in plain C++ of its own, the reference algorithm for the hot path:
//   * MaterialBase::prepare / average           material.C:37-110
//   * MaterialBase::getrstop / rstop / rpstop   material.C:114-281
//   * SampleLayers::lookupLayer                 sample_layers.C:27-43
//   * sampleClusters::lookupCluster             sample_clusters.C:42-130
//   * TrimBase::trim (one cascade member)       trim.C:36-425, with the universal,
//     Moliere and C-Kr potentials of TrimBase::_potential (trim.C:194-258)
//   * runmytrim's seeding and FIFO cascade loop apps/runmytrim.C:71-93, 287-304
//   * tallies with TrimVacCount / TrimVacEnergyCount / TrimRange / TrimPrimaries /
//     TrimRecoils / TrimPhononOut semantics (apps/src/TrimVacCount.C:32-54,
//     apps/src/TrimVacEnergyCount.C:32-53, apps/src/TrimRange.C:32-47,
//     trim.C:446-464, trim.C:504-527) and runmytrim's output files (runspec.h)
// Every floating-point expression is evaluated in the same order as the
// reference, and the same libm functions are called, so that with mt19937
// seeding ("seeding compat") the results are bit-identical to the reference
// library (checked by tests/test_oracle.py against oracle/_ref/ref_driver and
// against the committed fixtures in tests/golden/).
//
// "seeding philox" replaces the mt19937 stream by the counter-based Philox4x32-10
// streams the CUDA engine's FP64 path uses (keyed by cascade member and collision
// index), so that the GPU and this oracle draw the same random numbers.
//
// Usage:  mtoracle <tables.tsv> < spec      (spec format: oracle/runspec.h)

#include "runspec.h"

#include <cmath>
#include <cstdint>
#include <queue>
#include <random>
#include <chrono>
#include <algorithm>

namespace mto
{

// ---------------------------------------------------------------- potentials
// v(r) and v'(r) of the screened potential (trim.C:194-226): 0 universal,
// 1 Moliere (Utility::pow<4> and pow<5> multiply as (x x)(x x) and x (x^4),
// shim/pow.h), 2 C-Kr with the reference's derivative coefficients as written.
static inline void
screening(int pot, double r, double & v, double & v1)
{
  if (pot == 1)
  {
    const double ex1 = std::exp(-0.3 * r);
    const double e1s = ex1 * ex1;
    const double ex2 = e1s * e1s;
    const double e2s = ex2 * ex2;
    const double ex3 = ex2 * (e2s * e2s);
    v = (0.35 * ex1 + 0.55 * ex2 + 0.1 * ex3) / r;
    v1 = -(v + 0.105 * ex1 + 0.66 * ex2 + 0.6 * ex3) / r;
  }
  else if (pot == 2)
  {
    const double ex1 = std::exp(-0.279 * r);
    const double ex2 = std::exp(-0.637 * r);
    const double ex3 = std::exp(-1.1919 * r);
    v = (0.191 * ex1 + 0.474 * ex2 + 0.335 * ex3) / r;
    v1 = -(v + 0.531865 * ex1 + 0.30181 * ex2 + 0.6437 * ex3) / r;
  }
  else
  {
    const double ex1 = 0.18175 * std::exp(-3.1998 * r);
    const double ex2 = 0.50986 * std::exp(-0.94229 * r);
    const double ex3 = 0.28022 * std::exp(-0.4029 * r);
    const double ex4 = 0.028171 * std::exp(-0.20162 * r);
    v = (ex1 + ex2 + ex3 + ex4) / r;
    v1 = -(v + 3.1998 * ex1 + 0.94229 * ex2 + 0.4029 * ex3 + 0.20162 * ex4) / r;
  }
}

// magic-formula A and F of each potential (trim.C:236-258)
static inline void
magic(int pot, double eps, double sqe, double b, double & aa, double & ff)
{
  if (pot == 1)
  {
    const double cc = (0.009611 + sqe) / (0.005175 + sqe);
    aa = 2.0 * eps * (1.0 + (0.6743 / sqe)) * std::pow(b, cc);
    ff = (std::sqrt(aa * aa + 1.0) - aa) * ((6.314 + eps) / (10.0 + eps));
  }
  else if (pot == 2)
  {
    const double cc = (0.235809 + sqe) / (0.126000 + sqe);
    aa = 2.0 * eps * (1.0 + (1.0144 / sqe)) * std::pow(b, cc);
    ff = (std::sqrt(aa * aa + 1.0) - aa) * ((6935.0 + eps) / (83550.0 + eps));
  }
  else
  {
    const double cc = (0.011615 + sqe) / (0.0071222 + sqe);
    aa = 2.0 * eps * (1.0 + (0.99229 / sqe)) * std::pow(b, cc);
    ff = (std::sqrt(aa * aa + 1.0) - aa) * ((9.3066 + eps) / (14.813 + eps));
  }
}

// ---------------------------------------------------------------- data tables
struct Coef
{
  double mm1, m1, vfermi, lfctr;
  double pcoef[8];
};
static Coef g_coef[92];

static bool
load_tables(const char * path)
{
  std::ifstream in(path);
  if (!in)
    return false;
  std::string line;
  int rows = 0;
  while (std::getline(in, line))
  {
    if (line.empty() || line[0] == '#')
      continue;
    std::istringstream ls(line);
    int Z;
    std::string sym;
    double mm1, m1, mnat, rho, atrho, vfermi, heat, lfctr;
    ls >> Z >> sym >> mm1 >> m1 >> mnat >> rho >> atrho >> vfermi >> heat >> lfctr;
    if (!ls || Z < 1 || Z > 92)
      return false;
    Coef & c = g_coef[Z - 1];
    c.mm1 = mm1;
    c.m1 = m1;
    c.vfermi = vfermi;
    c.lfctr = lfctr;
    for (int j = 0; j < 8; ++j)
      ls >> c.pcoef[j];
    if (!ls)
      return false;
    ++rows;
  }
  return rows == 92;
}

// ---------------------------------------------------------------- RNG streams
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11 "Parallel random numbers: as
// easy as 1, 2, 3"), restated here independently of the CUDA engine's copy.
static inline void
philox4x32_10(uint32_t ctr[4], uint32_t k0, uint32_t k1)
{
  for (int r = 0; r < 10; ++r)
  {
    const uint64_t p0 = uint64_t(0xD2511F53u) * ctr[0];
    const uint64_t p1 = uint64_t(0xCD9E8D57u) * ctr[2];
    const uint32_t n0 = uint32_t(p1 >> 32) ^ ctr[1] ^ k0;
    const uint32_t n2 = uint32_t(p0 >> 32) ^ ctr[3] ^ k1;
    ctr[0] = n0;
    ctr[1] = uint32_t(p1);
    ctr[2] = n2;
    ctr[3] = uint32_t(p0);
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
}

// splitmix64 finaliser (Steele, Lea, Flood 2014) used to derive cascade-member keys
static inline uint64_t
mix64(uint64_t z)
{
  z ^= z >> 30;
  z *= 0xBF58476D1CE4E5B9ull;
  z ^= z >> 27;
  z *= 0x94D049BB133111EBull;
  z ^= z >> 31;
  return z;
}

static inline uint64_t
root_key(uint64_t sim, uint64_t primary)
{
  return mix64((sim << 40) ^ (primary + 1));
}

static inline uint64_t
child_key(uint64_t parent, uint32_t collision)
{
  return mix64(parent + 0x9E3779B97F4A7C15ull * uint64_t(collision));
}

// 53-bit uniform in (0, 1]
static inline double
u53(uint32_t hi, uint32_t lo)
{
  const uint64_t v = (uint64_t(hi) << 21) ^ uint64_t(lo >> 11);
  return double(v + 1) * (1.0 / 9007199254740992.0);
}

// 32-bit uniform in (0, 1]
static inline double
u32(uint32_t x)
{
  return (double(x) + 1.0) * (1.0 / 4294967296.0);
}

struct PhiloxDraw
{
  uint32_t k0, k1;
  uint64_t member;
  // r1 of the first flight (trim.C:71): the bits of the member's path key, which
  // mix64 has already mixed
  double r1() const { return u53(uint32_t(member >> 32), uint32_t(member)); }
  // block 0 of collision ic: impact parameter and target-atom draws (trim.C:143,147)
  void pair(uint32_t ic, double & r2, double & hh) const
  {
    uint32_t c[4] = {uint32_t(member), uint32_t(member >> 32), ic, 0u};
    philox4x32_10(c, k0, k1);
    r2 = u53(c[0], c[1]);
    hh = u53(c[2], c[3]);
  }
  // block 1+pass of collision ic: one rejection pass of the perpendicular vector
  // (trim.C:322-333)
  void ball(uint32_t ic, uint32_t pass, double r[3]) const
  {
    uint32_t c[4] = {uint32_t(member), uint32_t(member >> 32), ic, 1u + pass};
    philox4x32_10(c, k0, k1);
    for (int i = 0; i < 3; ++i)
      r[i] = 2.0 * u32(c[i]) - 1.0;
  }
};

// ---------------------------------------------------------------- materials
struct Elem
{
  int Z;
  double m, t, Edisp, Elbind;
  double my, ec, ai, fi; // projectile dependent
};

struct Mat
{
  double rho, am, az, arho;
  double mu, a, f, epsdg;
  std::vector<Elem> el;

  // MaterialBase::prepare (material.C:37-74)
  void prepare()
  {
    double tt = 0.0;
    for (auto & e : el)
    {
      if (e.t < 0.0)
        e.t = 0.0;
      tt += e.t;
    }
    for (auto & e : el)
      e.t /= tt;
    am = 0.0;
    az = 0.0;
    for (auto & e : el)
    {
      am += e.m * e.t;
      az += double(e.Z) * e.t;
    }
    arho = rho * 0.6022 / am;
  }

  // MaterialBase::average (material.C:78-110): projectile-dependent constants
  void average(int Z1, double m1, double tmin)
  {
    mu = m1 / am;
    const double fZ = double(Z1);
    const double fZ023 = std::pow(fZ, 0.23);
    a = .5292 * .8853 / (fZ023 + std::pow(az, 0.23));
    f = a * am / (az * fZ * 14.4 * (m1 + am));
    epsdg = tmin * f * ((1.0 + mu) * (1.0 + mu)) / (4.0 * mu);
    for (auto & e : el)
    {
      e.my = m1 / e.m;
      e.ec = 4.0 * e.my / ((1.0 + e.my) * (1.0 + e.my));
      e.ai = .5292 * .8853 / (fZ023 + std::pow(e.Z, 0.23));
      e.fi = e.ai * e.m / (fZ * double(e.Z) * 14.4 * (m1 + e.m));
    }
  }
};

// proton stopping in element z2p (material.C:134-158)
static double
proton_stopping(int z2p, double e)
{
  const Coef & c = g_coef[z2p - 1];
  const double pe0 = 25.0;
  const double pe = std::max(pe0, e);
  const double sl = (c.pcoef[0] * std::pow(pe, c.pcoef[1])) + (c.pcoef[2] * std::pow(pe, c.pcoef[3]));
  const double sh = c.pcoef[4] / std::pow(pe, c.pcoef[5]) * std::log(c.pcoef[6] / pe + c.pcoef[7] * pe);
  double sp = sl * sh / (sl + sh);
  if (e <= pe0)
    sp *= std::pow(e / pe0, z2p <= 6 ? 0.25 : 0.45);
  return sp;
}

// electronic stopping of ion (Z1, m, E[eV]) in element z2, eV/(1e15 atoms/cm^2)*10
// (material.C:161-281)
static double
ion_stopping(int z1, double m, double E, int z2)
{
  const double fz1 = double(z1);
  const double fz2 = double(z2);
  const double lfctr = g_coef[z1 - 1].lfctr;
  const double vfermi = g_coef[z2 - 1].vfermi;
  const double m1 = (m == 0.0) ? g_coef[z1 - 1].mm1 : m;
  const double ee = 0.001 * E;
  const double e = ee / m1;
  double se;

  if (z1 == 1)
    se = proton_stopping(z2, e);
  else if (z1 == 2)
  {
    const double he0 = 1.0;
    double he = std::max(he0, e);
    const double b = std::log(he);
    const double b2 = b * b;
    const double b4 = b2 * b2;
    double a = 0.2865 + 0.1266 * b - 0.001429 * b2 + 0.02402 * b * b2 - 0.01135 * b4 +
               0.001475 * b4 * b;
    double heh = 1.0 - std::exp(-std::min(30.0, a));
    he = std::max(he, 1.0);
    const double t = 7.6 - std::log(he);
    a = 1.0 + (0.007 + 0.00005 * fz2) * std::exp(-(t * t));
    heh *= a * a;
    const double sp = proton_stopping(z2, he);
    se = sp * heh * 4.0;
    if (e <= he0)
      se *= std::sqrt(e / he0);
  }
  else
  {
    const double yrmin = 0.13;
    double vrmin = 1.0;
    const double v = std::sqrt(e / 25.0) / vfermi;
    const double v2 = v * v;
    double vr;
    if (v >= 1.0)
      vr = v * vfermi * (1.0 + 1.0 / (5.0 * v2));
    else
      vr = (3.0 * vfermi / 4.0) * (1.0 + (2.0 * v2 / 3.0) - v2 * v2 / 15.0);
    const double cb = std::cbrt(fz1);
    const double cb2 = cb * cb;
    double yr = std::max(yrmin, vr / cb2);
    yr = std::max(yr, vrmin / cb2);
    const double yr03 = std::pow(yr, 0.3);
    double a = -0.803 * yr03 + 1.3167 * yr03 * yr03 + 0.38157 * yr + 0.008983 * yr * yr;
    const double q = std::min(1.0, std::max(0.0, 1.0 - std::exp(-std::min(a, 50.0))));
    const double b = (std::min(0.43, std::max(0.32, 0.12 + 0.025 * fz1))) / cb;
    const double l0 = (0.8 - q * std::min(1.2, 0.6 + fz1 / 30.0)) / cb;
    double l1;
    if (q < 0.2)
      l1 = 0.0;
    else if (q < std::max(0.0, 0.9 - 0.025 * fz1))
      l1 = b * (q - 0.2) / std::abs(std::max(0.0, 0.9 - 0.025 * fz1) - 0.2000001);
    else if (q < std::max(0.0, 1.0 - 0.025 * std::min(16.0, fz1)))
      l1 = b;
    else
      l1 = b * (1.0 - q) / (0.025 * std::min(16.0, fz1));
    const double l = std::max(l1, l0 * lfctr);
    const double w = 4.0 * l * vfermi / 1.919;
    double zeta = q + (1.0 / (2.0 * vfermi * vfermi)) * (1.0 - q) * std::log(1.0 + w * w);
    const double t = 7.6 - std::max(0.0, std::log(e));
    a = -(t * t);
    zeta *= 1.0 + (1.0 / (fz1 * fz1)) * (0.18 + 0.0015 * fz2) * std::exp(a);
    const double zf = zeta * fz1;
    if (yr <= std::max(yrmin, vrmin / cb2))
    {
      vrmin = std::max(vrmin, yrmin * cb2);
      const double vmin = 0.5 * (vrmin + std::sqrt(std::max(0.0, vrmin * vrmin - 0.8 * vfermi * vfermi)));
      const double eee = 25.0 * vmin * vmin;
      const double sp = proton_stopping(z2, eee);
      const double power = (z2 == 6 || ((z2 == 14 || z2 == 32) && z1 <= 19)) ? 0.375 : 0.5;
      se = sp * (zf * zf) * std::pow(e / eee, power);
    }
    else
    {
      const double sp = proton_stopping(z2, e);
      se = sp * (zf * zf);
    }
  }
  return se * 10.0;
}

// MaterialBase::getrstop (material.C:114-121), eV/Angstrom
static double
material_stopping(const Mat & mat, int Z1, double m1, double E)
{
  double se = 0.0;
  for (auto & e : mat.el)
    se += ion_stopping(Z1, m1, E, e.Z) * e.t;
  return se * mat.arho;
}

// ---------------------------------------------------------------- cascade
enum State
{
  MOVING,
  REPLACEMENT,
  SUBSTITUTIONAL,
  INTERSTITIAL,
  LOST,
  DELETE
};

struct Ion
{
  int Z;
  double m, E, Ef;
  double dir[3], pos[3];
  int gen;
  int state;
  uint64_t key;
  int md = 0; // IonMDTag::_md: 0 when spawned (ion.C:88-93)
};

struct Engine
{
  const runspec::Spec & spec;
  std::vector<Mat> mats;
  std::vector<double> thick;
  double tmin = 0.2, tau = 0.0, cw = 0.001;
  runspec::Tally t;
  runspec::PluginOut out; // runmytrim output plugin (spec key "output")
  // current primary
  long long p_vac = 0, p_coll = 0;
  double p_enuc = 0.0, p_eel = 0.0;
  double last_x = 0, last_y = 0, last_z = 0;
  int last_state = 0;

  std::mt19937 mt;
  std::uniform_real_distribution<double> ureal{0.0, 1.0};
  std::uniform_int_distribution<unsigned int> uint16{0, 65535};
  uint32_t pk0 = 0, pk1 = 0;

  explicit Engine(const runspec::Spec & s) : spec(s)
  {
    for (auto & l : s.layers)
    {
      Mat m;
      m.rho = l.rho;
      for (auto & e : l.el)
        m.el.push_back(Elem{e.Z, e.m, e.t, e.Edisp, e.Elbind, 0, 0, 0, 0});
      m.prepare();
      mats.push_back(m);
      thick.push_back(l.thickness);
    }
    t.hist_range.assign(s.hist_range_n, 0);
    t.hist_vac.assign(s.hist_vac_n, 0);
    t.hist_repl.assign(s.hist_vac_n, 0);
    t.spec = &s;
    t.vox_depth.assign(s.vox_n[0] > 0 ? s.vox_n[0] : 0, 0.0);
    out.type = s.out_type;
    out.base = s.out_base;
    if (s.clusters)
      hash.build(s);
    pk0 = s.seed;
    pk1 = 0x4D795452u; // fixed high key word for single-simulation runs
  }

  void reseed(unsigned int s)
  {
    mt.seed(s);
    ureal.reset();
    uint16.reset();
  }
  double drand() { return ureal(mt); }

  runspec::ClusterHash hash; // cluster samples only

  // material index at pos: SampleLayers::lookupLayer (sample_layers.C:27-43) or
  // sampleClusters::lookupMaterial (sample_clusters.C:42-53; -1 = no material)
  int material_at(const double pos[3]) const
  {
    if (!spec.clusters)
      return layer_of(pos[0]);
    const int l = hash.lookup(pos);
    return l == -2 ? -1 : (l >= 0 ? 1 : 0);
  }

  // SampleLayers::lookupLayer (sample_layers.C:27-43)
  int layer_of(double x) const
  {
    unsigned int i;
    double d = 0.0;
    for (i = 0; i < thick.size(); ++i)
    {
      d += thick[i];
      if (x < d)
        break;
    }
    if (i >= mats.size())
      i = mats.size() - 1;
    return int(i);
  }

  static void norm3(double v[3])
  {
    const double s = 1.0 / std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    v[0] *= s;
    v[1] *= s;
    v[2] *= s;
  }

  // One cascade member from start to rest: TrimBase::trim (trim.C:36-425).
  template <class Push>
  void run_member(Ion & pka, Push && push)
  {
    pka.state = MOVING;
    // the demo programs' MD-gap mark, set when the member is popped (mytrim_solid.C:156-159)
    if (spec.md_Z != 0 && pka.Z == spec.md_Z && pka.E > spec.md_Emin && pka.E < spec.md_Emax && pka.md == 0)
      pka.md = 1;
    const double scale = spec.scale;
    const double invscale = 1.0 / scale;
    PhiloxDraw ph{pk0, pk1, pka.key};
    const bool philox = spec.philox;
    for (auto & m : mats)
      m.average(pka.Z, pka.m, tmin);

    double r1 = philox ? ph.r1() : drand();
    uint32_t ic = 0;
    do
    {
      ++ic;
      const int mi = material_at(pka.pos);
      if (mi < 0)
        break; // outside the sample: the member is dropped (trim.C:81-83)
      Mat & mat = mats[mi];
      norm3(pka.dir);

      // maximum impact parameter and free flight (trim.C:88-94)
      double eps = pka.E * mat.f;
      const double eeg = std::sqrt(eps * mat.epsdg);
      const double pmax = mat.a / (eeg + std::sqrt(eeg) + 0.125 * std::pow(eeg, 0.1));
      double ls = 1.0 / (M_PI * (pmax * pmax) * mat.arho);
      if (ic == 1)
        ls = r1 * std::min(ls, cw);

      double r2, hh;
      if (philox)
        ph.pair(ic, r2, hh);
      else
      {
        r2 = drand();
        hh = 0.0;
      }
      const double p = pmax * std::sqrt(r2);
      if (!philox)
        hh = drand();
      unsigned int nn;
      const unsigned int nel = mat.el.size();
      for (nn = 0; nn < nel; ++nn)
      {
        hh -= mat.el[nn].t;
        if (hh <= 0)
          break;
      }
      if (nn >= nel) // rounding guard (the reference would read past its vector)
        nn = nel - 1;
      const Elem & el = mat.el[nn];

      eps = el.fi * pka.E;
      const double b = p / el.ai;
      const double see = material_stopping(mat, pka.Z, pka.m, pka.E);
      double dee = ls * see;

      // scattering angle (trim.C:172-271) in the chosen potential (trim.C:194-258)
      double s2, c2, ct, st;
      if (eps > 10.0)
      {
        const double w = 2.0 * eps * b;
        s2 = 1.0 / (1.0 + (1.0 + b * (1.0 + b)) * (w * w));
        c2 = 1.0 - s2;
        ct = 2.0 * c2 - 1.0;
        st = std::sqrt(1.0 - ct * ct);
      }
      else
      {
        double r = b;
        double rr = -2.7 * std::log(eps * b);
        if (rr >= b)
        {
          rr = -2.7 * std::log(eps * rr);
          if (rr >= b)
            r = rr;
        }
        double v, v1, q;
        do
        {
          screening(spec.potential, r, v, v1);
          const double fr = b * b / r + v * r / eps - r;
          const double fr1 = -b * b / (r * r) + (v + v1 * r) / eps - 1.0;
          q = fr / fr1;
          r -= q;
        } while (std::abs(q / r) > 0.001);
        const double roc = -2.0 * (eps - v) / v1;
        const double sqe = std::sqrt(eps);
        double aa, ff;
        magic(spec.potential, eps, sqe, b, aa, ff);
        const double delta = (r - b) * aa * ff / (ff + 1.0);
        const double co = (b + delta + roc) / (r + roc);
        c2 = co * co;
        s2 = 1.0 - c2;
        ct = 2.0 * c2 - 1.0;
        st = std::sqrt(1.0 - ct * ct);
      }

      // energy bookkeeping (trim.C:275-296)
      double den = el.ec * s2 * pka.E;
      if (dee > pka.E)
        dee = pka.E;
      pka.E -= dee;
      t.Eel += dee;
      p_eel += dee;
      const double p1 = std::sqrt(2.0 * pka.m * pka.E);
      if (den > pka.E)
        den = pka.E;
      pka.E -= den;
      const double p2 = std::sqrt(2.0 * pka.m * pka.E);

      // recoil spawn at the pre-flight position (trim.C:306-318, ion.C:55-68)
      Ion rec;
      rec.gen = pka.gen + 1;
      rec.pos[0] = pka.pos[0];
      rec.pos[1] = pka.pos[1];
      rec.pos[2] = pka.pos[2];
      rec.Ef = pka.Ef;
      const double fl = ls - tau;
      for (int i = 0; i < 3; ++i)
        pka.pos[i] += pka.dir[i] * fl * invscale;
      for (int i = 0; i < 3; ++i)
        rec.dir[i] = pka.dir[i] * p1;
      rec.E = den;
      rec.E -= el.Elbind;
      rec.m = el.m;
      rec.Z = el.Z;
      rec.state = MOVING;

      // random unit vector perpendicular to dir (trim.C:322-333)
      double perp[3], nrm;
      uint32_t pass = 0;
      do
      {
        double rd[3];
        do
        {
          if (philox)
            ph.ball(ic, pass++, rd);
          else
            for (int i = 0; i < 3; ++i)
              rd[i] = 2.0 * drand() - 1.0;
        } while (rd[0] * rd[0] + rd[1] * rd[1] + rd[2] * rd[2] > 1.0);
        for (int i = 0; i < 3; ++i)
          perp[i] = pka.dir[(i + 1) % 3] * rd[(i + 2) % 3] - pka.dir[(i + 2) % 3] * rd[(i + 1) % 3];
        nrm = std::sqrt(perp[0] * perp[0] + perp[1] * perp[1] + perp[2] * perp[2]);
      } while (nrm == 0.0);
      for (int i = 0; i < 3; ++i)
        perp[i] /= nrm;

      // new direction (trim.C:336-341)
      const double psi = std::atan2(st, ct + el.my);
      const double cp = std::cos(psi);
      for (int i = 0; i < 3; ++i)
        pka.dir[i] *= cp;
      const double sp = std::sin(psi);
      for (int i = 0; i < 3; ++i)
        pka.dir[i] += perp[i] * sp;
      for (int i = 0; i < 3; ++i)
        rec.dir[i] -= pka.dir[i] * p2;

      // CUT boundaries (trim.C:344-352)
      for (int i = 0; i < 3; ++i)
        if (spec.bc[i] == 2 && (pka.pos[i] > spec.size[i] || pka.pos[i] < 0.0))
        {
          pka.state = LOST;
          break;
        }

      // fate of recoil and projectile (trim.C:357-411)
      bool queued = false;
      if (pka.state != LOST)
      {
        if (rec.E > el.Edisp - el.Elbind)
        {
          emit(EV_HISTORY, pka.pos, pka.E, pka.Z, pka.m, pka.gen, 0, 0.0, pka.key, pka.md);
          emit(EV_BRANCH, rec.pos, rec.E, el.Z, el.m, rec.gen, 0, el.Elbind, pka.key);
          t.Enuc += el.Elbind;
          p_enuc += el.Elbind;
          t.deposit(rec.pos[0], rec.pos[1], rec.pos[2], el.Elbind);
          // followRecoil: TrimRange (TrimRange.h:16), TrimPrimaries / TrimRecoils
          // (trim.h:119), ThreadedTrimBase (ThreadedTrimBase.h:12)
          const bool follow = spec.range_mode       ? (rec.gen < 1)
                              : spec.primaries_mode ? (rec.gen < spec.max_gen)
                                                    : !spec.primaries_only;
          if (follow)
          {
            norm3(rec.dir);
            rec.key = child_key(pka.key, ic);
            push(rec);
            queued = true;
          }
          else
            t.Eunfollowed += rec.E;
          if (pka.E > el.Edisp)
          {
            emit(EV_VACANCY, rec.pos, rec.E, el.Z, el.m, rec.gen, 0, el.Elbind, pka.key);
            vacancy(rec, el, mat);
          }
          else
          {
            emit(EV_REPLACEMENT, rec.pos, rec.E, el.Z, el.m, rec.gen, 0, el.Elbind, pka.key);
            replacement(rec);
            pka.state = (pka.Z == el.Z) ? REPLACEMENT : SUBSTITUTIONAL;
          }
        }
        else
        {
          emit(EV_DISSIPATE, rec.pos, rec.E, el.Z, el.m, rec.gen, 0, el.Elbind, pka.key);
          const double e = rec.E + el.Elbind;
          out.dissipate(rec.Z, rec.pos[0]);
          t.Enuc += e;
          p_enuc += e;
          t.deposit(rec.pos[0], rec.pos[1], rec.pos[2], e);
          if (pka.E < pka.Ef)
            pka.state = INTERSTITIAL;
        }
      }
      (void)queued;
      // electronic loss deposited where the flight started, in the order the
      // reference's hooks see it (checkPKAState follows the fate hooks)
      t.deposit(rec.pos[0], rec.pos[1], rec.pos[2], dee);
      check_state(pka, rec.E + el.Elbind);
    } while (pka.state == MOVING);
  }

  void vacancy(const Ion & rec, const Elem & el, const Mat & mat)
  {
    if (spec.primaries_mode)
    {
      // TrimPrimaries::vacancyCreation (trim.C:446-464)
      long long add = 1;
      if (rec.gen == spec.max_gen)
      {
        const double ed = 0.0115 * std::pow(mat.az, -7.0 / 3.0) * rec.E;
        const double g = 3.4008 * std::pow(ed, 1.0 / 6.0) + 0.40244 * std::pow(ed, 3.0 / 4.0) + ed;
        const double kd = 0.1337 * std::pow(mat.az, 2.0 / 3.0) / std::sqrt(mat.am);
        const double Ev = rec.E / (1.0 + kd * g);
        add += int(0.8 * Ev / (2.0 * el.Edisp));
      }
      t.vacancies += add;
      p_vac += add;
      return;
    }
    if (spec.range_mode)
    {
      const double Ed = el.Edisp;
      const double ed = 0.0115 * std::pow(rec.Z, -7.0 / 3.0) * rec.E;
      const double kd = 0.1337 * std::pow(rec.Z, 2.0 / 3.0) / std::sqrt(rec.m);
      const double g = 3.4008 * std::pow(ed, 1.0 / 6.0) + 0.40244 * std::pow(ed, 3.0 / 4.0) + ed;
      const double Ev = rec.E / (1.0 + kd * g);
      long long add;
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
    out.vacancy(rec.pos[0], rec.E);
    const int b = runspec::bin_of(rec.pos[0], spec.hist_vac_bin, spec.hist_vac_n);
    if (b >= 0)
      t.hist_vac[b]++;
  }

  void replacement(const Ion & rec)
  {
    t.replacements++;
    out.replacement(rec.pos[0]);
    const int b = runspec::bin_of(rec.pos[0], spec.hist_vac_bin, spec.hist_vac_n);
    if (b >= 0)
      t.hist_repl[b]++;
  }

  void check_state(const Ion & pka, double recoil_energy)
  {
    t.collisions++;
    p_coll++;
    if (pka.state == MOVING)
      return;
    last_state = pka.state;
    if (pka.state == LOST)
    {
      emit(EV_LOST, pka.pos, pka.E, pka.Z, pka.m, pka.gen, LOST, recoil_energy, pka.key, pka.md);
      t.lost++;
      t.Elost += pka.E + recoil_energy;
      t.exit_surface(pka.pos[0], pka.gen, pka.E, pka.dir[0]);
      return;
    }
    emit(EV_REST, pka.pos, pka.E, pka.Z, pka.m, pka.gen, pka.state, 0.0, pka.key, pka.md);
    t.Enuc += pka.E;
    p_enuc += pka.E;
    t.deposit(pka.pos[0], pka.pos[1], pka.pos[2], pka.E);
    if (pka.state == INTERSTITIAL)
      t.interstitials++;
    else if (pka.state == SUBSTITUTIONAL)
      t.substitutionals++;
    if (pka.gen == 0)
    {
      const double x = pka.pos[0], y = pka.pos[1], z = pka.pos[2];
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
      const int b = runspec::bin_of(x, spec.hist_range_bin, spec.hist_range_n);
      if (b >= 0)
        t.hist_range[b]++;
    }
  }

  double seed_sq = 0.0; // compat seeding: sum over distinct seeds of their use count squared
  long long cur_primary = 0;

  // Event records with the fields of the GPU event log (mtg_event): the reference's
  // hook calls that TrimDefectLog, TrimPhononOut and TrimHistory stream
  // (trim.C:467-527, trim.h:139-153), one line each, floats in hex
  enum EvKind
  {
    EV_VACANCY = 1,
    EV_REPLACEMENT = 2,
    EV_BRANCH = 3,
    EV_DISSIPATE = 4,
    EV_REST = 5,
    EV_LOST = 6,
    EV_HISTORY = 7
  };
  void emit(int kind, const double pos[3], double E, int Z, double m, int gen, int state, double aux, uint64_t key,
            int md = 0)
  {
    if (!(spec.event_mask & (1u << kind)))
      return;
    printf("ev %d %llu %lld %d %d %d %d %a %a %a %a %a %a\n", kind, (unsigned long long)key, cur_primary, gen, Z,
           state, md, pos[0], pos[1], pos[2], E, aux, m);
  }

  void run()
  {
    std::vector<unsigned int> seeds;
    if (!spec.philox)
    {
      reseed(spec.seed);
      seeds.resize(spec.count);
      for (long long i = 0; i < spec.count; ++i)
        seeds[i] = uint16(mt);
      // primaries that draw the same 16-bit seed repeat one cascade exactly: the
      // sum over seeds of (primaries with that seed)^2 sets the variance of a
      // run-wide mean (sum n_s^2 / N^2 times the per-cascade variance)
      std::vector<long long> uses(65536, 0);
      for (long long i = 0; i < spec.count; ++i)
        uses[seeds[i] & 0xFFFFu]++;
      seed_sq = 0.0;
      for (long long u : uses)
        seed_sq += double(u) * double(u);
    }
    std::queue<Ion> fifo;
    for (long long n = spec.first; n < spec.first + spec.n; ++n)
    {
      Ion pka;
      pka.Z = spec.Z;
      pka.m = spec.m;
      pka.E = spec.E;
      pka.Ef = spec.Ef;
      pka.gen = 0;
      for (int i = 0; i < 3; ++i)
      {
        pka.dir[i] = spec.dir[i];
        pka.pos[i] = spec.pos[i];
      }
      pka.key = root_key(spec.sim_index, uint64_t(n));
      cur_primary = n;
      if (!spec.philox)
        reseed(seeds[n]);
      p_vac = 0;
      p_coll = 0;
      p_enuc = 0.0;
      p_eel = 0.0;
      long long members = 0;
      fifo.push(pka);
      while (!fifo.empty())
      {
        Ion ion = fifo.front();
        fifo.pop();
        run_member(ion, [&](const Ion & r) { fifo.push(r); });
        ++members;
      }
      t.primaries++;
      t.members += members;
      t.vac_s2 += double(p_vac) * double(p_vac);
      t.eel_s2 += p_eel * p_eel;
      t.enuc_s2 += p_enuc * p_enuc;
      t.coll_s2 += double(p_coll) * double(p_coll);
      if (n - spec.first < spec.records)
      {
        runspec::Record r{n, members, p_coll, p_vac, p_eel, p_enuc, last_x, last_y, last_z, last_state};
        runspec::print_record(stdout, r);
      }
    }
  }
};

} // namespace mto

int
main(int argc, char ** argv)
{
  if (argc < 2 || !mto::load_tables(argv[1]))
  {
    fprintf(stderr, "usage: mtoracle <stopping_tables.tsv> < spec\n");
    return 2;
  }
  if (argc >= 3 && std::string(argv[2]) == "--stopping")
  {
    // stopping-power service: lines "Z1 m1 E Z2" -> ion_stopping value
    int z1, z2;
    double m, E;
    while (std::cin >> z1 >> m >> E >> z2)
      printf("%.17g\n", mto::ion_stopping(z1, m, E, z2));
    return 0;
  }
  runspec::Spec spec;
  std::string err;
  if (!runspec::parse(std::cin, spec, err))
  {
    fprintf(stderr, "mtoracle: %s\n", err.c_str());
    return 2;
  }
  mto::Engine eng(spec);
  auto t0 = std::chrono::steady_clock::now();
  eng.run();
  auto t1 = std::chrono::steady_clock::now();
  eng.t.print(stdout);
  if (!spec.philox)
    printf("seed_sq %.17g\n", eng.seed_sq);
  printf("wall_s %.6f\n", std::chrono::duration<double>(t1 - t0).count());
  if (!spec.out_type.empty() && !eng.out.write())
  {
    fprintf(stderr, "mtoracle: cannot write %s output\n", spec.out_type.c_str());
    return 1;
  }
  return 0;
}
