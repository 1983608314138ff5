// Host replay build of the GPU engine's FP64 collision code (test infrastructure).
//
// Compiles the product's shared physics (mytrim_gb300/csrc/mtg_collide64.cuh,
// mtg_common.cuh) and table setup (mtg_setup.cpp) for the CPU with every multiply
// and add rounded separately (-ffp-contract=off), the same rounding the FP64 GPU
// engine is compiled with (-fmad=false).  It follows every cascade member of a
// run spec to rest and prints one record per member; the GPU engine's member
// records (mtg_get_records) must match these bit for bit, whatever order the GPU
// ran the members in, because every random number is keyed by the member's path
// and collision index.
//
// Usage: replay_host <stopping_tables.tsv> < spec     (spec format: runspec.h)
//
// Checks of single pieces of the same code, for the tests:
//   replay_host <tables> --stopping              "Z1 m1 rho n Z m t ...", then energies -> stopping (hex)
//   replay_host <tables> --scatter [potential]   lines "eps b" -> sin^2(theta/2) (hex)
//   replay_host <tables> --mathcheck [n]         exp64 / log64 short routes vs full forms
//   replay_host <tables> --eval exp|log|pow       lines of hex-float arguments -> results (hex)
//   replay_host <tables> --philox                lines of six hex words -> Philox outputs
//   replay_host <tables> --lookupcheck n < spec  cluster lookup with vs without the candidate lists

#include "runspec.h"

#include "mtg_collide64.cuh"
#include "mtg_geometry.cuh"
#include "mtg_setup.h"

#include <algorithm>
#include <cinttypes>
#include <vector>

using namespace mtg;

struct HostSink
{
  const SimDesc * sim;
  unsigned int m_vac = 0;
  int m_state = 0;
  double m_eel = 0.0;
  int range_mode = 0;

  void eel(double d, double, double, double) { m_eel += d; }
  void newton(int) {}
  void passes(int) {}
  void fallback() {}
  void numeric() {}
  void enuc(double, double, double, double) {}
  void unfollowed(double) {}
  template <class P>
  void history(const P &, int, double)
  {
  }
  template <class R, class E>
  void branch(const R &, const E &, uint64_t)
  {
  }
  template <class R, class E>
  void dissipate(const R &, double, const E &, uint64_t)
  {
  }
  template <class P>
  void lost(double, const P &, int, double)
  {
    m_state = ST_LOST;
  }
  template <class R, class E>
  void vacancy(const R & rec, const E & el, double Erec, uint64_t)
  {
    if (range_mode == 2)
    {
      // TrimPrimaries::vacancyCreation, as the engine's sink
      unsigned int add = 1;
      if (rec.gen == sim->kp_gen)
      {
        const double az = el.maz, am = el.mam;
        const double ed = 0.0115 * pow64(az, -7.0 / 3.0) * Erec;
        const double g = 3.4008 * pow64(ed, 1.0 / 6.0) + 0.40244 * pow64(ed, 3.0 / 4.0) + ed;
        const double kd = 0.1337 * pow64(az, 2.0 / 3.0) / sqrt(am);
        const double Ev = Erec / (1.0 + kd * g);
        add += (unsigned int)(int(0.8 * Ev / (2.0 * el.Edisp)));
      }
      m_vac += add;
      return;
    }
    if (range_mode)
    {
      const double Z = double(el.Z2), m = el.m2, Er = Erec;
      const double Ed = el.Edisp;
      const double ed = 0.0115 * pow64(Z, -7.0 / 3.0) * Er;
      const double kd = 0.1337 * pow64(Z, 2.0 / 3.0) / sqrt(m);
      const double g = 3.4008 * pow64(ed, 1.0 / 6.0) + 0.40244 * pow64(ed, 3.0 / 4.0) + ed;
      const double Ev = Er / (1.0 + kd * g);
      unsigned long long add = 0;
      if (Ev < Ed)
        add = 0;
      else if (Ev >= Ed / 0.4)
        add = (unsigned long long)(Ev * 0.4 / Ed);
      else
        add = 1;
      m_vac += (unsigned int)add;
      return;
    }
    ++m_vac;
  }
  template <class R, class E>
  void replacement(const R &, const E &, double, uint64_t)
  {
  }
  template <class P>
  void stop(int state, const P &, int, double)
  {
    m_state = state;
  }
};

int
main(int argc, char ** argv)
{
  if (argc < 2)
  {
    fprintf(stderr, "usage: replay_host <stopping_tables.tsv> < spec\n");
    return 2;
  }
  std::string err;
  mtg_scoef_row rows[MTG_SCOEF_ROWS];
  if (!read_table_file(argv[1], rows, err))
  {
    fprintf(stderr, "replay_host: %s\n", err.c_str());
    return 2;
  }
  if (argc >= 3 && std::string(argv[2]) == "--stopping")
  {
    // line 1: Z1 m1 rho n Z m t [Z m t ...]; then one energy per line
    int Z1, n;
    double m1, rho;
    std::cin >> Z1 >> m1 >> rho >> n;
    mtg_material mat;
    memset(&mat, 0, sizeof mat);
    mat.rho = rho;
    mat.n_elements = n;
    for (int j = 0; j < n && j < MTG_MAX_ELEMENTS; ++j)
    {
      std::cin >> mat.elements[j].Z >> mat.elements[j].m >> mat.elements[j].t;
      mat.elements[j].Edisp = 25.0;
      mat.elements[j].Elbind = 3.0;
    }
    SpeciesConst sc = make_species(rows, Z1, m1);
    MatConst mc;
    if (make_material(rows, sc, mat, 0.2, mc, err) != MTG_OK)
    {
      fprintf(stderr, "replay_host: %s\n", err.c_str());
      return 2;
    }
    double E;
    while (std::cin >> E)
      printf("%a\n", material_stop64(sc, mc, E));
    return 0;
  }
  if (argc >= 3 && std::string(argv[2]) == "--philox")
  {
    // lines "x y z w k0 k1" -> Philox4x32-10 of (x, y, z, w) under (k0, k1), then
    // Philox2x32-10 of (x, y) under k0 (hex words)
    unsigned long long v[6];
    while (std::cin >> std::hex >> v[0] >> v[1] >> v[2] >> v[3] >> v[4] >> v[5])
    {
      const U4 a = philox(U4{uint32_t(v[0]), uint32_t(v[1]), uint32_t(v[2]), uint32_t(v[3])}, uint32_t(v[4]),
                          uint32_t(v[5]));
      const U2 b = philox2(U2{uint32_t(v[0]), uint32_t(v[1])}, uint32_t(v[4]));
      printf("%08x %08x %08x %08x %08x %08x\n", a.x, a.y, a.z, a.w, b.x, b.y);
    }
    return 0;
  }
  if (argc >= 4 && std::string(argv[2]) == "--eval")
  {
    // lines of hex-float arguments -> the engine's exp64 / log64 (one argument) or
    // pow64 (two) of them, in hex
    const std::string f = argv[3];
    std::string line;
    while (std::getline(std::cin, line))
    {
      std::istringstream ls(line);
      std::string a, b;
      if (!(ls >> a))
        continue;
      const double x = std::strtod(a.c_str(), nullptr);
      double r;
      if (f == "exp")
        r = exp64(x);
      else if (f == "log")
        r = log64(x);
      else if (f == "pow" && (ls >> b))
        r = pow64(x, std::strtod(b.c_str(), nullptr));
      else
        return 2;
      printf("%a\n", r);
    }
    return 0;
  }
  if (argc >= 3 && std::string(argv[2]) == "--mathcheck")
  {
    // exp64 / log64 (short routes) against exp64_wide / log64_wide bit for bit on n
    // inputs: random bit patterns, random values of every magnitude, the edges of
    // the short routes; prints "checked mismatches"
    const long long n = argc >= 4 ? atoll(argv[3]) : 1000000;
    uint64_t st = 0x9e3779b97f4a7c15ull;
    auto next = [&]() {
      st += 0x9e3779b97f4a7c15ull;
      uint64_t z = st;
      z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
      z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
      return z ^ (z >> 31);
    };
    const double edges[] = {0.0, -0.0, 704.0, -704.0, 703.9999999999999, -703.9999999999999, 709.7, -745.2,
                            1.0, 0x1.6a09e667f3bcdp+0, 0x1.6a09e667f3bcep+0, 0x1p-1022, 0x1p-1023, 0x1.fffffffffffffp+1023,
                            HUGE_VAL, -HUGE_VAL, NAN, 0.703125, 0.70710678118654757};
    long long bad = 0, checked = 0;
    auto check = [&](double x) {
      const uint64_t a = double_to_bits(exp64(x)), b = double_to_bits(exp64_wide(x));
      const uint64_t c = double_to_bits(log64(x)), d = double_to_bits(log64_wide(x));
      const bool nan_ab = exp64(x) != exp64(x) && exp64_wide(x) != exp64_wide(x);
      const bool nan_cd = log64(x) != log64(x) && log64_wide(x) != log64_wide(x);
      if ((a != b && !nan_ab) || (c != d && !nan_cd))
      {
        if (bad < 5)
          printf("mismatch x=%a exp %a %a log %a %a\n", x, exp64(x), exp64_wide(x), log64(x), log64_wide(x));
        ++bad;
      }
      ++checked;
    };
    for (double x : edges)
      check(x);
    for (long long i = 0; i < n; ++i)
    {
      const uint64_t r = next();
      check(bits_to_double(r));                                          // any bit pattern
      check(double(int64_t(r >> 11) - (1ll << 52)) * 0x1p-43);           // |x| < 512
      check(ldexp(double(r >> 11) * 0x1p-53, int(next() % 2100) - 1074)); // every magnitude
      check((double(r >> 11) * 0x1p-53 - 0.5) * 1500.0);                 // around the exp edges
    }
    printf("%lld %lld\n", checked, bad);
    return bad ? 1 : 0;
  }
  if (argc >= 3 && std::string(argv[2]) == "--scatter")
  {
    // lines "eps b" -> s2; an optional argument after --scatter picks the potential
    const int pot = argc >= 4 ? atoi(argv[3]) : 0;
    double eps, b;
    while (std::cin >> eps >> b)
    {
      double s2, ct, st;
      int it;
      scatter64(eps, b, s2, ct, st, it, pot);
      printf("%a\n", s2);
    }
    return 0;
  }
  runspec::Spec spec;
  if (!runspec::parse(std::cin, spec, err))
  {
    fprintf(stderr, "replay_host: %s\n", err.c_str());
    return 2;
  }
  if (spec.layers.size() > MTG_MAX_LAYERS)
  {
    fprintf(stderr, "replay_host: too many layers\n");
    return 2;
  }
  mtg_sim sim;
  memset(&sim, 0, sizeof sim);
  sim.sample.n_layers = int(spec.layers.size());
  for (size_t k = 0; k < spec.layers.size(); ++k)
  {
    sim.sample.thickness[k] = spec.layers[k].thickness;
    mtg_material & m = sim.sample.material[k];
    m.rho = spec.layers[k].rho;
    m.n_elements = int(spec.layers[k].el.size());
    for (int j = 0; j < m.n_elements && j < MTG_MAX_ELEMENTS; ++j)
    {
      const auto & e = spec.layers[k].el[j];
      m.elements[j] = mtg_element{e.Z, e.m, e.t, e.Edisp, e.Elbind};
    }
  }
  for (int i = 0; i < 3; ++i)
  {
    sim.sample.w[i] = spec.size[i];
    sim.sample.bc[i] = spec.bc[i];
    sim.ion.dir[i] = spec.dir[i];
    sim.ion.pos[i] = spec.pos[i];
  }
  sim.ion.Z = spec.Z;
  sim.ion.m = spec.m;
  sim.ion.E = spec.E;
  sim.ion.Ef = spec.Ef;
  sim.n_primaries = spec.count;
  sim.first_primary = 0;
  sim.tally_mode = spec.primaries_mode ? MTG_TALLY_PRIMARIES : (spec.range_mode ? MTG_TALLY_RANGE : MTG_TALLY_VACCOUNT);
  sim.max_generation = spec.max_gen;
  sim.primaries_only = spec.primaries_only;
  sim.potential = spec.potential;
  if (spec.clusters)
  {
    sim.sample.geometry = MTG_GEOM_CLUSTERS;
    for (int i = 0; i < 3; ++i)
      sim.sample.cluster_hash[i] = spec.kn[i];
    sim.sample.n_clusters = (long long)(spec.cl.size() / 4);
    sim.sample.clusters = spec.cl.data();
  }
  mtg_config cfg;
  memset(&cfg, 0, sizeof cfg);
  cfg.tmin = 0.2;
  cfg.tau = 0.0;
  cfg.cw = 0.001;
  cfg.length_scale = spec.scale;
  cfg.seed = spec.seed;
  HostTables t;
  if (build_tables(rows, cfg, &sim, 1, t, err) != MTG_OK)
  {
    fprintf(stderr, "replay_host: %s\n", err.c_str());
    return 2;
  }
  patch_cluster_pointers(t.sims, t.clusters.data(), t.cl_next.data(), t.cl_head.data(), t.cl_mask.data());
  const SimDesc & sd = t.sims[0];
  if (argc >= 4 && std::string(argv[2]) == "--lookupcheck" && sd.geometry == 1)
  {
    // the cluster lookup with and without the candidate lists, in double and in float,
    // at n random points: inside the box, within 64 box lengths on periodic axes,
    // and near cluster surfaces; prints "checked mismatches"
    const long long n = atoll(argv[3]);
    std::vector<Cl4f> c32(t.clusters.size());
    for (size_t l = 0; l < c32.size(); ++l)
      c32[l] = Cl4f{float(t.clusters[l].x), float(t.clusters[l].y), float(t.clusters[l].z), float(t.clusters[l].r)};
    const float w32[3] = {float(sd.w[0]), float(sd.w[1]), float(sd.w[2])};
    const float kd32[3] = {float(sd.kd[0]), float(sd.kd[1]), float(sd.kd[2])};
    const float im32[3] = {float(sd.inv_mcell[0]), float(sd.inv_mcell[1]), float(sd.inv_mcell[2])};
    uint64_t st = 12345;
    auto uni = [&]() {
      st = st * 6364136223846793005ull + 1442695040888963407ull;
      return double(st >> 11) * 0x1p-53;
    };
    long long bad = 0;
    for (long long i = 0; i < n; ++i)
    {
      double q[3];
      const int kind = int(i % 3);
      if (kind == 2 && !t.clusters.empty())
      {
        // near a cluster surface (and its periodic images)
        const Cl4d & c = t.clusters[size_t(uni() * double(t.clusters.size())) % t.clusters.size()];
        double v[3], vv = 0.0;
        for (int k = 0; k < 3; ++k)
        {
          v[k] = uni() - 0.5;
          vv += v[k] * v[k];
        }
        const double rad = c.r * (1.0 + (uni() - 0.5) * 1e-6);
        const double shift[3] = {(&c.x)[0], (&c.x)[1], (&c.x)[2]};
        for (int k = 0; k < 3; ++k)
          q[k] = shift[k] + v[k] / std::sqrt(vv) * rad + (sd.bc[k] == 0 ? sd.w[k] * double(int(uni() * 9.0) - 4) : 0.0);
      }
      else
        for (int k = 0; k < 3; ++k)
          q[k] = sd.bc[k] == 0 && kind == 1 ? (uni() - 0.5) * 120.0 * sd.w[k] : uni() * sd.w[k];
      const int a = cluster_lookup<double>(q, sd.w, sd.bc, sd.kn, sd.kd, sd.cmr, sd.cl, sd.cl_next, sd.cl_head,
                                           sd.n_clusters, sd.cl_mask, sd.mn, sd.inv_mcell);
      const int b = cluster_lookup<double>(q, sd.w, sd.bc, sd.kn, sd.kd, sd.cmr, sd.cl, sd.cl_next, sd.cl_head,
                                           sd.n_clusters, nullptr, sd.mn, sd.inv_mcell);
      const float qf[3] = {float(q[0]), float(q[1]), float(q[2])};
      const int af = cluster_lookup<float>(qf, w32, sd.bc, sd.kn, kd32, float(sd.cmr), c32.data(), sd.cl_next,
                                           sd.cl_head, sd.n_clusters, sd.cl_mask, sd.mn, im32);
      const int bf = cluster_lookup<float>(qf, w32, sd.bc, sd.kn, kd32, float(sd.cmr), c32.data(), sd.cl_next,
                                           sd.cl_head, sd.n_clusters, nullptr, sd.mn, im32);
      if (a != b || af != bf)
      {
        if (bad < 5)
          printf("mismatch %.17g %.17g %.17g: %d %d / %d %d\n", q[0], q[1], q[2], a, b, af, bf);
        ++bad;
      }
    }
    // cells with candidates, and those of them marked for the hash search
    long long listed = 0, marked = 0;
    const long long ncell = (long long)sd.mn[0] * sd.mn[1] * sd.mn[2];
    for (long long q = 0; q < ncell; ++q)
    {
      const uint32_t s0 = sd.cl_mask[q], s1 = sd.cl_mask[q + 1] & 0x7fffffffu;
      if (s0 & 0x80000000u)
        ++marked;
      else if (s1 > s0)
        ++listed;
    }
    printf("cells %lld %lld\n", listed, marked);
    printf("%lld %lld\n", n, bad);
    return bad ? 1 : 0;
  }
  std::vector<P64> stack;
  for (long long n = spec.first; n < spec.first + spec.n; ++n)
  {
    P64 p;
    p.x = sd.pos[0];
    p.y = sd.pos[1];
    p.z = sd.pos[2];
    p.dx = sd.dir[0];
    p.dy = sd.dir[1];
    p.dz = sd.dir[2];
    p.E = sd.E0;
    p.key = root_key(sd.sim_key, uint64_t(n));
    p.species = 0;
    p.gen = 0;
    p.sim = 0;
    p.prim = uint32_t(n);
    p.tag = -1;
    stack.push_back(p);
    while (!stack.empty())
    {
      P64 m = stack.back();
      stack.pop_back();
      const SpeciesConst & sc = t.species[sd.species_base + m.species];
      const MatConst * mrow = &t.mats[sd.mat_base + m.species * sd.n_mat];
      const double r1 = key_u53(m.key);
      HostSink sink;
      sink.sim = &sd;
      sink.range_mode = sd.range_mode;
      uint32_t ic = 0;
      int flags = 0;
      do
      {
        ++ic;
        P64 rec;
        flags = collide64<true>(m, ic, r1, sd, sc, mrow, t.k0, t.k1, rec, sink);
        if (flags & CF_PUSH)
        {
          rec.sim = m.sim;
          rec.prim = m.prim;
          stack.push_back(rec);
        }
      } while (!(flags & CF_DONE) && ic < (1u << 24));
      printf("%" PRIu64 " %d %d %d %u %u %a %a %a %a %a\n", m.key, m.species, m.gen, sink.m_state, ic,
             sink.m_vac, m.E, m.x, m.y, m.z, sink.m_eel);
    }
  }
  return 0;
}
