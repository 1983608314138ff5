// runmytrim_gpu: the reference's runmytrim driver (apps/runmytrim.C) on the GB300
// cascade engine.
//
//   runmytrim_gpu [--precision fp64|fp32|surrogate] [--device N] [--tables FILE]
//                 [--surrogate-params FILE.npy] [--check-input] < input.json
//
// --check-input reads and checks the input, prints the simulation it describes
// (one "key values" line per item) and exits without touching the GPU.
//
// It reads the same JSON input (runmytrim.C:103-285; // and /* */ comments
// allowed), rejects the same malformed inputs with the same messages ("ERROR: ..."
// on stderr, exit status 1), runs every primary as one GPU batch through the
// C ABI (include/mytrim_gpu.h) and writes the output file of the chosen plugin in
// the reference's format:
//   vaccount        <base>_vac.dat    "x vacancies replacements" per 1-unit depth bin
//                                     (apps/src/TrimVacCount.C:70-79)
//   vacenergycount  <base>_evac.dat   "E x count" per int(ln E) row and depth bin, a
//                                     blank line after each row (TrimVacEnergyCount.C:71-81)
//   range           <base>_ranges.dat histogram of the x of every dissipated recoil by
//                                     recoil Z, bin width chosen from the data
//                                     (TrimRange.C:67-121)
// then the two summary lines of runmytrim.C:326-329 on stderr.
//
// Differences, by design: the random streams are the engine's counter-based
// streams keyed by the master seed (the statistics match, the individual
// cascades do not); options.threads is accepted and ignored (one GPU runs every
// primary); without options.seed a seed is drawn from /dev/urandom.  The default
// precision is fp64, the reference's arithmetic.  The depth histograms live on the
// device with a fixed number of bins; a run that records events past the last
// bin is repeated with four times the bins (the result does not depend on the
// bin count, so the repeat reproduces the same cascades).
#include "json_lite.h"
#include "mytrim_gpu.h"

#include <unistd.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <iterator>
#include <sstream>
#include <string>
#include <vector>

namespace
{

struct InputError
{
  std::string msg;
};

[[noreturn]] void
input_error(const std::string & m)
{
  throw InputError{m};
}

struct Run
{
  mtg_sim sim;
  std::string type, base;
  unsigned long long seed = 0;
  double scale = 1.0;
  long long npka = 0;
};

// apps/runmytrim.C:103-304, the same checks in the same order
Run
read_input(const mtg_json::Value & top)
{
  Run r;
  std::memset(&r.sim, 0, sizeof r.sim);
  if (!top["mytrim"].isObject())
    input_error("No 'mytrim' top level block found in input");
  const mtg_json::Value & root = top["mytrim"];
  const mtg_json::Value & opt = root["options"];
  if (opt.isObject() && opt["threads"].isNumeric())
    std::cerr << "Using " << opt["threads"].asInt() << " threads\n";
  bool have_seed = false;
  if (opt.isObject())
  {
    if (opt["seed"].isNumeric())
    {
      r.seed = (unsigned long long)(unsigned int)int(opt["seed"].asInt());
      have_seed = true;
      std::cerr << "Using provided master seed " << int(opt["seed"].asInt()) << '\n';
    }
    if (opt["scale"].isNumeric())
    {
      r.scale = opt["scale"].asDouble();
      std::cerr << "Using provided length scale " << r.scale << '\n';
    }
  }
  if (!have_seed)
  {
    unsigned int s = 0;
    std::ifstream ur("/dev/urandom", std::ios::binary);
    if (!ur.read(reinterpret_cast<char *>(&s), sizeof s))
      input_error("Unable to access /dev/urandom");
    r.seed = s;
  }

  const mtg_json::Value & sample = root["sample"];
  if (!sample.isObject())
    input_error("Must specify a 'sample' block in the input file");
  const mtg_json::Value & layers = sample["layers"];
  if (!layers.isArray())
    input_error("sample.layers must be an array");
  const size_t nlayers = layers.size();
  std::cerr << "Building " << nlayers << " layers\n";
  double thickness = 0.0;
  for (size_t i = 0; i < nlayers; ++i)
    if (layers[i]["thickness"].isNumeric())
      thickness += layers[i]["thickness"].asDouble();
    else
      input_error("No 'thickness' found for layer " + std::to_string(i));
  if (nlayers < 1 || nlayers > MTG_MAX_LAYERS)
    input_error("this engine supports 1 to " + std::to_string(MTG_MAX_LAYERS) + " layers");

  const mtg_json::Value & out = root["output"];
  if (!out.isObject())
    input_error("Must specify an 'output' block in the input file");
  if (!out["type"].isString())
    input_error("output.type must be a string");
  r.type = out["type"].asString();
  if (r.type != "vaccount" && r.type != "vacenergycount" && r.type != "range")
    input_error("Unknown output type " + r.type);
  if (out["base"].isString())
    r.base = out["base"].asString();
  const bool primaries_only = out["primaries_only"].isBool() && out["primaries_only"].asBool();

  mtg_sim & s = r.sim;
  s.sample.n_layers = int(nlayers);
  // one Element object is filled for all layers: an omitted edisp / elbind keeps
  // the previous element's value (runmytrim.C:208-251)
  double edisp = 25.0, elbind = 3.0;
  for (size_t i = 0; i < nlayers; ++i)
  {
    const mtg_json::Value & L = layers[i];
    if (!L["rho"].isNumeric())
      input_error("Missing 'rho' in layer " + std::to_string(i));
    if (!L["elements"].isArray())
      input_error("Missing 'elements' in layer " + std::to_string(i));
    const mtg_json::Value & els = L["elements"];
    if (els.size() > MTG_MAX_ELEMENTS)
      input_error("this engine supports at most " + std::to_string(MTG_MAX_ELEMENTS) + " elements per layer");
    mtg_material & m = s.sample.material[i];
    m.rho = L["rho"].asDouble();
    m.n_elements = int(els.size());
    for (size_t j = 0; j < els.size(); ++j)
    {
      const mtg_json::Value & E = els[j];
      const std::string where = " in element " + std::to_string(j) + " in layer " + std::to_string(i);
      if (!E["Z"].isNumeric())
        input_error("Missing 'Z'" + where);
      if (!E["mass"].isNumeric())
        input_error("Missing 'mass'" + where);
      if (!E["fraction"].isNumeric())
        input_error("Missing 'fraction'" + where);
      if (E["edisp"].isNumeric())
        edisp = E["edisp"].asDouble();
      if (E["elbind"].isNumeric())
        elbind = E["elbind"].asDouble();
      m.elements[j].Z = int(E["Z"].asInt());
      m.elements[j].m = E["mass"].asDouble();
      m.elements[j].t = E["fraction"].asDouble();
      m.elements[j].Edisp = edisp;
      m.elements[j].Elbind = elbind;
    }
    s.sample.thickness[i] = L["thickness"].asDouble();
  }
  // SampleLayers(thickness, 100, 100) with periodic boundaries (sample.C:31)
  s.sample.w[0] = thickness;
  s.sample.w[1] = 100.0;
  s.sample.w[2] = 100.0;
  for (int i = 0; i < 3; ++i)
    s.sample.bc[i] = MTG_BC_PBC;

  const mtg_json::Value & ion = root["ion"];
  if (!ion.isObject())
    input_error("Must specify an 'ion' block in the input file");
  if (!ion["Z"].isNumeric())
    input_error("Missing 'Z' in ion block");
  if (!ion["mass"].isNumeric())
    input_error("Missing 'mass' in ion block");
  if (!ion["energy"].isNumeric())
    input_error("Missing 'energy' in ion block");
  if (!ion["number"].isNumeric())
    input_error("Missing 'number' in ion block");
  s.ion.Z = int(ion["Z"].asInt());
  s.ion.m = ion["mass"].asDouble();
  s.ion.E = ion["energy"].asDouble();
  s.ion.Ef = ion["final_energy"].isNumeric() ? ion["final_energy"].asDouble() : 3.0;
  s.ion.dir[0] = 1.0;
  s.ion.pos[1] = s.sample.w[1] / 2.0;
  s.ion.pos[2] = s.sample.w[2] / 2.0;
  r.npka = (long long)(unsigned int)int(ion["number"].asInt());
  s.n_primaries = r.npka;
  s.tally_mode = r.type == "range" ? MTG_TALLY_RANGE : MTG_TALLY_VACCOUNT;
  s.primaries_only = primaries_only ? 1 : 0;
  return r;
}

// little-endian float32 .npy (version 1 or 2) with `n` values
bool
read_npy_f32(const std::string & path, std::vector<float> & out, size_t n)
{
  std::ifstream f(path, std::ios::binary);
  std::string data((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
  if (data.size() < 12 || data.compare(0, 6, "\x93NUMPY") != 0)
    return false;
  const int major = (unsigned char)data[6];
  size_t hlen, off;
  if (major == 1)
  {
    hlen = (unsigned char)data[8] | ((size_t)(unsigned char)data[9] << 8);
    off = 10;
  }
  else
  {
    hlen = (unsigned char)data[8] | ((size_t)(unsigned char)data[9] << 8) |
           ((size_t)(unsigned char)data[10] << 16) | ((size_t)(unsigned char)data[11] << 24);
    off = 12;
  }
  const std::string header = data.substr(off, hlen);
  if (header.find("'<f4'") == std::string::npos || header.find("'fortran_order': False") == std::string::npos)
    return false;
  off += hlen;
  if (data.size() < off + 4 * n)
    return false;
  out.resize(n);
  for (size_t i = 0; i < n; ++i)
  {
    const unsigned char * p = reinterpret_cast<const unsigned char *>(data.data() + off + 4 * i);
    const uint32_t u = uint32_t(p[0]) | (uint32_t(p[1]) << 8) | (uint32_t(p[2]) << 16) | (uint32_t(p[3]) << 24);
    std::memcpy(&out[i], &u, 4);
  }
  return true;
}

std::string
exe_dir()
{
  char buf[4096];
  const ssize_t n = readlink("/proc/self/exe", buf, sizeof buf - 1);
  if (n <= 0)
    return ".";
  buf[n] = '\0';
  std::string p(buf);
  const size_t k = p.rfind('/');
  return k == std::string::npos ? "." : p.substr(0, k);
}

// last index with a nonzero count, plus one
size_t
used_size(const long long * h, size_t n)
{
  while (n > 0 && h[n - 1] == 0)
    --n;
  return n;
}

bool
write_vac(const std::string & base, const long long * vac, const long long * repl, size_t n)
{
  const size_t size = std::max(used_size(vac, n), used_size(repl, n));
  std::ofstream out(base + "_vac.dat");
  for (size_t x = 0; x < size; ++x)
    out << x << ' ' << (unsigned int)vac[x] << ' ' << (unsigned int)repl[x] << '\n';
  return bool(out);
}

bool
write_evac(const std::string & base, const long long * evac, int rows, size_t n)
{
  int used_rows = 0;
  for (int e = 0; e < rows; ++e)
    if (used_size(evac + size_t(e) * n, n) > 0)
      used_rows = e + 1;
  std::ofstream out(base + "_evac.dat");
  for (int e = 0; e < used_rows; ++e)
  {
    const long long * row = evac + size_t(e) * n;
    const size_t size = used_size(row, n);
    for (size_t x = 0; x < size; ++x)
      out << (unsigned int)e << ' ' << x << ' ' << (unsigned int)row[x] << '\n';
    out << '\n';
  }
  return bool(out);
}

bool
write_ranges(const std::string & base, const std::vector<std::vector<double>> & range)
{
  unsigned int max_samples = 0;
  double x_min = 0.0, x_max = 0.0;
  for (auto & r : range)
  {
    max_samples = std::max(max_samples, (unsigned int)r.size());
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
    return bool(out); // nothing to bin: header only
  const double bin = std::min(xwidth * 100.0 / max_samples, xwidth / 10.0);
  const unsigned int nbin = (unsigned int)(xwidth / bin + 1);
  std::vector<std::vector<unsigned int>> hist;
  for (auto & r : range)
  {
    if (r.empty())
      continue;
    hist.emplace_back(nbin, 0u);
    for (double x : r)
      hist.back()[(size_t)std::floor((x - x_min) / bin)]++;
  }
  for (unsigned int k = 0; k < nbin; ++k)
  {
    out << (k * bin + x_min);
    for (auto & h : hist)
      out << ' ' << h[k];
    out << '\n';
  }
  return bool(out);
}

void
print_run(const Run & r)
{
  const mtg_sim & s = r.sim;
  std::printf("type %s\nbase %s\nseed %llu\nscale %.17g\nprimaries %lld\nprimaries_only %d\n", r.type.c_str(),
              r.base.c_str(), r.seed, r.scale, r.npka, s.primaries_only);
  std::printf("ion %d %.17g %.17g %.17g\n", s.ion.Z, s.ion.m, s.ion.E, s.ion.Ef);
  std::printf("box %.17g %.17g %.17g\n", s.sample.w[0], s.sample.w[1], s.sample.w[2]);
  for (int i = 0; i < s.sample.n_layers; ++i)
  {
    const mtg_material & m = s.sample.material[i];
    std::printf("layer %.17g %.17g\n", s.sample.thickness[i], m.rho);
    for (int j = 0; j < m.n_elements; ++j)
      std::printf("element %d %.17g %.17g %.17g %.17g\n", m.elements[j].Z, m.elements[j].m, m.elements[j].t,
                  m.elements[j].Edisp, m.elements[j].Elbind);
  }
}

int
engine_error(mtg_ctx * ctx, const char * what, mtg_status st)
{
  std::cerr << "ERROR: " << what << " failed (status " << int(st) << "): " << mtg_last_error(ctx) << '\n';
  return 1;
}

} // namespace

int
main(int argc, char ** argv)
{
  std::string precision = "fp64", tables, sg_params;
  int device = 0;
  bool check_only = false;
  for (int i = 1; i < argc; ++i)
  {
    const std::string a = argv[i];
    auto next = [&]() -> std::string {
      if (i + 1 >= argc)
      {
        std::cerr << "ERROR: " << a << " needs a value\n";
        std::exit(1);
      }
      return argv[++i];
    };
    if (a == "--precision")
      precision = next();
    else if (a == "--device")
      device = std::atoi(next().c_str());
    else if (a == "--tables")
      tables = next();
    else if (a == "--surrogate-params")
      sg_params = next();
    else if (a == "--check-input")
      check_only = true;
    else
    {
      std::cerr << "ERROR: Please supply the input file via stdin (e.g. ./runmytrim_gpu < input.json); "
                   "options: --precision fp64|fp32|surrogate, --device N, --tables FILE, "
                   "--surrogate-params FILE, --check-input\n";
      return 1;
    }
  }
  int prec;
  if (precision == "fp64")
    prec = MTG_PREC_FP64;
  else if (precision == "fp32")
    prec = MTG_PREC_FP32;
  else if (precision == "surrogate")
    prec = MTG_PREC_FP32_SURROGATE;
  else
  {
    std::cerr << "ERROR: unknown precision " << precision << '\n';
    return 1;
  }
  const std::string data = exe_dir() + "/../data/";
  if (tables.empty())
    tables = data + "stopping_tables.tsv";
  if (sg_params.empty())
    sg_params = data + "surrogate_params.npy";

  // parse and check the whole input before touching the GPU
  std::string text((std::istreambuf_iterator<char>(std::cin)), std::istreambuf_iterator<char>());
  mtg_json::Value top;
  std::string perr;
  if (!mtg_json::parse(text, top, perr))
  {
    std::cerr << "ERROR: cannot parse the input: " << perr << '\n';
    return 1;
  }
  Run run;
  try
  {
    run = read_input(top);
  }
  catch (const InputError & e)
  {
    std::cerr << "ERROR: " << e.msg << '\n' << std::flush;
    return 1;
  }
  if (check_only)
  {
    print_run(run);
    return 0;
  }

  mtg_ctx * ctx = nullptr;
  mtg_status st = mtg_create(device, &ctx);
  if (st != MTG_OK)
  {
    std::cerr << "ERROR: no usable CUDA device " << device << " (status " << int(st) << ")\n";
    return 1;
  }
  struct Closer
  {
    mtg_ctx * c;
    ~Closer() { mtg_destroy(c); }
  } closer{ctx};
  if ((st = mtg_load_tables(ctx, tables.c_str())) != MTG_OK)
    return engine_error(ctx, "loading the stopping tables", st);
  mtg_config cfg;
  std::memset(&cfg, 0, sizeof cfg);
  cfg.tmin = 0.2; // runmytrim.C:126
  cfg.tau = 0.0;
  cfg.cw = 0.001;
  cfg.length_scale = run.scale;
  cfg.precision = prec;
  cfg.seed = run.seed;
  if (prec == MTG_PREC_FP32_SURROGATE)
  {
    std::vector<float> p;
    if (!read_npy_f32(sg_params, p, MTG_SURROGATE_NPARAM))
    {
      std::cerr << "ERROR: cannot read the surrogate parameters " << sg_params << '\n';
      return 1;
    }
    if ((st = mtg_surrogate_set_params(ctx, p.data(), (long long)p.size())) != MTG_OK)
      return engine_error(ctx, "loading the surrogate", st);
  }
  if ((st = mtg_configure(ctx, &cfg)) != MTG_OK)
    return engine_error(ctx, "configuring the engine", st);

  mtg_sim & sim = run.sim;
  const bool range = run.type == "range";
  const bool evac = run.type == "vacenergycount";
  // depth bins of 1 length unit, as int(x) in the reference
  long long nbins = std::min<long long>(std::max<long long>((long long)std::ceil(sim.sample.w[0]) + 2, 4096), 65536);
  const int rows = evac ? std::max(1, int(std::log(std::max(sim.ion.E, 1.0))) + 2) : 0;
  long long ev_cap = range ? std::max<long long>(1 << 20, 64 * run.npka) : 0;
  mtg_totals tot;
  std::vector<long long> hist;
  for (int attempt = 0;; ++attempt)
  {
    sim.hist_vac_bin = 1.0;
    sim.hist_vac_n = range ? 0 : int(nbins);
    sim.hist_evac_rows = rows;
    if ((st = mtg_set_event_log(ctx, range ? (1u << MTG_EV_DISSIPATE) : 0u, ev_cap)) != MTG_OK)
      return engine_error(ctx, "setting up the event log", st);
    const long long nh = sim.hist_vac_n * (2LL + rows);
    hist.assign(size_t(std::max<long long>(nh, 1)), 0);
    st = mtg_run(ctx, &sim, 1, &tot, hist.data());
    long long n_written = 0, n_total = 0;
    if (range && st == MTG_ERR_QUEUE_FULL)
    {
      mtg_get_events(ctx, nullptr, 0, &n_written, &n_total);
      if (n_total > ev_cap && attempt < 4)
      {
        ev_cap = n_total + n_total / 8 + 1024; // the repeat logs exactly as many events
        continue;
      }
    }
    if (st != MTG_OK)
      return engine_error(ctx, "the cascade run", st);
    if (tot.hist_dropped > 0 && !range)
    {
      if (nbins >= (1LL << 25))
      {
        std::cerr << "ERROR: vacancies deeper than " << nbins << " length units\n";
        return 1;
      }
      nbins *= 4;
      continue;
    }
    break;
  }

  bool ok = true;
  if (run.type == "vaccount")
    ok = write_vac(run.base, hist.data(), hist.data() + nbins, size_t(nbins));
  else if (evac)
    ok = write_evac(run.base, hist.data() + 2 * nbins, rows, size_t(nbins));
  else
  {
    std::vector<mtg_event> ev(size_t(std::max<long long>(ev_cap, 1)));
    long long n_written = 0, n_total = 0;
    if ((st = mtg_get_events(ctx, ev.data(), ev_cap, &n_written, &n_total)) != MTG_OK)
      return engine_error(ctx, "reading the event log", st);
    std::vector<std::vector<double>> samples(112);
    for (long long i = 0; i < n_written; ++i)
      if (ev[i].Z >= 0 && ev[i].Z < 112)
        samples[ev[i].Z].push_back(ev[i].x);
    ok = write_ranges(run.base, samples);
  }
  if (!ok)
  {
    std::cerr << "ERROR: cannot write the output file for base '" << run.base << "'\n";
    return 1;
  }
  const double n = double(run.npka);
  std::cerr << "Vacancies/ion: " << double(tot.vacancies) / n << '\n'
            << "Electronic energy loss/ion: " << tot.Eel / n << '\n';
  return 0;
}
