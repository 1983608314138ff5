// runstopping_gpu: the reference's runstopping driver (apps/runstopping.C) on the
// GB300 engine's stopping service.
//
//   runstopping_gpu [--precision fp64|fp32] [--device N] [--tables FILE] < input.json
//
// It reads the same JSON input (a "stopping" block with a material and an ion
// whose energy is a number, an array, or a {begin, end, step | mult} range;
// runstopping.C:66-175), rejects malformed inputs with the same messages
// ("ERROR: ..." on stderr, exit status 1, all checks done before the GPU is
// touched), evaluates the electronic stopping of every energy in one call of
// mtg_stopping (include/mytrim_gpu.h) and prints "E S_e" per line as
// runstopping.C:175-179 does (S_e in eV/Angstrom, MaterialBase::getrstop).
// fp64 (default) is the reference's formula in double precision; fp32 reads the
// FP32 cascade engine's stopping table.
#include "json_lite.h"
#include "mytrim_gpu.h"

#include <unistd.h>

#include <cstdio>
#include <cstring>
#include <iostream>
#include <iterator>
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

struct Request
{
  int Z1 = 0;
  double m1 = 0.0;
  mtg_material mat;
  std::vector<double> energies;
};

Request
read_input(const mtg_json::Value & top)
{
  Request r;
  std::memset(&r.mat, 0, sizeof r.mat);
  if (!top["stopping"].isObject())
    input_error("No 'stopping' top level block found in input");
  const mtg_json::Value & root = top["stopping"];
  const mtg_json::Value & mat = root["material"];
  if (!mat.isObject())
    input_error("Must specify a 'material' block in the input file");
  if (!mat["rho"].isNumeric())
    input_error("Missing 'rho'");
  r.mat.rho = mat["rho"].asDouble();
  if (!mat["elements"].isArray())
    input_error("Missing 'elements' in material");
  const mtg_json::Value & els = mat["elements"];
  if (els.size() > MTG_MAX_ELEMENTS)
    input_error("this engine supports at most " + std::to_string(MTG_MAX_ELEMENTS) + " elements per material");
  r.mat.n_elements = int(els.size());
  for (size_t j = 0; j < els.size(); ++j)
  {
    const mtg_json::Value & E = els[j];
    if (!E["Z"].isNumeric())
      input_error("Missing 'Z' in element " + std::to_string(j));
    if (!E["mass"].isNumeric())
      input_error("Missing 'mass' in element " + std::to_string(j));
    if (!E["fraction"].isNumeric())
      input_error("Missing 'fraction' in element " + std::to_string(j));
    r.mat.elements[j].Z = int(E["Z"].asInt());
    r.mat.elements[j].m = E["mass"].asDouble();
    r.mat.elements[j].t = E["fraction"].asDouble();
    r.mat.elements[j].Edisp = 25.0; // not used by the stopping
    r.mat.elements[j].Elbind = 3.0;
  }

  const mtg_json::Value & ion = root["ion"];
  if (!ion.isObject())
    input_error("Must specify an 'ion' block in the input file");
  if (!ion["Z"].isNumeric())
    input_error("Missing 'Z' in ion block");
  r.Z1 = int(ion["Z"].asInt());
  if (!ion["mass"].isNumeric())
    input_error("Missing 'mass' in ion block");
  r.m1 = ion["mass"].asDouble();

  // a number, an array, or a range with a step or a factor (runstopping.C:128-169)
  const mtg_json::Value & en = ion["energy"];
  if (en.isNumeric())
    r.energies.push_back(en.asDouble());
  else if (en.isArray())
  {
    for (size_t j = 0; j < en.size(); ++j)
      r.energies.push_back(en[j].asDouble());
  }
  else if (en.isObject())
  {
    if (!en["begin"].isNumeric())
      input_error("Missing 'begin' in energy block");
    const double ebegin = en["begin"].asDouble();
    if (!en["end"].isNumeric())
      input_error("Missing 'end' in energy block");
    const double eend = en["end"].asDouble();
    const bool has_step = en["step"].isNumeric();
    const bool has_mult = en["mult"].isNumeric();
    if (has_step == has_mult)
      input_error("Specify either 'step' or 'mult' energy block");
    // the same accumulation as the reference, so the energies are the same doubles
    if (has_step)
    {
      const double estep = en["step"].asDouble();
      if (!(estep > 0.0))
        input_error("'step' must be positive");
      for (double E = ebegin; E <= eend; E += estep)
        r.energies.push_back(E);
    }
    if (has_mult)
    {
      const double emult = en["mult"].asDouble();
      if (emult <= 1.0)
        input_error("'mult' must be larger than 1.0");
      for (double E = ebegin; E <= eend; E *= emult)
        r.energies.push_back(E);
    }
  }
  else
    input_error("Missing or invalid 'energy' in ion block");
  return r;
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

} // namespace

int
main(int argc, char ** argv)
{
  std::string precision = "fp64", tables;
  int device = 0;
  for (int i = 1; i < argc; ++i)
  {
    const std::string a = argv[i];
    if ((a == "--precision" || a == "--device" || a == "--tables") && i + 1 < argc)
    {
      const std::string v = argv[++i];
      if (a == "--precision")
        precision = v;
      else if (a == "--device")
        device = std::atoi(v.c_str());
      else
        tables = v;
    }
    else
    {
      std::cerr << "ERROR: Please supply the input file via stdin (e.g. ./runstopping_gpu < input.json); "
                   "options: --precision fp64|fp32, --device N, --tables FILE\n";
      return 1;
    }
  }
  if (precision != "fp64" && precision != "fp32")
  {
    std::cerr << "ERROR: unknown precision " << precision << '\n';
    return 1;
  }
  if (tables.empty())
    tables = exe_dir() + "/../data/stopping_tables.tsv";

  std::string text((std::istreambuf_iterator<char>(std::cin)), std::istreambuf_iterator<char>());
  mtg_json::Value top;
  std::string perr;
  if (!mtg_json::parse(text, top, perr))
  {
    std::cerr << "ERROR: cannot parse the input: " << perr << '\n';
    return 1;
  }
  Request req;
  try
  {
    req = read_input(top);
  }
  catch (const InputError & e)
  {
    std::cerr << "ERROR: " << e.msg << '\n' << std::flush;
    return 1;
  }

  mtg_ctx * ctx = nullptr;
  mtg_status st = mtg_create(device, &ctx);
  if (st != MTG_OK)
  {
    std::cerr << "ERROR: no usable CUDA device " << device << " (status " << int(st) << ")\n";
    return 1;
  }
  std::vector<double> se(req.energies.size());
  st = mtg_load_tables(ctx, tables.c_str());
  if (st == MTG_OK)
    st = mtg_stopping(ctx, req.Z1, req.m1, &req.mat, req.energies.data(), (long long)req.energies.size(),
                      precision == "fp64" ? MTG_PREC_FP64 : MTG_PREC_FP32, se.data());
  if (st != MTG_OK)
  {
    std::cerr << "ERROR: stopping evaluation failed (status " << int(st) << "): " << mtg_last_error(ctx) << '\n';
    mtg_destroy(ctx);
    return 1;
  }
  mtg_destroy(ctx);
  for (size_t n = 0; n < se.size(); ++n)
    std::cout << req.energies[n] << ' ' << se[n] << '\n';
  return 0;
}
