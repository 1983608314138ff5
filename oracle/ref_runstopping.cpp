// runstopping's evaluation with the reference library itself, built from the
// reference's sources by oracle/Makefile (test infrastructure: it makes the
// golden stopping tables; never part of the product).
//
// apps/runstopping.C cannot be built here (jsoncpp is absent).  This program takes
// a line-oriented request instead of its JSON and prints what runstopping.C:175-179
// prints: "E S_e" per energy, S_e = MaterialBase::getrstop (material.C:114-121).
//
//   ion <Z> <mass>
//   rho <g/cm3>
//   element <Z> <mass> <fraction>      (one line per element)
//   energies <E1> <E2> ...
#include "simconf.h"
#include "element.h"
#include "material.h"
#include "ion.h"

#include <iostream>
#include <sstream>
#include <string>
#include <vector>

using namespace MyTRIM_NS;

int
main()
{
  SimconfType simconf;
  simconf.fullTraj = false;
  simconf.tmin = 0.2;
  int Z1 = 1;
  double m1 = 1.0, rho = 1.0;
  std::vector<Element> els;
  std::vector<double> energies;
  std::string line;
  while (std::getline(std::cin, line))
  {
    std::istringstream ls(line);
    std::string key;
    if (!(ls >> key))
      continue;
    if (key == "ion")
      ls >> Z1 >> m1;
    else if (key == "rho")
      ls >> rho;
    else if (key == "element")
    {
      Element e;
      ls >> e._Z >> e._m >> e._t;
      els.push_back(e);
    }
    else if (key == "energies")
    {
      double E;
      while (ls >> E)
        energies.push_back(E);
    }
  }
  MaterialBase material(&simconf, rho);
  for (auto & e : els)
    material._element.push_back(e);
  material.prepare();
  IonBase pka;
  pka._Z = Z1;
  pka._m = m1;
  for (double E : energies)
  {
    pka._E = E;
    std::cout << pka._E << ' ' << material.getrstop(&pka) << '\n';
  }
  return 0;
}
