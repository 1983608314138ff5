// Builds reference objects the way runmytrim does and prints what TrimGPU sends
// through the C ABI (compiled against the reference's own headers and sources).
#include "trim.h"
#include "simconf.h"
#include "material.h"
#include "sample_layers.h"
#include "sample_clusters.h"
#include "trim_gpu.h"

#include <cstdio>

using namespace MyTRIM_NS;

int main()
{
  SimconfType simconf;
  simconf.setLengthScale(1.0);
  SampleLayers sample(1100.0, 100.0, 100.0);
  sample.bc[0] = SampleBase::CUT;
  MaterialBase * m1 = new MaterialBase(&simconf, 2.2);
  Element e;
  e._Z = 14; e._m = 28.086; e._t = 1.0; e._Edisp = 15.0; e._Elbind = 3.0;
  m1->_element.push_back(e);
  e._Z = 8; e._m = 15.999; e._t = 2.0; e._Edisp = 28.0;
  m1->_element.push_back(e);
  m1->prepare();
  MaterialBase * m2 = new MaterialBase(&simconf, 2.33);
  e._Z = 14; e._m = 28.086; e._t = 1.0; e._Edisp = 15.0;
  m2->_element.push_back(e);
  m2->prepare();
  sample.material.push_back(m1);
  sample.layerThickness.push_back(100.0);
  sample.material.push_back(m2);
  sample.layerThickness.push_back(1000.0);
  IonBase pka(33, 74.922, 50000.0);
  pka._dir = Point(0.99, 0.1, 0.0);
  pka._pos = Point(0.0, 50.0, 50.0);
  pka._Ef = 5.0;

  std::vector<mtg_scoef_row> rows = mtg::flatten_tables(simconf);
  mtg_sample s = mtg::flatten_sample(sample, &sample.layerThickness);
  mtg_ion ion = mtg::flatten_ion(pka);
  printf("rows %zu %.17g %.17g %.17g %.17g\n", rows.size(), rows[28].m1, rows[28].vfermi, rows[28].lfctr,
         rows[28].pcoef[7]);
  printf("layers %d %.17g %.17g bc %d %d %d\n", s.n_layers, s.thickness[0], s.thickness[1], s.bc[0], s.bc[1],
         s.bc[2]);
  for (int k = 0; k < s.n_layers; ++k)
    for (int j = 0; j < s.material[k].n_elements; ++j)
      printf("el %d %d %.17g %d %.17g %.17g %.17g %.17g\n", k, j, s.material[k].rho, s.material[k].elements[j].Z,
             s.material[k].elements[j].m, s.material[k].elements[j].t, s.material[k].elements[j].Edisp,
             s.material[k].elements[j].Elbind);
  printf("ion %d %.17g %.17g %.17g %.17g %.17g %.17g\n", ion.Z, ion.m, ion.E, ion.Ef, ion.dir[0], ion.dir[1],
         ion.pos[1]);

  // a cluster sample built with the reference's own hash and insertion
  sampleClusters cs(400.0, 300.0, 200.0);
  cs.initSpatialhash(8, 6, 4);
  cs.addCluster(10.0, 20.0, 30.0, 5.0);
  cs.addCluster(200.0, 150.0, 100.0, 7.5);
  cs.material.push_back(m2);
  cs.material.push_back(m1);
  std::vector<double> storage;
  mtg_sample c = mtg::flatten_clusters(cs, storage);
  printf("clusters %d %d %lld %d %d %d %.17g %.17g\n", c.geometry, c.n_layers, c.n_clusters, c.cluster_hash[0],
         c.cluster_hash[1], c.cluster_hash[2], c.clusters[4], c.clusters[7]);
  return 0;
}
