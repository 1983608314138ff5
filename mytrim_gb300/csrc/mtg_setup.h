// Host-side table construction: turns the reference-style inputs (stopping rows,
// materials, layers, ion template) into the POD tables of mtg_tables.h.
// Plain C++ (no CUDA), so the host replay check builds exactly the same tables.
#pragma once

#include <string>
#include <vector>

#include "mytrim_gpu.h"
#include "mtg_tables.h"

namespace mtg
{

struct HostTables
{
  std::vector<SimDesc> sims;
  std::vector<long long> prim_end;        // exclusive end of each simulation's primaries
  std::vector<SpeciesConst> species;
  std::vector<MatConst> mats;
  long long total_primaries = 0;
  long long hist_total = 0;               // entries of the concatenated histograms
  long long voxel_total = 0;              // cells of the concatenated voxel grids
  uint32_t k0 = 0, k1 = 0;                // Philox key
  double emax = 0.0;                      // largest primary energy
  int any_evac = 0;                       // some simulation keeps a vacancy-energy histogram
  int any_mode = 0;                       // some simulation tallies in TrimRange / TrimPrimaries mode
  int any_extended = 0;                   // some simulation has the cluster geometry or a
                                          // potential other than the universal one
  int any_clusters = 0;                   // some simulation has the cluster geometry
  int any_potential = 0;                  // some simulation has a non-universal potential
  double members_est = 1.0;               // expected cascade members per primary (launch heuristics)
  // stopping-table rows of the FP32 engine, one per distinct (species, material):
  // the MatConst entry and the species each row is built from
  std::vector<int> stop_row_mat, stop_row_species;
  // clusters of all cluster samples of the run (SimDesc::cl_base / cell_base index them)
  std::vector<Cl4d> clusters;
  std::vector<int> cl_next, cl_head;
  std::vector<uint32_t> cl_mask; // cluster candidate lists (SimDesc::mask_base indexes them)
};

// Point the simulations' cluster pointers at arrays holding HostTables::clusters,
// cl_next, cl_head and cl_mask (host or device copies).
void patch_cluster_pointers(std::vector<SimDesc> & sims, const Cl4d * cl, const int * next, const int * head,
                            const uint32_t * mask);

// Build the tables; returns MTG_OK or MTG_ERR_BAD_INPUT with `err` set.
int build_tables(const mtg_scoef_row * rows, const mtg_config & cfg, const mtg_sim * sims,
                 int n_sims, HostTables & out, std::string & err);

// Species constants of projectile (Z1, m1) and its stopping constants in Z2.
SpeciesConst make_species(const mtg_scoef_row * rows, int Z1, double m1);
StopPair make_stop_pair(const mtg_scoef_row * rows, const SpeciesConst & sc, int Z2);

// One material as seen by species sc (MaterialBase::prepare + average,
// material.C:37-110); rspecies is filled by the caller.
int make_material(const mtg_scoef_row * rows, const SpeciesConst & sc, const mtg_material & m,
                  double tmin, MatConst & out, std::string & err);

// Single-precision copies of the tables for the FP32 engine.
void build_fp32_tables(const HostTables & t, std::vector<Species32> & species, std::vector<Mat32> & mats,
                       std::vector<Sim32> & sims);

// Philox key of a run seed
void seed_key(unsigned long long seed, uint32_t & k0, uint32_t & k1);

// Parse stopping_tables.tsv (92 rows); returns false on a malformed file.
bool read_table_file(const char * path, mtg_scoef_row * rows, std::string & err);

} // namespace mtg
