// Plain-old-data tables the cascade kernels read.  Built on the host from the
// reference-style inputs (stopping coefficients, materials, layers, ion template)
// by mtg_setup.cpp and copied to the device once per run.
//
// Everything that depends only on the projectile species and the material is
// precomputed here in FP64 on the host, exactly as the reference computes it once
// per cascade member (MaterialBase::average, material.C:78-110), and the
// velocity-independent parts of the electronic stopping (material.C:161-281).
#pragma once

#include <stdint.h>

namespace mtg
{

constexpr int MAX_EL = 4;      // elements per material
constexpr int MAX_LAYERS = 8;  // layers per sample (the last extends to +inf)

// stopping branch of the projectile (material.C:187, 192, 213)
enum StopBranch : int
{
  STOP_H = 1,
  STOP_HE = 2,
  STOP_HEAVY = 3
};

// Constants of projectile species s that the stopping and scattering use.
struct SpeciesConst
{
  int Z1;
  int branch;
  double m1;        // mass [u] used for momenta and reduced energies
  double inv_m1k;   // 0.001 / m_stop, m_stop = m1 or SCOEF mm1 if m1 == 0 (material.C:178-185)
  double fz1;
  double cb, cb2;   // cbrt(Z1), cbrt(Z1)^2
  double lfctr;     // SLFCTR screening factor
  double bq;        // min(.43, max(.32, .12 + .025 Z1)) / cbrt(Z1)
  double l0a;       // min(1.2, 0.6 + Z1 / 30)
  double qlo, qden; // max(0, .9 - .025 Z1), |qlo - .2000001|
  double qhi, qden2;// max(0, 1 - .025 min(16, Z1)), .025 min(16, Z1)
  double inv_z1sq;  // 1 / Z1^2
};

// Electronic-stopping constants of species s in target element Z2.
struct StopPair
{
  double pcoef[8];  // SCOEF.95A proton coefficients of Z2
  double vfermi;    // Fermi velocity of Z2
  double inv2vf2;   // 1 / (2 vfermi^2)
  double velpwr;    // 0.25 for Z2 <= 6, else 0.45 (material.C:148-152)
  double yrcut;     // max(yrmin, vrmin / cbrt(Z1)^2)
  double eee;       // low-velocity matching energy (material.C:259-261)
  double sp_eee;    // proton stopping at eee
  double power;     // low-velocity exponent (material.C:264-267)
  double zc;        // 0.18 + 0.0015 Z2
  double hez;       // 0.007 + 0.00005 Z2 (helium)
  int Z2;
  int pad;
};

// One target element as seen by species s.
struct ElemConst
{
  double t;         // normalised stoichiometric fraction (material.C:52-55)
  double my;        // m1 / m2
  double ec;        // 4 my / (1 + my)^2
  double ai;        // screening length with Z1
  double fi;        // reduced-energy factor with Z1
  double Edisp, Elbind, m2;
  double maz, mam;  // the material's mean Z and mass (MaterialBase::_az, _am), for TrimPrimaries
  int Z2;
  int rspecies;     // species index (within the simulation) of a recoil of this element
};

// Material k as seen by species s.
struct MatConst
{
  double a, f, epsdg, arho;
  double am, az;
  int nel;
  int row; // stopping-table row (FP32 engine); equal (species, material) pairs share one
  ElemConst el[MAX_EL];
  StopPair sp[MAX_EL];
};

// One simulation: sample, ion template, run parameters, tally layout.
struct SimDesc
{
  // species and material tables: MatConst index = mat_base + s * n_mat + k
  int species_base, n_species;
  int mat_base, n_mat;
  // SampleLayers: x < layer_end[i] selects layer i, the last extends to +inf
  int n_layers;
  int layer_mat[MAX_LAYERS];
  double layer_end[MAX_LAYERS];
  int bc[3];        // 0 PBC, 1 INF, 2 CUT (sample.h:49-54)
  double w[3];
  // primary template (IonBase as built by runmytrim.C:290-304)
  double E0, Ef;
  double dir[3], pos[3];
  // run control
  double scale, invscale, tau, cw;
  int range_mode;       // tally mode: 0 TrimVacCount, 1 TrimRange, 2 TrimPrimaries / TrimRecoils
  int primaries_only;   // ThreadedTrimBase::_primaries_only
  int follow_gen;       // a displaced recoil is followed iff its generation is below this
  int kp_gen;           // TrimPrimaries: generation whose displaced recoils add a KP count
  int potential;        // TrimBase::Potential: 0 universal, 1 Moliere, 2 C-Kr
  int md_Z;             // IonMDTag rule: members of this Z born in (md_Emin, md_Emax) get _md = 1 (0 = off)
  double md_Emin, md_Emax;
  float md_Emin_f, md_Emax_f; // single-precision copies (FP32 engine)
  long long prim_begin; // first global primary index of this simulation
  long long n_primaries;
  uint64_t sim_key;     // simulation number used in the member keys
  long long key_offset; // primary index offset of the member keys (sharded runs)
  // tallies
  int hist_range_n, hist_vac_n;
  long long hist_range_base, hist_vac_base;
  double inv_hist_range_bin, inv_hist_vac_bin;
  float inv_hist_range_bin_f, inv_hist_vac_bin_f; // single-precision copies (FP32 engine)
  // extensions: sputter counting and energy-deposition voxels
  float surface_binding;   // 0 = off
  int voxel_n[3];          // 0 = off
  float voxel_origin[3], voxel_inv_cell[3];
  long long voxel_base;    // offset into the run's voxel buffer
  // lateral (y, z) histogram of stopping points around the start position
  int hist_lat_n;
  float inv_hist_lat_bin, lat_y0, lat_z0; // y0, z0: lower corner of the histogram
  long long hist_lat_base;
  // vacancy-energy histogram (TrimVacEnergyCount): rows by int(ln E) of the
  // recoil, columns the vacancy depth bins
  int hist_evac_rows;
  long long hist_evac_base;
  // sampleClusters geometry (geometry 1): spatial hash of kn cells of size kd,
  // largest radius cmr; cluster arrays of the run (x, y, z, r; next in cell list;
  // first cluster per cell) patched in as pointers where the tables live
  int geometry;
  int kn[3];
  int n_clusters;
  double kd[3];
  double cmr;
  long long cl_base, cell_base; // offsets into the run's cluster and cell arrays
  const struct Cl4d * cl;
  const int * cl_next;
  const int * cl_head;
  // candidate lists on a finer grid (mn cells per axis): per cell the clusters that
  // (dilated by a rounding margin) reach into it, or a mark sending the cell's points
  // to the hash search (layout in mtg_setup.cpp, build_cluster_cells)
  int mn[3];
  double inv_mcell[3];
  long long mask_base; // offset of this simulation's lists in the run's words
  const uint32_t * cl_mask;
};

// one cluster: centre and radius
struct Cl4d
{
  double x, y, z, r;
};
struct Cl4f
{
  float x, y, z, r;
};

// Totals per simulation (device accumulators, reduced on the host).
struct SimTotals
{
  unsigned long long members, replacements, interstitials, substitutionals, lost;
  unsigned long long newton_iters, rejection_passes, fallbacks;
  double Elost, Eunfollowed;
  unsigned long long sputtered, backscattered;
  double Esputtered;
  unsigned long long hist_dropped; // depth-histogram events beyond the last bin
};

// One entry of the event log (layout of mtg_event).
struct EventRec
{
  double x, y, z, E, aux, m;
  uint64_t key;
  long long primary;
  int sim, kind, Z, gen, state, tag;
  int md; // IonMDTag::_md of the atom
};

// event kinds (bit k of the log's mask selects kind k)
enum EventKind : int
{
  EV_VACANCY = 1,
  EV_REPLACEMENT = 2,
  EV_BRANCH = 3,
  EV_DISSIPATE = 4,
  EV_REST = 5,
  EV_LOST = 6,
  EV_HISTORY = 7,
  EV_UNUSED = -1 // a reserved slot of the log that no event filled (see LaneSink::event)
};

// ---- single-precision copies used by the FP32 engine (built from the tables above)
struct Elem32
{
  float t, my, ec, inv_ai, fi, Edisp, Elbind, m2;
  float disp_thresh; // Edisp - Elbind (trim.C:359)
  float maz, mam;    // material mean Z and mass (TrimPrimaries)
  int Z2, rspecies;
};

struct Mat32
{
  float a, f, epsdg, inv_pi_arho; // 1 / (pi * atomic density)
  int nel, row, pad0, pad1;       // row: stopping-table row of this (species, material)
  Elem32 el[MAX_EL];
};

struct Species32
{
  float m1, two_m1;
  int Z1, pad;
};

// byte offset of the surrogate network in the FP32 engine's staged shared-memory
// tables: after the species and material rows, 16-byte aligned
#ifdef __CUDACC__
__host__ __device__
#endif
inline size_t
stage_net_offset(int n_species, int n_mats)
{
  return (sizeof(Species32) * size_t(n_species) + sizeof(Mat32) * size_t(n_mats) + 15) / 16 * 16;
}

struct Sim32
{
  float layer_end[MAX_LAYERS];
  int layer_mat[MAX_LAYERS];
  float w[3];
  int bc[3];
  int n_layers, n_mat, mat_base, species_base;
  float Ef, flscale, tau, cw; // flscale = 1 / length scale
  int range_mode, primaries_only, any_cut, geometry;
  int follow_gen, kp_gen, potential, pad1;
  // sampleClusters geometry (see SimDesc)
  int kn[3];
  int n_clusters;
  float kd[3];
  float cmr;
  const Cl4f * cl;
  const int * cl_next;
  const int * cl_head;
  int mn[3];
  float inv_mcell[3];
  const uint32_t * cl_mask;
};

// final state of a cascade member (IonBase::StateType, ion.h:75-84)
enum MemberState : int
{
  ST_MOVING = 0,
  ST_REPLACEMENT = 1,
  ST_SUBSTITUTIONAL = 2,
  ST_INTERSTITIAL = 3,
  ST_LOST = 4
};

// outcome flags of one collision
enum CollideFlags : int
{
  CF_PUSH = 1, // the collision displaced a recoil to follow
  CF_DONE = 2, // the member came to rest or left the sample
  CF_VOID = 4  // no collision happened: the member found no material and was dropped
};

enum ErrorBits : unsigned int
{
  ERRB_QUEUE_FULL = 1u,
  ERRB_NUMERIC = 2u,
  ERRB_BUDGET = 4u,
  ERRB_BAD_INDEX = 8u,
  ERRB_EVENTS_FULL = 16u
};

} // namespace mtg
