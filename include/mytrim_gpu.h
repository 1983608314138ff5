/*
 * mytrim_gpu.h -- C ABI of the GB300 cascade engine (libmytrim_gpu.so).
 *
 * The engine runs MyTRIM's binary-collision cascade (TrimBase::trim, trim.C:36-425,
 * driven by the FIFO loop of apps/runmytrim.C:71-93) on one GPU.  The ABI uses
 * plain C types only: POD structs, pointers and sizes.  The caller owns every
 * host buffer; a context owns the device memory it allocates.  All calls are
 * synchronous unless named *_async.  A context is not thread-safe: use one per
 * host thread, as the reference uses one SimconfType/TrimBase per thread
 * (apps/runmytrim.C:59-67).  No call aborts the process; every call returns an
 * mtg_status and mtg_last_error() describes the last failure.
 *
 * The reference has no foreign-function interface: each entry point below names
 * the C++ interface of the reference it stands in for.
 */
#ifndef MYTRIM_GPU_H
#define MYTRIM_GPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MTG_MAX_ELEMENTS 4
#define MTG_MAX_LAYERS 8
#define MTG_SCOEF_ROWS 92

typedef enum
{
  MTG_OK = 0,
  MTG_ERR_BAD_INPUT = 1,  /* invalid argument or unsupported sample */
  MTG_ERR_DATA = 2,       /* stopping tables missing or unreadable */
  MTG_ERR_OOM = 3,        /* device allocation failed */
  MTG_ERR_QUEUE_FULL = 4, /* recoil overflow list still exhausted after 3 enlargements:
                             results incomplete; or a full event log: tallies complete
                             (mtg_set_event_log) */
  MTG_ERR_TIMEOUT = 5,    /* a member exceeded the collision budget */
  MTG_ERR_NUMERIC = 6,    /* NaN energy or degenerate geometry met */
  MTG_ERR_CUDA = 7,       /* CUDA runtime error */
  MTG_ERR_NO_DEVICE = 8,  /* no CUDA device */
  MTG_ERR_STATE = 9       /* call out of order (e.g. run before tables) */
} mtg_status;

typedef enum
{
  MTG_PREC_FP64 = 0,          /* plain path: FP64 exact scattering (Newton + magic formula) */
  MTG_PREC_FP32 = 1,          /* FP32 flight/stopping/scattering, compensated energy bookkeeping */
  MTG_PREC_FP32_SURROGATE = 2 /* FP32 path with the learned scattering surrogate */
} mtg_precision;

typedef enum
{
  MTG_BC_PBC = 0, /* SampleBase::PBC (sample.h:49-54); positions are not wrapped, as in trim.C */
  MTG_BC_INF = 1, /* SampleBase::INF */
  MTG_BC_CUT = 2  /* SampleBase::CUT: a member leaving [0, w] is lost (trim.C:344-352) */
} mtg_boundary;

typedef enum
{
  MTG_TALLY_VACCOUNT = 0, /* TrimVacCount semantics (apps/src/TrimVacCount.C:32-54) */
  MTG_TALLY_RANGE = 1,    /* TrimRange semantics: no recoil followed, Kinchin-Pease
                             vacancies (apps/src/TrimRange.C:32-47) */
  MTG_TALLY_PRIMARIES = 2 /* TrimPrimaries (max_generation 1) / TrimRecoils (2): recoils
                             of a generation below max_generation are followed; every
                             displaced recoil is a vacancy, and one of generation
                             max_generation adds the modified Kinchin-Pease count with
                             the material's mean Z and mass (trim.C:446-464) */
} mtg_tally_mode;

/* One row of the stopping tables (SimconfType::ScoefLine, simconf.h:71-90). */
typedef struct
{
  double mm1, m1, mnat, rho, atrho, vfermi, heat, lfctr;
  double pcoef[8];
} mtg_scoef_row;

/* Element (element.h:29-41): _Z, _m, _t, _Edisp, _Elbind. */
typedef struct
{
  int Z;
  double m;
  double t;
  double Edisp;
  double Elbind;
} mtg_element;

/* MaterialBase (material.h:34-75) before prepare(): density in g/cm^3. */
typedef struct
{
  double rho;
  int n_elements;
  mtg_element elements[MTG_MAX_ELEMENTS];
} mtg_material;

/* TrimBase::Potential (trim.h:63-69): the screened interatomic potential of the
 * scattering, with its magic-formula constants (trim.C:194-258). */
typedef enum
{
  MTG_POT_UNIVERSAL = 0, /* ZBL universal (the reference's default, trim.h:40) */
  MTG_POT_MOLIERE = 1,
  MTG_POT_CKR = 2        /* C-Kr, with the reference's derivative coefficients as written */
} mtg_potential;

typedef enum
{
  MTG_GEOM_LAYERS = 0,  /* SampleLayers / SampleSolid */
  MTG_GEOM_CLUSTERS = 1 /* sampleClusters (sample_clusters.h:30-57) */
} mtg_geometry;

/* SampleLayers (sample_layers.h:33-43) or SampleSolid (n_layers = 1): layers stacked
 * along x from 0; x < 0 belongs to layer 0, the last layer extends to +infinity.
 * With geometry MTG_GEOM_CLUSTERS the sample is sampleClusters: material[0] fills the
 * box w, material[1] fills spheres (x, y, z, r) listed in `clusters` (host memory,
 * read during mtg_prepare / mtg_run), found through a spatial hash of
 * cluster_hash[0..2] cells (sampleClusters::initSpatialhash, addCluster); n_layers
 * must be 2 and thickness is not used.  A member that reaches a CUT boundary's
 * outside at the start of a collision is dropped without a tally, as in trim.C:81-83. */
typedef struct
{
  int n_layers;
  double thickness[MTG_MAX_LAYERS];
  mtg_material material[MTG_MAX_LAYERS];
  double w[3];
  int bc[3];
  int geometry;            /* mtg_geometry */
  int cluster_hash[3];     /* spatial-hash cells per axis (clusters only) */
  long long n_clusters;
  const double * clusters; /* n_clusters x (x, y, z, r) */
} mtg_sample;

/* IonBase template of the primaries (ion.h:30-85, runmytrim.C:263-304). */
typedef struct
{
  int Z;
  double m;      /* mass [u]; 0 selects the SCOEF MAI mass for stopping */
  double E;      /* energy [eV] */
  double Ef;     /* final energy [eV] (IonBase::_Ef, default 3) */
  double dir[3]; /* direction (normalised by the engine) */
  double pos[3]; /* start position */
} mtg_ion;

/* One independent simulation. */
typedef struct
{
  mtg_sample sample;
  mtg_ion ion;
  long long n_primaries;
  long long first_primary; /* index of the first primary: the random streams of primary i
                              depend only on (simulation, first_primary + i), so a run split
                              into primary ranges reproduces the unsplit run exactly */
  int tally_mode;         /* mtg_tally_mode */
  int primaries_only;     /* ThreadedTrimBase::_primaries_only */
  double hist_range_bin;  /* primary stopping-depth histogram: bin width [length unit] */
  int hist_range_n;       /*   and number of bins (0 = none) */
  double hist_vac_bin;    /* vacancy / replacement depth histograms (TrimVacCount uses 1) */
  int hist_vac_n;
  /* extensions with no counterpart in the reference (0 disables them): */
  double surface_binding; /* E_surf [eV]: a recoil leaving through x < 0 with
                             E cos^2(angle to the surface normal) > E_surf counts as sputtered */
  int voxel_n[3];         /* energy-deposition voxel tally: cells per axis (all > 0 to enable) */
  double voxel_origin[3]; /* corner of the voxel box [length unit] */
  double voxel_size[3];   /* edge lengths of the voxel box [length unit] */
  double hist_lateral_bin; /* 2-D histogram of the primaries' stopping points in (y, z) around
                              the start position: bin width [length unit] */
  int hist_lateral_n;     /* bins per axis (0 = none); appended after the replacement bins */
  int max_generation;     /* MTG_TALLY_PRIMARIES: TrimPrimaries::maxGen (1 for TrimPrimaries,
                             2 for TrimRecoils, trim.h:113-133); ignored otherwise */
  int hist_evac_rows;     /* vacancy-energy histogram (TrimVacEnergyCount, apps/src/
                             TrimVacEnergyCount.C:32-53): rows int(ln E) of the displaced
                             recoil's energy (below 0 in row 0), hist_vac_n depth columns
                             each; 0 = none; appended after the lateral bins */
  int potential;          /* TrimBase::_potential, an mtg_potential value; 0 = universal.  The
                             learned surrogate covers the universal potential only: the
                             other two scatter exactly on the surrogate path as well */
  int md_tag_Z;           /* IonMDTag::_md (ion.h:89-100) as the reference's demo programs
                             set it (apps/mytrim_solid.C:156-159): a member of atomic number
                             md_tag_Z whose energy at the start of its trajectory lies in
                             (md_tag_Emin, md_tag_Emax) gets _md = 1; every other member, and
                             every recoil when it is spawned (ion.C:88-93), 0.  0 = off */
  double md_tag_Emin, md_tag_Emax; /* the MD energy gap [eV], e.g. 200 and 12000 */
} mtg_sim;

/* Run-wide settings (SimconfType scalars, simconf.h:66). */
typedef struct
{
  double tmin;           /* minimum energy transfer setting p_max [eV] (0.2 in runmytrim) */
  double tau;            /* flight-path correction (0) */
  double cw;             /* first-flight cap [Angstrom] (0.001) */
  double length_scale;   /* SimconfType::setLengthScale */
  int precision;         /* mtg_precision */
  unsigned long long seed;
  long long max_collisions_per_member; /* 0 = default (2^24) */
  int stack_capacity;    /* recoil stack entries per warp, 0 = default */
  int block_threads;     /* threads per block of the cascade kernel: 64 or 128, 0 = 128 */
  int max_primaries_per_refill; /* fresh primaries one warp takes at a time, 1..32;
                                   0 = chosen from the expected cascade size (one for
                                   large cascades), the batch size and the grid */
  int refill_min_idle;   /* lanes of a warp that must be idle before the warp gives them
                            new members (recoils from its stack, fresh primaries), 1..32;
                            waiting lets the member-start code run for several lanes at
                            once instead of for one or two; 0 = 8 (FP32, surrogate) or 1
                            (FP64, whose FP64 pipe an idle lane leaves unused) */
} mtg_config;

/* Results of one simulation. */
typedef struct
{
  long long primaries, members, collisions;
  long long vacancies, replacements, interstitials, substitutionals, lost;
  double Eel, Enuc, Elost, Eunfollowed;
  long long range_n; /* primaries that came to rest (not lost) */
  double sx, sxx, sy, syy, sz, szz;
  double vac_s2, eel_s2, enuc_s2, coll_s2; /* sums of per-primary squares */
  long long newton_iterations, rejection_passes, surrogate_fallbacks;
  long long sputtered, backscattered; /* recoils / primaries lost through x < 0 */
  double Esputtered;                  /* kinetic energy carried out by sputtered atoms */
  double Evoxel;                      /* energy deposited inside the voxel box */
  long long hist_dropped;             /* vacancy, replacement or vacancy-energy events past the
                                         last depth bin or energy row (the reference grows its
                                         histograms instead; rerun with more bins to keep them) */
} mtg_totals;

/* Per-member trajectory summary (replay checks). */
typedef struct
{
  unsigned long long key;
  int sim, species, gen, state;
  unsigned int ncoll, nvac;
  double E, x, y, z, eel;
} mtg_member_record;

typedef struct
{
  double kernel_ms;        /* device time of the cascade launches of the last run */
  double reduce_ms;        /* device time of the tally reduction of the last run */
  int launches;            /* kernels launched by the last run */
  int drains;              /* overflow drain passes of the last run */
  int grid, block;         /* cascade launch shape */
  int stack_capacity;
  long long overflowed;    /* members spilled to the overflow list */
  long long collisions;
  size_t device_bytes;     /* device memory held by the context */
  long long h2d_bytes;     /* host-to-device bytes of the last prepare */
  long long d2h_bytes;     /* device-to-host bytes of the last collect */
  long long warp_steps;    /* collision-loop iterations of all warps in the last run; the
                              lane occupancy is collisions / (32 warp_steps) */
  int kernel_level;        /* feature level of the last run's cascade kernel: 0 lean, 1 member
                              records / voxels / tally modes, 2 + event log, 3 cluster geometry
                              or a non-universal potential, 4 + event log, 5 cluster geometry
                              with the universal potential only (plain FP32), 6 + event log */
  int max_take;            /* fresh primaries one warp took per refill in the last run */
  int events_overflowed;   /* 1 when the last collect's only error was a full event log (its
                              status is MTG_ERR_QUEUE_FULL and the tallies are complete) */
  int overflow_retries;    /* times the last run was made again because its recoil overflow
                              list filled (each time with lists four times larger, kept for
                              later runs; at most 3, then MTG_ERR_QUEUE_FULL) */
} mtg_stats;

typedef struct mtg_ctx mtg_ctx;

/* Create a context on CUDA device `device`.
 * Replaces: constructing SimconfType + TrimBase per thread (runmytrim.C:121-127). */
mtg_status mtg_create(int device, mtg_ctx ** out);

/* Release all device memory of the context. */
mtg_status mtg_destroy(mtg_ctx * ctx);

/* Text of the last error on this context (never NULL). */
const char * mtg_last_error(const mtg_ctx * ctx);

/* Stopping tables, 92 rows for Z = 1..92.
 * Replaces: SimconfType::readDataFiles (simconf.C:82-137). */
mtg_status mtg_set_tables(mtg_ctx * ctx, const mtg_scoef_row * rows, int n_rows);

/* Read the tables from a stopping_tables.tsv file (mytrim_gb300/data).
 * Replaces: SimconfType::readDataFiles with $MYTRIM_DATADIR (simconf.C:39, 82-137). */
mtg_status mtg_load_tables(mtg_ctx * ctx, const char * path);

/* Run-wide settings.  Replaces: SimconfType fields tmin/tau/cw and setLengthScale
 * (simconf.C:44-49, 75-80). */
mtg_status mtg_configure(mtg_ctx * ctx, const mtg_config * cfg);

/* Run n_sims simulations to completion (full cascades), host in, host out.
 * totals: n_sims entries.  hist: NULL or, per simulation in order, hist_range_n
 * range bins, then hist_vac_n vacancy bins, then hist_vac_n replacement bins, then
 * hist_lateral_n^2 lateral bins (z major), then hist_evac_rows x hist_vac_n
 * vacancy-energy bins (row major).
 * Replaces: the cascade loop computeThread (runmytrim.C:71-93) over
 * TrimBase::trim (trim.C:36-425) with the tally plugins (apps/src/Trim*.C). */
mtg_status mtg_run(mtg_ctx * ctx, const mtg_sim * sims, int n_sims, mtg_totals * totals,
                   long long * hist);

/* Split form of mtg_run for callers that keep inputs resident: prepare uploads the
 * tables of the simulations, launch runs the cascades on `stream` (a cudaStream_t,
 * NULL = default stream) without host copies, collect waits and copies the results. */
mtg_status mtg_prepare(mtg_ctx * ctx, const mtg_sim * sims, int n_sims);
mtg_status mtg_launch_async(mtg_ctx * ctx, void * stream);
mtg_status mtg_collect(mtg_ctx * ctx, mtg_totals * totals, long long * hist);

/* Per-primary results of the last run, primaries [first, first + n) of the global
 * index space (simulation after simulation).  Any pointer may be NULL.
 * Replaces: the per-ion quantities the reference tallies through checkPKAState and
 * vacancyCreation (trim.h:76-84). */
mtg_status mtg_get_primaries(mtg_ctx * ctx, long long first, long long n, long long * vacancies,
                             long long * collisions, double * eel, double * enuc, double * x,
                             double * y, double * z, int * state);

/* Energy-deposition voxels of simulation `sim` of the last run (voxel_n[0] * voxel_n[1] *
 * voxel_n[2] cells, x fastest): electronic loss at the start of each flight path,
 * nuclear deposits (binding energy, sub-threshold recoils, stopped members) where
 * they happen, in eV.  Each lane sums its consecutive deposits into one cell in
 * FP32 and adds the sum to the cell's FP64 total, so a cell that collects ~1e8
 * deposits keeps them all (an FP32 total would stop growing once it passed 2^24
 * deposits' worth); mtg_get_voxels rounds each cell's total to FP32 once,
 * mtg_get_voxels64 returns the FP64 totals.  The run's in-box total (Evoxel) is a
 * compensated FP64 reduction over the cells.  No counterpart in the reference. */
mtg_status mtg_get_voxels(mtg_ctx * ctx, int sim, float * out, long long n);
mtg_status mtg_get_voxels64(mtg_ctx * ctx, int sim, double * out, long long n);

/* Record one summary per cascade member (up to `capacity`) in subsequent runs;
 * 0 disables.  Replaces: the fullTraj trajectory dump (trim.C:370-371, 421-422). */
mtg_status mtg_set_record_capacity(mtg_ctx * ctx, long long capacity);
mtg_status mtg_get_records(mtg_ctx * ctx, mtg_member_record * out, long long capacity,
                           long long * n_written);

/* ---- event log: one record per hook call of the selected kinds ----
 * The reference streams such events from its hooks: TrimDefectLog (vacancies and
 * the rest states, trim.C:467-483), TrimPhononOut (binding energy of followed
 * recoils, dissipated recoil energy and residual energy of stopped members,
 * trim.C:504-527) and TrimRange (x of every dissipated recoil by Z,
 * apps/src/TrimRange.C:49-54).  Here the cascade kernel appends them to a device
 * buffer; the order of the records is not defined (sort them by primary, key).
 * Members are identified by their path key instead of the reference's sequential
 * _id. */
typedef enum
{
  MTG_EV_VACANCY = 1,     /* vacancyCreation: the displaced recoil (position, energy E after
                             the binding energy, Z of the target atom, its generation) */
  MTG_EV_REPLACEMENT = 2, /* replacementCollision: the displaced recoil */
  MTG_EV_BRANCH = 3,      /* followRecoil: a displaced recoil (whether followed or not);
                             aux = binding energy left at its site */
  MTG_EV_DISSIPATE = 4,   /* dissipateRecoilEnergy: a recoil below the displacement energy;
                             E = its energy, aux = binding energy (E + aux stays there) */
  MTG_EV_REST = 5,        /* checkPKAState: the member came to rest; state = 1 replacement,
                             2 substitutional, 3 interstitial; E = residual energy */
  MTG_EV_LOST = 6,        /* the member left through a CUT boundary; aux = energy of the
                             recoil dropped with it */
  MTG_EV_HISTORY = 7      /* TrimHistory's followRecoil (trim.h:139-153): the moving atom's
                             position after its flight at each displaced recoil; E = its
                             energy after the collision */
} mtg_event_kind;

typedef struct
{
  double x, y, z;          /* position [length unit] */
  double E, aux;           /* energies [eV], meaning by kind */
  double m;                /* mass [u] of the atom the event describes */
  unsigned long long key;  /* path key of the member that raised the event */
  long long primary;       /* primary index within its simulation (first_primary based) */
  int sim, kind, Z, gen, state;
  int tag;                 /* IonBase::_tag of the atom: for a followed recoil created inside a
                              cluster of a sampleClusters sample, that cluster's index
                              (trim.C:365, sample_clusters.C:53); -1 otherwise */
  int md;                  /* IonMDTag::_md of the atom (mtg_sim.md_tag_*): the member's own
                              for rest, loss and history events, 0 for the recoil of a vacancy,
                              replacement, branch or dissipation event (a recoil is spawned
                              with _md = 0, ion.C:88-93) */
} mtg_event;

/* Log events of the kinds whose bit (1 << kind) is set in kind_mask (0 disables)
 * in subsequent runs, up to `capacity` records; a run that raises more fails with
 * MTG_ERR_QUEUE_FULL after its tallies are complete.  A log of fewer than 128 slots
 * per resident GPU thread fills slot by slot (one global atomic per event); a larger
 * one is filled eight slots at a time per thread (sixteen from 256 slots per thread),
 * and the slots a thread leaves unused, fewer than one such chunk per thread and
 * pass, count toward the capacity: such a log can fill up to 1/16 early.
 * mtg_get_events returns the records without the unused slots either way. */
mtg_status mtg_set_event_log(mtg_ctx * ctx, unsigned int kind_mask, long long capacity);
/* Copy the last run's records; *n_total receives the number logged (may exceed the
 * capacity when the log overflowed), *n_written the number copied. */
mtg_status mtg_get_events(mtg_ctx * ctx, mtg_event * out, long long capacity, long long * n_written,
                          long long * n_total);

/* Electronic stopping [eV/Angstrom] of ion (Z1, m1) in `material` at n energies,
 * evaluated on the GPU in FP64 (precision MTG_PREC_FP64) or through the FP32
 * engine's stopping table (MTG_PREC_FP32).
 * Replaces: MaterialBase::getrstop (material.C:114-121) as driven by runstopping
 * (apps/runstopping.C:175-179). */
mtg_status mtg_stopping(mtg_ctx * ctx, int Z1, double m1, const mtg_material * material,
                        const double * E, long long n, int precision, double * out);

/* Centre-of-mass scattering for n (reduced energy, reduced impact parameter) pairs:
 * s2 = sin^2(theta/2).  precision selects the FP64 exact, FP32 exact or surrogate path.
 * Replaces: the scattering block of TrimBase::trim (trim.C:172-271). */
mtg_status mtg_scatter(mtg_ctx * ctx, const double * eps, const double * b, long long n,
                       int precision, double * s2);
/* mtg_scatter in the potential given as an mtg_potential value; the surrogate
 * precision accepts only MTG_POT_UNIVERSAL.
 * Replaces: the same block with TrimBase::_potential set (trim.C:194-258). */
mtg_status mtg_scatter_potential(mtg_ctx * ctx, const double * eps, const double * b, long long n,
                                 int precision, int potential, double * s2);

/* Launch settings chosen by mtg_autotune. */
typedef struct
{
  int block_threads;            /* cascade kernel block shape: 64 or 128 */
  int max_primaries_per_refill; /* fresh primaries per warp refill, 1..32; 0 = the built-in
                                   estimate, which each run makes from its own size */
  int stack_capacity;           /* recoil stack entries per warp (queue depth) */
  int refill_min_idle;          /* idle lanes a warp waits for before refilling, 1..32 */
  int heuristic_take;           /* the refill size the built-in estimate picks for this run */
  double default_collisions_per_s; /* trial rate of the built-in settings */
  double best_collisions_per_s;    /* trial rate of the chosen settings */
  int trials;                   /* trial launches made */
  int changed;                  /* 1 if the chosen settings differ from the built-in ones */
} mtg_tuning;

/* Choose the cascade kernel's launch settings for a run by measurement: the
 * simulations' primaries are scaled to about `trial_primaries` in total (0 = 262,144)
 * and launched with the built-in settings, then, one setting at a time, with each
 * candidate refill size (1, 2, 4, 8, 16, 32 primaries per warp refill and the
 * built-in estimate), refill threshold (1, 4, 8, 16 idle lanes), block shape (64,
 * 128 threads) and recoil stack depth (the default, half of it); the fastest in
 * collisions per second of kernel time is kept in the context's configuration for
 * the runs that follow, if it beats the built-in settings by more than 2 %.  A
 * candidate whose trial fails (a stack too shallow for the cascades fills the
 * overflow list) is skipped, and so is one whose trial spilled members to the
 * overflow list at a rate that, over the run's full primaries, would fill a quarter
 * of it.  The trials use the context like ordinary runs (their
 * results are discarded).  No counterpart in the reference, whose threads take
 * primaries one at a time (apps/runmytrim.C:71-93). */
mtg_status mtg_autotune(mtg_ctx * ctx, const mtg_sim * sims, int n_sims, long long trial_primaries,
                        mtg_tuning * out);

/* Counters of the last run. */
mtg_status mtg_get_stats(const mtg_ctx * ctx, mtg_stats * out);

/* ---- learned scattering surrogate (MTG_PREC_FP32_SURROGATE) ----
 * An MLP 2 -> 64 -> 64 -> 64 -> 2 (SiLU) from (log10 reduced energy, reduced impact
 * parameter) to sin^2(theta/2) and the reduced time integral, trained on FP64
 * quadrature of the universal-potential scattering integral.  No counterpart in the
 * reference, which evaluates the magic formula (trim.C:235-271) every collision; the
 * exact path stays the fallback outside log10(eps) in [-4, 4], b in [0, 12]. */
#define MTG_SURROGATE_NPARAM 8642

typedef struct
{
  long long n_train;       /* quadrature samples generated on the GPU (e.g. 2e7) */
  int batch;               /* mini-batch size */
  int epochs;              /* passes over the samples */
  int qat_epochs;          /* last epochs with BF16-rounded hidden layers in the forward pass */
  float lr;                /* Adam learning rate (cosine decay to 2 %) */
  unsigned long long seed;
  float w_tau;             /* loss weight of the time-integral output */
  int target;              /* sin^2(theta/2) target of each sample: MTG_SURROGATE_TARGET_* */
  int weighting;           /* loss weight of each sample's sin^2(theta/2): MTG_SURROGATE_WEIGHT_* */
} mtg_surrogate_config;

/* Training targets for sin^2(theta/2); the time-integral output is always the
 * quadrature's.  QUADRATURE: FP64 Gauss-Mehler quadrature of the scattering integral
 * (the true integral).  MAGIC: the FP64 magic formula with the reference's Newton
 * solve (trim.C:180-271) at the same samples, the formula the plain path and the
 * FP64 oracle evaluate. */
#define MTG_SURROGATE_TARGET_QUADRATURE 0
#define MTG_SURROGATE_TARGET_MAGIC 1
/* Loss weights.  UNIFORM: every sample's error in ln sin^2(theta/2) counts the same.
 * TRANSFER: weighted by the sample's sin^2(theta/2) (plus 1e-6), the share of the
 * beam energy and of the angular diffusion theta^2 the collision carries; the
 * weights are normalised to mean 1 over the training set. */
#define MTG_SURROGATE_WEIGHT_UNIFORM 0
#define MTG_SURROGATE_WEIGHT_TRANSFER 1

typedef struct
{
  double final_loss;       /* mean loss of the last mini-batch */
  double train_seconds;    /* device time of data generation + training */
  long long steps;
} mtg_surrogate_report;

/* Train the network on the GPU with the project's own kernels; the context keeps it. */
mtg_status mtg_surrogate_train(mtg_ctx * ctx, const mtg_surrogate_config * cfg, mtg_surrogate_report * rep);

/* Flat FP32 parameter vector (MTG_SURROGATE_NPARAM floats: W1[64][2] b1 W2[64][64] b2
 * W3[64][64] b3 W4[2][64] b4) of the context's network, or load one into it. */
mtg_status mtg_surrogate_get_params(mtg_ctx * ctx, float * params, long long n);
mtg_status mtg_surrogate_set_params(mtg_ctx * ctx, const float * params, long long n);

/* Loss and gradient of the training loss for a batch (x: n x 2 normalised inputs, y:
 * n x 2 targets) at `params`, computed by the training kernels (gradient check). */
mtg_status mtg_surrogate_gradients(mtg_ctx * ctx, const float * params, const float * x, const float * y,
                                   long long n, float w_tau, float * loss, float * grads);

/* FP64 Gauss-Mehler quadrature of the scattering integral (the training target):
 * s2 = sin^2(theta/2) and the reduced time integral (tau may be NULL). */
mtg_status mtg_surrogate_quadrature(mtg_ctx * ctx, const double * eps, const double * b, long long n,
                                    double * s2, double * tau);

/* Allocation-free reduction of per-primary tallies held in caller-owned device
 * buffers (n entries each, layout of mtg_get_primaries: vacancies, collisions,
 * electronic and nuclear energy, stopping point x/y/z, final state) into 15
 * doubles at device pointer `out`: sum and sum of squares of vacancies, of
 * collisions, of electronic energy and of nuclear energy; then the number of
 * primaries that came to rest and the sums and sums of squares of their x, y, z.
 * The same bits as the totals mtg_collect reports for a single simulation.
 *
 * For hosts that cannot let the library call cudaMalloc (for instance because
 * their own pool allocator owns all device memory): this call allocates nothing.
 * Its scratch is a fixed 120 KiB array in the library's device memory, so n is
 * limited to 67,108,864 primaries; larger n fails with MTG_ERR_BAD_INPUT and a
 * message in errbuf (may be NULL).  It works on the current device and queues its
 * kernels on `stream` (a cudaStream_t, NULL = default stream) without waiting.
 * The first call on each device looks up the scratch array's device address,
 * so make that first call before any stream capture.  The address belongs to the
 * device's CUDA context: after cudaDeviceReset, or under another context, the
 * next call looks it up again (it keeps the context's unique id beside it), and
 * that call too should come before any stream capture.  All calls on a device
 * share the scratch array: calls whose kernels could overlap on the GPU race,
 * so order them (one stream, or synchronise between them).
 * This entry point has no counterpart in the reference. */
mtg_status mtg_reduce_primaries_noalloc(const unsigned long long * vacancies,
                                        const unsigned long long * collisions, const double * eel,
                                        const double * enuc, const double * x, const double * y,
                                        const double * z, const int * state, long long n,
                                        double * out, void * stream, char * errbuf,
                                        size_t errbuf_len);

#ifdef __cplusplus
}
#endif

#endif /* MYTRIM_GPU_H */
