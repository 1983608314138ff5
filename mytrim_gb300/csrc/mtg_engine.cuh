// Persistent, warp-cooperative cascade kernel.
//
// The reference follows one cascade with a host FIFO: pop a member, run
// TrimBase::trim on it until it stops, push every recoil it displaces
// (apps/runmytrim.C:71-93, trim.C:369).  Here every lane of a warp holds one
// cascade member in registers and the 32 lanes advance one collision per loop
// iteration.  Each warp owns a LIFO recoil stack in HBM:
//   * a lane whose member came to rest pops the next recoil from its warp's
//     stack (warp-synchronous ballot + prefix count, no atomics);
//   * with the stack empty, idle lanes take fresh primaries from one global
//     counter (one atomicAdd per warp refill);
//   * recoils are pushed with a ballot + prefix count; a full stack spills into
//     a global overflow list that a follow-up launch drains.
// No warp ever waits on another, so the kernel needs no spin loops; every loop
// is bounded (collisions per member, Newton iterations, rejection passes).
//
// Random numbers are keyed by the member's path key and collision index, so the
// result does not depend on which lane or warp ran which member.
//
// Tallies: per-lane accumulators flushed to per-primary arrays when a lane
// switches primary (vacancies, collisions, electronic and nuclear energy), the
// primary's stopping point written once, depth histograms through per-lane
// atomics, per-simulation counters flushed once per lane.
#pragma once

#include "mtg_tables.h"
#include "mtg_common.cuh"

namespace mtg
{

struct PrimaryTallies
{
  unsigned long long * vac;  // vacancies (KP count in range mode)
  unsigned long long * coll; // collisions
  double * eel;              // electronic loss [eV]
  double * enuc;             // nuclear (phonon) deposit [eV]
  double * fx;               // stopping point of the primary (generation 0)
  double * fy;
  double * fz;
  int * fstate;              // final state of the primary, 0 if lost / not stopped
};

struct MemberRecord
{
  uint64_t key;
  int sim, species, gen, state;
  unsigned int ncoll, nvac;
  double E, x, y, z, eel;
};

struct EngineParams
{
  const SimDesc * sims;
  int n_sims;
  const long long * sim_prim_end; // exclusive prefix end of each simulation's primaries
  const SpeciesConst * species;
  const MatConst * mats;
  int stage_tables;               // stage species+mats of simulation 0 into shared memory
  int n_stage_species, n_stage_mats;
  long long total_primaries;
  unsigned long long * next_primary;
  // drain mode: members read from `in_records` (count in device memory) instead
  // of fresh primaries
  const void * in_records;
  const unsigned long long * in_count;
  long long in_cap;
  // per-warp stacks and overflow list
  void * stacks;
  int stack_cap;
  void * overflow;
  unsigned long long * overflow_count;
  long long overflow_cap;
  // tallies
  PrimaryTallies prim;
  SimTotals * totals;
  unsigned long long * hist; // all histograms, per-simulation bases in SimDesc
  double * voxels;           // energy-deposition voxels of all simulations (may be NULL):
                             // FP64 sums in global memory (L2 atomics), fed by each lane's
                             // short FP32 run of deposits into one cell
  unsigned int * error_flags;
  uint32_t k0, k1;
  unsigned int max_collisions; // per member
  int max_take;                // fresh primaries one warp takes per refill (load balance)
  int refill_min;              // idle lanes a warp waits for before refilling them
  int cold_offset;             // byte offset of the per-thread LaneCold slots in dynamic shared memory
  // optional per-member records (replay checks)
  MemberRecord * records;
  unsigned long long * n_records;
  long long records_cap;
  // optional event log (mask bit k selects EventKind k; 0 = off)
  EventRec * events;
  unsigned long long * n_events;       // slots reserved
  unsigned long long * n_event_unused; // reserved slots that no event filled
  long long events_cap;
  int event_chunk;                     // slots a lane reserves at a time (1, 8 or 16)
  unsigned int event_mask;
  int any_evac; // some simulation keeps a vacancy-energy histogram
  int level;    // KernelLevel of the launched variant
  unsigned long long * warp_steps; // loop iterations of all warps (lane occupancy = collisions / 32 steps)
  // single-simulation runs with few depth bins count vacancies and replacements in
  // a per-block shared-memory histogram (hist_smem_bins counters from byte offset
  // hist_smem_offset), added to the global one when the block ends; 0 = global atomics
  int hist_smem_bins;
  int hist_smem_offset;
  long long hist_smem_base; // global index of shared bin 0
};

// largest vacancy + replacement histogram counted in shared memory (u32 counters)
constexpr int HIST_SMEM_MAX = 2048;

__device__ __forceinline__ unsigned int
lanemask_lt()
{
  unsigned int m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

__device__ __forceinline__ int
find_sim(const long long * ends, int n, long long g)
{
  int lo = 0, hi = n - 1;
  while (lo < hi)
  {
    const int mid = (lo + hi) >> 1;
    if (g < ends[mid])
      hi = mid;
    else
      lo = mid + 1;
  }
  return lo;
}

// Plain FP64 accumulator (FP64 engine)
struct AccF64
{
  double s;
  __device__ void reset() { s = 0.0; }
  __device__ void add(double x) { s += x; }
  __device__ double value() const { return s; }
  __device__ bool nonzero() const { return s != 0.0; }
  __device__ void atomic_add_to(double * dst) const { atomicAdd(dst, s); }
};

// float -> double by exponent rebias on the bit pattern (no FP64 instruction; the
// FP32 engine flushes denormals, so a zero exponent means zero)
__device__ __forceinline__ double
widen_f32(float f)
{
  const uint32_t u = __float_as_uint(f);
  const uint32_t e = (u >> 23) & 0xffu;
  if (e == 0u)
    return 0.0;
  const unsigned long long bits = ((unsigned long long)(u >> 31) << 63) | ((unsigned long long)(e + 896u) << 52) |
                                  ((unsigned long long)(u & 0x7fffffu) << 29);
  return __longlong_as_double((long long)bits);
}

// Plain FP32 accumulator for the per-collision energy sums of the FP32 engine;
// the engine hands it to the FP64 per-primary arrays every few dozen collisions
// (Pol::FLUSH_EVERY), so each float sum stays short and accurate to ~1e-7
struct AccF32
{
  float s;
  __device__ void reset() { s = 0.0f; }
  __device__ void add(float x) { s += x; }
  __device__ double value() const { return double(s); }
  __device__ bool nonzero() const { return s != 0.0f; }
  __device__ void atomic_add_to(double * dst) const { atomicAdd(dst, widen_f32(s)); }
};

// Kahan-compensated FP32 accumulator (FP32 engine, long-lived rare sums): keeps
// FP64 work out of the engine.  The error of a compensated sum is bounded by about
// 2u sum|x_i| (u = 2^-24, so ~1.2e-7 of the summed magnitudes) independent of the
// number of terms, where a plain FP32 sum grows as n u sum|x_i|.
struct AccKahan32
{
  float s, c;
  __device__ void reset() { s = c = 0.0f; }
  __device__ void add(float x)
  {
    const float y = x - c;
    const float t = s + y;
    c = (t - s) - y;
    s = t;
  }
  __device__ double value() const { return double(s) - double(c); }
  __device__ bool nonzero() const { return s != 0.0f; }
  // add the sum to a double in global memory without FP64 instructions
  __device__ void atomic_add_to(double * dst) const
  {
    atomicAdd(dst, widen_f32(s));
    if (c != 0.0f)
      atomicAdd(dst, widen_f32(-c));
  }
};

// Rarely-updated tally state of one lane, kept in a per-thread slot of shared
// memory instead of registers (the collision loop needs its registers).
template <class Acc>
struct LaneCold
{
  unsigned int n_repl, n_inter, n_subst, n_lost, n_members, n_passes, n_fallbacks, n_sput, n_back;
  unsigned int m_vac;
  int m_state;
  unsigned int n_dropped; // depth-histogram events beyond the last bin
  Acc e_lost, e_unf, e_sput, m_eel;
  long long vcell; // pending voxel deposit: cell and value
  float vacc;
  int m_md;        // IonMDTag::_md of the lane's member (event-logging levels)
  int evac_bin;    // vacancy-energy bin of the current collision (-1 = none)
  unsigned int ev_next, ev_end; // the lane's reserved event-log slots [ev_next, ev_end)
};

// Kernel feature levels.  Code for a feature a run does not use still costs the
// collision loop (instruction fetch, registers), so the cascade kernel comes in
// up to seven variants and each run takes the smallest that has what it needs:
//   LVL_LEAN    layered samples, universal potential, TrimVacCount tallies (depth,
//               range and lateral histograms), CUT boundaries and sputter counting;
//   LVL_MID     + member records, deposition voxels, the vacancy-energy histogram,
//               TrimRange / TrimPrimaries tally modes;
//   LVL_EVENTS  LVL_MID + the event log (no cluster geometry, universal potential);
//   LVL_GEO     LVL_MID + the cluster geometry, the Moliere and C-Kr potentials;
//   LVL_FULL    LVL_GEO + the event log;
//   LVL_CLU     LVL_MID + the cluster geometry, universal potential only (the plain
//               FP32 engine; the others run LVL_GEO);
//   LVL_CLU_EV  LVL_CLU + the event log (the others run LVL_FULL).
enum KernelLevel : int
{
  LVL_LEAN = 0,
  LVL_MID = 1,
  LVL_EVENTS = 2,
  LVL_GEO = 3,
  LVL_FULL = 4,
  LVL_CLU = 5,
  LVL_CLU_EV = 6,
  LVL_COUNT = 7
};

// the level's cluster geometry, its non-universal potentials, its event log
MTG_HD constexpr bool
level_clusters(int lvl)
{
  return lvl == LVL_GEO || lvl == LVL_FULL || lvl == LVL_CLU || lvl == LVL_CLU_EV;
}
MTG_HD constexpr bool
level_potentials(int lvl)
{
  return lvl == LVL_GEO || lvl == LVL_FULL;
}
MTG_HD constexpr bool
level_events(int lvl)
{
  return lvl == LVL_EVENTS || lvl == LVL_FULL || lvl == LVL_CLU_EV;
}

// Device tally sink for one lane of a kernel of level LVL.
template <class Pol, int LVL>
struct LaneSink
{
  static constexpr bool EV = level_events(LVL); // feeds the event log
  static constexpr bool MID = LVL >= LVL_MID;
  using Acc = typename Pol::Acc;       // rare sums (kept in shared memory)
  using AccHot = typename Pol::AccHot; // per-collision sums (registers)
  using Real = typename Pol::Real;
  LaneCold<Acc> * cold;
  const EngineParams * prm;
  const SimDesc * sim;
  long long gprim;     // global primary index of the current member
  int range_mode;
  // per-primary accumulators
  unsigned int a_vac, a_coll;
  AccHot a_eel, a_enuc;
  // per-simulation Newton-iteration count (every collision), the rest in `cold`
  unsigned int n_newton;
  bool vox;  // this simulation tallies energy deposition in voxels
  bool dep_in; // the last deposit's point lies in the voxel box (its cell is pending)
  // events of the current collision, aggregated per warp after it
  int vac_bin, repl_bin;

  __device__ void reset_sim()
  {
    LaneCold<Acc> & c = *cold;
    c.n_repl = c.n_inter = c.n_subst = c.n_lost = c.n_members = c.n_passes = c.n_fallbacks = 0;
    c.n_sput = c.n_back = c.n_dropped = 0;
    n_newton = 0;
    c.e_lost.reset();
    c.e_unf.reset();
    c.e_sput.reset();
  }
  // when the lane leaves the kernel: its reserved slots that no event filled are
  // marked unused (the host skips them) and counted
  __device__ void flush_events()
  {
    if constexpr (EV)
    {
      LaneCold<Acc> & c = *cold;
      if (c.ev_end > c.ev_next)
      {
        atomicAdd(prm->n_event_unused, (unsigned long long)(c.ev_end - c.ev_next));
        for (unsigned int s = c.ev_next; s < c.ev_end && (long long)s < prm->events_cap; ++s)
          prm->events[s].kind = EV_UNUSED;
      }
      c.ev_next = c.ev_end = 0;
    }
  }
  // per-member summaries feed the optional member records only
  __device__ void reset_member()
  {
    if (!MID || !prm->records)
      return;
    cold->m_vac = 0;
    cold->m_state = 0;
    cold->m_eel.reset();
  }
  __device__ void reset_prim()
  {
    a_vac = a_coll = 0;
    a_eel.reset();
    a_enuc.reset();
  }

  // ---- event log (opt-in): one entry per selected hook call
  __device__ void event(int kind, Real x, Real y, Real z, Real E, int Z, Real m, int gen, int state, Real aux,
                        uint64_t key, int tag, int md = 0)
  {
    if (!(prm->event_mask & (1u << kind)))
      return;
    // a lane takes its slots event_chunk at a time: the atomic that reserves them
    // returns through L2, and the lane waits for it before writing the record
    LaneCold<Acc> & c = *cold;
    if (c.ev_next == c.ev_end)
    {
      // slot indexes fit 32 bits: a log of 2^32 88-byte records exceeds the device
      // memory; the reservation saturates there once a full log keeps reserving
      const unsigned long long base = atomicAdd(prm->n_events, (unsigned long long)prm->event_chunk);
      c.ev_next = base < 0xfffffff0ull ? (unsigned int)base : 0xfffffff0u;
      c.ev_end = c.ev_next + (unsigned int)prm->event_chunk;
    }
    const unsigned int slot = c.ev_next++;
    if ((long long)slot >= prm->events_cap)
    {
      atomicOr(prm->error_flags, ERRB_EVENTS_FULL);
      return;
    }
    EventRec & r = prm->events[slot];
    r.x = double(x);
    r.y = double(y);
    r.z = double(z);
    r.E = double(E);
    r.aux = double(aux);
    r.key = key;
    r.primary = gprim - sim->prim_begin + sim->key_offset;
    r.sim = int(sim - prm->sims);
    r.kind = kind;
    r.Z = Z;
    r.m = double(m);
    r.gen = gen;
    r.state = state;
    r.tag = tag;
    r.md = md;
  }
  // TrimHistory::followRecoil (trim.h:146-150): the moving atom's position (after
  // its flight, trim.C:310) at each displaced recoil
  template <class P>
  __device__ void history(const P & p, int Z1, Real m1)
  {
    if constexpr (EV)
      event(EV_HISTORY, Real(p.x), Real(p.y), Real(p.z), Real(p.E), Z1, m1, p.gen, 0, Real(0), p.key, p.tag,
            cold->m_md);
  }
  // followRecoil (trim.C:362): a displaced recoil, followed or not
  template <class R, class E>
  __device__ void branch(const R & rec, const E & el, uint64_t key)
  {
    if constexpr (EV)
      event(EV_BRANCH, Real(rec.x), Real(rec.y), Real(rec.z), Real(rec.E), el.Z2, Real(el.m2), rec.gen, 0,
            Real(el.Elbind), key, rec.tag);
  }
  // dissipateRecoilEnergy (trim.C:397-401): a recoil below the displacement energy
  template <class R, class E>
  __device__ void dissipate(const R & rec, Real Erec, const E & el, uint64_t key)
  {
    if constexpr (EV)
      event(EV_DISSIPATE, Real(rec.x), Real(rec.y), Real(rec.z), Erec, el.Z2, Real(el.m2), rec.gen, 0,
            Real(el.Elbind), key, rec.tag);
  }

  // ---- events raised by the collision code (the reference's hooks, trim.h:72-84)
  // energy-deposition voxel tally (extension): one float atomic per deposit
  __device__ void deposit(Real x, Real y, Real z, Real e)
  {
    if (!MID || !vox)
      return;
    const int ix = int(floorf(float(x - Real(sim->voxel_origin[0])) * sim->voxel_inv_cell[0]));
    const int iy = int(floorf(float(y - Real(sim->voxel_origin[1])) * sim->voxel_inv_cell[1]));
    const int iz = int(floorf(float(z - Real(sim->voxel_origin[2])) * sim->voxel_inv_cell[2]));
    dep_in = false;
    if (ix < 0 || iy < 0 || iz < 0 || ix >= sim->voxel_n[0] || iy >= sim->voxel_n[1] || iz >= sim->voxel_n[2])
      return;
    dep_in = true;
    const long long cell = sim->voxel_base + ((long long)iz * sim->voxel_n[1] + iy) * sim->voxel_n[0] + ix;
    LaneCold<Acc> & c = *cold;
    if (cell == c.vcell)
    {
      c.vacc += float(e);
      return;
    }
    flush_voxel();
    c.vcell = cell;
    c.vacc = float(e);
  }
  __device__ void flush_voxel()
  {
    if constexpr (!MID)
      return;
    LaneCold<Acc> & c = *cold;
    // the lane's run of deposits into one cell is short (FP32 is exact enough for
    // it); the cell's sum over the whole run takes up to ~1e8 of them, which FP32
    // would round away once the sum passes 2^24 deposits' worth, so it is kept in
    // FP64 (the float is widened on its bit pattern, no FP64 instruction here)
    if (c.vcell >= 0)
      atomicAdd(prm->voxels + c.vcell, widen_f32(c.vacc));
    c.vcell = -1;
    c.vacc = 0.0f;
  }

  // electronic loss d over the flight path that starts at (x, y, z)
  __device__ void eel(Real d, Real x, Real y, Real z)
  {
    a_eel.add(d);
    if (MID && prm->records)
      cold->m_eel.add(d);
    deposit(x, y, z, d);
  }
  __device__ void newton(int n) { n_newton += (unsigned int)n; }
  __device__ void passes(int n) { cold->n_passes += (unsigned int)n; }
  __device__ void fallback() { ++cold->n_fallbacks; }
  __device__ void numeric() { atomicOr(prm->error_flags, ERRB_NUMERIC); }
  // nuclear (phonon) deposit e at (x, y, z)
  // The collision code deposits a collision's nuclear loss where it deposited the
  // electronic loss just before (the flight's starting point, which is the recoil's
  // position, trim.C:306-318), so the pending voxel cell is already the right one:
  // the same sum as a full deposit, without recomputing the cell.
  __device__ void enuc(Real e, Real /*x*/, Real /*y*/, Real /*z*/)
  {
    a_enuc.add(e);
    if (MID && vox && dep_in)
      cold->vacc += float(e);
  }
  __device__ void unfollowed(Real e) { cold->e_unf.add(e); }
  // the member left the sample carrying `e` (its own energy plus the recoil dropped
  // with it, trim.C:357); through the entrance surface a recoil counts as sputtered
  // when E cos^2 > E_surf, a primary as backscattered
  template <class P>
  __device__ void lost(Real e, const P & p, int Z1, Real m1)
  {
    LaneCold<Acc> & c = *cold;
    if constexpr (EV)
      event(EV_LOST, Real(p.x), Real(p.y), Real(p.z), Real(p.E), Z1, m1, p.gen, ST_LOST, e - Real(p.E), p.key, p.tag,
            cold->m_md);
    ++c.n_lost;
    c.e_lost.add(e);
    if (MID && prm->records)
      c.m_state = ST_LOST;
    if (p.x < Real(0) && sim->bc[0] == 2)
    {
      if (p.gen == 0)
        ++c.n_back;
      else if (sim->surface_binding > 0.0f && Real(p.E) * p.dx * p.dx > Real(sim->surface_binding))
      {
        ++c.n_sput;
        c.e_sput.add(Real(p.E));
      }
    }
  }

  template <class R, class E>
  __device__ void vacancy(const R & rec, const E & el, Real Erec, uint64_t key)
  {
    if constexpr (EV)
      event(EV_VACANCY, Real(rec.x), Real(rec.y), Real(rec.z), Erec, el.Z2, Real(el.m2), rec.gen, 0,
            Real(el.Elbind), key, rec.tag);
    if (MID && range_mode == 2)
    {
      // TrimPrimaries::vacancyCreation (trim.C:446-464): one vacancy per displaced
      // recoil and, for a recoil of the cutoff generation (not followed), the
      // modified Kinchin-Pease count with the material's mean Z and mass
      unsigned int add = 1;
      if (rec.gen == sim->kp_gen)
      {
        const Real az = Real(el.maz), am = Real(el.mam), Er = Erec;
        const Real ed = Real(0.0115) * powr(az, Real(-7.0 / 3.0)) * Er;
        const Real g = Real(3.4008) * powr(ed, Real(1.0 / 6.0)) + Real(0.40244) * powr(ed, Real(3.0 / 4.0)) + ed;
        const Real kd = Real(0.1337) * powr(az, Real(2.0 / 3.0)) / sqrt(am);
        const Real Ev = Er / (Real(1) + kd * g);
        add += (unsigned int)(int(Real(0.8) * Ev / (Real(2) * Real(el.Edisp))));
      }
      a_vac += add;
      if (prm->records)
        cold->m_vac += add;
      return;
    }
    if (MID && range_mode)
    {
      // TrimRange::vacancyCreation (apps/src/TrimRange.C:32-47): Kinchin-Pease
      // count of the displaced recoil, each increment truncated like the
      // reference's int accumulator
      const Real Z = Real(el.Z2), m = Real(el.m2), Er = Erec;
      const Real Ed = Real(el.Edisp);
      const Real ed = Real(0.0115) * powr(Z, Real(-7.0 / 3.0)) * Er;
      const Real kd = Real(0.1337) * powr(Z, Real(2.0 / 3.0)) / sqrt(m);
      const Real g = Real(3.4008) * powr(ed, Real(1.0 / 6.0)) + Real(0.40244) * powr(ed, Real(3.0 / 4.0)) + ed;
      const Real Ev = Er / (Real(1) + kd * g);
      unsigned int add = 0;
      if (Ev < Ed)
        add = 0;
      else if (Ev >= Ed / Real(0.4))
        add = (unsigned int)(Ev * Real(0.4) / Ed);
      else
        add = 1;
      a_vac += add;
      if (prm->records)
        cold->m_vac += add;
      return;
    }
    ++a_vac;
    if (MID && prm->records)
      ++cold->m_vac;
    const int b = depth_bin(Real(rec.x), inv_vac_bin(), sim->hist_vac_n);
    if (b >= 0)
    {
      vac_bin = int(sim->hist_vac_base) + b;
      if (MID && prm->any_evac && sim->hist_evac_rows > 0)
      {
        // TrimVacEnergyCount::vacancyCreation (apps/src/TrimVacEnergyCount.C:32-53):
        // row int(ln E) of the recoil energy, negative rows in row 0
        int row = int(loge(Erec));
        row = row < 0 ? 0 : row;
        if (row < sim->hist_evac_rows)
          cold->evac_bin = int(sim->hist_evac_base) + row * sim->hist_vac_n + b;
        else
          ++cold->n_dropped;
      }
    }
    else if (b == BIN_BEYOND)
      ++cold->n_dropped;
  }
  template <class R, class E>
  __device__ void replacement(const R & rec, const E & el, Real Erec, uint64_t key)
  {
    if constexpr (EV)
      event(EV_REPLACEMENT, Real(rec.x), Real(rec.y), Real(rec.z), Erec, el.Z2, Real(el.m2), rec.gen, 0,
            Real(el.Elbind), key, rec.tag);
    ++cold->n_repl;
    const int b = depth_bin(Real(rec.x), inv_vac_bin(), sim->hist_vac_n);
    if (b >= 0)
      repl_bin = int(sim->hist_vac_base + sim->hist_vac_n) + b;
    else if (b == BIN_BEYOND)
      ++cold->n_dropped;
  }
  template <class P>
  __device__ void stop(int state, const P & p, int Z1, Real m1)
  {
    if constexpr (EV)
      event(EV_REST, Real(p.x), Real(p.y), Real(p.z), Real(p.E), Z1, m1, p.gen, state, Real(0), p.key, p.tag,
            cold->m_md);
    if (MID && prm->records)
      cold->m_state = state;
    a_enuc.add(Real(p.E));
    deposit(Real(p.x), Real(p.y), Real(p.z), Real(p.E));
    if (state == ST_INTERSTITIAL)
      ++cold->n_inter;
    else if (state == ST_SUBSTITUTIONAL)
      ++cold->n_subst;
    if (p.gen == 0)
    {
      prm->prim.fx[gprim] = double(p.x);
      prm->prim.fy[gprim] = double(p.y);
      prm->prim.fz[gprim] = double(p.z);
      prm->prim.fstate[gprim] = state;
      const int b = depth_bin(Real(p.x), inv_range_bin(), sim->hist_range_n);
      if (b >= 0)
        atomicAdd(prm->hist + sim->hist_range_base + b, 1ull);
      if (sim->hist_lat_n > 0)
      {
        const float qy = (float(p.y) - sim->lat_y0) * sim->inv_hist_lat_bin;
        const float qz = (float(p.z) - sim->lat_z0) * sim->inv_hist_lat_bin;
        const int n = sim->hist_lat_n;
        if (qy >= 0.0f && qz >= 0.0f && qy < float(n) && qz < float(n))
          atomicAdd(prm->hist + sim->hist_lat_base + (long long)int(qz) * n + int(qy), 1ull);
      }
    }
  }

  // truncation toward zero like int(x) in the reference (TrimVacCount.C:36-39),
  // in the engine's own precision; BIN_BEYOND past the last bin, -1 before the
  // first (where the reference drops the event too) or without a histogram
  static constexpr int BIN_BEYOND = -2;
  static __device__ int depth_bin(Real x, Real inv_bin, int n)
  {
    const Real q = x * inv_bin;
    if (n <= 0 || !(q > Real(-1)))
      return -1;
    if (q >= Real(n))
      return BIN_BEYOND;
    return int(q);
  }
  static __device__ Real loge(Real x)
  {
    if constexpr (sizeof(Real) == sizeof(float))
      return __logf(x);
    else
      return log64(x);
  }
  __device__ Real inv_vac_bin() const
  {
    if constexpr (sizeof(Real) == sizeof(float))
      return sim->inv_hist_vac_bin_f;
    else
      return sim->inv_hist_vac_bin;
  }
  __device__ Real inv_range_bin() const
  {
    if constexpr (sizeof(Real) == sizeof(float))
      return sim->inv_hist_range_bin_f;
    else
      return sim->inv_hist_range_bin;
  }
  static __device__ Real powr(Real x, Real y)
  {
    if constexpr (sizeof(Real) == sizeof(float))
      return __powf(x, y);
    else
      return pow64(x, y);
  }

  // every Pol::FLUSH_EVERY collisions of a lane, hand the energy sums to the
  // per-primary arrays (no-op for FLUSH_EVERY = 0)
  __device__ void tick()
  {
    if constexpr (Pol::FLUSH_EVERY > 0)
      if ((a_coll & unsigned(Pol::FLUSH_EVERY - 1)) == 0u)
      {
        if (a_eel.nonzero())
          a_eel.atomic_add_to(prm->prim.eel + gprim);
        if (a_enuc.nonzero())
          a_enuc.atomic_add_to(prm->prim.enuc + gprim);
        a_eel.reset();
        a_enuc.reset();
      }
  }

  __device__ void flush_prim()
  {
    if (gprim < 0)
      return;
    if (a_vac)
      atomicAdd(prm->prim.vac + gprim, (unsigned long long)a_vac);
    if (a_coll)
      atomicAdd(prm->prim.coll + gprim, (unsigned long long)a_coll);
    if (a_eel.nonzero())
      a_eel.atomic_add_to(prm->prim.eel + gprim);
    if (a_enuc.nonzero())
      a_enuc.atomic_add_to(prm->prim.enuc + gprim);
    reset_prim();
  }
  __device__ void flush_sim(int s)
  {
    if (s < 0)
      return;
    SimTotals * t = prm->totals + s;
    const LaneCold<Acc> & c = *cold;
    using ull = unsigned long long;
    if (c.n_members)
      atomicAdd(&t->members, ull(c.n_members));
    if (c.n_repl)
      atomicAdd(&t->replacements, ull(c.n_repl));
    if (c.n_inter)
      atomicAdd(&t->interstitials, ull(c.n_inter));
    if (c.n_subst)
      atomicAdd(&t->substitutionals, ull(c.n_subst));
    if (c.n_lost)
      atomicAdd(&t->lost, ull(c.n_lost));
    if (n_newton)
      atomicAdd(&t->newton_iters, ull(n_newton));
    if (c.n_passes)
      atomicAdd(&t->rejection_passes, ull(c.n_passes));
    if (c.n_fallbacks)
      atomicAdd(&t->fallbacks, ull(c.n_fallbacks));
    if (c.e_lost.nonzero())
      c.e_lost.atomic_add_to(&t->Elost);
    if (c.e_unf.nonzero())
      c.e_unf.atomic_add_to(&t->Eunfollowed);
    if (c.n_sput)
      atomicAdd(&t->sputtered, ull(c.n_sput));
    if (c.n_back)
      atomicAdd(&t->backscattered, ull(c.n_back));
    if (c.e_sput.nonzero())
      c.e_sput.atomic_add_to(&t->Esputtered);
    if (c.n_dropped)
      atomicAdd(&t->hist_dropped, ull(c.n_dropped));
    reset_sim();
  }
};

// LVL: the feature level (KernelLevel); the collision code knows the cluster
// geometry at LVL_GEO, LVL_FULL, LVL_CLU and LVL_CLU_EV, the non-universal
// potentials at LVL_GEO and LVL_FULL
template <class Pol, int LVL>
__global__ void __launch_bounds__(128, Pol::min_blocks(LVL))
cascade_kernel(const EngineParams prm, const typename Pol::Tables tabs)
{
  constexpr bool MID = LVL >= LVL_MID;
  constexpr bool EXT = level_clusters(LVL);   // the cluster geometry
  constexpr bool POT = level_potentials(LVL); // the Moliere and C-Kr potentials
  using Particle = typename Pol::Particle;
  extern __shared__ __align__(16) unsigned char smem[];

  // stage the tables of a single-simulation run in shared memory
  // per-block vacancy / replacement counters (zeroed before the staging barrier)
  unsigned int * s_hist = reinterpret_cast<unsigned int *>(smem + prm.hist_smem_offset);
  for (int i = threadIdx.x; i < prm.hist_smem_bins; i += blockDim.x)
    s_hist[i] = 0u;
  if (prm.hist_smem_bins)
    __syncthreads();
  const typename Pol::Tables tab = Pol::stage(prm, tabs, smem);

  const unsigned int FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const unsigned int lt = lanemask_lt();
  const long long warp_id = (long long)(blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  Particle * stack = reinterpret_cast<Particle *>(prm.stacks) + warp_id * prm.stack_cap;
  Particle * overflow = reinterpret_cast<Particle *>(prm.overflow);
  const Particle * in_records = reinterpret_cast<const Particle *>(prm.in_records);
  long long n_work = prm.total_primaries;
  if (prm.in_records)
  {
    const long long c = (long long)*prm.in_count;
    n_work = c < prm.in_cap ? c : prm.in_cap;
  }

  int top = 0;
  bool work_done = false; // no more primaries / input records for this warp
  // members per refill: the launch's choice for fresh primaries; for the records of
  // a drain pass, a quarter of a warp's fair share (at most one per lane)
  int max_take = prm.max_take;
  if (prm.in_records)
  {
    const long long nwarps = (long long)gridDim.x * (blockDim.x >> 5);
    const long long share = n_work / (nwarps * 4);
    max_take = share < 1 ? 1 : (share > 32 ? 32 : int(share));
  }
  bool live = false;
  Particle p;
  uint32_t ic = 0;
  typename Pol::Real r1 = 0;
  int cur_sim = -1;
  const SimDesc * sim = nullptr;
  typename Pol::MemberCtx mctx;

  LaneSink<Pol, LVL> sink;
  sink.cold = reinterpret_cast<LaneCold<typename Pol::Acc> *>(smem + prm.cold_offset) + threadIdx.x;
  sink.cold->vcell = -1;
  sink.cold->vacc = 0.0f;
  sink.cold->evac_bin = -1;
  sink.cold->ev_next = sink.cold->ev_end = 0;
  sink.prm = &prm;
  sink.sim = nullptr;
  sink.gprim = -1;
  sink.range_mode = 0;
  sink.vox = false;
  sink.dep_in = false;
  sink.reset_prim();
  sink.reset_sim();
  sink.reset_member();

  auto start_member = [&](const Particle & q) {
    p = q;
    ic = 0;
    if (p.sim != cur_sim)
    {
      sink.flush_prim();
      sink.flush_sim(cur_sim);
      cur_sim = p.sim;
      sim = prm.sims + cur_sim;
      sink.sim = sim;
      sink.range_mode = sim->range_mode;
      sink.vox = MID && prm.voxels != nullptr && sim->voxel_n[0] > 0;
      sink.gprim = -1;
    }
    if ((long long)p.prim != sink.gprim)
    {
      sink.flush_prim();
      sink.gprim = (long long)p.prim;
      if (sink.n_newton > 0x40000000u || sink.cold->n_passes > 0x40000000u)
        sink.flush_sim(cur_sim);
    }
    Pol::begin_member(mctx, prm, tab, *sim, p);
    if constexpr (LaneSink<Pol, LVL>::EV)
    {
      // IonMDTag: the demo programs' MD-gap mark, taken when the member starts
      // (apps/mytrim_solid.C:156-159); a spawned recoil's _md is 0 (ion.C:88-93)
      bool gap;
      if constexpr (sizeof(typename Pol::Real) == 8)
        gap = double(p.E) > sim->md_Emin && double(p.E) < sim->md_Emax;
      else
        gap = float(p.E) > sim->md_Emin_f && float(p.E) < sim->md_Emax_f; // no FP64 in the FP32 engine
      sink.cold->m_md = (sim->md_Z != 0 && mctx.sc->Z1 == sim->md_Z && gap) ? 1 : 0;
    }
    r1 = Pol::first_draw(p.key, prm.k0, prm.k1);
    sink.reset_member();
    ++sink.cold->n_members;
  };

  unsigned int steps = 0;
  while (true)
  {
    ++steps;
    // ---- refill idle lanes: recoils from the warp stack first, then new work
    // idle lanes wait until refill_min (at most 32) of them need a member, so that
    // the member-start code below runs for several lanes at once: without waiting
    // it runs in nearly every iteration, for about four lanes of the 32
    const unsigned int idle = __ballot_sync(FULL, !live);
    if (idle && __popc(idle) >= prm.refill_min)
    {
      const int nidle = __popc(idle);
      const int rank = __popc(idle & lt);
      const int npop = nidle < top ? nidle : top;
      if (!live && rank < npop)
      {
        start_member(stack[top - 1 - rank]);
        live = true;
      }
      top -= npop;
      int need = nidle - npop;
      if (need > max_take)
        need = max_take;
      if (need > 0 && !work_done)
      {
        unsigned long long base = 0;
        const int leader = __ffs(idle) - 1;
        if (lane == leader)
          base = atomicAdd(prm.next_primary, (unsigned long long)need);
        base = __shfl_sync(FULL, base, leader);
        const long long avail = n_work - (long long)base;
        if (avail <= need)
          work_done = true;
        const int r = rank - npop;
        if (!live && r >= 0 && r < need && r < avail)
        {
          const long long g = (long long)base + r;
          if (prm.in_records)
            start_member(in_records[g]);
          else
          {
            const int s = prm.n_sims > 1 ? find_sim(prm.sim_prim_end, prm.n_sims, g) : 0;
            start_member(Pol::make_primary(prm.sims[s], s, g));
          }
          live = true;
        }
      }
    }
    if (__ballot_sync(FULL, live) == 0)
      break;

    // ---- one collision per live lane
    Particle rec;
    int flags = 0;
    sink.vac_bin = -1;
    sink.repl_bin = -1;
    if (live)
    {
      ++ic;
      ++sink.a_coll;
    }
    // every lane takes part (a policy may evaluate warp-collective code); lanes
    // without a member do no work and get no flags
    flags = Pol::template collide<EXT, POT>(live, p, ic, r1, mctx, prm.k0, prm.k1, rec, sink);
    if (live)
    {
      if (flags & CF_VOID)
        --sink.a_coll; // the member left without a collision (no checkPKAState)
      sink.tick();
      if (!(flags & CF_DONE) && ic >= prm.max_collisions)
      {
        atomicOr(prm.error_flags, ERRB_BUDGET);
        flags |= CF_DONE;
      }
      if (flags & CF_DONE)
      {
        live = false;
        if (MID && prm.records)
        {
          const unsigned long long slot = atomicAdd(prm.n_records, 1ull);
          if ((long long)slot < prm.records_cap)
          {
            MemberRecord m;
            m.key = p.key;
            m.sim = p.sim;
            m.species = p.species;
            m.gen = p.gen;
            m.state = sink.cold->m_state;
            m.ncoll = ic;
            m.nvac = sink.cold->m_vac;
            m.E = double(p.E);
            m.x = double(p.x);
            m.y = double(p.y);
            m.z = double(p.z);
            m.eel = sink.cold->m_eel.value();
            prm.records[slot] = m;
          }
        }
      }
      if (flags & CF_PUSH)
      {
        rec.sim = p.sim;
        rec.prim = p.prim;
      }
    }
    // depth histograms: a collision makes a vacancy or a replacement, never both;
    // about one lane in ten has an event, so each adds its own count (aggregating
    // lanes with __match_any_sync cost more than it saved)
    {
      const int hb = sink.vac_bin >= 0 ? sink.vac_bin : sink.repl_bin;
      if (hb >= 0)
      {
        if (prm.hist_smem_bins)
          atomicAdd(s_hist + (hb - prm.hist_smem_base), 1u);
        else
          atomicAdd(prm.hist + hb, 1ull);
      }
    }
    if (MID && prm.any_evac)
    {
      if (sink.cold->evac_bin >= 0)
        atomicAdd(prm.hist + sink.cold->evac_bin, 1ull);
      sink.cold->evac_bin = -1;
    }

    // ---- push displaced recoils onto the warp stack
    const bool push = (flags & CF_PUSH) != 0;
    const unsigned int pm = __ballot_sync(FULL, push);
    if (pm)
    {
      if (push)
      {
        const int slot = top + __popc(pm & lt);
        if (slot < prm.stack_cap)
          stack[slot] = rec;
        else
        {
          const unsigned long long o = atomicAdd(prm.overflow_count, 1ull);
          if ((long long)o < prm.overflow_cap)
            overflow[o] = rec;
          else
            atomicOr(prm.error_flags, ERRB_QUEUE_FULL);
        }
      }
      top += __popc(pm);
      if (top > prm.stack_cap)
        top = prm.stack_cap;
    }

  }
  sink.flush_prim();
  sink.flush_sim(cur_sim);
  sink.flush_voxel();
  sink.flush_events();
  if (prm.hist_smem_bins)
  {
    // every warp of the block has left its loop: add the block's counts
    __syncthreads();
    for (int i = threadIdx.x; i < prm.hist_smem_bins; i += blockDim.x)
      if (s_hist[i])
        atomicAdd(prm.hist + prm.hist_smem_base + i, (unsigned long long)s_hist[i]);
  }
  if (lane == 0)
  {
    atomicAdd(prm.warp_steps, (unsigned long long)(steps - 1)); // the last pass finds no work
  }
}

} // namespace mtg
