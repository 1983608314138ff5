// FP32 cascade path: the same collision loop as the FP64 plain path
// (TrimBase::trim, trim.C:74-424) in single precision, with three changes of
// evaluation that keep FP32 accurate and fast:
//   * electronic stopping and the maximum impact parameter of the free flight are
//     read from a per-(species, material) table of (S(E), p_max(E)) pairs, uniform
//     in ln E with 2048 points and filled by the FP64 code, instead of
//     re-evaluating ~11 transcendentals per element (S) and a chain of two square
//     roots, a power and two divisions (p_max) per collision;
//   * the Newton solve for the distance of closest approach iterates on
//     d = r - b (the same Newton steps as trim.C:192-233 written in a variable
//     that does not cancel), and sin^2(theta/2) is formed as (1 - co)(1 + co)
//     with 1 - co = d (1 - A F / (F + 1)) / (r + roc), algebraically equal to
//     1 - co^2 of trim.C:266-269 without its cancellation at small angles; the
//     solve starts from a tabulated first guess (mtg_newton_guess.h), so one
//     step nearly always meets the reference's stopping test;
//   * the random azimuth is drawn directly (uniform angle around the flight
//     direction) instead of by unit-ball rejection; the two give the same
//     distribution, and the direct draw has no data-dependent loop.
// Energies are kept as a float pair (value + rounding remainder) so that
// the small per-collision losses are not rounded away, and the lane tallies use
// Kahan-compensated sums; FP64 instructions stay out of the collision loop.
#include <mutex>
#include <vector>

#include "mtg_common.cuh"
#include "mtg_collide64.cuh"
#include "mtg_engine.cuh"
#include "mtg_geometry.cuh"
#include "mtg_kernels.h"
#include "mtg_scatter32.cuh"
#include "mtg_surrogate.cuh"

// resident 128-thread blocks per SM the register budget of each feature level is
// cut for: lean, mid and events 8 (64 registers), full and clusters+events 7 (72),
// geometry and clusters 6 (80).
// Measured per level: eight blocks beat seven for the mid and events levels in spite
// of their spills (32 and 80 bytes): +14 % (mid), +7 % (events, full log), +25 %
// (events, log nearly empty) on B 10 keV into SiO2/Si; the full level gains 7.5 % at
// seven (Xe into UO2 with bubbles, event log on; 214 bytes of spill), while the
// geometry level loses 3.5 % at seven and 4 % at eight; the lean level loses 2 to
// 4 % at nine (56 registers)
#ifndef MTG_FP32_MIN_BLOCKS
#define MTG_FP32_MIN_BLOCKS 7
#endif
#ifndef MTG_FP32_MIN_BLOCKS_MID
#define MTG_FP32_MIN_BLOCKS_MID 8
#endif
#ifndef MTG_FP32_MIN_BLOCKS_EVENTS
#define MTG_FP32_MIN_BLOCKS_EVENTS 8
#endif
#ifndef MTG_FP32_MIN_BLOCKS_GEO
#define MTG_FP32_MIN_BLOCKS_GEO 6
#endif
#ifndef MTG_FP32_MIN_BLOCKS_CLU
#define MTG_FP32_MIN_BLOCKS_CLU 6
#endif
#ifndef MTG_FP32_MIN_BLOCKS_CLU_EV
#define MTG_FP32_MIN_BLOCKS_CLU_EV 7
#endif
#ifndef MTG_FP32_MIN_BLOCKS_LEAN
#define MTG_FP32_MIN_BLOCKS_LEAN 8
#endif

namespace mtg
{

struct P32
{
  float x, y, z;
  float dx, dy, dz;
  float E, El;   // energy as value + remainder
  uint64_t key;
  int species;
  int gen;
  int sim;
  uint32_t prim;
  int tag; // IonBase::_tag: cluster index where a followed recoil was created, else -1
};

struct Tables32
{
  const Species32 * species;
  const Mat32 * mats;
  const Sim32 * sims;
  const float2 * stop; // (S, p_max) pairs, STOP_N per row
  float lnE_min, inv_dlnE;
  const SurrogateNet * net;
};

// E -= d, keeping the rounding remainder (TwoSum followed by FastTwoSum)
__device__ __forceinline__ void
ff_sub(float & hi, float & lo, float d)
{
  const float s = hi - d;
  const float bb = s - hi;
  const float err = (hi - (s - bb)) + (-d - bb);
  const float l = lo + err;
  const float h = s + l;
  lo = l - (h - s);
  hi = h;
}

// S(E) and p_max(E) from one row of the table; false below its first point, where
// S scales as sqrt(E) from there and p_max is left to the formula
__device__ __forceinline__ bool
stop_lookup(const float2 * row, float lnE_min, float inv_d, float E, float & S, float & pmax)
{
  const float u = (__logf(E) - lnE_min) * inv_d;
  if (!(u > 0.0f))
  {
    S = row[0].x * sqrtf(E * float(1.0 / STOP_EMIN));
    return false;
  }
  const int i = min(int(u), STOP_N - 2);
  const float f = u - float(i);
  const float2 a = row[i], b = row[i + 1];
  S = fmaf(f, b.x - a.x, a.x);
  pmax = fmaf(f, b.y - a.y, a.y);
  return true;
}

template <bool SURROGATE>
struct Fp32Policy
{
  using Particle = P32;
  using Real = float;
  using Acc = AccKahan32;
  using AccHot = AccF32;
  static constexpr int FLUSH_EVERY = 64; // collisions per hand-over of the hot energy sums (power of 2)
  using Tables = Tables32;
  // resident 128-thread blocks per SM the register budget of the variant of level
  // `lvl` is cut for (the surrogate's tensor-core fragments need more registers)
  static constexpr int min_blocks(int lvl)
  {
    return SURROGATE ? 4
                     : lvl == LVL_LEAN   ? MTG_FP32_MIN_BLOCKS_LEAN
                     : lvl == LVL_MID    ? MTG_FP32_MIN_BLOCKS_MID
                     : lvl == LVL_EVENTS ? MTG_FP32_MIN_BLOCKS_EVENTS
                     : lvl == LVL_GEO    ? MTG_FP32_MIN_BLOCKS_GEO
                     : lvl == LVL_CLU    ? MTG_FP32_MIN_BLOCKS_CLU
                     : lvl == LVL_CLU_EV ? MTG_FP32_MIN_BLOCKS_CLU_EV
                                         : MTG_FP32_MIN_BLOCKS;
  }

  struct MemberCtx
  {
    const Sim32 * sim;
    const Species32 * sc;
    const Mat32 * mrow;
    const float2 * stop;
    float lnE_min, inv_dlnE;
    const SurrogateNet * net;
  };

  static __device__ Tables stage(const EngineParams & prm, const Tables & g, unsigned char * smem)
  {
    if (!prm.stage_tables)
    {
      if constexpr (!SURROGATE)
        return g;
      // the network always lives in shared memory
      Tables t = g;
      SurrogateNet * s_net = reinterpret_cast<SurrogateNet *>(smem);
      for (int i = threadIdx.x; i < int(sizeof(SurrogateNet) / 4); i += blockDim.x)
        reinterpret_cast<float *>(s_net)[i] = reinterpret_cast<const float *>(g.net)[i];
      __syncthreads();
      t.net = s_net;
      return t;
    }
    Tables t = g;
    unsigned char * q = smem;
    const int ns = prm.n_stage_species, nm = prm.n_stage_mats;
    Species32 * s_sp = reinterpret_cast<Species32 *>(q);
    q += sizeof(Species32) * ns;
    Mat32 * s_mc = reinterpret_cast<Mat32 *>(q);
    q += sizeof(Mat32) * nm;
    const int n1 = int(sizeof(Species32) / 4) * ns;
    const int n2 = int(sizeof(Mat32) / 4) * nm;
    for (int i = threadIdx.x; i < n1; i += blockDim.x)
      reinterpret_cast<float *>(s_sp)[i] = reinterpret_cast<const float *>(g.species)[i];
    for (int i = threadIdx.x; i < n2; i += blockDim.x)
      reinterpret_cast<float *>(s_mc)[i] = reinterpret_cast<const float *>(g.mats)[i];
    // the stopping tables stay in global memory (L1-resident): the shared memory
    // they would take is worth more as an eighth resident block
    if (SURROGATE)
    {
      SurrogateNet * s_net = reinterpret_cast<SurrogateNet *>(smem + stage_net_offset(ns, nm));
      for (int i = threadIdx.x; i < int(sizeof(SurrogateNet) / 4); i += blockDim.x)
        reinterpret_cast<float *>(s_net)[i] = reinterpret_cast<const float *>(g.net)[i];
      t.net = s_net;
    }
    __syncthreads();
    t.species = s_sp;
    t.mats = s_mc;
    return t;
  }

  static __device__ __forceinline__ void begin_member(MemberCtx & m, const EngineParams & prm, const Tables & t,
                                                      const SimDesc & /*sim*/, const P32 & p)
  {
    const Sim32 * s = t.sims + p.sim;
    const int sbase = prm.stage_tables ? 0 : s->species_base;
    const int mbase = prm.stage_tables ? 0 : s->mat_base;
    m.sim = s;
    m.sc = t.species + sbase + p.species;
    m.mrow = t.mats + mbase + p.species * s->n_mat;
    m.stop = t.stop;
    m.lnE_min = t.lnE_min;
    m.inv_dlnE = t.inv_dlnE;
    m.net = t.net;
  }

  static __device__ __forceinline__ float first_draw(uint64_t key, uint32_t, uint32_t)
  {
    return key_u24f(key);
  }

  static __device__ __forceinline__ P32 make_primary(const SimDesc & s, int si, long long g)
  {
    P32 p;
    p.x = float(s.pos[0]);
    p.y = float(s.pos[1]);
    p.z = float(s.pos[2]);
    p.dx = float(s.dir[0]);
    p.dy = float(s.dir[1]);
    p.dz = float(s.dir[2]);
    p.E = float(s.E0);
    p.El = float(s.E0 - double(p.E));
    p.key = root_key(s.sim_key, uint64_t(g - s.prim_begin + s.key_offset));
    p.species = 0;
    p.gen = 0;
    p.sim = si;
    p.prim = uint32_t(g);
    p.tag = -1;
    return p;
  }

  // what the first half of a collision hands to the scattering and the second half
  struct PhaseA
  {
    const Mat32 * mc;
    int nn;        // target element
    float eps, b;  // reduced energy and impact parameter
    float ls, dee; // flight length and electronic loss
    uint32_t azimuth;
    bool gone;     // outside the sample: no collision, the member is dropped
    int tag;       // the material's _tag: the cluster index inside a cluster, else -1
  };

  // flight, target atom and electronic loss (trim.C:80-170)
  template <bool EXT>
  static __device__ __forceinline__ PhaseA phase_a(P32 & p, uint32_t ic, float r1, const MemberCtx & m, uint32_t k0,
                                                   uint32_t k1)
  {
    const Sim32 & sim = *m.sim;
    PhaseA a;
    // material lookup: SampleLayers (sample_layers.C:27-43) or sampleClusters
    // (sample_clusters.C:42-53)
    int k;
    a.gone = false;
    a.tag = -1;
    if (EXT && sim.geometry == 1)
    {
      const float pos[3] = {p.x, p.y, p.z};
      const int l = cluster_lookup<float>(pos, sim.w, sim.bc, sim.kn, sim.kd, sim.cmr, sim.cl, sim.cl_next,
                                          sim.cl_head, sim.n_clusters, sim.cl_mask, sim.mn, sim.inv_mcell);
      a.gone = l == -2; // no material: the member is dropped (trim.C:81-83)
      k = l >= 0 ? 1 : 0;
      a.tag = l >= 0 ? l : -1; // sampleClusters::lookupMaterial sets material[1]->_tag = l
    }
    else
    {
      int layer = 0;
      while (layer < sim.n_layers - 1 && !(p.x < sim.layer_end[layer]))
        ++layer;
      k = sim.layer_mat[layer];
    }
    a.mc = m.mrow + k;
    const Mat32 & mc = *a.mc;

    // normalise direction
    {
      const float s = rsqrtf(p.dx * p.dx + p.dy * p.dy + p.dz * p.dz);
      p.dx *= s;
      p.dy *= s;
      p.dz *= s;
    }
    const float E = p.E;

    // electronic stopping (material.C:114-121) and maximum impact parameter
    // (trim.C:88-94) from the table; the formula below its first point
    float S, pmax;
    if (!stop_lookup(m.stop + (long long)mc.row * STOP_N, m.lnE_min, m.inv_dlnE, E, S, pmax))
    {
      const float eeg = sqrtf(E * mc.f * mc.epsdg);
      pmax = mc.a / (eeg + sqrtf(eeg) + 0.125f * __expf(0.1f * __logf(eeg)));
    }
    // free flight (trim.C:88-94)
    float ls = mc.inv_pi_arho / (pmax * pmax);
    if (ic == 1)
      ls = r1 * fminf(ls, sim.cw);
    a.ls = ls;

    // impact parameter and azimuth from one Philox2x32-10 block per collision; the
    // target atom of a multi-element material from a second block whose counter is
    // the member key with its top bit flipped
    uint32_t u_imp, u_el = 0u;
    {
      const U2 d = draw_pair(p.key, ic, k0, k1);
      u_imp = d.x;
      a.azimuth = d.y;
      if (mc.nel > 1)
        u_el = draw_pair(p.key ^ 0x8000000000000000ull, ic, k0, k1).x;
    }
    const float r2 = u24f(u_imp);
    float hh = u24f(u_el);
    const float pimp = pmax * sqrtf(r2);
    int nn = 0;
    for (; nn < mc.nel - 1; ++nn)
    {
      hh -= mc.el[nn].t;
      if (hh <= 0.0f)
        break;
    }
    a.nn = nn;
    a.eps = mc.el[nn].fi * E;
    a.b = pimp * mc.el[nn].inv_ai;

    // electronic loss
    a.dee = ls * S;
    return a;
  }

  // EXT: the cluster geometry; POT: the Moliere and C-Kr potentials
  template <bool EXT, bool POT, class Sink>
  static __device__ __forceinline__ int collide(bool live, P32 & p, uint32_t ic, float r1, const MemberCtx & m,
                                                uint32_t k0, uint32_t k1, P32 & rec, Sink & sink)
  {
    PhaseA a;
    float s2, c2;
    int niter = 0;
    if constexpr (SURROGATE)
    {
      bool nn = false;
      if (live)
      {
        a = phase_a<EXT>(p, ic, r1, m, k0, k1);
        // the network is trained on the universal potential only
        nn = !a.gone && (!POT || m.sim->potential == 0) && surrogate_in_domain(a.eps, a.b);
      }
      // warp-collective: the lanes whose collision is in the network's domain are
      // evaluated together, the others (no member, or the exact fallback) only take
      // part in the shuffles
      const float o0 = surrogate_eval_warp(m.net, nn, nn ? surrogate_x1(a.eps) : 0.0f, nn ? surrogate_x2(a.b) : 0.0f);
      if (!live)
        return 0;
      if (a.gone)
        return CF_DONE | CF_VOID;
      if (nn)
        surrogate_s2_from(a.eps, a.b, o0, s2, c2);
      else
      {
        sink.fallback();
        scatter32(a.eps, a.b, s2, c2, niter, POT ? m.sim->potential : 0);
      }
    }
    else
    {
      if (!live)
        return 0;
      a = phase_a<EXT>(p, ic, r1, m, k0, k1);
      if (a.gone)
        return CF_DONE | CF_VOID;
      scatter32(a.eps, a.b, s2, c2, niter, POT ? m.sim->potential : 0);
    }
    sink.newton(niter);
    const Sim32 & sim = *m.sim;
    const Mat32 & mc = *a.mc;
    const Elem32 & el = mc.el[a.nn];
    const float E = p.E;
    const float ls = a.ls;
    float dee = a.dee;

    // energy transfer, electronic loss, momenta (trim.C:275-296)
    float den = el.ec * s2 * E;
    if (dee >= E)
    {
      dee = E + p.El;
      p.E = 0.0f;
      p.El = 0.0f;
    }
    else
      ff_sub(p.E, p.El, dee);
    sink.eel(dee, p.x, p.y, p.z);
    const float p1 = sqrtf(m.sc->two_m1 * p.E);
    if (den >= p.E)
    {
      den = p.E + p.El;
      p.E = 0.0f;
      p.El = 0.0f;
    }
    else
      ff_sub(p.E, p.El, den);
    const float p2 = sqrtf(m.sc->two_m1 * p.E);

    // recoil at the pre-flight position (trim.C:306-318)
    rec.x = p.x;
    rec.y = p.y;
    rec.z = p.z;
    rec.gen = p.gen + 1;
    const float fl = (ls - sim.tau) * sim.flscale;
    p.x = fmaf(p.dx, fl, p.x);
    p.y = fmaf(p.dy, fl, p.y);
    p.z = fmaf(p.dz, fl, p.z);
    rec.dx = p.dx * p1;
    rec.dy = p.dy * p1;
    rec.dz = p.dz * p1;
    const float recE = den - el.Elbind;
    rec.E = recE;
    rec.El = 0.0f;
    rec.species = el.rspecies;
    rec.tag = -1; // a new IonBase (ion.C:26)

    // azimuth around the flight direction: orthonormal basis by Duff et al.,
    // "Building an Orthonormal Basis, Revisited" (JCGT 2017)
    const float sgn = copysignf(1.0f, p.dz);
    const float ia = -1.0f / (sgn + p.dz);
    const float bxy = p.dx * p.dy * ia;
    const float ux = 1.0f + sgn * p.dx * p.dx * ia, uy = sgn * bxy, uz = -sgn * p.dx;
    const float vx = bxy, vy = sgn + p.dy * p.dy * ia, vz = -p.dy;
    float sphi, cphi;
    __sincosf(6.283185307179586f * u24f(a.azimuth), &sphi, &cphi);
    const float px = cphi * ux + sphi * vx;
    const float py = cphi * uy + sphi * vy;
    const float pz = cphi * uz + sphi * vz;

    // new direction: cos(psi), sin(psi) of psi = atan2(st, ct + my) (trim.C:336-341)
    const float ct = c2 - s2;
    const float st = 2.0f * sqrtf(s2 * c2);
    const float cy = ct + el.my;
    const float ih = rsqrtf(st * st + cy * cy);
    const float cpsi = cy * ih, spsi = st * ih;
    p.dx = p.dx * cpsi + px * spsi;
    p.dy = p.dy * cpsi + py * spsi;
    p.dz = p.dz * cpsi + pz * spsi;
    rec.dx -= p.dx * p2;
    rec.dy -= p.dy * p2;
    rec.dz -= p.dz * p2;

    // CUT boundaries (trim.C:344-352)
    if (sim.any_cut)
    {
      const float pos[3] = {p.x, p.y, p.z};
      for (int i = 0; i < 3; ++i)
        if (sim.bc[i] == 2 && (pos[i] > sim.w[i] || pos[i] < 0.0f))
        {
          sink.lost(p.E + p.El + den, p, m.sc->Z1, m.sc->m1);
          return CF_DONE;
        }
    }

    // fate of recoil and projectile (trim.C:357-411)
    int flags = 0;
    int state = ST_MOVING;
    if (recE > el.disp_thresh)
    {
      sink.enuc(el.Elbind, rec.x, rec.y, rec.z);
      sink.history(p, m.sc->Z1, m.sc->m1);
      sink.branch(rec, el, p.key);
      const bool follow = rec.gen < sim.follow_gen;
      if (follow)
      {
        const float s = rsqrtf(rec.dx * rec.dx + rec.dy * rec.dy + rec.dz * rec.dz);
        rec.dx *= s;
        rec.dy *= s;
        rec.dz *= s;
        rec.key = child_key(p.key, ic);
        rec.tag = a.tag; // trim.C:365, after followRecoil's output
        flags |= CF_PUSH;
      }
      else
        sink.unfollowed(recE);
      if (p.E > el.Edisp)
        sink.vacancy(rec, el, recE, p.key);
      else
      {
        sink.replacement(rec, el, recE, p.key);
        state = (m.sc->Z1 == el.Z2) ? ST_REPLACEMENT : ST_SUBSTITUTIONAL;
      }
    }
    else
    {
      sink.dissipate(rec, recE, el, p.key);
      sink.enuc(den, rec.x, rec.y, rec.z);
      if (p.E < sim.Ef)
        state = ST_INTERSTITIAL;
    }
    if (state != ST_MOVING)
    {
      p.E += p.El;
      p.El = 0.0f;
      sink.stop(state, p, m.sc->Z1, m.sc->m1);
      flags |= CF_DONE;
    }
    else if (!(p.E == p.E))
    {
      sink.numeric();
      flags |= CF_DONE;
    }
    return flags;
  }
};

cudaError_t
launch_cascade32(const EngineParams & prm, const Fp32Tables & t, int grid, int block, size_t smem, cudaStream_t st,
                 int surrogate)
{
  Tables32 tabs;
  tabs.species = reinterpret_cast<const Species32 *>(prm.species);
  tabs.mats = reinterpret_cast<const Mat32 *>(prm.mats);
  tabs.sims = reinterpret_cast<const Sim32 *>(t.sims32);
  tabs.stop = reinterpret_cast<const float2 *>(t.stop);
  tabs.lnE_min = t.lnE_min;
  tabs.inv_dlnE = t.inv_dlnE;
  tabs.net = reinterpret_cast<const SurrogateNet *>(t.mlp);
  if (surrogate)
    switch (prm.level)
    {
      case LVL_LEAN: cascade_kernel<Fp32Policy<true>, LVL_LEAN><<<grid, block, smem, st>>>(prm, tabs); break;
      case LVL_MID: cascade_kernel<Fp32Policy<true>, LVL_MID><<<grid, block, smem, st>>>(prm, tabs); break;
      case LVL_EVENTS: cascade_kernel<Fp32Policy<true>, LVL_EVENTS><<<grid, block, smem, st>>>(prm, tabs); break;
      // the surrogate engine runs the cluster-only levels in the geometry variants
      case LVL_GEO:
      case LVL_CLU: cascade_kernel<Fp32Policy<true>, LVL_GEO><<<grid, block, smem, st>>>(prm, tabs); break;
      default: cascade_kernel<Fp32Policy<true>, LVL_FULL><<<grid, block, smem, st>>>(prm, tabs); break;
    }
  else
    switch (prm.level)
    {
      case LVL_LEAN: cascade_kernel<Fp32Policy<false>, LVL_LEAN><<<grid, block, smem, st>>>(prm, tabs); break;
      case LVL_MID: cascade_kernel<Fp32Policy<false>, LVL_MID><<<grid, block, smem, st>>>(prm, tabs); break;
      case LVL_EVENTS: cascade_kernel<Fp32Policy<false>, LVL_EVENTS><<<grid, block, smem, st>>>(prm, tabs); break;
      case LVL_GEO: cascade_kernel<Fp32Policy<false>, LVL_GEO><<<grid, block, smem, st>>>(prm, tabs); break;
      case LVL_CLU: cascade_kernel<Fp32Policy<false>, LVL_CLU><<<grid, block, smem, st>>>(prm, tabs); break;
      case LVL_CLU_EV: cascade_kernel<Fp32Policy<false>, LVL_CLU_EV><<<grid, block, smem, st>>>(prm, tabs); break;
      default: cascade_kernel<Fp32Policy<false>, LVL_FULL><<<grid, block, smem, st>>>(prm, tabs); break;
    }
  return cudaGetLastError();
}

template <class K>
static cudaError_t
occupancy_of(K kernel, int block, size_t smem, int * blocks_per_sm)
{
  if (smem > 48 * 1024)
  {
    cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e != cudaSuccess)
      return e;
  }
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, kernel, block, smem);
}

template <bool SG>
static cudaError_t
occupancy_variants(int block, size_t smem, int * occ)
{
  cudaError_t e;
  if ((e = occupancy_of(cascade_kernel<Fp32Policy<SG>, LVL_LEAN>, block, smem, &occ[LVL_LEAN])) != cudaSuccess ||
      (e = occupancy_of(cascade_kernel<Fp32Policy<SG>, LVL_MID>, block, smem, &occ[LVL_MID])) != cudaSuccess ||
      (e = occupancy_of(cascade_kernel<Fp32Policy<SG>, LVL_EVENTS>, block, smem, &occ[LVL_EVENTS])) != cudaSuccess ||
      (e = occupancy_of(cascade_kernel<Fp32Policy<SG>, LVL_GEO>, block, smem, &occ[LVL_GEO])) != cudaSuccess ||
      (e = occupancy_of(cascade_kernel<Fp32Policy<SG>, LVL_FULL>, block, smem, &occ[LVL_FULL])) != cudaSuccess)
    return e;
  if constexpr (SG)
  {
    occ[LVL_CLU] = occ[LVL_GEO];
    occ[LVL_CLU_EV] = occ[LVL_FULL];
    return cudaSuccess;
  }
  else
  {
    if ((e = occupancy_of(cascade_kernel<Fp32Policy<SG>, LVL_CLU>, block, smem, &occ[LVL_CLU])) != cudaSuccess)
      return e;
    return occupancy_of(cascade_kernel<Fp32Policy<SG>, LVL_CLU_EV>, block, smem, &occ[LVL_CLU_EV]);
  }
}

// residency of the variant of feature level `level` (KernelLevel); every variant
// gets the shared-memory opt-in
cudaError_t
occupancy32(int block, size_t smem, int * blocks_per_sm, int surrogate, int level)
{
  int occ[LVL_COUNT] = {};
  cudaError_t e = surrogate ? occupancy_variants<true>(block, smem, occ) : occupancy_variants<false>(block, smem, occ);
  if (e != cudaSuccess)
    return e;
  *blocks_per_sm = occ[level < 0 ? 0 : (level >= LVL_COUNT ? LVL_COUNT - 1 : level)];
  return cudaSuccess;
}

size_t
record_size32()
{
  return sizeof(P32);
}

size_t
cold_slot_bytes32()
{
  return sizeof(LaneCold<AccKahan32>);
}

// ---- scattering service (FP32 exact)
__global__ void
scatter32_kernel(const double * eps, const double * b, long long n, double * s2, int potential)
{
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n)
    return;
  const float e = float(eps[i]), bb = float(b[i]);
  float s, c;
  int it;
  scatter32(e, bb, s, c, it, potential);
  s2[i] = double(s);
}

cudaError_t
launch_scatter32(const double * eps, const double * b, long long n, double * s2, int potential, cudaStream_t st)
{
  const int block = 256;
  if (n > 0)
    scatter32_kernel<<<(unsigned int)((n + block - 1) / block), block, 0, st>>>(eps, b, n, s2, potential);
  return cudaGetLastError();
}

// ---- first-guess table of the FP32 Newton solve
// phi(r) of the universal (pot 0) or Moliere (1) potential in FP64 (trim.C:197-213),
// with the project's exp64 so that the table has the same bits on every host
static double
screening_phi64(int pot, double r)
{
  if (pot == 1)
    return 0.35 * exp64(-0.3 * r) + 0.55 * exp64(-1.2 * r) + 0.1 * exp64(-6.0 * r);
  return 0.18175 * exp64(-3.1998 * r) + 0.50986 * exp64(-0.94229 * r) + 0.28022 * exp64(-0.4029 * r) +
         0.028171 * exp64(-0.20162 * r);
}

const float *
newton_guess_table32()
{
  // f(r) = b^2 / r + phi(r) / eps - r falls strictly with r, f(b) = phi(b) / eps > 0
  // and f(b + 2 / eps) < 0 because phi <= 1.000001: 72 halvings of that bracket
  // (at most 2^19 wide) leave the root to 1e-16, far below float resolution of d
  static std::vector<float> table;
  static std::once_flag once;
  std::call_once(once, [] {
    table.resize(NG_CELLS);
    for (int pot = 0; pot < NG_POT; ++pot)
      for (int i = 0; i < NG_U; ++i)
      {
        const double eps = exp64((NG_U0 + i * NG_DU) * 0.69314718055994531);
        for (int j = 0; j < NG_B; ++j)
        {
          const double b = j * NG_DB;
          double lo = b, hi = b + 2.0 / eps;
          for (int it = 0; it < 72; ++it)
          {
            const double m = 0.5 * (lo + hi);
            const double f = b * b / m + screening_phi64(pot, m) / eps - m;
            (f > 0.0 ? lo : hi) = m;
          }
          const double d = 0.5 * (lo + hi) - b;
          table[(size_t(pot) * NG_U + i) * NG_B + j] = float(log64(d) * 1.4426950408889634);
        }
      }
  });
  return table.data();
}

cudaError_t
upload_newton_guess32()
{
  return upload_newton_guess32_here(newton_guess_table32());
}

// ---- stopping through the FP32 table (one (species, material) row)
__global__ void
stopping32_kernel(const float * row, float lnE_min, float inv_d, const double * E, long long n, double * out)
{
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n)
  {
    float S = 0.0f, pmax = 0.0f;
    stop_lookup(reinterpret_cast<const float2 *>(row), lnE_min, inv_d, float(E[i]), S, pmax);
    out[i] = double(S);
  }
}

cudaError_t
launch_stopping32(const float * row, float lnE_min, float inv_d, const double * E, long long n, double * out,
                  cudaStream_t st)
{
  const int block = 256;
  if (n > 0)
    stopping32_kernel<<<(unsigned int)((n + block - 1) / block), block, 0, st>>>(row, lnE_min, inv_d, E, n, out);
  return cudaGetLastError();
}

} // namespace mtg
