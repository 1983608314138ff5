// One binary collision of one cascade member in FP64 -- the plain ("exact") path.
//
// This is the per-iteration body of TrimBase::trim (trim.C:74-424) with the
// universal ZBL potential: free flight and maximum impact parameter, target-atom
// choice, electronic loss (MaterialBase::getrstop, material.C:114-281), the
// Newton solve for the distance of closest approach and Biersack's "magic"
// scattering formula, energy and momentum bookkeeping, recoil creation, the
// random azimuth by unit-ball rejection, the CUT boundary and the fate of recoil
// and projectile.  The reference's virtual tally hooks become calls on a Sink.
//
// Differences from the reference that do not change the algorithm:
//   * random numbers come from Philox streams keyed by (member, collision, block)
//     instead of one mt19937 stream per primary;
//   * exp / log / pow are the project's own FP64 functions (mtg_common.cuh);
//   * psi = atan2(st, ct + my) followed by cos(psi), sin(psi) is evaluated as
//     (ct + my) / h and st / h with h = sqrt(st^2 + (ct + my)^2), the same numbers
//     without trigonometric calls;
//   * projectile-dependent material constants come from a table precomputed once
//     instead of MaterialBase::average per member.
// Compiled for the GPU (mtg_engine64.cu, -fmad=false) and for the host replay
// check, which must give the same bits.
#pragma once

#include "mtg_common.cuh"
#include "mtg_geometry.cuh"
#include "mtg_tables.h"

namespace mtg
{

struct P64
{
  double x, y, z;
  double dx, dy, dz;
  double E;
  uint64_t key;
  int species;   // species index within the simulation
  int gen;       // 0 for the primary
  int sim;       // simulation index
  uint32_t prim; // global primary index (tally slot)
  int tag;       // IonBase::_tag: cluster index where a followed recoil was created, else -1
};

// proton electronic stopping in one element (material.C:134-158)
MTG_HD double
proton_stop64(const StopPair & sp, double e)
{
  const double pe = e > 25.0 ? e : 25.0;
  const double lpe = log64(pe);
  const double sl = sp.pcoef[0] * exp64(sp.pcoef[1] * lpe) + sp.pcoef[2] * exp64(sp.pcoef[3] * lpe);
  const double sh = sp.pcoef[4] / exp64(sp.pcoef[5] * lpe) * log64(sp.pcoef[6] / pe + sp.pcoef[7] * pe);
  double s = sl * sh / (sl + sh);
  if (e <= 25.0)
    s *= pow64(e / 25.0, sp.velpwr);
  return s;
}

// electronic stopping of species sc with energy E [eV] in element sp, in the
// reference's units (material.C:161-281, result * 10)
MTG_HD double
ion_stop64(const SpeciesConst & sc, const StopPair & sp, double E)
{
  const double e = E * sc.inv_m1k; // keV/u
  double se;
  if (sc.branch == STOP_H)
    se = proton_stop64(sp, e);
  else if (sc.branch == STOP_HE)
  {
    const double he = e > 1.0 ? e : 1.0;
    const double b = log64(he);
    const double b2 = b * b;
    const double b4 = b2 * b2;
    double a = 0.2865 + 0.1266 * b - 0.001429 * b2 + 0.02402 * b * b2 - 0.01135 * b4 + 0.001475 * b4 * b;
    double heh = 1.0 - exp64(-(a < 30.0 ? a : 30.0));
    const double t = 7.6 - b;
    a = 1.0 + sp.hez * exp64(-(t * t));
    heh *= a * a;
    se = proton_stop64(sp, he) * heh * 4.0;
    if (e <= 1.0)
      se *= sqrt(e);
  }
  else
  {
    const double vf = sp.vfermi;
    const double v = sqrt(e / 25.0) / vf;
    const double v2 = v * v;
    double vr;
    if (v >= 1.0)
      vr = v * vf * (1.0 + 1.0 / (5.0 * v2));
    else
      vr = (3.0 * vf / 4.0) * (1.0 + (2.0 * v2 / 3.0) - v2 * v2 / 15.0);
    double yr = vr / sc.cb2;
    if (yr < sp.yrcut)
      yr = sp.yrcut;
    const double yr03 = pow64(yr, 0.3);
    double a = -0.803 * yr03 + 1.3167 * yr03 * yr03 + 0.38157 * yr + 0.008983 * yr * yr;
    double q = 1.0 - exp64(-(a < 50.0 ? a : 50.0));
    q = q < 0.0 ? 0.0 : (q > 1.0 ? 1.0 : q);
    const double b = sc.bq;
    const double l0 = (0.8 - q * sc.l0a) / sc.cb;
    double l1;
    if (q < 0.2)
      l1 = 0.0;
    else if (q < sc.qlo)
      l1 = b * (q - 0.2) / sc.qden;
    else if (q < sc.qhi)
      l1 = b;
    else
      l1 = b * (1.0 - q) / sc.qden2;
    const double l0f = l0 * sc.lfctr;
    const double l = l1 > l0f ? l1 : l0f;
    const double w = 4.0 * l * vf / 1.919;
    double zeta = q + sp.inv2vf2 * (1.0 - q) * log64(1.0 + w * w);
    const double le = log64(e);
    const double t = 7.6 - (le > 0.0 ? le : 0.0);
    zeta *= 1.0 + sc.inv_z1sq * sp.zc * exp64(-(t * t));
    const double zf = zeta * sc.fz1;
    if (yr <= sp.yrcut)
      se = sp.sp_eee * (zf * zf) * exp64(sp.power * (le - log64(sp.eee)));
    else
      se = proton_stop64(sp, e) * (zf * zf);
  }
  return se * 10.0;
}

// MaterialBase::getrstop (material.C:114-121), eV/Angstrom
MTG_HD double
material_stop64(const SpeciesConst & sc, const MatConst & mc, double E)
{
  double se = 0.0;
  for (int j = 0; j < mc.nel; ++j)
    se += ion_stop64(sc, mc.sp[j], E) * mc.el[j].t;
  return se * mc.arho;
}

// Scattering (trim.C:172-271) for the universal (pot 0), Moliere (1) or C-Kr (2)
// screened potential, each with its magic-formula constants; the reference's
// expressions as written, the C-Kr derivative coefficients included.  Returns
// s2 = sin^2(theta_cm/2) and ct, st = cos, sin of theta_cm; niter counts Newton
// iterations.
MTG_HD void
scatter64(double eps, double b, double & s2, double & ct, double & st, int & niter, int pot = 0)
{
  niter = 0;
  if (eps > 10.0)
  {
    const double w = 2.0 * eps * b;
    s2 = 1.0 / (1.0 + (1.0 + b * (1.0 + b)) * (w * w));
    const double c2 = 1.0 - s2;
    ct = 2.0 * c2 - 1.0;
    st = sqrt(1.0 - ct * ct);
    return;
  }
  double r = b;
  double rr = -2.7 * log64(eps * b);
  if (rr >= b)
  {
    rr = -2.7 * log64(eps * rr);
    if (rr >= b)
      r = rr;
  }
  double v, v1, q;
  do
  {
    if (pot == 1)
    {
      // Moliere (trim.C:206-213); Utility::pow<4> and pow<5> as the reference's
      // shim/pow.h multiplies: (x x)(x x) and x ((x x)(x x))
      const double ex1 = exp64(-0.3 * r);
      const double e1s = ex1 * ex1;
      const double ex2 = e1s * e1s;
      const double e2s = ex2 * ex2;
      const double ex3 = ex2 * (e2s * e2s);
      v = (0.35 * ex1 + 0.55 * ex2 + 0.1 * ex3) / r;
      v1 = -(v + 0.105 * ex1 + 0.66 * ex2 + 0.6 * ex3) / r;
    }
    else if (pot == 2)
    {
      // C-Kr (trim.C:215-222)
      const double ex1 = exp64(-0.279 * r);
      const double ex2 = exp64(-0.637 * r);
      const double ex3 = exp64(-1.1919 * r);
      v = (0.191 * ex1 + 0.474 * ex2 + 0.335 * ex3) / r;
      v1 = -(v + 0.531865 * ex1 + 0.30181 * ex2 + 0.6437 * ex3) / r;
    }
    else
    {
      const double ex1 = 0.18175 * exp64(-3.1998 * r);
      const double ex2 = 0.50986 * exp64(-0.94229 * r);
      const double ex3 = 0.28022 * exp64(-0.4029 * r);
      const double ex4 = 0.028171 * exp64(-0.20162 * r);
      v = (ex1 + ex2 + ex3 + ex4) / r;
      v1 = -(v + 3.1998 * ex1 + 0.94229 * ex2 + 0.4029 * ex3 + 0.20162 * ex4) / r;
    }
    const double fr = b * b / r + v * r / eps - r;
    const double fr1 = -b * b / (r * r) + (v + v1 * r) / eps - 1.0;
    q = fr / fr1;
    r -= q;
    ++niter;
  } while (fabs(q / r) > 0.001 && niter < 100);
  const double roc = -2.0 * (eps - v) / v1;
  const double sqe = sqrt(eps);
  double cc, aa, ff;
  if (pot == 1)
  {
    cc = (0.009611 + sqe) / (0.005175 + sqe);
    aa = 2.0 * eps * (1.0 + (0.6743 / sqe)) * pow64(b, cc);
    ff = (sqrt(aa * aa + 1.0) - aa) * ((6.314 + eps) / (10.0 + eps));
  }
  else if (pot == 2)
  {
    cc = (0.235809 + sqe) / (0.126000 + sqe);
    aa = 2.0 * eps * (1.0 + (1.0144 / sqe)) * pow64(b, cc);
    ff = (sqrt(aa * aa + 1.0) - aa) * ((6935.0 + eps) / (83550.0 + eps));
  }
  else
  {
    cc = (0.011615 + sqe) / (0.0071222 + sqe);
    aa = 2.0 * eps * (1.0 + (0.99229 / sqe)) * pow64(b, cc);
    ff = (sqrt(aa * aa + 1.0) - aa) * ((9.3066 + eps) / (14.813 + eps));
  }
  const double delta = (r - b) * aa * ff / (ff + 1.0);
  const double co = (b + delta + roc) / (r + roc);
  const double c2 = co * co;
  s2 = 1.0 - c2;
  ct = 2.0 * c2 - 1.0;
  st = sqrt(1.0 - ct * ct);
}

// One collision.  `mats` points at this species' MatConst row of the simulation
// (n_mat entries), ic is the 1-based collision index, r1 the member's first-flight
// draw.  Sink receives the tally events (see the engine and the host replay).  EXT
// enables the cluster geometry, POT the non-universal potentials.
template <bool EXT, bool POT = EXT, class Sink>
MTG_HD int
collide64(P64 & p, uint32_t ic, double r1, const SimDesc & sim, const SpeciesConst & sc,
          const MatConst * mats, uint32_t k0, uint32_t k1, P64 & rec, Sink & sink)
{
  // which material: SampleLayers::lookupLayer (sample_layers.C:27-43) or
  // sampleClusters::lookupMaterial (sample_clusters.C:42-53)
  int mat_index;
  int mat_tag = -1; // the material's _tag (sampleClusters sets material[1]->_tag = l)
  if (EXT && sim.geometry == 1)
  {
    const double pos[3] = {p.x, p.y, p.z};
    const int l = cluster_lookup<double>(pos, sim.w, sim.bc, sim.kn, sim.kd, sim.cmr, sim.cl, sim.cl_next,
                                         sim.cl_head, sim.n_clusters, sim.cl_mask, sim.mn, sim.inv_mcell);
    if (l == -2)
      return CF_DONE | CF_VOID; // no material: the member is dropped (trim.C:81-83)
    mat_index = l >= 0 ? 1 : 0;
    mat_tag = l >= 0 ? l : -1;
  }
  else
  {
    int layer = 0;
    while (layer < sim.n_layers - 1 && !(p.x < sim.layer_end[layer]))
      ++layer;
    mat_index = sim.layer_mat[layer];
  }
  const MatConst & mc = mats[mat_index];

  // normalise direction (trim.C:85)
  {
    const double s = 1.0 / sqrt(p.dx * p.dx + p.dy * p.dy + p.dz * p.dz);
    p.dx *= s;
    p.dy *= s;
    p.dz *= s;
  }

  // maximum impact parameter and free flight (trim.C:88-94)
  double eps = p.E * mc.f;
  const double eeg = sqrt(eps * mc.epsdg);
  const double pmax = mc.a / (eeg + sqrt(eeg) + 0.125 * pow64(eeg, 0.1));
  double ls = 1.0 / (3.14159265358979323846 * (pmax * pmax) * mc.arho);
  if (ic == 1)
    ls = r1 * (ls < sim.cw ? ls : sim.cw);

  // impact parameter and target atom (trim.C:143-160)
  const U4 d0 = draw_block(p.key, ic, 0u, k0, k1);
  const double r2 = u53(d0.x, d0.y);
  double hh = u53(d0.z, d0.w);
  const double pimp = pmax * sqrt(r2);
  int nn = 0;
  for (; nn < mc.nel - 1; ++nn)
  {
    hh -= mc.el[nn].t;
    if (hh <= 0)
      break;
  }
  const ElemConst & el = mc.el[nn];
  eps = el.fi * p.E;
  const double b = pimp / el.ai;

  // electronic loss along the flight path (trim.C:166-170)
  double dee = ls * material_stop64(sc, mc, p.E);

  double s2, ct, st;
  int niter;
  scatter64(eps, b, s2, ct, st, niter, POT ? sim.potential : 0);
  sink.newton(niter);

  // energy transfer, electronic loss, momenta (trim.C:275-296)
  double den = el.ec * s2 * p.E;
  if (dee > p.E)
    dee = p.E;
  p.E -= dee;
  sink.eel(dee, p.x, p.y, p.z);
  const double p1 = sqrt(2.0 * sc.m1 * p.E);
  if (den > p.E)
    den = p.E;
  p.E -= den;
  const double p2 = sqrt(2.0 * sc.m1 * p.E);

  // recoil at the pre-flight position (trim.C:306-318)
  rec.x = p.x;
  rec.y = p.y;
  rec.z = p.z;
  rec.gen = p.gen + 1;
  const double fl = (ls - sim.tau) * sim.invscale;
  p.x += p.dx * fl;
  p.y += p.dy * fl;
  p.z += p.dz * fl;
  rec.dx = p.dx * p1;
  rec.dy = p.dy * p1;
  rec.dz = p.dz * p1;
  rec.E = den - el.Elbind;
  rec.species = el.rspecies;
  rec.tag = -1; // a new IonBase (ion.C:26)

  // random unit vector perpendicular to dir by unit-ball rejection (trim.C:322-333)
  double px, py, pz, nrm;
  uint32_t pass = 0;
  do
  {
    double rx, ry, rz;
    do
    {
      const U4 dr = draw_block(p.key, ic, 1u + pass, k0, k1);
      ++pass;
      rx = 2.0 * u32d(dr.x) - 1.0;
      ry = 2.0 * u32d(dr.y) - 1.0;
      rz = 2.0 * u32d(dr.z) - 1.0;
    } while (rx * rx + ry * ry + rz * rz > 1.0 && pass < 64);
    px = p.dy * rz - p.dz * ry;
    py = p.dz * rx - p.dx * rz;
    pz = p.dx * ry - p.dy * rx;
    nrm = sqrt(px * px + py * py + pz * pz);
  } while (nrm == 0.0 && pass < 64);
  sink.passes(int(pass));
  if (nrm == 0.0)
  {
    sink.numeric();
    px = 0.0;
    py = 0.0;
    pz = 1.0;
    nrm = 1.0;
  }
  px /= nrm;
  py /= nrm;
  pz /= nrm;

  // new projectile direction (trim.C:336-341)
  const double cy = ct + el.my;
  const double h = sqrt(st * st + cy * cy);
  const double cpsi = cy / h, spsi = st / h;
  p.dx = p.dx * cpsi + px * spsi;
  p.dy = p.dy * cpsi + py * spsi;
  p.dz = p.dz * cpsi + pz * spsi;
  rec.dx -= p.dx * p2;
  rec.dy -= p.dy * p2;
  rec.dz -= p.dz * p2;

  // CUT boundaries (trim.C:344-352)
  const double pos[3] = {p.x, p.y, p.z};
  for (int i = 0; i < 3; ++i)
    if (sim.bc[i] == 2 && (pos[i] > sim.w[i] || pos[i] < 0.0))
    {
      sink.lost(p.E + den, p, sc.Z1, sc.m1);
      return CF_DONE;
    }

  // fate of recoil and projectile (trim.C:357-411)
  int flags = 0;
  int state = ST_MOVING;
  if (rec.E > el.Edisp - el.Elbind)
  {
    sink.enuc(el.Elbind, rec.x, rec.y, rec.z);
    sink.history(p, sc.Z1, sc.m1);
    sink.branch(rec, el, p.key);
    const bool follow = rec.gen < sim.follow_gen;
    if (follow)
    {
      const double s = 1.0 / sqrt(rec.dx * rec.dx + rec.dy * rec.dy + rec.dz * rec.dz);
      rec.dx *= s;
      rec.dy *= s;
      rec.dz *= s;
      rec.key = child_key(p.key, ic);
      rec.tag = mat_tag; // trim.C:365, after followRecoil's output
      flags |= CF_PUSH;
    }
    else
      sink.unfollowed(rec.E);
    if (p.E > el.Edisp)
      sink.vacancy(rec, el, rec.E, p.key);
    else
    {
      sink.replacement(rec, el, rec.E, p.key);
      state = (sc.Z1 == el.Z2) ? ST_REPLACEMENT : ST_SUBSTITUTIONAL;
    }
  }
  else
  {
    sink.dissipate(rec, rec.E, el, p.key);
    sink.enuc(rec.E + el.Elbind, rec.x, rec.y, rec.z);
    if (p.E < sim.Ef)
      state = ST_INTERSTITIAL;
  }
  if (state != ST_MOVING)
  {
    sink.stop(state, p, sc.Z1, sc.m1);
    flags |= CF_DONE;
  }
  else if (!(p.E == p.E))
  {
    sink.numeric();
    flags |= CF_DONE;
  }
  return flags;
}

} // namespace mtg
