// sampleClusters geometry: spheres of the cluster material in a matrix, found
// through a spatial hash (sample_clusters.C).  Shared by the FP64 engine, the FP32
// engine and the host replay build.
#pragma once

#include <cmath>

#include "mtg_common.cuh"
#include "mtg_tables.h"

namespace mtg
{

template <class Real>
MTG_HD Real
geo_floor(Real x)
{
  if constexpr (sizeof(Real) == sizeof(float))
    return floorf(x);
  else
    return floor(x);
}

template <class Real>
MTG_HD Real
geo_round(Real x)
{
  if constexpr (sizeof(Real) == sizeof(float))
    return roundf(x);
  else
    return round(x);
}

// Whether cluster q contains pos: the distance test of sampleClusters::lookupCluster
// with dr = 0 (sample_clusters.C:60-130), to the nearest image on periodic axes.
template <class Real, class C4>
MTG_HD bool
cluster_contains(const Real pos[3], const C4 & q, const Real w[3], const int bc[3])
{
  Real d0 = pos[0] - Real(q.x), d1 = pos[1] - Real(q.y), d2 = pos[2] - Real(q.z);
  if (bc[0] == 0)
    d0 -= geo_round(d0 / w[0]) * w[0];
  if (bc[1] == 0)
    d1 -= geo_round(d1 / w[1]) * w[1];
  if (bc[2] == 0)
    d2 -= geo_round(d2 / w[2]) * w[2];
  const Real r2 = d0 * d0 + d1 * d1 + d2 * d2;
  const Real rr = Real(q.r) + Real(0);
  return r2 < rr * rr;
}

// sampleClusters::lookupCluster with dr = 0 (sample_clusters.C:60-130): the index
// of the cluster that contains pos, -1 in the matrix, -2 outside a CUT boundary.
// The hash cells within ceil(cmr / kd) of pos's cell are searched in the
// reference's order; periodic axes measure the distance to the nearest image.
// Every cell list is walked at most n_clusters steps.  Before the search, the
// candidate lists (`cells`, mn cells per axis, built by mtg_setup.cpp) answer for
// most points: a cell not marked for the search lists every cluster that can
// contain a point of it, and at most one of them does, the cluster the search
// would return; no candidate containing pos means the matrix.  They are consulted
// only for periodic coordinates within 64 box lengths, where their rounding margin
// holds.
template <class Real, class C4>
MTG_HD int
cluster_lookup(const Real pos[3], const Real w[3], const int bc[3], const int kn[3], const Real kd[3], Real cmr,
               const C4 * c, const int * next, const int * head, int n_clusters, const uint32_t * cells,
               const int mn[3], const Real inv_mcell[3])
{
  int k[3];
  for (int i = 0; i < 3; ++i)
  {
    k[i] = int(geo_floor((pos[i] * Real(kn[i])) / w[i]));
    if (pos[i] < Real(0) || pos[i] >= w[i])
    {
      if (bc[i] == 2)
        return -2; // CUT
      if (bc[i] == 1)
        return -1; // INF
      k[i] = k[i] % kn[i];
      if (k[i] < 0)
        k[i] += kn[i];
    }
  }
  if (cells)
  {
    bool use = true;
    long long cell = 0, stride = 1;
    for (int i = 0; i < 3 && use; ++i)
    {
      Real x = pos[i];
      if (bc[i] == 0)
      {
        use = x >= -Real(64) * w[i] && x <= Real(64) * w[i];
        x -= geo_floor(x / w[i]) * w[i];
      }
      int m = int(x * inv_mcell[i]);
      m = m < 0 ? 0 : (m >= mn[i] ? mn[i] - 1 : m);
      cell += stride * m;
      stride *= mn[i];
    }
    if (use)
    {
      const uint32_t s0 = cells[cell];
      if (!(s0 & 0x80000000u))
      {
        const uint32_t s1 = cells[cell + 1] & 0x7fffffffu;
        for (uint32_t j = s0; j < s1; ++j)
        {
          const int l = int(cells[j]);
          if (cluster_contains(pos, c[l], w, bc))
            return l;
        }
        return -1;
      }
    }
  }
  int k1[3], k2[3];
  for (int i = 0; i < 3; ++i)
  {
    const int ks = int((cmr + Real(0)) / kd[i]) + 1;
    k1[i] = k[i] - ks;
    k2[i] = k[i] + ks;
    if (k1[i] < 0 && bc[i] != 0)
      k1[i] = 0;
    if (k2[i] >= kn[i] && bc[i] != 0)
      k2[i] = kn[i] - 1;
  }
  for (int j0 = k1[0]; j0 <= k2[0]; ++j0)
    for (int j1 = k1[1]; j1 <= k2[1]; ++j1)
      for (int j2 = k1[2]; j2 <= k2[2]; ++j2)
      {
        int m0 = j0 % kn[0], m1 = j1 % kn[1], m2 = j2 % kn[2];
        m0 += m0 < 0 ? kn[0] : 0;
        m1 += m1 < 0 ? kn[1] : 0;
        m2 += m2 < 0 ? kn[2] : 0;
        int l = head[m0 + kn[0] * (m1 + kn[1] * m2)];
        for (int guard = 0; l >= 0 && guard < n_clusters; ++guard)
        {
          if (cluster_contains(pos, c[l], w, bc))
            return l;
          l = next[l];
        }
      }
  return -1;
}

} // namespace mtg
