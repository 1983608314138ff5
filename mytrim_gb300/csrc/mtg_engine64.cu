// FP64 ("plain", exact scattering) instantiation of the cascade kernel, plus the
// FP64 stopping and scattering service kernels.  Compiled with -fmad=false so
// that every multiply and add is rounded separately, exactly as in the host
// replay build of the same code.
#include "mtg_collide64.cuh"

// resident 128-thread blocks per SM the register budget is cut for
#ifndef MTG_FP64_MIN_BLOCKS
#define MTG_FP64_MIN_BLOCKS 3
#endif
#include "mtg_engine.cuh"
#include "mtg_kernels.h"

namespace mtg
{

struct Fp64Policy
{
  using Particle = P64;
  using Real = double;
  using Acc = AccF64;
  using AccHot = AccF64;
  static constexpr int FLUSH_EVERY = 0;
  static constexpr int min_blocks(int) { return MTG_FP64_MIN_BLOCKS; } // 3: <= 170 registers, 12 warps per SM

  struct Tables
  {
    const SpeciesConst * species;
    const MatConst * mats;
  };

  struct MemberCtx
  {
    const SimDesc * sim;
    const SpeciesConst * sc;
    const MatConst * mrow;
  };

  // copy the species and material rows of a single-simulation run to shared memory
  static __device__ Tables stage(const EngineParams & prm, const Tables & g, unsigned char * smem)
  {
    if (!prm.stage_tables)
      return g;
    SpeciesConst * s_sp = reinterpret_cast<SpeciesConst *>(smem);
    MatConst * s_mc = reinterpret_cast<MatConst *>(smem + sizeof(SpeciesConst) * prm.n_stage_species);
    const int n1 = int(sizeof(SpeciesConst) / 8) * prm.n_stage_species;
    const int n2 = int(sizeof(MatConst) / 8) * prm.n_stage_mats;
    for (int i = threadIdx.x; i < n1; i += blockDim.x)
      reinterpret_cast<double *>(s_sp)[i] = reinterpret_cast<const double *>(g.species)[i];
    for (int i = threadIdx.x; i < n2; i += blockDim.x)
      reinterpret_cast<double *>(s_mc)[i] = reinterpret_cast<const double *>(g.mats)[i];
    __syncthreads();
    return Tables{s_sp, s_mc};
  }

  static __device__ __forceinline__ void begin_member(MemberCtx & m, const EngineParams & prm, const Tables & t,
                                                      const SimDesc & sim, const P64 & p)
  {
    const int sbase = prm.stage_tables ? 0 : sim.species_base;
    const int mbase = prm.stage_tables ? 0 : sim.mat_base;
    m.sim = &sim;
    m.sc = t.species + sbase + p.species;
    m.mrow = t.mats + mbase + p.species * sim.n_mat;
  }

  static __device__ __forceinline__ double first_draw(uint64_t key, uint32_t, uint32_t)
  {
    return key_u53(key);
  }

  static __device__ __forceinline__ P64 make_primary(const SimDesc & s, int si, long long g)
  {
    P64 p;
    p.x = s.pos[0];
    p.y = s.pos[1];
    p.z = s.pos[2];
    p.dx = s.dir[0];
    p.dy = s.dir[1];
    p.dz = s.dir[2];
    p.E = s.E0;
    p.key = root_key(s.sim_key, uint64_t(g - s.prim_begin + s.key_offset));
    p.species = 0;
    p.gen = 0;
    p.sim = si;
    p.prim = uint32_t(g);
    p.tag = -1;
    return p;
  }

  template <bool EXT, bool POT, class Sink>
  static __device__ __forceinline__ int collide(bool live, P64 & p, uint32_t ic, double r1, const MemberCtx & m,
                                                uint32_t k0, uint32_t k1, P64 & rec, Sink & sink)
  {
    if (!live)
      return 0;
    return collide64<EXT, POT>(p, ic, r1, *m.sim, *m.sc, m.mrow, k0, k1, rec, sink);
  }
};

cudaError_t
launch_cascade64(const EngineParams & prm, int grid, int block, size_t smem, cudaStream_t st)
{
  const Fp64Policy::Tables tabs{prm.species, prm.mats};
  switch (prm.level)
  {
    case LVL_LEAN: cascade_kernel<Fp64Policy, LVL_LEAN><<<grid, block, smem, st>>>(prm, tabs); break;
    case LVL_MID: cascade_kernel<Fp64Policy, LVL_MID><<<grid, block, smem, st>>>(prm, tabs); break;
    case LVL_EVENTS: cascade_kernel<Fp64Policy, LVL_EVENTS><<<grid, block, smem, st>>>(prm, tabs); break;
    // the FP64 engine runs the cluster-only levels in the geometry variants
    case LVL_GEO:
    case LVL_CLU: cascade_kernel<Fp64Policy, LVL_GEO><<<grid, block, smem, st>>>(prm, tabs); break;
    default: cascade_kernel<Fp64Policy, LVL_FULL><<<grid, block, smem, st>>>(prm, tabs); break;
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

// residency of the variant of feature level `level` (KernelLevel); every variant
// gets the shared-memory opt-in
cudaError_t
occupancy64(int block, size_t smem, int * blocks_per_sm, int level)
{
  int occ[LVL_COUNT] = {};
  cudaError_t e;
  if ((e = occupancy_of(cascade_kernel<Fp64Policy, LVL_LEAN>, block, smem, &occ[LVL_LEAN])) != cudaSuccess ||
      (e = occupancy_of(cascade_kernel<Fp64Policy, LVL_MID>, block, smem, &occ[LVL_MID])) != cudaSuccess ||
      (e = occupancy_of(cascade_kernel<Fp64Policy, LVL_EVENTS>, block, smem, &occ[LVL_EVENTS])) != cudaSuccess ||
      (e = occupancy_of(cascade_kernel<Fp64Policy, LVL_GEO>, block, smem, &occ[LVL_GEO])) != cudaSuccess ||
      (e = occupancy_of(cascade_kernel<Fp64Policy, LVL_FULL>, block, smem, &occ[LVL_FULL])) != cudaSuccess)
    return e;
  occ[LVL_CLU] = occ[LVL_GEO];
  occ[LVL_CLU_EV] = occ[LVL_FULL];
  *blocks_per_sm = occ[level < 0 ? 0 : (level >= LVL_COUNT ? LVL_COUNT - 1 : level)];
  return cudaSuccess;
}

size_t
record_size64()
{
  return sizeof(P64);
}

size_t
cold_slot_bytes64()
{
  return sizeof(LaneCold<AccF64>);
}

// ---- service kernels

__global__ void
stopping64_kernel(const SpeciesConst * sc, const MatConst * mc, const double * E, long long n,
                  double * out)
{
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n)
    out[i] = material_stop64(*sc, *mc, E[i]);
}

cudaError_t
launch_stopping64(const SpeciesConst * sc, const MatConst * mc, const double * E, long long n,
                  double * out, cudaStream_t st)
{
  const int block = 256;
  const long long grid = (n + block - 1) / block;
  if (grid > 0)
    stopping64_kernel<<<(unsigned int)grid, block, 0, st>>>(sc, mc, E, n, out);
  return cudaGetLastError();
}

__global__ void
scatter64_kernel(const double * eps, const double * b, long long n, double * s2, int potential)
{
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n)
  {
    double ct, st, s;
    int it;
    scatter64(eps[i], b[i], s, ct, st, it, potential);
    s2[i] = s;
  }
}

cudaError_t
launch_scatter64(const double * eps, const double * b, long long n, double * s2, int potential,
                 cudaStream_t st)
{
  const int block = 256;
  const long long grid = (n + block - 1) / block;
  if (grid > 0)
    scatter64_kernel<<<(unsigned int)grid, block, 0, st>>>(eps, b, n, s2, potential);
  return cudaGetLastError();
}

} // namespace mtg

namespace mtg
{

// FP32-path stopping tables: for every (species, material) row, on a grid uniform
// in ln E, the pair S(E) (the FP64 stopping above) and p_max(E), the maximum impact
// parameter of the free flight (trim.C:88-94, the FP64 formula of collide64).
__global__ void
build_stop_tables_kernel(const SpeciesConst * species, const MatConst * mats, const int * row_mat, int n_rows,
                         const int * row_species, float * out, double lnE_min, double dlnE)
{
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (long long)n_rows * STOP_N)
    return;
  const int row = int(i / STOP_N);
  const int j = int(i % STOP_N);
  const double E = exp64(lnE_min + dlnE * double(j));
  const MatConst & mc = mats[row_mat ? row_mat[row] : row];
  const double eeg = sqrt(E * mc.f * mc.epsdg);
  const double pmax = mc.a / (eeg + sqrt(eeg) + 0.125 * pow64(eeg, 0.1));
  out[2 * i] = float(material_stop64(species[row_species[row]], mc, E));
  out[2 * i + 1] = float(pmax);
}

cudaError_t
launch_build_stop_tables(const SpeciesConst * species, const MatConst * mats, const int * row_mat, int n_rows,
                         const int * row_species, float * out, double lnE_min, double dlnE, cudaStream_t st)
{
  const long long n = (long long)n_rows * STOP_N;
  const int block = 256;
  if (n > 0)
    build_stop_tables_kernel<<<(unsigned int)((n + block - 1) / block), block, 0, st>>>(
        species, mats, row_mat, n_rows, row_species, out, lnE_min, dlnE);
  return cudaGetLastError();
}

} // namespace mtg
