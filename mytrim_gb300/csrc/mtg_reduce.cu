// Deterministic compensated reduction of the per-primary tallies.
//
// The reference sums its tallies in double as the cascades run and joins the
// threads' copies at the end (apps/runmytrim.C:315-323).  Here the per-primary
// arrays are reduced after the cascade kernel in a fixed order -- a block per job
// (a contiguous primary range of one simulation), a fixed thread-to-primary map,
// a fixed tree in shared memory, then the jobs of a simulation in index order --
// with plain FP64 sums per thread and Neumaier-compensated FP64 merges
// (mtg_reduce.cuh), so the totals are reproducible bit for bit run to run.  It
// streams 60 bytes per primary and does about 20 FP64 operations on them.
#include "mtg_engine.cuh"
#include "mtg_kernels.h"
#include "mtg_reduce.cuh"

namespace mtg
{

static_assert(NQ == NQ_SUM, "the reduction sums the NQ quantities of mtg_kernels.h");

__global__ void __launch_bounds__(RBLOCK)
reduce_primaries_kernel(const ReduceJob * jobs, PrimaryTallies prim, double * partials)
{
  const ReduceJob job = jobs[blockIdx.x];
  block_sum_primaries(prim.vac, prim.coll, prim.eel, prim.enuc, prim.fx, prim.fy, prim.fz, prim.fstate, job.begin,
                      job.end, partials + (long long)blockIdx.x * NQ);
}

// one block per simulation, one thread per quantity: the simulation's job sums in
// job order (a thread per simulation walking all quantities took 0.6 ms at 153 jobs)
__global__ void
reduce_finish_kernel(const int * job_first, int nsims, const double * partials, double * out)
{
  const int s = blockIdx.x, k = threadIdx.x;
  if (s >= nsims || k >= NQ)
    return;
  Comp a{0.0, 0.0};
  for (int j = job_first[s]; j < job_first[s + 1]; ++j)
    comp_add(a, partials[(long long)j * NQ + k]);
  out[(long long)s * NQ + k] = a.s + a.c;
}

// Compensated sum of each simulation's voxel grid in two fixed-order stages: block
// b of simulation s sums the cells of its stretch [b n / B, (b+1) n / B) into
// partials[s B + b], then one thread per simulation adds its B partials in order.
// (One block per grid read a 256^3 grid at 4 GB/s on one SM: 34 ms.)
constexpr int VOX_BLOCKS = 256; // blocks per simulation

__global__ void __launch_bounds__(RBLOCK)
voxel_partial_kernel(const double * vox, const long long * range, double * partials)
{
  const int sim = blockIdx.y, b = blockIdx.x;
  const long long base = range[2 * sim], n = range[2 * sim + 1];
  const long long lo = n * b / VOX_BLOCKS, hi = n * (b + 1) / VOX_BLOCKS;
  double a = 0.0; // plain FP64 per thread, compensated merges (mtg_reduce.cuh)
  for (long long i = lo + threadIdx.x; i < hi; i += RBLOCK)
    a += vox[base + i];
  __shared__ Comp red[RBLOCK];
  red[threadIdx.x] = Comp{a, 0.0};
  __syncthreads();
  for (int w = RBLOCK / 2; w > 0; w >>= 1)
  {
    if (threadIdx.x < w)
      comp_merge(red[threadIdx.x], red[threadIdx.x + w]);
    __syncthreads();
  }
  if (threadIdx.x == 0)
    partials[(long long)sim * VOX_BLOCKS + b] = red[0].s + red[0].c;
}

__global__ void
voxel_finish_kernel(const double * partials, int nsims, double * out)
{
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nsims)
    return;
  Comp a{0.0, 0.0};
  for (int b = 0; b < VOX_BLOCKS; ++b)
    comp_add(a, partials[(long long)s * VOX_BLOCKS + b]);
  out[s] = a.s + a.c;
}

size_t
voxel_partials_bytes(int nsims)
{
  return sizeof(double) * size_t(VOX_BLOCKS) * size_t(nsims > 0 ? nsims : 1);
}

cudaError_t
launch_voxel_sum(const double * vox, const long long * range, int nsims, double * partials, double * out,
                 cudaStream_t st)
{
  if (nsims > 0)
  {
    voxel_partial_kernel<<<dim3(VOX_BLOCKS, nsims), RBLOCK, 0, st>>>(vox, range, partials);
    voxel_finish_kernel<<<(nsims + 127) / 128, 128, 0, st>>>(partials, nsims, out);
  }
  return cudaGetLastError();
}

cudaError_t
launch_reduce(const ReduceJob * jobs, int njobs, const PrimaryTallies & prim, double * partials,
              const int * job_first, int nsims, double * out, cudaStream_t st)
{
  if (njobs > 0)
    reduce_primaries_kernel<<<njobs, RBLOCK, 0, st>>>(jobs, prim, partials);
  if (nsims > 0)
    reduce_finish_kernel<<<nsims, 32, 0, st>>>(job_first, nsims, partials, out);
  return cudaGetLastError();
}

} // namespace mtg
