// Deterministic compensated reduction of the per-primary tallies.
//
// The reference sums its tallies in double as the cascades run and joins the
// threads' copies at the end (apps/runmytrim.C:315-323).  Here the per-primary
// arrays are reduced after the cascade kernel in a fixed order -- a block per job
// (a contiguous primary range of one simulation), a fixed thread-to-primary map,
// a fixed tree in shared memory, then the jobs of a simulation in index order --
// with Neumaier-compensated FP64 sums, so the totals are reproducible bit for bit
// run to run.  This kernel is HBM-bound: it streams 60 bytes per primary.
#include "mtg_engine.cuh"
#include "mtg_kernels.h"

namespace mtg
{

struct Comp
{
  double s, c;
};

__device__ __forceinline__ void
comp_add(Comp & a, double x)
{
  const double t = a.s + x;
  if (fabs(a.s) >= fabs(x))
    a.c += (a.s - t) + x;
  else
    a.c += (x - t) + a.s;
  a.s = t;
}

__device__ __forceinline__ void
comp_merge(Comp & a, const Comp & b)
{
  comp_add(a, b.s);
  a.c += b.c;
}

constexpr int RBLOCK = 256;

__global__ void __launch_bounds__(RBLOCK)
reduce_primaries_kernel(const ReduceJob * jobs, PrimaryTallies prim, double * partials)
{
  const ReduceJob job = jobs[blockIdx.x];
  Comp q[NQ];
#pragma unroll
  for (int k = 0; k < NQ; ++k)
    q[k] = Comp{0.0, 0.0};
  for (long long i = job.begin + threadIdx.x; i < job.end; i += RBLOCK)
  {
    const double v = double(prim.vac[i]);
    const double c = double(prim.coll[i]);
    const double e = prim.eel[i];
    const double n = prim.enuc[i];
    comp_add(q[0], v);
    comp_add(q[1], v * v);
    comp_add(q[2], c);
    comp_add(q[3], c * c);
    comp_add(q[4], e);
    comp_add(q[5], e * e);
    comp_add(q[6], n);
    comp_add(q[7], n * n);
    const int st = prim.fstate[i];
    if (st >= 1 && st <= 3)
    {
      const double x = prim.fx[i], y = prim.fy[i], z = prim.fz[i];
      comp_add(q[8], 1.0);
      comp_add(q[9], x);
      comp_add(q[10], x * x);
      comp_add(q[11], y);
      comp_add(q[12], y * y);
      comp_add(q[13], z);
      comp_add(q[14], z * z);
    }
  }
  __shared__ Comp red[RBLOCK];
  for (int k = 0; k < NQ; ++k)
  {
    red[threadIdx.x] = q[k];
    __syncthreads();
    for (int w = RBLOCK / 2; w > 0; w >>= 1)
    {
      if (threadIdx.x < w)
        comp_merge(red[threadIdx.x], red[threadIdx.x + w]);
      __syncthreads();
    }
    if (threadIdx.x == 0)
      partials[(long long)blockIdx.x * NQ + k] = red[0].s + red[0].c;
    __syncthreads();
  }
}

__global__ void
reduce_finish_kernel(const int * job_first, int nsims, const double * partials, double * out)
{
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nsims)
    return;
  for (int k = 0; k < NQ; ++k)
  {
    Comp a{0.0, 0.0};
    for (int j = job_first[s]; j < job_first[s + 1]; ++j)
      comp_add(a, partials[(long long)j * NQ + k]);
    out[(long long)s * NQ + k] = a.s + a.c;
  }
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
  Comp a{0.0, 0.0};
  for (long long i = lo + threadIdx.x; i < hi; i += RBLOCK)
    comp_add(a, vox[base + i]);
  __shared__ Comp red[RBLOCK];
  red[threadIdx.x] = a;
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
  reduce_finish_kernel<<<(nsims + 127) / 128, 128, 0, st>>>(job_first, nsims, partials, out);
  return cudaGetLastError();
}

} // namespace mtg
