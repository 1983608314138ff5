// Arithmetic of the per-primary tally reduction, shared by mtg_collect's kernel
// (mtg_reduce.cu) and the allocation-free variant (mtg_noalloc.cu), so that the two
// give the same bits.
//
// A block of RBLOCK threads sums one stretch of primaries: each thread adds its
// primaries (every RBLOCK-th) in plain FP64 -- a few hundred values, so its error
// stays near 1e-14 of their magnitude -- and the threads' sums are merged with
// Neumaier-compensated FP64 adds in a fixed tree.  Compensating every single add
// made the reduction FP64-issue-bound (GB300 executes FP64 at 1/64 of the FP32
// rate): 2 ms for a stretch of 65,536 primaries on one SM.
#pragma once

namespace mtg
{

constexpr int RBLOCK = 256;
constexpr int NQ_SUM = 15;

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

// The 15 sums of primaries [begin, end) over the block, into out[0..14] (thread 0
// writes): sum and sum of squares of vacancies, collisions, electronic and nuclear
// energy; primaries at rest (states 1..3) and the sums and sums of squares of
// their x, y, z.
__device__ __forceinline__ void
block_sum_primaries(const unsigned long long * vac, const unsigned long long * coll, const double * eel,
                    const double * enuc, const double * fx, const double * fy, const double * fz, const int * fstate,
                    long long begin, long long end, double * out)
{
  double q[NQ_SUM];
#pragma unroll
  for (int k = 0; k < NQ_SUM; ++k)
    q[k] = 0.0;
  for (long long i = begin + threadIdx.x; i < end; i += RBLOCK)
  {
    const double v = double(vac[i]);
    const double c = double(coll[i]);
    const double e = eel[i];
    const double n = enuc[i];
    q[0] += v;
    q[1] += v * v;
    q[2] += c;
    q[3] += c * c;
    q[4] += e;
    q[5] += e * e;
    q[6] += n;
    q[7] += n * n;
    const int st = fstate[i];
    if (st >= 1 && st <= 3)
    {
      const double x = fx[i], y = fy[i], z = fz[i];
      q[8] += 1.0;
      q[9] += x;
      q[10] += x * x;
      q[11] += y;
      q[12] += y * y;
      q[13] += z;
      q[14] += z * z;
    }
  }
  __shared__ Comp red[RBLOCK];
  for (int k = 0; k < NQ_SUM; ++k)
  {
    red[threadIdx.x] = Comp{q[k], 0.0};
    __syncthreads();
    for (int w = RBLOCK / 2; w > 0; w >>= 1)
    {
      if (threadIdx.x < w)
        comp_merge(red[threadIdx.x], red[threadIdx.x + w]);
      __syncthreads();
    }
    if (threadIdx.x == 0)
      out[k] = red[0].s + red[0].c;
    __syncthreads();
  }
}

} // namespace mtg
