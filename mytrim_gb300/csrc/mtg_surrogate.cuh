// Learned scattering surrogate: an MLP 2 -> 64 -> 64 -> 64 -> 2 (SiLU) that maps
// (log10 reduced energy, reduced impact parameter) to the centre-of-mass
// scattering, trained on FP64 Gauss-Mehler quadrature of the universal-potential
// scattering integral.
//
// Output 0 is a correction to an analytic baseline that carries the dynamic range
// of sin^2(theta/2) (about 36 e-folds over the domain):
//     ln s2 = ln s2_0(eps, b) + Y0 * o0,
//     s2_0 = 1 / (1 + (2 eps b)^2 exp(2 d4 b)),  d4 = 0.20162,
// i.e. the small-angle Coulomb limit times the screening of the potential's slowest
// exponential, so the network only learns an O(1) correction.  Output 1 is the
// reduced time integral tau / Y1 (not used by the transport: tau = 0 in the
// reference, trim.C:303, 310).
//
// Inference in the FP32 engine is warp-collective: the inputs of the lanes whose
// collision lies in the network's domain are compacted into 16-row tiles (one tile
// for up to 16 such lanes, none without); the two 64x64 hidden layers run on the tensor cores
// (mma.sync m16n8k16, BF16 operands, FP32 accumulation) with the accumulator
// fragments of one layer reused in registers as the A fragments of the next; the
// 2x64 input and 64x2 output layers stay in FP32.  Weights are staged in shared
// memory.
#pragma once

#include <cstddef>
#include <stdint.h>
#include <cuda_bf16.h>

namespace mtg
{

constexpr int SG_H = 64;        // hidden width
constexpr int SG_LD = 72;       // padded row length of the BF16 weight tiles (bank-conflict free)
constexpr int SG_NPARAM = 2 * SG_H + SG_H + SG_H * SG_H + SG_H + SG_H * SG_H + SG_H + 2 * SG_H + 2;
constexpr float SG_LOGEPS_MIN = -4.0f, SG_LOGEPS_MAX = 4.0f;
constexpr float SG_B_MAX = 12.0f;
constexpr float SG_D4 = 0.20162f;
constexpr float SG_Y0 = 4.0f;   // output 0 scale (e-folds)
constexpr float SG_Y1 = 10.0f;  // output 1 scale (reduced length)
constexpr float SG_EPS_NET_MAX = 10.0f; // above: the closed-form Rutherford branch (trim.C:172-179)
constexpr double SG_WEIGHT_FLOOR = 1e-6; // floor of the energy-transfer loss weight

// Inference layout of the network (built from the flat FP32 parameter vector).
// 16-byte aligned: the BF16 weight rows (144 bytes apart, from byte offsets 768 and
// 10240) are read with ldmatrix, which wants 16-byte aligned row addresses.
struct alignas(16) SurrogateNet
{
  float w1[SG_H][2];
  float b1[SG_H];
  __nv_bfloat16 w2[SG_H][SG_LD]; // [out][in]
  float b2[SG_H];
  __nv_bfloat16 w3[SG_H][SG_LD];
  float b3[SG_H];
  float w4[2][SG_H];
  float b4[2];
  float pad[2];
};
static_assert(sizeof(SurrogateNet) % 16 == 0 && offsetof(SurrogateNet, w2) % 16 == 0 &&
                  offsetof(SurrogateNet, w3) % 16 == 0 && (SG_LD * 2) % 16 == 0,
              "ldmatrix alignment of the weight rows");

// Where the network replaces the exact scattering: the trained domain (log10 eps in
// [-4, 4], b in [0, 12]) cut at eps = 10, above which the exact path is the reference's
// closed-form Rutherford branch (trim.C:172-179) -- cheaper than the network, and
// exact.  The network stands in for the Newton solve and magic formula only.
__host__ __device__ __forceinline__ bool
surrogate_in_domain(float eps, float b)
{
  return eps >= 1e-4f && eps <= SG_EPS_NET_MAX && b <= SG_B_MAX;
}

// Weight reads from shared memory that the compiler may not hoist out of the
// persistent cascade loop (hoisting them would need hundreds of registers).
__device__ __forceinline__ uint32_t
lds_u32(const void * p)
{
  uint32_t v;
  asm volatile("ld.shared.b32 %0, [%1];" : "=r"(v) : "r"((uint32_t)__cvta_generic_to_shared(p)));
  return v;
}

__device__ __forceinline__ float
lds_f32(const void * p)
{
  return __uint_as_float(lds_u32(p));
}

// SiLU for inference: x sigmoid(x) = x (1 + tanh(x/2)) / 2 with the hardware tanh
// (one special-function operation instead of an exponential and a reciprocal)
__device__ __forceinline__ float
silu(float x)
{
  const float h = 0.5f * x;
  float t;
  asm("tanh.approx.f32 %0, %1;" : "=f"(t) : "f"(h));
  return fmaf(h, t, h);
}

__device__ __forceinline__ uint32_t
pack_bf16(float lo, float hi)
{
  __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<uint32_t *>(&v);
}

__device__ __forceinline__ void
mma_bf16(float (&c)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1)
{
  asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
               "{%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, {%0, %1, %2, %3};\n"
               : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
               : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// Four 8x8 BF16 tiles of shared memory into the B fragments of two m16n8k16
// products: lanes 8i..8i+7 give the row addresses of tile i (16-byte aligned rows).
__device__ __forceinline__ void
ldsm_x4(uint32_t (&r)[4], const void * p)
{
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0, %1, %2, %3}, [%4];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"((uint32_t)__cvta_generic_to_shared(p)));
}

// One 64x64 hidden layer for one 16-row tile: A fragments in, accumulator
// fragments of the 8 column tiles out (bias added).  The weights w[out][in] are the
// B operand in column-major form; each ldmatrix.x4 brings the B fragments of two
// consecutive 16-wide k chunks of one 8-wide column tile (tile i of the four:
// k chunk 2 kp + i / 2, its lower or upper 8 columns by i % 2).
__device__ __forceinline__ void
hidden_layer(const __nv_bfloat16 (*w)[SG_LD], const float * bias, const uint32_t (&a)[4][4], float (&c)[8][4],
             int g, int t)
{
  const int lane = threadIdx.x & 31;
  const int mrow = lane & 7, msel = lane >> 3;
#pragma unroll
  for (int nt = 0; nt < 8; ++nt)
  {
    const float b0 = lds_f32(bias + nt * 8 + 2 * t), b1v = lds_f32(bias + nt * 8 + 2 * t + 1);
    c[nt][0] = b0;
    c[nt][1] = b1v;
    c[nt][2] = b0;
    c[nt][3] = b1v;
#pragma unroll
    for (int kp = 0; kp < 2; ++kp)
    {
      uint32_t r[4];
      ldsm_x4(r, &w[nt * 8 + mrow][(2 * kp + (msel >> 1)) * 16 + (msel & 1) * 8]);
      mma_bf16(c[nt], a[2 * kp], r[0], r[1]);
      mma_bf16(c[nt], a[2 * kp + 1], r[2], r[3]);
    }
  }
}

// accumulator fragments -> SiLU -> A fragments of the next layer
__device__ __forceinline__ void
to_a_fragments(const float (&c)[8][4], uint32_t (&a)[4][4])
{
#pragma unroll
  for (int kc = 0; kc < 4; ++kc)
  {
    a[kc][0] = pack_bf16(silu(c[2 * kc][0]), silu(c[2 * kc][1]));
    a[kc][1] = pack_bf16(silu(c[2 * kc][2]), silu(c[2 * kc][3]));
    a[kc][2] = pack_bf16(silu(c[2 * kc + 1][0]), silu(c[2 * kc + 1][1]));
    a[kc][3] = pack_bf16(silu(c[2 * kc + 1][2]), silu(c[2 * kc + 1][3]));
  }
}

// Lane of the (n+1)-th set bit of m (n < popc(m)): binary search on popcounts.
__device__ __forceinline__ int
nth_set_lane(unsigned m, int n)
{
  int pos = 0;
#pragma unroll
  for (int w = 16; w > 0; w >>= 1)
  {
    const int c = __popc(m & ((1u << w) - 1u));
    const bool up = n >= c;
    n -= up ? c : 0;
    pos += up ? w : 0;
    m = up ? (m >> w) : m;
  }
  return pos;
}

// Warp-collective evaluation: every lane of the warp calls it (converged) with its
// own inputs; lanes with `active` set get output 0 (the correction) for their
// sample, the others 0.  The active lanes' samples are compacted into the first rows
// of the 16-row tiles (row r holds the active lane of rank r), so a warp evaluates
// ceil(active / 16) tiles: none when no lane is active, one for up to 16.  `net`
// must point to shared memory.
__device__ __forceinline__ float
surrogate_eval_warp(const SurrogateNet * net, bool active, float x1, float x2)
{
  const unsigned m = __ballot_sync(0xffffffffu, active);
  const int count = __popc(m);
  const int lane = threadIdx.x & 31;
  const int g = lane >> 2, t = lane & 3;
  const int rank = __popc(m & ((1u << lane) - 1u));
  const int tiles = (count + 15) >> 4;
  float out0 = 0.0f;
#pragma unroll 1
  for (int mt = 0; mt < tiles; ++mt)
  {
    // rows of this tile owned by the thread: mt*16 + g and mt*16 + g + 8; a row past
    // the last active sample reads any lane's input and its result is not used
    const int s0 = mt * 16 + g, s1 = s0 + 8;
    const int l0 = s0 < count ? nth_set_lane(m, s0) : lane;
    const int l1 = s1 < count ? nth_set_lane(m, s1) : lane;
    const float ax1 = __shfl_sync(0xffffffffu, x1, l0), ax2 = __shfl_sync(0xffffffffu, x2, l0);
    const float bx1 = __shfl_sync(0xffffffffu, x1, l1), bx2 = __shfl_sync(0xffffffffu, x2, l1);
    // input layer (FP32) directly in A-fragment layout
    uint32_t a[4][4];
#pragma unroll
    for (int kc = 0; kc < 4; ++kc)
    {
      const int c0 = kc * 16 + 2 * t, c1 = c0 + 8;
      float h[8];
      const int cols[4] = {c0, c0 + 1, c1, c1 + 1};
#pragma unroll
      for (int q = 0; q < 4; ++q)
      {
        const int j = cols[q];
        const float w0 = lds_f32(&net->w1[j][0]), w1v = lds_f32(&net->w1[j][1]), bj = lds_f32(&net->b1[j]);
        h[2 * q] = silu(fmaf(w0, ax1, fmaf(w1v, ax2, bj)));
        h[2 * q + 1] = silu(fmaf(w0, bx1, fmaf(w1v, bx2, bj)));
      }
      a[kc][0] = pack_bf16(h[0], h[2]); // row s0, cols c0, c0+1
      a[kc][1] = pack_bf16(h[1], h[3]); // row s1, cols c0, c0+1
      a[kc][2] = pack_bf16(h[4], h[6]); // row s0, cols c1, c1+1
      a[kc][3] = pack_bf16(h[5], h[7]); // row s1, cols c1, c1+1
    }
    float c[8][4];
    hidden_layer(net->w2, net->b2, a, c, g, t);
    to_a_fragments(c, a);
    hidden_layer(net->w3, net->b3, a, c, g, t);
    // output layer (FP32): partial dot products over the thread's 16 columns,
    // reduced over the 4 threads of the group
    float p0 = 0.0f, p1 = 0.0f; // rows s0 and s1, output 0
#pragma unroll
    for (int nt = 0; nt < 8; ++nt)
    {
      const int j = nt * 8 + 2 * t;
      const float wa = lds_f32(&net->w4[0][j]), wb = lds_f32(&net->w4[0][j + 1]);
      p0 = fmaf(silu(c[nt][0]), wa, fmaf(silu(c[nt][1]), wb, p0));
      p1 = fmaf(silu(c[nt][2]), wa, fmaf(silu(c[nt][3]), wb, p1));
    }
    p0 += __shfl_xor_sync(0xffffffffu, p0, 1);
    p0 += __shfl_xor_sync(0xffffffffu, p0, 2);
    p1 += __shfl_xor_sync(0xffffffffu, p1, 1);
    p1 += __shfl_xor_sync(0xffffffffu, p1, 2);
    // the active lane of rank r gets row r's value from the group owning that row
    const int r = rank - mt * 16;
    const int src = ((r & 7) << 2);
    const float v0 = __shfl_sync(0xffffffffu, p0, src);
    const float v1 = __shfl_sync(0xffffffffu, p1, src);
    if (active && r >= 0 && r < 16)
      out0 = (r < 8 ? v0 : v1) + lds_f32(&net->b4[0]);
  }
  return out0;
}

// s2 and c2 from the network output and the analytic baseline
__device__ __forceinline__ void
surrogate_s2_from(float eps, float b, float o0, float & s2, float & c2)
{
  const float w = 2.0f * eps * b;
  const float ln_s20 = -__logf(1.0f + w * w * __expf(2.0f * SG_D4 * b));
  s2 = __expf(ln_s20 + SG_Y0 * o0);
  s2 = fminf(s2, 1.0f);
  c2 = 1.0f - s2;
}

__device__ __forceinline__ float
surrogate_x1(float eps)
{
  return __log10f(eps) * 0.25f;
}

__device__ __forceinline__ float
surrogate_x2(float b)
{
  return b * (1.0f / 6.0f) - 1.0f;
}

} // namespace mtg
