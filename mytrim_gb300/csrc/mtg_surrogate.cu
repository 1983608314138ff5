// Learned scattering surrogate: training data, training, packing, evaluation.
//
// * Training data: FP64 Gauss-Mehler (Gauss-Chebyshev) quadrature of the classical
//   scattering integral of the universal (ZBL) potential,
//       theta = pi - 2 beta Int_0^1 du / g(u),   g(u)^2 = 1 - Phi(r0/u) u / (r0 eps) - beta^2 u^2,
//   beta = b / r0, r0 the distance of closest approach (safeguarded Newton to 1e-14),
//   and of Biersack's time integral
//       tau = sqrt(r0^2 - b^2) - r0 Int_0^1 [1/g(u) - 1/sqrt(1 - beta^2 u^2)] du / u^2,
//   both with the weight 1/sqrt(1 - u^2) absorbed: the integrands are evaluated as
//   F(u) = sqrt(1 - u^2) / g(u) at the positive Chebyshev nodes u_j = cos((2j-1) pi / 2N).
//   Samples are log-uniform in eps over [1e-4, 1e4] and area-weighted in b over
//   [0, 12] (b = 12 sqrt(U)), drawn from Philox.  The sin^2(theta/2) target is the
//   quadrature's or, on request, the FP64 magic formula's at the same samples
//   (scatter64: the reference's Newton solve and magic formula, trim.C:180-271).
// * Training: the project's own FP32 kernels -- dense forward, backward (data and
//   weight gradients, deterministic two-stage reduction), MSE loss, Adam -- with the
//   whole step captured in a CUDA graph.  The last epochs are quantisation-aware:
//   the two hidden 64x64 layers see BF16-rounded weights and inputs in the forward
//   pass, as in inference.
// * Inference: mtg_surrogate.cuh.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "mytrim_gpu.h"
#include "mtg_collide64.cuh"
#include "mtg_common.cuh"
#include "mtg_kernels.h"
#include "mtg_scatter32.cuh"
#include "mtg_surrogate.cuh"

namespace mtg
{

constexpr int QN = 256; // Gauss-Chebyshev nodes (QN / 2 evaluations per integral)
__constant__ double c_nodes[QN / 2];

// universal screening function and its derivative (trim.C:196-203)
__host__ __device__ __forceinline__ void
screening(double r, double & phi, double & dphi)
{
  const double e1 = 0.18175 * exp64(-3.1998 * r);
  const double e2 = 0.50986 * exp64(-0.94229 * r);
  const double e3 = 0.28022 * exp64(-0.4029 * r);
  const double e4 = 0.028171 * exp64(-0.20162 * r);
  phi = e1 + e2 + e3 + e4;
  dphi = -(3.1998 * e1 + 0.94229 * e2 + 0.4029 * e3 + 0.20162 * e4);
}

// distance of closest approach: root of f(r) = 1 - Phi(r)/(r eps) - b^2/r^2
__device__ double
closest_approach(double eps, double b)
{
  const double ie = 1.0 / eps;
  double hi = 0.5 * (ie + sqrt(ie * ie + 4.0 * b * b)) * (1.0 + 1e-12) + 1e-300;
  double lo = b > 0.0 ? b : hi * 1e-9;
  double r = 0.5 * (lo + hi);
  for (int it = 0; it < 200; ++it)
  {
    double phi, dphi;
    screening(r, phi, dphi);
    const double f = 1.0 - phi * ie / r - b * b / (r * r);
    if (f > 0.0)
      hi = r;
    else
      lo = r;
    const double fp = -dphi * ie / r + phi * ie / (r * r) + 2.0 * b * b / (r * r * r);
    double rn = r - f / fp;
    if (!(rn > lo && rn < hi))
      rn = 0.5 * (lo + hi);
    if (fabs(rn - r) <= 1e-14 * r)
    {
      r = rn;
      break;
    }
    r = rn;
  }
  return r;
}

// theta and tau by quadrature
__device__ void
scatter_quadrature(double eps, double b, double & s2, double & tau)
{
  const double r0 = closest_approach(eps, b);
  const double beta = b / r0;
  const double ie = 1.0 / (r0 * eps);
  double I = 0.0, J = 0.0;
  for (int j = 0; j < QN / 2; ++j)
  {
    const double u = c_nodes[j];
    double phi, dphi;
    screening(r0 / u, phi, dphi);
    const double omu2 = 1.0 - u * u;
    const double g2 = 1.0 - phi * u * ie - beta * beta * u * u;
    const double ig = sqrt(omu2 / g2); // sqrt(1-u^2)/g
    I += ig;
    J += (ig - sqrt(omu2 / (1.0 - beta * beta * u * u))) / (u * u);
  }
  const double w = 3.14159265358979323846 / QN;
  const double theta = 3.14159265358979323846 - 2.0 * beta * w * I;
  const double sh = sin(0.5 * theta);
  s2 = sh * sh;
  tau = sqrt(fmax(r0 * r0 - b * b, 0.0)) - r0 * w * J;
}

__global__ void
quadrature_kernel(const double * eps, const double * b, long long n, double * s2, double * tau)
{
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n)
    return;
  double s, t;
  scatter_quadrature(eps[i], b[i], s, t);
  s2[i] = s;
  if (tau)
    tau[i] = t;
}

// normalised network inputs / targets for one sample
__host__ __device__ __forceinline__ double
baseline_ln_s2(double eps, double b)
{
  const double w = 2.0 * eps * b;
  return -log(1.0 + w * w * exp(2.0 * double(SG_D4) * b));
}

__global__ void
make_training_data(long long n, uint32_t k0, uint32_t k1, uint32_t offset, int target, float * x, float * y,
                   float * wts)
{
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n)
    return;
  const U4 d = philox(U4{uint32_t(i), uint32_t(i >> 32), offset, 0x5347u}, k0, k1);
  const double le = -4.0 + 8.0 * (u53(d.x, d.y) - 0.5 / 9007199254740992.0);
  const double b = 12.0 * sqrt(u53(d.z, d.w) - 0.5 / 9007199254740992.0);
  const double eps = exp64(le * 2.302585092994046);
  double s2, tau;
  scatter_quadrature(eps, b, s2, tau);
  if (target == MTG_SURROGATE_TARGET_MAGIC)
  {
    double ct, st;
    int niter;
    scatter64(eps, b, s2, ct, st, niter, 0);
  }
  x[2 * i] = float(le * 0.25);
  x[2 * i + 1] = float(b / 6.0 - 1.0);
  y[2 * i] = float((log(fmax(s2, 1e-300)) - baseline_ln_s2(eps, b)) / SG_Y0);
  y[2 * i + 1] = float(tau / SG_Y1);
  // energy-transfer weight of the sample's sin^2(theta/2) error: the energy given to
  // the recoil is proportional to s2, and so is theta^2 at small angles (the angular
  // diffusion); a floor keeps every sample in the fit
  if (wts)
    wts[i] = float(s2 + SG_WEIGHT_FLOOR);
}

__global__ void
scale_weights(float * w, long long n, float f)
{
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n)
    w[i] *= f;
}

// ------------------------------------------------------------------ training
// Parameter vector layout: W1[64][2] b1[64] W2[64][64] b2[64] W3[64][64] b3[64] W4[2][64] b4[2]
struct Offsets
{
  int w1, b1, w2, b2, w3, b3, w4, b4;
};
constexpr Offsets OFF{0, 128, 192, 4288, 4352, 8448, 8512, 8640};
static_assert(OFF.b4 + 2 == SG_NPARAM, "parameter layout");

__device__ __forceinline__ float
bf16_round(float v)
{
  return __bfloat162float(__float2bfloat16_rn(v));
}

__device__ __forceinline__ float
silu_d(float z)
{
  const float s = 1.0f / (1.0f + expf(-z));
  return s * (1.0f + z * (1.0f - s));
}

__device__ __forceinline__ float
silu_acc(float z)
{
  return z / (1.0f + expf(-z));
}

// Z = X W^T + b, H = silu(Z) (act) or Z; X [B][K], W [N][K]; one thread per (sample, output)
__global__ void
dense_fwd(const float * X, int K, const float * W, const float * bias, int N, long long B, float * Z, float * H,
          int act, int quant)
{
  extern __shared__ float sw[]; // W [N][K]
  for (int i = threadIdx.x; i < N * K; i += blockDim.x)
    sw[i] = quant ? bf16_round(W[i]) : W[i];
  __syncthreads();
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= B * N)
    return;
  const long long s = idx / N;
  const int n = int(idx % N);
  float z = bias[n];
  const float * xr = X + s * K;
  for (int k = 0; k < K; ++k)
    z = fmaf(quant ? bf16_round(xr[k]) : xr[k], sw[n * K + k], z);
  Z[idx] = z;
  if (H)
    H[idx] = act ? silu_acc(z) : z;
}

// loss and output gradient: dO = 2 w_c (O - Y) / B; output 0 weighted per sample
// by W (NULL: 1), output 1 by w1
__global__ void
loss_grad(const float * O, const float * Y, const float * W, long long B, float w1, float * dO, float * loss_partial)
{
  __shared__ float red[256];
  float acc = 0.0f;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < B * 2; i += (long long)gridDim.x * blockDim.x)
  {
    const float wc = (i & 1) ? w1 : (W ? W[i >> 1] : 1.0f);
    const float d = O[i] - Y[i];
    dO[i] = 2.0f * wc * d / float(B);
    acc += wc * d * d;
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1)
  {
    if (threadIdx.x < w)
      red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0)
    loss_partial[blockIdx.x] = red[0];
}

// dX[s][k] = sum_n dZ[s][n] W[n][k], then times silu'(Zprev[s][k])
__global__ void
dense_bwd_data(const float * dZ, const float * W, int N, int K, long long B, const float * Zprev, float * dX,
               int quant)
{
  extern __shared__ float sw[];
  for (int i = threadIdx.x; i < N * K; i += blockDim.x)
    sw[i] = quant ? bf16_round(W[i]) : W[i];
  __syncthreads();
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= B * K)
    return;
  const long long s = idx / K;
  const int k = int(idx % K);
  float g = 0.0f;
  const float * dz = dZ + s * N;
  for (int n = 0; n < N; ++n)
    g = fmaf(dz[n], sw[n * K + k], g);
  dX[idx] = g * silu_d(Zprev[idx]);
}

// partial weight gradients over a slice of the batch: P[p][n][k] = sum_s dZ[s][n] X[s][k]
// and P[p][N][n] for the bias; grid (N, parts)
__global__ void
dense_bwd_weight(const float * dZ, const float * X, int N, int K, long long B, int parts, float * P, int quant)
{
  const int n = blockIdx.x;
  const int p = blockIdx.y;
  const long long s0 = B * p / parts, s1 = B * (p + 1) / parts;
  const int k = threadIdx.x; // blockDim.x == 64 >= K
  float acc = 0.0f, accb = 0.0f;
  for (long long s = s0; s < s1; ++s)
  {
    const float d = dZ[s * N + n];
    if (k < K)
      acc = fmaf(d, quant ? bf16_round(X[s * K + k]) : X[s * K + k], acc);
    accb += d;
  }
  const long long base = (long long)p * (N * K + N);
  if (k < K)
    P[base + n * K + k] = acc;
  if (k == 0)
    P[base + N * K + n] = accb;
}

// G[i] = sum_p P[p][i] in order; scatter into the flat gradient vector
__global__ void
reduce_parts(const float * P, int count, int parts, float * gW, float * gb, int N, int K)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count)
    return;
  float a = 0.0f;
  for (int p = 0; p < parts; ++p)
    a += P[(long long)p * count + i];
  if (i < N * K)
    gW[i] = a;
  else
    gb[i - N * K] = a;
}

__global__ void
adam_step(float * w, const float * g, float * m, float * v, int n, const int * step, float lr, float b1, float b2,
          float eps_adam, float lr_final_frac, int total_steps)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n)
    return;
  const int t = *step + 1;
  // cosine decay from lr to lr * lr_final_frac
  const float prog = fminf(1.0f, float(t) / float(total_steps));
  const float lrt = lr * (lr_final_frac + (1.0f - lr_final_frac) * 0.5f * (1.0f + cosf(3.14159265f * prog)));
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.0f - b1) * gi;
  const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  const float mh = mi / (1.0f - powf(b1, float(t)));
  const float vh = vi / (1.0f - powf(b2, float(t)));
  w[i] -= lrt * mh / (sqrtf(vh) + eps_adam);
}

__global__ void
bump_step(int * step)
{
  *step += 1;
}

// gather batch rows by a device-side step counter (epoch-cyclic)
__global__ void
gather_batch(const float * x, const float * y, const float * w, long long n, long long B, const int * step, float * bx,
             float * by, float * bw)
{
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= B)
    return;
  const long long src = ((long long)(*step) * B + i) % n;
  bx[2 * i] = x[2 * src];
  bx[2 * i + 1] = x[2 * src + 1];
  by[2 * i] = y[2 * src];
  by[2 * i + 1] = y[2 * src + 1];
  if (w)
    bw[i] = w[src];
}

// flat parameters -> inference layout
__global__ void
pack_net(const float * w, SurrogateNet * net)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < 128)
    net->w1[i / 2][i % 2] = w[OFF.w1 + i];
  if (i < 64)
  {
    net->b1[i] = w[OFF.b1 + i];
    net->b2[i] = w[OFF.b2 + i];
    net->b3[i] = w[OFF.b3 + i];
    net->w4[0][i] = w[OFF.w4 + i];
    net->w4[1][i] = w[OFF.w4 + 64 + i];
  }
  if (i < 2)
    net->b4[i] = w[OFF.b4 + i];
  if (i < 64 * SG_LD)
  {
    const int r = i / SG_LD, c = i % SG_LD;
    net->w2[r][c] = __float2bfloat16_rn(c < 64 ? w[OFF.w2 + r * 64 + c] : 0.0f);
    net->w3[r][c] = __float2bfloat16_rn(c < 64 ? w[OFF.w3 + r * 64 + c] : 0.0f);
  }
}

// surrogate evaluation for the scatter service (whole warps; tail lanes use dummy input)
__global__ void
surrogate_eval_kernel(const SurrogateNet * gnet, const double * eps, const double * b, long long n, double * s2,
                      int fallback_exact)
{
  __shared__ SurrogateNet net;
  for (int i = threadIdx.x; i < int(sizeof(SurrogateNet) / 4); i += blockDim.x)
    reinterpret_cast<float *>(&net)[i] = reinterpret_cast<const float *>(gnet)[i];
  __syncthreads();
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const float e = i < n ? float(eps[i]) : 1.0f;
  const float bb = i < n ? float(b[i]) : 1.0f;
  const bool in = surrogate_in_domain(e, bb);
  const float o0 = surrogate_eval_warp(&net, in && i < n, surrogate_x1(in ? e : 1.0f), surrogate_x2(in ? bb : 1.0f));
  if (i >= n)
    return;
  float s, c;
  if (in)
    surrogate_s2_from(e, bb, o0, s, c);
  else
  {
    // outside the trained domain the exact FP32 path applies, as in the engine
    int it;
    scatter32(e, bb, s, c, it);
  }
  s2[i] = double(s);
}

} // namespace mtg

// ------------------------------------------------------------------ host side
namespace mtg
{

static void
upload_nodes_once()
{
  static bool done = false;
  if (done)
    return;
  double nodes[QN / 2];
  for (int j = 1; j <= QN / 2; ++j)
    nodes[j - 1] = std::cos((2.0 * j - 1.0) * 3.14159265358979323846 / (2.0 * QN));
  cudaMemcpyToSymbol(c_nodes, nodes, sizeof nodes);
  done = true;
}

cudaError_t
launch_quadrature(const double * eps, const double * b, long long n, double * s2, double * tau, cudaStream_t st)
{
  upload_nodes_once();
  if (n > 0)
    quadrature_kernel<<<(unsigned int)((n + 127) / 128), 128, 0, st>>>(eps, b, n, s2, tau);
  return cudaGetLastError();
}

cudaError_t
launch_surrogate_eval(const void * net, const double * eps, const double * b, long long n, double * s2,
                      cudaStream_t st)
{
  if (n > 0)
    surrogate_eval_kernel<<<(unsigned int)((n + 127) / 128), 128, 0, st>>>(
        reinterpret_cast<const SurrogateNet *>(net), eps, b, n, s2, 0);
  return cudaGetLastError();
}

cudaError_t
launch_pack_net(const float * params, void * net, cudaStream_t st)
{
  pack_net<<<(64 * SG_LD + 127) / 128, 128, 0, st>>>(params, reinterpret_cast<SurrogateNet *>(net));
  return cudaGetLastError();
}

size_t
surrogate_net_bytes()
{
  return sizeof(SurrogateNet);
}

// One forward + backward pass over a batch (device buffers), gradients into g.
struct TrainBuffers
{
  long long B;
  int parts;
  float *bx, *by;                // batch inputs/targets [B][2]
  float * bw;                    // per-sample loss weights of output 0 [B], or NULL
  float *z1, *h1, *z2, *h2, *z3, *h3, *o;
  float *d3, *d2, *d1, *dO;      // gradients of pre-activations
  float * P;                     // partial weight gradients
  float * lossp;                 // loss partials
};

static cudaError_t
fwd_bwd(const float * w, float * g, const TrainBuffers & t, int quant, float w_tau, cudaStream_t st)
{
  const long long B = t.B;
  const int T = 256;
  auto blocks = [&](long long n) { return (unsigned int)((n + T - 1) / T); };
  dense_fwd<<<blocks(B * 64), T, 64 * 2 * 4, st>>>(t.bx, 2, w + OFF.w1, w + OFF.b1, 64, B, t.z1, t.h1, 1, 0);
  dense_fwd<<<blocks(B * 64), T, 64 * 64 * 4, st>>>(t.h1, 64, w + OFF.w2, w + OFF.b2, 64, B, t.z2, t.h2, 1, quant);
  dense_fwd<<<blocks(B * 64), T, 64 * 64 * 4, st>>>(t.h2, 64, w + OFF.w3, w + OFF.b3, 64, B, t.z3, t.h3, 1, quant);
  dense_fwd<<<blocks(B * 2), T, 2 * 64 * 4, st>>>(t.h3, 64, w + OFF.w4, w + OFF.b4, 2, B, t.o, nullptr, 0, 0);
  loss_grad<<<64, 256, 0, st>>>(t.o, t.by, t.bw, B, w_tau, t.dO, t.lossp);
  // output layer
  dense_bwd_weight<<<dim3(2, t.parts), 64, 0, st>>>(t.dO, t.h3, 2, 64, B, t.parts, t.P, 0);
  reduce_parts<<<(2 * 64 + 2 + 127) / 128, 128, 0, st>>>(t.P, 2 * 64 + 2, t.parts, g + OFF.w4, g + OFF.b4, 2, 64);
  dense_bwd_data<<<blocks(B * 64), T, 2 * 64 * 4, st>>>(t.dO, w + OFF.w4, 2, 64, B, t.z3, t.d3, 0);
  // hidden layer 3
  dense_bwd_weight<<<dim3(64, t.parts), 64, 0, st>>>(t.d3, t.h2, 64, 64, B, t.parts, t.P, quant);
  reduce_parts<<<(64 * 64 + 64 + 127) / 128, 128, 0, st>>>(t.P, 64 * 64 + 64, t.parts, g + OFF.w3, g + OFF.b3, 64, 64);
  dense_bwd_data<<<blocks(B * 64), T, 64 * 64 * 4, st>>>(t.d3, w + OFF.w3, 64, 64, B, t.z2, t.d2, quant);
  // hidden layer 2
  dense_bwd_weight<<<dim3(64, t.parts), 64, 0, st>>>(t.d2, t.h1, 64, 64, B, t.parts, t.P, quant);
  reduce_parts<<<(64 * 64 + 64 + 127) / 128, 128, 0, st>>>(t.P, 64 * 64 + 64, t.parts, g + OFF.w2, g + OFF.b2, 64, 64);
  dense_bwd_data<<<blocks(B * 64), T, 64 * 64 * 4, st>>>(t.d2, w + OFF.w2, 64, 64, B, t.z1, t.d1, quant);
  // input layer
  dense_bwd_weight<<<dim3(64, t.parts), 64, 0, st>>>(t.d1, t.bx, 64, 2, B, t.parts, t.P, 0);
  reduce_parts<<<(64 * 2 + 64 + 127) / 128, 128, 0, st>>>(t.P, 64 * 2 + 64, t.parts, g + OFF.w1, g + OFF.b1, 64, 2);
  return cudaGetLastError();
}

// ---- exported to the C ABI layer (mtg_api.cu)

struct SurrogateTrainer
{
  float * w = nullptr; // parameters
  void * net = nullptr;
  bool trained = false;
};

cudaError_t
surrogate_gradients(const float * params_h, const float * x_h, const float * y_h, long long n, float w_tau,
                    float * loss_h, float * grads_h)
{
  TrainBuffers t{};
  t.B = n;
  t.parts = 4;
  std::vector<void *> allocs;
  auto alloc = [&](float *& p, size_t count) {
    cudaError_t e = cudaMalloc(&p, count * sizeof(float));
    allocs.push_back(p);
    return e;
  };
  float *w = nullptr, *g = nullptr;
  cudaError_t e = cudaSuccess;
  const size_t B = size_t(n);
  e = e ? e : alloc(w, SG_NPARAM);
  e = e ? e : alloc(g, SG_NPARAM);
  e = e ? e : alloc(t.bx, 2 * B);
  e = e ? e : alloc(t.by, 2 * B);
  e = e ? e : alloc(t.z1, 64 * B);
  e = e ? e : alloc(t.h1, 64 * B);
  e = e ? e : alloc(t.z2, 64 * B);
  e = e ? e : alloc(t.h2, 64 * B);
  e = e ? e : alloc(t.z3, 64 * B);
  e = e ? e : alloc(t.h3, 64 * B);
  e = e ? e : alloc(t.o, 2 * B);
  e = e ? e : alloc(t.d3, 64 * B);
  e = e ? e : alloc(t.d2, 64 * B);
  e = e ? e : alloc(t.d1, 64 * B);
  e = e ? e : alloc(t.dO, 2 * B);
  e = e ? e : alloc(t.P, size_t(t.parts) * (64 * 64 + 64));
  e = e ? e : alloc(t.lossp, 64);
  if (!e)
    e = cudaMemcpy(w, params_h, SG_NPARAM * 4, cudaMemcpyHostToDevice);
  if (!e)
    e = cudaMemcpy(t.bx, x_h, 2 * B * 4, cudaMemcpyHostToDevice);
  if (!e)
    e = cudaMemcpy(t.by, y_h, 2 * B * 4, cudaMemcpyHostToDevice);
  if (!e)
    e = fwd_bwd(w, g, t, 0, w_tau, nullptr);
  if (!e)
    e = cudaMemcpy(grads_h, g, SG_NPARAM * 4, cudaMemcpyDeviceToHost);
  if (!e)
  {
    float lp[64];
    e = cudaMemcpy(lp, t.lossp, sizeof lp, cudaMemcpyDeviceToHost);
    double s = 0.0;
    for (float v : lp)
      s += v;
    *loss_h = float(s / double(n));
  }
  for (void * p : allocs)
    if (p)
      cudaFree(p);
  return e;
}

// Train from scratch.  params_out: SG_NPARAM floats; net_out: device SurrogateNet.
cudaError_t
surrogate_train(long long n_train, int batch, int epochs, int qat_epochs, float lr, unsigned long long seed,
                float w_tau, int target, int weighting, float * params_dev, void * net_dev, double * final_loss,
                double * train_seconds)
{
  upload_nodes_once();
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0);
  std::vector<void *> allocs;
  auto alloc = [&](void ** p, size_t bytes) {
    cudaError_t e = cudaMalloc(p, bytes);
    allocs.push_back(*p);
    return e;
  };
  cudaError_t e = cudaSuccess;
  float *x = nullptr, *y = nullptr, *wts = nullptr, *g = nullptr, *m = nullptr, *v = nullptr;
  int * step = nullptr;
  TrainBuffers t{};
  t.B = batch;
  t.parts = 32;
  const size_t B = size_t(batch);
  e = e ? e : alloc((void **)&x, 2 * sizeof(float) * n_train);
  e = e ? e : alloc((void **)&y, 2 * sizeof(float) * n_train);
  if (weighting)
  {
    e = e ? e : alloc((void **)&wts, sizeof(float) * n_train);
    e = e ? e : alloc((void **)&t.bw, 4 * B);
  }
  e = e ? e : alloc((void **)&g, 4 * SG_NPARAM);
  e = e ? e : alloc((void **)&m, 4 * SG_NPARAM);
  e = e ? e : alloc((void **)&v, 4 * SG_NPARAM);
  e = e ? e : alloc((void **)&step, 4);
  float ** bufs[] = {&t.bx, &t.by, &t.o, &t.dO};
  for (float ** p : bufs)
    e = e ? e : alloc((void **)p, 2 * 4 * B);
  float ** wide[] = {&t.z1, &t.h1, &t.z2, &t.h2, &t.z3, &t.h3, &t.d3, &t.d2, &t.d1};
  for (float ** p : wide)
    e = e ? e : alloc((void **)p, 64 * 4 * B);
  e = e ? e : alloc((void **)&t.P, 4 * size_t(t.parts) * (64 * 64 + 64));
  e = e ? e : alloc((void **)&t.lossp, 4 * 64);
  if (e)
  {
    for (void * p : allocs)
      if (p)
        cudaFree(p);
    return e;
  }
  uint32_t k0 = uint32_t(seed), k1 = uint32_t(seed >> 32) ^ 0x53474E4Eu;
  make_training_data<<<(unsigned int)((n_train + 127) / 128), 128>>>(n_train, k0, k1, 0u, target, x, y, wts);
  if (wts)
  {
    // normalise the weights to mean 1 over the training set
    std::vector<float> hw(n_train);
    e = cudaMemcpy(hw.data(), wts, sizeof(float) * n_train, cudaMemcpyDeviceToHost);
    double sum = 0.0;
    for (float w : hw)
      sum += double(w);
    if (!e && sum > 0.0)
      scale_weights<<<(unsigned int)((n_train + 255) / 256), 256>>>(wts, n_train, float(double(n_train) / sum));
  }
  // initial weights: uniform(-1/sqrt(fan_in), 1/sqrt(fan_in)) from a host LCG
  std::vector<float> w0(SG_NPARAM, 0.0f);
  uint64_t st = seed * 6364136223846793005ull + 1442695040888963407ull;
  auto uni = [&]() {
    st = st * 6364136223846793005ull + 1442695040888963407ull;
    return float((st >> 11) * (1.0 / 9007199254740992.0)) * 2.0f - 1.0f;
  };
  for (int i = 0; i < 128; ++i)
    w0[OFF.w1 + i] = uni() * 1.2f;
  for (int i = 0; i < 4096; ++i)
    w0[OFF.w2 + i] = uni() * 0.3f;
  for (int i = 0; i < 4096; ++i)
    w0[OFF.w3 + i] = uni() * 0.3f;
  for (int i = 0; i < 128; ++i)
    w0[OFF.w4 + i] = uni() * 0.2f;
  cudaMemcpy(params_dev, w0.data(), 4 * SG_NPARAM, cudaMemcpyHostToDevice);
  cudaMemset(m, 0, 4 * SG_NPARAM);
  cudaMemset(v, 0, 4 * SG_NPARAM);
  cudaMemset(step, 0, 4);
  const long long steps_per_epoch = std::max<long long>(1, n_train / batch);
  const int total = int(steps_per_epoch * epochs);
  cudaStream_t s;
  cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
  cudaGraphExec_t exec[2] = {nullptr, nullptr};
  for (int q = 0; q < 2 && !e; ++q)
  {
    cudaGraph_t graph;
    e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
    if (e)
      break;
    gather_batch<<<(unsigned int)((batch + 255) / 256), 256, 0, s>>>(x, y, wts, n_train, batch, step, t.bx, t.by,
                                                                      t.bw);
    fwd_bwd(params_dev, g, t, q, w_tau, s);
    adam_step<<<(SG_NPARAM + 255) / 256, 256, 0, s>>>(params_dev, g, m, v, SG_NPARAM, step, lr, 0.9f, 0.999f, 1e-8f,
                                                      0.02f, total);
    bump_step<<<1, 1, 0, s>>>(step);
    e = cudaStreamEndCapture(s, &graph);
    if (!e)
      e = cudaGraphInstantiate(&exec[q], graph, 0);
    cudaGraphDestroy(graph);
  }
  for (int it = 0; it < total && !e; ++it)
  {
    const bool quant = it >= int(steps_per_epoch * (epochs - qat_epochs));
    e = cudaGraphLaunch(exec[quant ? 1 : 0], s);
  }
  if (!e)
    e = cudaStreamSynchronize(s);
  if (!e)
  {
    float lp[64];
    cudaMemcpy(lp, t.lossp, sizeof lp, cudaMemcpyDeviceToHost);
    double sum = 0.0;
    for (float val : lp)
      sum += val;
    *final_loss = sum / double(batch);
    e = launch_pack_net(params_dev, net_dev, nullptr);
  }
  if (!e)
    e = cudaDeviceSynchronize();
  cudaEventRecord(e1);
  cudaEventSynchronize(e1);
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, e0, e1);
  *train_seconds = ms / 1e3;
  for (auto & ge : exec)
    if (ge)
      cudaGraphExecDestroy(ge);
  cudaStreamDestroy(s);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  for (void * p : allocs)
    if (p)
      cudaFree(p);
  return e;
}

cudaError_t
upload_newton_guess32_surrogate(const float * table)
{
  return upload_newton_guess32_here(table);
}

} // namespace mtg
