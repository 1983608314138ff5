// Launch wrappers shared between the engine translation units and the C ABI.
#pragma once

#include <cuda_runtime.h>

#include "mtg_tables.h"

namespace mtg
{

struct EngineParams;
struct PrimaryTallies;

// FP64 exact path (mtg_engine64.cu)
cudaError_t launch_cascade64(const EngineParams & prm, int grid, int block, size_t smem, cudaStream_t st);
cudaError_t occupancy64(int block, size_t smem, int * blocks_per_sm, int level);
size_t record_size64();
size_t cold_slot_bytes64(); // per-thread shared-memory tally slot
cudaError_t launch_stopping64(const SpeciesConst * sc, const MatConst * mc, const double * E, long long n,
                              double * out, cudaStream_t st);
cudaError_t launch_scatter64(const double * eps, const double * b, long long n, double * s2, int potential,
                             cudaStream_t st);

// FP32 path (mtg_engine32.cu)
constexpr int STOP_N = 2048;      // points per stopping table (uniform in ln E)
constexpr double STOP_EMIN = 1e-2; // eV
struct Fp32Tables
{
  const float * stop;   // STOP_N pairs (S, p_max) per MatConst row (same row index as the MatConst table)
  float lnE_min;        // ln(STOP_EMIN)
  float inv_dlnE;       // 1 / spacing in ln E
  const void * mlp;     // surrogate weights, NULL without the surrogate
  const void * sims32;  // Sim32 per simulation
};
cudaError_t launch_build_stop_tables(const SpeciesConst * species, const MatConst * mats, const int * row_mat,
                                     int n_rows, const int * row_species, float * out, double lnE_min,
                                     double dlnE, cudaStream_t st);
cudaError_t launch_cascade32(const EngineParams & prm, const Fp32Tables & t, int grid, int block, size_t smem,
                             cudaStream_t st, int surrogate);
cudaError_t occupancy32(int block, size_t smem, int * blocks_per_sm, int surrogate, int level);
size_t record_size32();
size_t cold_slot_bytes32();
cudaError_t launch_scatter32(const double * eps, const double * b, long long n, double * s2, int potential,
                             cudaStream_t st);
cudaError_t launch_stopping32(const float * row, float lnE_min, float inv_d, const double * E, long long n,
                              double * out, cudaStream_t st);
// the FP32 Newton solve's first-guess table (built once per process) and its
// upload to the current device, for the engine and for the surrogate's service
const float * newton_guess_table32();
cudaError_t upload_newton_guess32();
cudaError_t upload_newton_guess32_surrogate(const float * table);

// Surrogate (mtg_surrogate.cu)
cudaError_t launch_quadrature(const double * eps, const double * b, long long n, double * s2, double * tau,
                              cudaStream_t st);
cudaError_t launch_surrogate_eval(const void * net, const double * eps, const double * b, long long n, double * s2,
                                  cudaStream_t st);
cudaError_t launch_pack_net(const float * params, void * net, cudaStream_t st);
size_t surrogate_net_bytes();
cudaError_t surrogate_gradients(const float * params_h, const float * x_h, const float * y_h, long long n,
                                float w_tau, float * loss_h, float * grads_h);
cudaError_t surrogate_train(long long n_train, int batch, int epochs, int qat_epochs, float lr,
                            unsigned long long seed, float w_tau, int target, int weighting, float * params_dev,
                            void * net_dev,
                            double * final_loss, double * train_seconds);

// Tally reduction (mtg_reduce.cu)
constexpr int NQ = 15; // reduced quantities per simulation
struct ReduceJob
{
  int sim;
  long long begin, end;
};
size_t voxel_partials_bytes(int nsims);
cudaError_t launch_voxel_sum(const double * vox, const long long * range, int nsims, double * partials, double * out,
                             cudaStream_t st);
cudaError_t launch_reduce(const ReduceJob * jobs, int njobs, const PrimaryTallies & prim, double * partials,
                          const int * job_first, int nsims, double * out, cudaStream_t st);

} // namespace mtg
