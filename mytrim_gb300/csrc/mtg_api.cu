// C ABI of the cascade engine (include/mytrim_gpu.h): context, table upload,
// launch sequence (cascade pass, overflow drains, tally reduction) and result
// collection.  No CPU fallback exists: without a CUDA device every call that
// needs one fails with MTG_ERR_NO_DEVICE.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "mytrim_gpu.h"
#include "mtg_engine.cuh"
#include "mtg_kernels.h"
#include "mtg_setup.h"

using namespace mtg;

namespace
{

struct DevBuf
{
  void * p = nullptr;
  size_t bytes = 0;
};

cudaError_t
ensure(DevBuf & b, size_t bytes)
{
  if (b.bytes >= bytes && b.p)
    return cudaSuccess;
  if (b.p)
    cudaFree(b.p);
  b.p = nullptr;
  b.bytes = 0;
  if (bytes == 0)
    return cudaSuccess;
  cudaError_t e = cudaMalloc(&b.p, bytes);
  if (e == cudaSuccess)
    b.bytes = bytes;
  return e;
}

template <class T>
T *
ptr(DevBuf & b)
{
  return reinterpret_cast<T *>(b.p);
}

// counters block layout (unsigned long long)
enum Counter
{
  C_NEXT0 = 0, // work counters of up to MAX_PASSES passes
  C_OVF0 = 64, // overflow counts of the two ping-pong lists
  C_OVF1 = 65,
  C_NREC = 66,
  C_NEV = 67,   // event-log slots reserved
  C_STEPS = 68,
  C_NEV_UNUSED = 69, // reserved event-log slots that no event filled
  C_COUNT = 72
};
constexpr int MAX_PASSES = 64;
constexpr int MAX_OVF_RETRIES = 3; // runs redone with a larger overflow list

} // namespace

struct mtg_ctx
{
  int device = 0;
  int n_sm = 0;
  cudaStream_t stream = nullptr; // stream of the current launch
  std::string err;
  mtg_scoef_row rows[MTG_SCOEF_ROWS];
  bool have_tables = false;
  mtg_config cfg;
  HostTables tables;
  std::vector<Species32> sp32; // single-precision copies (FP32 engine), storage kept across batches
  std::vector<Mat32> mc32;
  std::vector<Sim32> sm32;
  bool prepared = false;
  bool launched = false;
  // device buffers
  DevBuf d_sims, d_prim_end, d_species, d_mats, d_row_species, d_stop;
  DevBuf d_species32, d_mats32, d_sims32;
  DevBuf d_sg_params, d_sg_net; // surrogate network
  DevBuf d_vox, d_vox_range, d_vox_sum, d_vox_part; // energy-deposition voxels
  DevBuf d_cl, d_cl32, d_cl_next, d_cl_head, d_cl_mask; // sampleClusters geometry
  std::vector<SimDesc> sims_dev;             // SimDesc copies with device cluster pointers
  bool sg_ready = false;
  DevBuf p_vac, p_coll, p_eel, p_enuc, p_fx, p_fy, p_fz, p_state;
  DevBuf d_totals, d_hist, d_err, d_counters, d_stacks, d_ovf0, d_ovf1, d_records, d_events;
  DevBuf d_jobs, d_job_first, d_partials, d_out;
  DevBuf d_tmp0, d_tmp1, d_tmp2, d_tmp3;
  std::vector<ReduceJob> jobs;
  std::vector<int> job_first;
  int block = 128, grid = 0;
  size_t smem = 0;
  int cold_offset = 0;
  int hist_smem_bins = 0, hist_smem_offset = 0;
  int stage = 0;
  int stack_cap = 0;
  long long ovf_cap = 0;
  long long ovf_floor = 0; // smallest overflow list of later runs, raised when a run exhausted one
  long long record_cap = 0;
  long long event_cap = 0;
  unsigned int event_mask = 0;
  int passes = 0; // cascade passes launched for the current run
  int ovf_last = 0;
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  mtg_stats stats;
};

namespace
{

mtg_status
fail(mtg_ctx * ctx, mtg_status st, const std::string & msg)
{
  if (ctx)
    ctx->err = msg;
  return st;
}

#define CK(call)                                                                                   \
  do                                                                                               \
  {                                                                                                \
    cudaError_t e_ = (call);                                                                       \
    if (e_ != cudaSuccess)                                                                         \
      return fail(ctx, e_ == cudaErrorMemoryAllocation ? MTG_ERR_OOM : MTG_ERR_CUDA,             \
                  std::string(#call) + ": " + cudaGetErrorString(e_));                           \
  } while (0)

mtg_config
default_config()
{
  mtg_config c;
  std::memset(&c, 0, sizeof c);
  c.tmin = 0.2;
  c.tau = 0.0;
  c.cw = 0.001;
  c.length_scale = 1.0;
  c.precision = MTG_PREC_FP64;
  c.seed = 1;
  c.max_collisions_per_member = 1 << 24;
  c.stack_capacity = 0;
  c.block_threads = 0;
  c.max_primaries_per_refill = 0;
  return c;
}

size_t
record_size(int precision)
{
  return precision == MTG_PREC_FP64 ? record_size64() : record_size32();
}

// the smallest cascade-kernel variant (KernelLevel) with every feature the run uses
int
kernel_level(const mtg_ctx * ctx)
{
  const HostTables & t = ctx->tables;
  // cluster geometry with the universal potential only: the plain FP32 engine has
  // variants without the other potentials' code
  const bool clu_only = t.any_clusters && !t.any_potential && ctx->cfg.precision == MTG_PREC_FP32;
  if (ctx->event_cap > 0 && ctx->event_mask)
    return clu_only ? LVL_CLU_EV : (t.any_extended ? LVL_FULL : LVL_EVENTS);
  if (t.any_extended)
    return clu_only ? LVL_CLU : LVL_GEO;
  if (ctx->record_cap > 0 || t.voxel_total > 0 || t.any_evac || t.any_mode)
    return LVL_MID;
  return LVL_LEAN;
}

mtg_status
setup_launch_shape(mtg_ctx * ctx)
{
  const int prec = ctx->cfg.precision;
  const HostTables & t = ctx->tables;
  // stage species and material tables in shared memory for single-simulation runs
  size_t tab = 0;
  ctx->stage = 0;
  if (t.sims.size() == 1)
  {
    if (prec == MTG_PREC_FP64)
      tab = sizeof(SpeciesConst) * t.species.size() + sizeof(MatConst) * t.mats.size();
    else if (prec == MTG_PREC_FP32_SURROGATE)
      tab = stage_net_offset(int(t.species.size()), int(t.mats.size())) + surrogate_net_bytes();
    else
      tab = sizeof(Species32) * t.species.size() + sizeof(Mat32) * t.mats.size();
    if (tab <= 160 * 1024)
      ctx->stage = 1;
    else
      tab = 0;
  }
  ctx->block = ctx->cfg.block_threads > 0 ? ctx->cfg.block_threads : 128;
  size_t tables = ctx->stage ? tab : 0;
  if (!ctx->stage && prec == MTG_PREC_FP32_SURROGATE)
    tables = surrogate_net_bytes();
  // per-thread tally slots follow the tables, 16-byte aligned, then the shared
  // vacancy / replacement histogram of a single-simulation run with few bins
  ctx->cold_offset = int((tables + 15) / 16 * 16);
  const size_t slot = prec == MTG_PREC_FP64 ? cold_slot_bytes64() : cold_slot_bytes32();
  ctx->smem = size_t(ctx->cold_offset) + slot * size_t(ctx->block);
  ctx->hist_smem_bins = 0;
  int bps = 0;
  const int level = kernel_level(ctx);
  auto occupancy = [&](size_t smem, int * b) {
    return prec == MTG_PREC_FP64 ? occupancy64(ctx->block, smem, b, level)
                                 : occupancy32(ctx->block, smem, b, prec == MTG_PREC_FP32_SURROGATE, level);
  };
  cudaError_t e = occupancy(ctx->smem, &bps);
  if (e != cudaSuccess)
    return fail(ctx, MTG_ERR_CUDA, std::string("occupancy query: ") + cudaGetErrorString(e));
  if (t.sims.size() == 1 && t.sims[0].hist_vac_n > 0 && 2 * t.sims[0].hist_vac_n <= HIST_SMEM_MAX)
  {
    // only where it leaves the resident blocks per SM unchanged
    const int off = int((ctx->smem + 15) / 16 * 16);
    const size_t smem2 = size_t(off) + sizeof(unsigned int) * 2 * size_t(t.sims[0].hist_vac_n);
    int bps2 = 0;
    if (occupancy(smem2, &bps2) == cudaSuccess && bps2 >= bps)
    {
      ctx->hist_smem_offset = off;
      ctx->hist_smem_bins = 2 * t.sims[0].hist_vac_n;
      ctx->smem = smem2;
      bps = bps2;
    }
  }
  if (bps < 1)
    return fail(ctx, MTG_ERR_CUDA, "cascade kernel cannot be resident with this launch shape");
  ctx->grid = ctx->n_sm * bps;
  const long long warps = (long long)ctx->grid * (ctx->block / 32);
  const size_t rec = record_size(prec);
  int cap = ctx->cfg.stack_capacity;
  if (cap <= 0)
    cap = prec == MTG_PREC_FP64 ? 4096 : 8192;
  ctx->stack_cap = cap;
  ctx->ovf_cap = std::max<long long>({1LL << 20, warps * 64, ctx->ovf_floor});
  mtg_status st = MTG_OK;
  auto chk = [&](cudaError_t ce, const char * what) {
    if (ce != cudaSuccess && st == MTG_OK)
      st = fail(ctx, ce == cudaErrorMemoryAllocation ? MTG_ERR_OOM : MTG_ERR_CUDA,
                std::string(what) + ": " + cudaGetErrorString(ce));
  };
  chk(ensure(ctx->d_stacks, size_t(warps) * cap * rec), "stack allocation");
  chk(ensure(ctx->d_ovf0, size_t(ctx->ovf_cap) * rec), "overflow allocation");
  chk(ensure(ctx->d_ovf1, size_t(ctx->ovf_cap) * rec), "overflow allocation");
  return st;
}

void
fill_params(mtg_ctx * ctx, EngineParams & prm)
{
  const HostTables & t = ctx->tables;
  std::memset(&prm, 0, sizeof prm);
  prm.sims = ptr<SimDesc>(ctx->d_sims);
  prm.n_sims = int(t.sims.size());
  prm.sim_prim_end = ptr<long long>(ctx->d_prim_end);
  if (ctx->cfg.precision == MTG_PREC_FP64)
  {
    prm.species = ptr<SpeciesConst>(ctx->d_species);
    prm.mats = ptr<MatConst>(ctx->d_mats);
  }
  else
  {
    // the FP32 engine reads the single-precision copies through the same pointers
    prm.species = reinterpret_cast<const SpeciesConst *>(ctx->d_species32.p);
    prm.mats = reinterpret_cast<const MatConst *>(ctx->d_mats32.p);
  }
  prm.stage_tables = ctx->stage;
  prm.cold_offset = ctx->cold_offset;
  prm.hist_smem_bins = ctx->hist_smem_bins;
  prm.hist_smem_offset = ctx->hist_smem_offset;
  prm.hist_smem_base = ctx->hist_smem_bins ? t.sims[0].hist_vac_base : 0;
  prm.n_stage_species = int(t.species.size());
  prm.n_stage_mats = int(t.mats.size());
  prm.total_primaries = t.total_primaries;
  prm.stacks = ctx->d_stacks.p;
  prm.stack_cap = ctx->stack_cap;
  prm.overflow_cap = ctx->ovf_cap;
  prm.prim.vac = ptr<unsigned long long>(ctx->p_vac);
  prm.prim.coll = ptr<unsigned long long>(ctx->p_coll);
  prm.prim.eel = ptr<double>(ctx->p_eel);
  prm.prim.enuc = ptr<double>(ctx->p_enuc);
  prm.prim.fx = ptr<double>(ctx->p_fx);
  prm.prim.fy = ptr<double>(ctx->p_fy);
  prm.prim.fz = ptr<double>(ctx->p_fz);
  prm.prim.fstate = ptr<int>(ctx->p_state);
  prm.totals = ptr<SimTotals>(ctx->d_totals);
  prm.hist = ptr<unsigned long long>(ctx->d_hist);
  prm.voxels = t.voxel_total > 0 ? ptr<double>(ctx->d_vox) : nullptr;
  prm.error_flags = ptr<unsigned int>(ctx->d_err);
  prm.k0 = t.k0;
  prm.k1 = t.k1;
  long long mc = ctx->cfg.max_collisions_per_member;
  prm.max_collisions = (unsigned int)(mc <= 0 ? (1 << 24) : std::min<long long>(mc, 0xffffffffLL));
  // fresh primaries per warp refill.  A warp that follows few cascades at a time
  // switches primary (and flushes the per-primary tallies) rarely, so large cascades
  // want one primary per refill, while small ones need several to keep 32 lanes
  // busy: about 64 expected members per refill.  At most a quarter of a warp's fair
  // share of the batch, so that every warp refills several times (load balance).
  int take = ctx->cfg.max_primaries_per_refill;
  if (take <= 0)
  {
    const long long warps = std::max<long long>(1, (long long)ctx->grid * (ctx->block / 32));
    const long long balance = std::max<long long>(1, t.total_primaries / (warps * 4));
    const long long fill = std::max<long long>(1, llround(64.0 / std::max(t.members_est, 1.0)));
    take = int(std::min<long long>(32, std::min(balance, fill)));
  }
  prm.max_take = take;
  ctx->stats.max_take = take;
  // waiting for idle lanes pays where lanes are cheap (FP32: +3 %); the FP64 kernel is
  // bound by its FP64 pipe, where an idle lane is lost throughput (-8 % at 8)
  prm.refill_min = ctx->cfg.refill_min_idle > 0 ? ctx->cfg.refill_min_idle
                                                : (ctx->cfg.precision == MTG_PREC_FP64 ? 1 : 8);
  if (ctx->record_cap > 0)
  {
    prm.records = ptr<MemberRecord>(ctx->d_records);
    prm.n_records = ptr<unsigned long long>(ctx->d_counters) + C_NREC;
    prm.records_cap = ctx->record_cap;
  }
  if (ctx->event_cap > 0 && ctx->event_mask)
  {
    prm.events = ptr<EventRec>(ctx->d_events);
    prm.n_events = ptr<unsigned long long>(ctx->d_counters) + C_NEV;
    prm.n_event_unused = ptr<unsigned long long>(ctx->d_counters) + C_NEV_UNUSED;
    prm.events_cap = ctx->event_cap;
    prm.event_mask = ctx->event_mask;
    // slots 16 or 8 at a time per lane where the log holds at least 16 such chunks per
    // resident lane (the slots left unused, fewer than a chunk per lane and pass, then
    // take at most 1/16 of it); one at a time in smaller logs, which fill exactly
    const long long lanes = (long long)ctx->grid * ctx->block;
    prm.event_chunk = 1;
    for (int c : {16, 8})
      if (ctx->event_cap >= 16LL * c * lanes)
      {
        prm.event_chunk = c;
        break;
      }
  }
  prm.any_evac = t.any_evac;
  prm.level = kernel_level(ctx);
  ctx->stats.kernel_level = prm.level;
  prm.warp_steps = ptr<unsigned long long>(ctx->d_counters) + C_STEPS;
}

// Launch cascade pass `pass` (0 = fresh primaries, >0 = drain of the previous
// pass's overflow list).
mtg_status
launch_pass(mtg_ctx * ctx, int pass)
{
  EngineParams prm;
  fill_params(ctx, prm);
  unsigned long long * cnt = ptr<unsigned long long>(ctx->d_counters);
  prm.next_primary = cnt + C_NEXT0 + (pass % MAX_PASSES);
  CK(cudaMemsetAsync(prm.next_primary, 0, sizeof(unsigned long long), ctx->stream));
  const int out_list = pass & 1;
  prm.overflow = out_list ? ctx->d_ovf1.p : ctx->d_ovf0.p;
  prm.overflow_count = cnt + (out_list ? C_OVF1 : C_OVF0);
  CK(cudaMemsetAsync(prm.overflow_count, 0, sizeof(unsigned long long), ctx->stream));
  if (pass > 0)
  {
    prm.in_records = out_list ? ctx->d_ovf0.p : ctx->d_ovf1.p;
    prm.in_count = cnt + (out_list ? C_OVF0 : C_OVF1);
    prm.in_cap = ctx->ovf_cap;
  }

  cudaError_t e;
  const int prec = ctx->cfg.precision;
  if (prec == MTG_PREC_FP64)
    e = launch_cascade64(prm, ctx->grid, ctx->block, ctx->smem, ctx->stream);
  else
  {
    Fp32Tables ft;
    ft.stop = ptr<float>(ctx->d_stop);
    ft.lnE_min = float(std::log(STOP_EMIN));
    ft.inv_dlnE = float(1.0 / ((std::log(ctx->tables.emax * 1.05) - std::log(STOP_EMIN)) / (STOP_N - 1)));
    ft.mlp = ctx->sg_ready ? ctx->d_sg_net.p : nullptr;
    ft.sims32 = ctx->d_sims32.p;
    e = launch_cascade32(prm, ft, ctx->grid, ctx->block, ctx->smem, ctx->stream,
                         prec == MTG_PREC_FP32_SURROGATE);
  }
  if (e != cudaSuccess)
    return fail(ctx, MTG_ERR_CUDA, std::string("cascade launch: ") + cudaGetErrorString(e));
  ctx->passes = pass + 1;
  ctx->ovf_last = out_list;
  ctx->stats.launches += 1;
  return MTG_OK;
}

mtg_status
launch_reduction(mtg_ctx * ctx)
{
  PrimaryTallies pt;
  pt.vac = ptr<unsigned long long>(ctx->p_vac);
  pt.coll = ptr<unsigned long long>(ctx->p_coll);
  pt.eel = ptr<double>(ctx->p_eel);
  pt.enuc = ptr<double>(ctx->p_enuc);
  pt.fx = ptr<double>(ctx->p_fx);
  pt.fy = ptr<double>(ctx->p_fy);
  pt.fz = ptr<double>(ctx->p_fz);
  pt.fstate = ptr<int>(ctx->p_state);
  cudaError_t e = launch_reduce(ptr<ReduceJob>(ctx->d_jobs), int(ctx->jobs.size()), pt, ptr<double>(ctx->d_partials),
                                ptr<int>(ctx->d_job_first), int(ctx->tables.sims.size()), ptr<double>(ctx->d_out),
                                ctx->stream);
  if (e != cudaSuccess)
    return fail(ctx, MTG_ERR_CUDA, std::string("reduction launch: ") + cudaGetErrorString(e));
  ctx->stats.launches += (ctx->jobs.empty() ? 1 : 2);
  return MTG_OK;
}

cudaError_t
h2d(mtg_ctx * ctx, void * dst, const void * src, size_t bytes)
{
  ctx->stats.h2d_bytes += (long long)bytes;
  return cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice);
}

mtg_status
require_device(mtg_ctx * ctx)
{
  if (!ctx)
    return MTG_ERR_BAD_INPUT;
  CK(cudaSetDevice(ctx->device));
  return MTG_OK;
}

} // namespace

extern "C" {

mtg_status
mtg_create(int device, mtg_ctx ** out)
{
  if (!out)
    return MTG_ERR_BAD_INPUT;
  *out = nullptr;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n <= 0)
    return MTG_ERR_NO_DEVICE;
  if (device < 0 || device >= n)
    return MTG_ERR_BAD_INPUT;
  if (cudaSetDevice(device) != cudaSuccess)
    return MTG_ERR_CUDA;
  mtg_ctx * ctx = new mtg_ctx();
  ctx->device = device;
  ctx->cfg = default_config();
  std::memset(&ctx->stats, 0, sizeof ctx->stats);
  cudaDeviceGetAttribute(&ctx->n_sm, cudaDevAttrMultiProcessorCount, device);
  for (auto & e : ctx->ev)
    if (cudaEventCreate(&e) != cudaSuccess)
    {
      delete ctx;
      return MTG_ERR_CUDA;
    }
  if (mtg::upload_newton_guess32() != cudaSuccess ||
      mtg::upload_newton_guess32_surrogate(mtg::newton_guess_table32()) != cudaSuccess)
  {
    mtg_destroy(ctx);
    return MTG_ERR_CUDA;
  }
  *out = ctx;
  return MTG_OK;
}

mtg_status
mtg_destroy(mtg_ctx * ctx)
{
  if (!ctx)
    return MTG_OK;
  cudaSetDevice(ctx->device);
  DevBuf * bufs[] = {&ctx->d_sims,   &ctx->d_prim_end, &ctx->d_species, &ctx->d_mats,    &ctx->d_row_species,
                     &ctx->d_stop,   &ctx->p_vac,      &ctx->p_coll,    &ctx->p_eel,     &ctx->p_enuc,
                     &ctx->p_fx,     &ctx->p_fy,       &ctx->p_fz,      &ctx->p_state,   &ctx->d_totals,
                     &ctx->d_hist,   &ctx->d_err,      &ctx->d_counters, &ctx->d_stacks, &ctx->d_ovf0,
                     &ctx->d_ovf1,   &ctx->d_records,  &ctx->d_events,  &ctx->d_jobs,    &ctx->d_job_first,
                     &ctx->d_partials,
                     &ctx->d_out,    &ctx->d_tmp0,     &ctx->d_tmp1,    &ctx->d_tmp2,    &ctx->d_tmp3,
                     &ctx->d_species32, &ctx->d_mats32, &ctx->d_sims32, &ctx->d_sg_params, &ctx->d_sg_net,
                     &ctx->d_vox,    &ctx->d_vox_range, &ctx->d_vox_sum, &ctx->d_vox_part, &ctx->d_cl, &ctx->d_cl32,
                     &ctx->d_cl_next, &ctx->d_cl_head, &ctx->d_cl_mask};
  for (DevBuf * b : bufs)
    if (b->p)
      cudaFree(b->p);
  for (auto & e : ctx->ev)
    if (e)
      cudaEventDestroy(e);
  delete ctx;
  return MTG_OK;
}

const char *
mtg_last_error(const mtg_ctx * ctx)
{
  return ctx ? ctx->err.c_str() : "no context";
}

mtg_status
mtg_set_tables(mtg_ctx * ctx, const mtg_scoef_row * rows, int n_rows)
{
  if (!ctx)
    return MTG_ERR_BAD_INPUT;
  if (!rows || n_rows != MTG_SCOEF_ROWS)
    return fail(ctx, MTG_ERR_DATA, "stopping tables must hold 92 rows");
  std::memcpy(ctx->rows, rows, sizeof(mtg_scoef_row) * MTG_SCOEF_ROWS);
  ctx->have_tables = true;
  ctx->prepared = false;
  return MTG_OK;
}

mtg_status
mtg_load_tables(mtg_ctx * ctx, const char * path)
{
  if (!ctx)
    return MTG_ERR_BAD_INPUT;
  if (!path)
    return fail(ctx, MTG_ERR_DATA, "no table path");
  std::string err;
  mtg_scoef_row rows[MTG_SCOEF_ROWS];
  if (!read_table_file(path, rows, err))
    return fail(ctx, MTG_ERR_DATA, err);
  return mtg_set_tables(ctx, rows, MTG_SCOEF_ROWS);
}

mtg_status
mtg_configure(mtg_ctx * ctx, const mtg_config * cfg)
{
  if (!ctx || !cfg)
    return MTG_ERR_BAD_INPUT;
  if (cfg->precision < MTG_PREC_FP64 || cfg->precision > MTG_PREC_FP32_SURROGATE)
    return fail(ctx, MTG_ERR_BAD_INPUT, "unknown precision");
  if (!(cfg->length_scale > 0.0) || !(cfg->tmin > 0.0) || !(cfg->cw > 0.0) || cfg->stack_capacity < 0)
    return fail(ctx, MTG_ERR_BAD_INPUT, "length_scale, tmin and cw must be positive");
  if (cfg->block_threads != 0 && cfg->block_threads != 64 && cfg->block_threads != 128)
    return fail(ctx, MTG_ERR_BAD_INPUT, "block_threads must be 0, 64 or 128");
  if (cfg->max_primaries_per_refill < 0 || cfg->max_primaries_per_refill > 32)
    return fail(ctx, MTG_ERR_BAD_INPUT, "max_primaries_per_refill must be 0..32");
  if (cfg->refill_min_idle < 0 || cfg->refill_min_idle > 32)
    return fail(ctx, MTG_ERR_BAD_INPUT, "refill_min_idle must be 0..32");
  ctx->cfg = *cfg;
  ctx->prepared = false;
  return MTG_OK;
}

mtg_status
mtg_prepare(mtg_ctx * ctx, const mtg_sim * sims, int n_sims)
{
  mtg_status st = require_device(ctx);
  if (st != MTG_OK)
    return st;
  ctx->stats.h2d_bytes = 0;
  if (!ctx->have_tables)
    return fail(ctx, MTG_ERR_STATE, "stopping tables not loaded");
  if (ctx->cfg.precision == MTG_PREC_FP32_SURROGATE && !ctx->sg_ready)
    return fail(ctx, MTG_ERR_STATE, "no trained surrogate: call mtg_surrogate_train or mtg_surrogate_set_params");
  std::string err;
  int rc = build_tables(ctx->rows, ctx->cfg, sims, n_sims, ctx->tables, err);
  if (rc != MTG_OK)
    return fail(ctx, mtg_status(rc), err);
  const HostTables & t = ctx->tables;
  const size_t ns = t.sims.size();
  const size_t np = size_t(std::max<long long>(t.total_primaries, 1));
  CK(ensure(ctx->d_sims, sizeof(SimDesc) * ns));
  CK(ensure(ctx->d_prim_end, sizeof(long long) * ns));
  CK(ensure(ctx->d_species, sizeof(SpeciesConst) * t.species.size()));
  CK(ensure(ctx->d_mats, sizeof(MatConst) * t.mats.size()));
  CK(ensure(ctx->p_vac, 8 * np));
  CK(ensure(ctx->p_coll, 8 * np));
  CK(ensure(ctx->p_eel, 8 * np));
  CK(ensure(ctx->p_enuc, 8 * np));
  CK(ensure(ctx->p_fx, 8 * np));
  CK(ensure(ctx->p_fy, 8 * np));
  CK(ensure(ctx->p_fz, 8 * np));
  CK(ensure(ctx->p_state, 4 * np));
  CK(ensure(ctx->d_totals, sizeof(SimTotals) * ns));
  CK(ensure(ctx->d_hist, 8 * size_t(std::max<long long>(t.hist_total, 1))));
  CK(ensure(ctx->d_err, 16));
  CK(ensure(ctx->d_counters, 8 * C_COUNT));
  if (t.voxel_total > 0)
  {
    std::vector<long long> vr(2 * ns);
    for (size_t s = 0; s < ns; ++s)
    {
      const SimDesc & d = t.sims[s];
      vr[2 * s] = d.voxel_base;
      vr[2 * s + 1] = d.voxel_n[0] > 0 ? (long long)d.voxel_n[0] * d.voxel_n[1] * d.voxel_n[2] : 0;
    }
    CK(ensure(ctx->d_vox, sizeof(double) * size_t(t.voxel_total)));
    CK(ensure(ctx->d_vox_range, sizeof(long long) * vr.size()));
    CK(ensure(ctx->d_vox_sum, sizeof(double) * ns));
    CK(ensure(ctx->d_vox_part, voxel_partials_bytes(int(ns))));
    CK(h2d(ctx, ctx->d_vox_range.p, vr.data(), sizeof(long long) * vr.size()));
  }
  // cluster samples: the cluster arrays, and the simulations pointing at them
  ctx->sims_dev = t.sims;
  if (!t.clusters.empty() || !t.cl_head.empty())
  {
    CK(ensure(ctx->d_cl, sizeof(Cl4d) * std::max<size_t>(t.clusters.size(), 1)));
    CK(ensure(ctx->d_cl_next, sizeof(int) * std::max<size_t>(t.cl_next.size(), 1)));
    CK(ensure(ctx->d_cl_head, sizeof(int) * std::max<size_t>(t.cl_head.size(), 1)));
    if (!t.clusters.empty())
    {
      CK(h2d(ctx, ctx->d_cl.p, t.clusters.data(), sizeof(Cl4d) * t.clusters.size()));
      CK(h2d(ctx, ctx->d_cl_next.p, t.cl_next.data(), sizeof(int) * t.cl_next.size()));
    }
    CK(h2d(ctx, ctx->d_cl_head.p, t.cl_head.data(), sizeof(int) * t.cl_head.size()));
    CK(ensure(ctx->d_cl_mask, sizeof(uint32_t) * std::max<size_t>(t.cl_mask.size(), 1)));
    if (!t.cl_mask.empty())
      CK(h2d(ctx, ctx->d_cl_mask.p, t.cl_mask.data(), sizeof(uint32_t) * t.cl_mask.size()));
    patch_cluster_pointers(ctx->sims_dev, ptr<Cl4d>(ctx->d_cl), ptr<int>(ctx->d_cl_next), ptr<int>(ctx->d_cl_head),
                           ptr<uint32_t>(ctx->d_cl_mask));
  }
  CK(h2d(ctx, ctx->d_sims.p, ctx->sims_dev.data(), sizeof(SimDesc) * ns));
  CK(h2d(ctx, ctx->d_prim_end.p, t.prim_end.data(), sizeof(long long) * ns));
  CK(h2d(ctx, ctx->d_species.p, t.species.data(), sizeof(SpeciesConst) * t.species.size()));
  CK(h2d(ctx, ctx->d_mats.p, t.mats.data(), sizeof(MatConst) * t.mats.size()));

  // reduction jobs: contiguous chunks of at most 65536 primaries per simulation
  ctx->jobs.clear();
  ctx->job_first.assign(1, 0);
  for (size_t s = 0; s < ns; ++s)
  {
    const long long b = t.sims[s].prim_begin, n = t.sims[s].n_primaries;
    const long long chunk = 65536;
    for (long long o = 0; o < n; o += chunk)
      ctx->jobs.push_back(ReduceJob{int(s), b + o, b + std::min(n, o + chunk)});
    ctx->job_first.push_back(int(ctx->jobs.size()));
  }
  CK(ensure(ctx->d_jobs, sizeof(ReduceJob) * std::max<size_t>(ctx->jobs.size(), 1)));
  CK(ensure(ctx->d_job_first, sizeof(int) * ctx->job_first.size()));
  CK(ensure(ctx->d_partials, sizeof(double) * NQ * std::max<size_t>(ctx->jobs.size(), 1)));
  CK(ensure(ctx->d_out, sizeof(double) * NQ * ns));
  if (!ctx->jobs.empty())
    CK(h2d(ctx, ctx->d_jobs.p, ctx->jobs.data(), sizeof(ReduceJob) * ctx->jobs.size()));
  CK(h2d(ctx, ctx->d_job_first.p, ctx->job_first.data(), sizeof(int) * ctx->job_first.size()));

  if (ctx->cfg.precision != MTG_PREC_FP64)
  {
    // FP32 path: stopping tables evaluated on the device in FP64, one row per
    // distinct (species, material) of the run
    const size_t nrows = t.stop_row_mat.size();
    CK(ensure(ctx->d_row_species, 2 * sizeof(int) * nrows));
    CK(ensure(ctx->d_stop, 2 * sizeof(float) * STOP_N * nrows)); // (S, p_max) pairs
    int * d_row_species = ptr<int>(ctx->d_row_species);
    int * d_row_mat = d_row_species + nrows;
    CK(h2d(ctx, d_row_species, t.stop_row_species.data(), sizeof(int) * nrows));
    CK(h2d(ctx, d_row_mat, t.stop_row_mat.data(), sizeof(int) * nrows));
    const double lo = std::log(STOP_EMIN), hi = std::log(t.emax * 1.05);
    CK(launch_build_stop_tables(ptr<SpeciesConst>(ctx->d_species), ptr<MatConst>(ctx->d_mats), d_row_mat,
                                int(nrows), d_row_species, ptr<float>(ctx->d_stop), lo, (hi - lo) / (STOP_N - 1),
                                nullptr));
    CK(cudaDeviceSynchronize());
    std::vector<Species32> & sp32 = ctx->sp32;
    std::vector<Mat32> & mc32 = ctx->mc32;
    std::vector<Sim32> & sm32 = ctx->sm32;
    build_fp32_tables(t, sp32, mc32, sm32);
    if (!t.clusters.empty() || !t.cl_head.empty())
    {
      std::vector<Cl4f> c32(t.clusters.size());
      for (size_t l = 0; l < c32.size(); ++l)
        c32[l] = Cl4f{float(t.clusters[l].x), float(t.clusters[l].y), float(t.clusters[l].z),
                      float(t.clusters[l].r)};
      CK(ensure(ctx->d_cl32, sizeof(Cl4f) * std::max<size_t>(c32.size(), 1)));
      if (!c32.empty())
        CK(h2d(ctx, ctx->d_cl32.p, c32.data(), sizeof(Cl4f) * c32.size()));
      for (size_t i = 0; i < sm32.size(); ++i)
        if (sm32[i].geometry == 1)
        {
          sm32[i].cl = ptr<Cl4f>(ctx->d_cl32) + t.sims[i].cl_base;
          sm32[i].cl_next = ptr<int>(ctx->d_cl_next) + t.sims[i].cl_base;
          sm32[i].cl_head = ptr<int>(ctx->d_cl_head) + t.sims[i].cell_base;
          sm32[i].cl_mask = ptr<uint32_t>(ctx->d_cl_mask) + t.sims[i].mask_base;
        }
    }
    CK(ensure(ctx->d_species32, sizeof(Species32) * sp32.size()));
    CK(ensure(ctx->d_mats32, sizeof(Mat32) * mc32.size()));
    CK(ensure(ctx->d_sims32, sizeof(Sim32) * sm32.size()));
    CK(h2d(ctx, ctx->d_species32.p, sp32.data(), sizeof(Species32) * sp32.size()));
    CK(h2d(ctx, ctx->d_mats32.p, mc32.data(), sizeof(Mat32) * mc32.size()));
    CK(h2d(ctx, ctx->d_sims32.p, sm32.data(), sizeof(Sim32) * sm32.size()));
  }
  if (ctx->record_cap > 0)
    CK(ensure(ctx->d_records, sizeof(MemberRecord) * size_t(ctx->record_cap)));
  if (ctx->event_cap > 0 && ctx->event_mask)
    CK(ensure(ctx->d_events, sizeof(EventRec) * size_t(ctx->event_cap)));
  st = setup_launch_shape(ctx);
  if (st != MTG_OK)
    return st;
  ctx->prepared = true;
  ctx->launched = false;
  return MTG_OK;
}

mtg_status
mtg_launch_async(mtg_ctx * ctx, void * stream)
{
  mtg_status st = require_device(ctx);
  if (st != MTG_OK)
    return st;
  if (!ctx->prepared)
    return fail(ctx, MTG_ERR_STATE, "mtg_prepare must come first");
  ctx->stream = reinterpret_cast<cudaStream_t>(stream);
  const HostTables & t = ctx->tables;
  const size_t np = size_t(std::max<long long>(t.total_primaries, 1));
  ctx->stats.launches = 0;
  ctx->stats.drains = 0;
  cudaStream_t s = ctx->stream;
  CK(cudaMemsetAsync(ctx->p_vac.p, 0, 8 * np, s));
  CK(cudaMemsetAsync(ctx->p_coll.p, 0, 8 * np, s));
  CK(cudaMemsetAsync(ctx->p_eel.p, 0, 8 * np, s));
  CK(cudaMemsetAsync(ctx->p_enuc.p, 0, 8 * np, s));
  CK(cudaMemsetAsync(ctx->p_state.p, 0, 4 * np, s));
  CK(cudaMemsetAsync(ctx->d_totals.p, 0, sizeof(SimTotals) * t.sims.size(), s));
  CK(cudaMemsetAsync(ctx->d_hist.p, 0, 8 * size_t(std::max<long long>(t.hist_total, 1)), s));
  CK(cudaMemsetAsync(ctx->d_err.p, 0, 16, s));
  if (t.voxel_total > 0)
    CK(cudaMemsetAsync(ctx->d_vox.p, 0, sizeof(double) * size_t(t.voxel_total), s));
  CK(cudaMemsetAsync(ctx->d_counters.p, 0, 8 * C_COUNT, s));
  CK(cudaEventRecord(ctx->ev[0], s));
  st = launch_pass(ctx, 0);
  if (st != MTG_OK)
    return st;
  st = launch_pass(ctx, 1); // drains whatever the first pass spilled (usually nothing)
  if (st != MTG_OK)
    return st;
  CK(cudaEventRecord(ctx->ev[1], s));
  if (t.voxel_total > 0)
  {
    CK(launch_voxel_sum(ptr<double>(ctx->d_vox), ptr<long long>(ctx->d_vox_range), int(t.sims.size()),
                        ptr<double>(ctx->d_vox_part), ptr<double>(ctx->d_vox_sum), s));
    ctx->stats.launches += 2;
  }
  st = launch_reduction(ctx);
  if (st != MTG_OK)
    return st;
  CK(cudaEventRecord(ctx->ev[2], s));
  ctx->launched = true;
  return MTG_OK;
}

// Grows both overflow lists to `cap` records; on failure restores the old size (the
// lists must never be left unallocated under a prepared context).
static bool
grow_overflow(mtg_ctx * ctx, long long cap)
{
  const size_t rec = record_size(ctx->cfg.precision);
  if (ensure(ctx->d_ovf0, size_t(cap) * rec) == cudaSuccess && ensure(ctx->d_ovf1, size_t(cap) * rec) == cudaSuccess)
  {
    ctx->ovf_cap = cap;
    ctx->ovf_floor = std::max(ctx->ovf_floor, cap);
    return true;
  }
  cudaGetLastError();
  if (ensure(ctx->d_ovf0, size_t(ctx->ovf_cap) * rec) != cudaSuccess ||
      ensure(ctx->d_ovf1, size_t(ctx->ovf_cap) * rec) != cudaSuccess)
  {
    cudaGetLastError();
    ctx->prepared = false; // the next mtg_prepare allocates again (or reports MTG_ERR_OOM)
  }
  return false;
}

static mtg_status
collect_run(mtg_ctx * ctx, mtg_totals * totals, long long * hist, int retry);

mtg_status
mtg_collect(mtg_ctx * ctx, mtg_totals * totals, long long * hist)
{
  mtg_status st = require_device(ctx);
  if (st != MTG_OK)
    return st;
  if (!ctx->launched)
    return fail(ctx, MTG_ERR_STATE, "nothing launched");
  return collect_run(ctx, totals, hist, 0);
}

static mtg_status
collect_run(mtg_ctx * ctx, mtg_totals * totals, long long * hist, int retry)
{
  mtg_status st = MTG_OK;
  CK(cudaStreamSynchronize(ctx->stream));
  const HostTables & t = ctx->tables;
  unsigned long long cnt[C_COUNT];
  ctx->stats.d2h_bytes = sizeof cnt + sizeof(unsigned int) + (long long)(sizeof(double) * NQ + sizeof(SimTotals)) *
                         (long long)t.sims.size() + (hist ? 8LL * t.hist_total : 0LL);
  CK(cudaMemcpy(cnt, ctx->d_counters.p, sizeof cnt, cudaMemcpyDeviceToHost));
  // further drain passes while the last pass spilled members
  long long overflowed = (long long)cnt[C_OVF0];
  int extra = 0;
  while (cnt[ctx->ovf_last ? C_OVF1 : C_OVF0] > 0 && ctx->passes < MAX_PASSES)
  {
    overflowed += (long long)cnt[ctx->ovf_last ? C_OVF1 : C_OVF0];
    st = launch_pass(ctx, ctx->passes);
    if (st != MTG_OK)
      return st;
    ++extra;
    CK(cudaStreamSynchronize(ctx->stream));
    CK(cudaMemcpy(cnt, ctx->d_counters.p, sizeof cnt, cudaMemcpyDeviceToHost));
  }
  const bool unfinished = cnt[ctx->ovf_last ? C_OVF1 : C_OVF0] > 0;
  // an overflow list that filled dropped members: the run is made again with lists
  // four times larger, kept for later runs.  The random draws depend on the members'
  // keys, not on the schedule, so the repeated run is the run the larger lists would
  // have given in the first place.
  {
    unsigned int errq = 0;
    CK(cudaMemcpy(&errq, ctx->d_err.p, sizeof errq, cudaMemcpyDeviceToHost));
    if ((errq & ERRB_QUEUE_FULL) && retry < MAX_OVF_RETRIES && grow_overflow(ctx, ctx->ovf_cap * 4))
    {
      const int launched_before = ctx->stats.launches; // the count covers every attempt
      st = mtg_launch_async(ctx, ctx->stream);
      if (st != MTG_OK)
        return st;
      ctx->stats.launches += launched_before;
      return collect_run(ctx, totals, hist, retry + 1);
    }
  }
  if (extra)
  {
    CK(cudaEventRecord(ctx->ev[3], ctx->stream)); // end of the extra drain passes
    st = launch_reduction(ctx);
    if (st != MTG_OK)
      return st;
    CK(cudaEventRecord(ctx->ev[2], ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
  }
  // with extra drain passes the kernel time runs to the end of the last one (it
  // includes the first reduction and the host's turnaround between the passes)
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, ctx->ev[0], extra ? ctx->ev[3] : ctx->ev[1]);
  ctx->stats.kernel_ms = ms;
  cudaEventElapsedTime(&ms, extra ? ctx->ev[3] : ctx->ev[1], ctx->ev[2]);
  ctx->stats.reduce_ms = ms;
  ctx->stats.overflow_retries = retry;
  ctx->stats.drains = ctx->passes - 1;
  ctx->stats.warp_steps = (long long)cnt[C_STEPS];
  ctx->stats.grid = ctx->grid;
  ctx->stats.block = ctx->block;
  ctx->stats.stack_capacity = ctx->stack_cap;
  ctx->stats.overflowed = overflowed;

  ctx->stats.events_overflowed = 0;
  unsigned int errf = 0;
  CK(cudaMemcpy(&errf, ctx->d_err.p, sizeof errf, cudaMemcpyDeviceToHost));
  const size_t ns = t.sims.size();
  std::vector<double> out(NQ * ns);
  std::vector<SimTotals> tot(ns);
  CK(cudaMemcpy(out.data(), ctx->d_out.p, sizeof(double) * NQ * ns, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(tot.data(), ctx->d_totals.p, sizeof(SimTotals) * ns, cudaMemcpyDeviceToHost));
  std::vector<double> vsum(ns, 0.0);
  if (t.voxel_total > 0)
  {
    if (extra)
    {
      CK(launch_voxel_sum(ptr<double>(ctx->d_vox), ptr<long long>(ctx->d_vox_range), int(ns),
                          ptr<double>(ctx->d_vox_part), ptr<double>(ctx->d_vox_sum), ctx->stream));
      CK(cudaStreamSynchronize(ctx->stream));
    }
    CK(cudaMemcpy(vsum.data(), ctx->d_vox_sum.p, sizeof(double) * ns, cudaMemcpyDeviceToHost));
  }
  long long coll_all = 0;
  if (totals)
    for (size_t s = 0; s < ns; ++s)
    {
      mtg_totals & o = totals[s];
      std::memset(&o, 0, sizeof o);
      const double * q = &out[NQ * s];
      o.primaries = t.sims[s].n_primaries;
      o.members = (long long)tot[s].members;
      o.collisions = (long long)llround(q[2]);
      o.vacancies = (long long)llround(q[0]);
      o.replacements = (long long)tot[s].replacements;
      o.interstitials = (long long)tot[s].interstitials;
      o.substitutionals = (long long)tot[s].substitutionals;
      o.lost = (long long)tot[s].lost;
      o.Eel = q[4];
      o.Enuc = q[6];
      o.Elost = tot[s].Elost;
      o.Eunfollowed = tot[s].Eunfollowed;
      o.range_n = (long long)llround(q[8]);
      o.sx = q[9];
      o.sxx = q[10];
      o.sy = q[11];
      o.syy = q[12];
      o.sz = q[13];
      o.szz = q[14];
      o.vac_s2 = q[1];
      o.eel_s2 = q[5];
      o.enuc_s2 = q[7];
      o.coll_s2 = q[3];
      o.newton_iterations = (long long)tot[s].newton_iters;
      o.rejection_passes = (long long)tot[s].rejection_passes;
      o.surrogate_fallbacks = (long long)tot[s].fallbacks;
      o.sputtered = (long long)tot[s].sputtered;
      o.backscattered = (long long)tot[s].backscattered;
      o.Esputtered = tot[s].Esputtered;
      o.Evoxel = vsum[s];
      o.hist_dropped = (long long)tot[s].hist_dropped;
      coll_all += o.collisions;
    }
  ctx->stats.collisions = coll_all;
  if (hist && t.hist_total > 0)
  {
    std::vector<unsigned long long> h(t.hist_total);
    CK(cudaMemcpy(h.data(), ctx->d_hist.p, 8 * h.size(), cudaMemcpyDeviceToHost));
    for (long long i = 0; i < t.hist_total; ++i)
      hist[i] = (long long)h[i];
  }
  size_t bytes = 0;
  DevBuf * bufs[] = {&ctx->d_sims,   &ctx->d_prim_end, &ctx->d_species, &ctx->d_mats,    &ctx->d_row_species,
                     &ctx->d_stop,   &ctx->p_vac,      &ctx->p_coll,    &ctx->p_eel,     &ctx->p_enuc,
                     &ctx->p_fx,     &ctx->p_fy,       &ctx->p_fz,      &ctx->p_state,   &ctx->d_totals,
                     &ctx->d_hist,   &ctx->d_err,      &ctx->d_counters, &ctx->d_stacks, &ctx->d_ovf0,
                     &ctx->d_ovf1,   &ctx->d_records,  &ctx->d_events,  &ctx->d_jobs,    &ctx->d_job_first,
                     &ctx->d_partials,
                     &ctx->d_out,    &ctx->d_species32, &ctx->d_mats32, &ctx->d_sims32, &ctx->d_vox, &ctx->d_vox_part};
  for (DevBuf * b : bufs)
    bytes += b->bytes;
  ctx->stats.device_bytes = bytes;

  // a full event log is reported last: any other error of the run takes precedence
  if (unfinished || (errf & ERRB_QUEUE_FULL))
    return fail(ctx, MTG_ERR_QUEUE_FULL, "recoil overflow list exhausted; results incomplete");
  if (errf & ERRB_BUDGET)
    return fail(ctx, MTG_ERR_TIMEOUT, "a cascade member exceeded the collision budget");
  if (errf & ERRB_NUMERIC)
    return fail(ctx, MTG_ERR_NUMERIC, "non-finite energy or degenerate direction met");
  if (errf & ERRB_EVENTS_FULL)
  {
    ctx->stats.events_overflowed = 1; // the run itself is complete (the autotuner times it)
    return fail(ctx, MTG_ERR_QUEUE_FULL,
                "event log capacity " + std::to_string(ctx->event_cap) + " exceeded; the tallies are complete");
  }
  return MTG_OK;
}

mtg_status
mtg_run(mtg_ctx * ctx, const mtg_sim * sims, int n_sims, mtg_totals * totals, long long * hist)
{
  mtg_status st = mtg_prepare(ctx, sims, n_sims);
  if (st != MTG_OK)
    return st;
  st = mtg_launch_async(ctx, nullptr);
  if (st != MTG_OK)
    return st;
  return mtg_collect(ctx, totals, hist);
}

mtg_status
mtg_autotune(mtg_ctx * ctx, const mtg_sim * sims, int n_sims, long long trial_primaries, mtg_tuning * out)
{
  mtg_status st = require_device(ctx);
  if (st != MTG_OK)
    return st;
  if (!sims || n_sims < 1 || !out || trial_primaries < 0)
    return fail(ctx, MTG_ERR_BAD_INPUT, "mtg_autotune: simulations, a result and trial_primaries >= 0 are needed");
  if (trial_primaries == 0)
    trial_primaries = 262144; // smaller trials are ruled by the end-of-batch tail
  long long total = 0;
  for (int i = 0; i < n_sims; ++i)
    total += std::max<long long>(0, sims[i].n_primaries);
  if (total == 0)
    return fail(ctx, MTG_ERR_BAD_INPUT, "mtg_autotune: no primaries to time");
  // the trial: the same simulations, primaries scaled to about trial_primaries
  const double f = total > trial_primaries ? double(trial_primaries) / double(total) : 1.0;
  std::vector<mtg_sim> trial(sims, sims + n_sims);
  for (mtg_sim & s : trial)
    if (s.n_primaries > 0)
      s.n_primaries = std::max<long long>(1, llround(double(s.n_primaries) * f));
  const mtg_config base = ctx->cfg;
  std::vector<mtg_totals> tot(static_cast<size_t>(n_sims));
  int trials = 0;
  struct Setting
  {
    int block, take, cap, refill;
  };
  long long trial_total = 0;
  for (const mtg_sim & s : trial)
    trial_total += std::max<long long>(0, s.n_primaries);
  const double run_scale = double(total) / double(std::max<long long>(1, trial_total));
  // collisions per second of kernel time of one trial launch.  A launch that fails
  // (an overflow list filled by a stack too shallow for the cascades) rates 0, and so
  // does a candidate whose trial spills, scaled from the trial's primaries to the
  // run's, would fill more than a quarter of the overflow list: spills grow with the
  // primaries of a pass, and a trial that passes can still exhaust the list at the
  // run's full size
  auto rate = [&](const Setting & x, bool guard) -> double {
    mtg_config c = base;
    c.block_threads = x.block;
    c.max_primaries_per_refill = x.take;
    c.stack_capacity = x.cap;
    c.refill_min_idle = x.refill;
    if (mtg_configure(ctx, &c) != MTG_OK)
      return 0.0;
    const mtg_status s = mtg_run(ctx, trial.data(), n_sims, tot.data(), nullptr);
    if (s != MTG_OK && !(s == MTG_ERR_QUEUE_FULL && ctx->stats.events_overflowed)) // a full event log still times the run
      return 0.0;
    ++trials;
    if (guard && (ctx->stats.overflow_retries > 0 ||
                  double(ctx->stats.overflowed) * run_scale > 0.25 * double(ctx->ovf_cap)))
      return 0.0;
    return ctx->stats.kernel_ms > 0.0 ? double(ctx->stats.collisions) / (ctx->stats.kernel_ms * 1e-3) : 0.0;
  };
  const Setting built_in{base.block_threads > 0 ? base.block_threads : 128, base.max_primaries_per_refill,
                         base.stack_capacity, base.refill_min_idle};
  rate(built_in, false); // warm-up (module load, first allocations)
  const double r_def = rate(built_in, false);
  if (!(r_def > 0.0))
    return fail(ctx, MTG_ERR_BAD_INPUT, std::string("mtg_autotune: the trial run failed: ") + ctx->err);
  const int heuristic = ctx->stats.max_take;
  const int default_cap = ctx->stats.stack_capacity;
  Setting best = built_in;
  double r_best = r_def;
  // coordinate search, one setting at a time
  auto consider = [&](Setting x) {
    const double r = rate(x, true);
    if (r > r_best)
    {
      r_best = r;
      best = x;
    }
  };
  for (int take : {1, 2, 4, 8, 16, 32})
    if (take != heuristic)
      consider(Setting{best.block, take, best.cap, best.refill});
  const int refill0 = built_in.refill > 0 ? built_in.refill : (base.precision == MTG_PREC_FP64 ? 1 : 8);
  for (int refill : {1, 4, 8, 16})
    if (refill != refill0)
      consider(Setting{best.block, best.take, best.cap, refill});
  consider(Setting{best.block == 128 ? 64 : 128, best.take, best.cap, best.refill});
  if (default_cap > 1024)
    consider(Setting{best.block, best.take, default_cap / 2, best.refill});
  const bool change = r_best > 1.02 * r_def;
  const Setting chosen = change ? best : built_in;
  mtg_config c = base;
  c.block_threads = chosen.block;
  c.max_primaries_per_refill = chosen.take;
  c.stack_capacity = chosen.cap;
  c.refill_min_idle = chosen.refill;
  st = mtg_configure(ctx, &c);
  if (st != MTG_OK)
    return st;
  out->block_threads = chosen.block;
  out->max_primaries_per_refill = chosen.take;
  out->stack_capacity = chosen.cap > 0 ? chosen.cap : default_cap;
  out->refill_min_idle = chosen.refill > 0 ? chosen.refill : refill0;
  out->heuristic_take = heuristic;
  out->default_collisions_per_s = r_def;
  out->best_collisions_per_s = change ? r_best : r_def;
  out->trials = trials;
  out->changed = change ? 1 : 0;
  return MTG_OK;
}

mtg_status
mtg_get_primaries(mtg_ctx * ctx, long long first, long long n, long long * vacancies, long long * collisions,
                  double * eel, double * enuc, double * x, double * y, double * z, int * state)
{
  mtg_status st = require_device(ctx);
  if (st != MTG_OK)
    return st;
  if (!ctx->launched)
    return fail(ctx, MTG_ERR_STATE, "no run to read");
  if (first < 0 || n < 0 || first + n > ctx->tables.total_primaries)
    return fail(ctx, MTG_ERR_BAD_INPUT, "primary range out of bounds");
  if (n == 0)
    return MTG_OK;
  auto get_u64 = [&](DevBuf & b, long long * dst) -> cudaError_t {
    if (!dst)
      return cudaSuccess;
    return cudaMemcpy(dst, ptr<unsigned long long>(b) + first, 8 * n, cudaMemcpyDeviceToHost);
  };
  auto get_f64 = [&](DevBuf & b, double * dst) -> cudaError_t {
    if (!dst)
      return cudaSuccess;
    return cudaMemcpy(dst, ptr<double>(b) + first, 8 * n, cudaMemcpyDeviceToHost);
  };
  CK(get_u64(ctx->p_vac, vacancies));
  CK(get_u64(ctx->p_coll, collisions));
  CK(get_f64(ctx->p_eel, eel));
  CK(get_f64(ctx->p_enuc, enuc));
  CK(get_f64(ctx->p_fx, x));
  CK(get_f64(ctx->p_fy, y));
  CK(get_f64(ctx->p_fz, z));
  if (state)
    CK(cudaMemcpy(state, ptr<int>(ctx->p_state) + first, 4 * n, cudaMemcpyDeviceToHost));
  return MTG_OK;
}

// the voxel cells of simulation `sim` of the last run (FP64 sums on the device)
static mtg_status
voxel_cells(mtg_ctx * ctx, int sim, const void * out, long long n, const double ** src, long long * cells)
{
  mtg_status st = require_device(ctx);
  if (st != MTG_OK)
    return st;
  if (!ctx->launched)
    return fail(ctx, MTG_ERR_STATE, "no run to read");
  if (sim < 0 || sim >= int(ctx->tables.sims.size()) || !out)
    return fail(ctx, MTG_ERR_BAD_INPUT, "bad simulation index or buffer");
  const SimDesc & d = ctx->tables.sims[sim];
  *cells = d.voxel_n[0] > 0 ? (long long)d.voxel_n[0] * d.voxel_n[1] * d.voxel_n[2] : 0;
  if (n != *cells)
    return fail(ctx, MTG_ERR_BAD_INPUT, "buffer size must equal the simulation's voxel count");
  *src = ptr<double>(ctx->d_vox) + d.voxel_base;
  return MTG_OK;
}

mtg_status
mtg_get_voxels(mtg_ctx * ctx, int sim, float * out, long long n)
{
  const double * src = nullptr;
  long long cells = 0;
  mtg_status st = voxel_cells(ctx, sim, out, n, &src, &cells);
  if (st != MTG_OK || cells == 0)
    return st;
  // FP32 tally: each cell's FP64 sum rounded once
  std::vector<double> tmp(static_cast<size_t>(cells));
  CK(cudaMemcpy(tmp.data(), src, sizeof(double) * cells, cudaMemcpyDeviceToHost));
  for (long long i = 0; i < cells; ++i)
    out[i] = float(tmp[static_cast<size_t>(i)]);
  return MTG_OK;
}

mtg_status
mtg_get_voxels64(mtg_ctx * ctx, int sim, double * out, long long n)
{
  const double * src = nullptr;
  long long cells = 0;
  mtg_status st = voxel_cells(ctx, sim, out, n, &src, &cells);
  if (st != MTG_OK || cells == 0)
    return st;
  CK(cudaMemcpy(out, src, sizeof(double) * cells, cudaMemcpyDeviceToHost));
  return MTG_OK;
}

mtg_status
mtg_set_record_capacity(mtg_ctx * ctx, long long capacity)
{
  if (!ctx || capacity < 0)
    return MTG_ERR_BAD_INPUT;
  ctx->record_cap = capacity;
  ctx->prepared = false;
  return MTG_OK;
}

mtg_status
mtg_get_records(mtg_ctx * ctx, mtg_member_record * out, long long capacity, long long * n_written)
{
  mtg_status st = require_device(ctx);
  if (st != MTG_OK)
    return st;
  if (!out || !n_written || capacity < 0)
    return fail(ctx, MTG_ERR_BAD_INPUT, "bad record buffer");
  *n_written = 0;
  if (ctx->record_cap <= 0 || !ctx->launched)
    return MTG_OK;
  unsigned long long n = 0;
  CK(cudaMemcpy(&n, ptr<unsigned long long>(ctx->d_counters) + C_NREC, 8, cudaMemcpyDeviceToHost));
  long long m = std::min<long long>((long long)n, std::min(capacity, ctx->record_cap));
  static_assert(sizeof(mtg_member_record) == sizeof(MemberRecord), "record layout");
  if (m > 0)
    CK(cudaMemcpy(out, ctx->d_records.p, sizeof(MemberRecord) * m, cudaMemcpyDeviceToHost));
  *n_written = m;
  if ((long long)n > ctx->record_cap)
    return fail(ctx, MTG_ERR_QUEUE_FULL, "record buffer too small; records truncated");
  return MTG_OK;
}

mtg_status
mtg_set_event_log(mtg_ctx * ctx, unsigned int kind_mask, long long capacity)
{
  if (!ctx)
    return MTG_ERR_BAD_INPUT;
  if (capacity < 0 || (kind_mask & ~0xfeu))
    return fail(ctx, MTG_ERR_BAD_INPUT, "event kinds are 1..7 and the capacity must not be negative");
  ctx->event_cap = capacity;
  ctx->event_mask = kind_mask;
  ctx->prepared = false;
  return MTG_OK;
}

mtg_status
mtg_get_events(mtg_ctx * ctx, mtg_event * out, long long capacity, long long * n_written, long long * n_total)
{
  mtg_status st = require_device(ctx);
  if (st != MTG_OK)
    return st;
  if ((capacity > 0 && !out) || capacity < 0 || !n_written)
    return fail(ctx, MTG_ERR_BAD_INPUT, "bad event buffer");
  *n_written = 0;
  if (n_total)
    *n_total = 0;
  if (ctx->event_cap <= 0 || !ctx->event_mask || !ctx->launched)
    return MTG_OK;
  unsigned long long n = 0, unused = 0;
  CK(cudaMemcpy(&n, ptr<unsigned long long>(ctx->d_counters) + C_NEV, 8, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(&unused, ptr<unsigned long long>(ctx->d_counters) + C_NEV_UNUSED, 8, cudaMemcpyDeviceToHost));
  static_assert(sizeof(mtg_event) == sizeof(EventRec), "event layout");
  const long long filled = (long long)std::min<unsigned long long>(n, (unsigned long long)ctx->event_cap);
  if (n_total)
    *n_total = (long long)(n - unused);
  if (unused == 0)
  {
    // slots taken one at a time: the records are contiguous
    const long long m = std::min<long long>(filled, capacity);
    if (m > 0)
      CK(cudaMemcpy(out, ctx->d_events.p, sizeof(EventRec) * m, cudaMemcpyDeviceToHost));
    *n_written = m;
    return MTG_OK;
  }
  // slots taken in chunks: copy in blocks and leave out the slots no event filled
  constexpr long long BLOCK = 1 << 20;
  std::vector<EventRec> buf(static_cast<size_t>(std::min(BLOCK, std::max(filled, 1LL))));
  long long m = 0;
  for (long long at = 0; at < filled && m < capacity; at += BLOCK)
  {
    const long long k = std::min(BLOCK, filled - at);
    CK(cudaMemcpy(buf.data(), ptr<EventRec>(ctx->d_events) + at, sizeof(EventRec) * k, cudaMemcpyDeviceToHost));
    for (long long i = 0; i < k && m < capacity; ++i)
      if (buf[size_t(i)].kind != EV_UNUSED)
        std::memcpy(out + m++, &buf[size_t(i)], sizeof(EventRec));
  }
  *n_written = m;
  return MTG_OK;
}

mtg_status
mtg_stopping(mtg_ctx * ctx, int Z1, double m1, const mtg_material * material, const double * E, long long n,
             int precision, double * out)
{
  mtg_status st = require_device(ctx);
  if (st != MTG_OK)
    return st;
  if (!ctx->have_tables)
    return fail(ctx, MTG_ERR_STATE, "stopping tables not loaded");
  if (!material || (n > 0 && (!E || !out)) || n < 0 || Z1 < 1 || Z1 > MTG_SCOEF_ROWS)
    return fail(ctx, MTG_ERR_BAD_INPUT, "bad stopping request");
  if (precision != MTG_PREC_FP64 && precision != MTG_PREC_FP32)
    return fail(ctx, MTG_ERR_BAD_INPUT, "stopping precision must be FP64 or FP32");
  std::string err;
  SpeciesConst sc = make_species(ctx->rows, Z1, m1);
  MatConst mc;
  int rc = make_material(ctx->rows, sc, *material, ctx->cfg.tmin, mc, err);
  if (rc != MTG_OK)
    return fail(ctx, mtg_status(rc), err);
  if (n == 0)
    return MTG_OK;
  CK(ensure(ctx->d_tmp0, sizeof sc + sizeof mc));
  CK(ensure(ctx->d_tmp1, 8 * size_t(n)));
  CK(ensure(ctx->d_tmp2, 8 * size_t(n)));
  SpeciesConst * d_sc = ptr<SpeciesConst>(ctx->d_tmp0);
  MatConst * d_mc = reinterpret_cast<MatConst *>(reinterpret_cast<char *>(ctx->d_tmp0.p) + sizeof sc);
  CK(cudaMemcpy(d_sc, &sc, sizeof sc, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(d_mc, &mc, sizeof mc, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(ctx->d_tmp1.p, E, 8 * n, cudaMemcpyHostToDevice));
  if (precision == MTG_PREC_FP64)
    CK(launch_stopping64(d_sc, d_mc, ptr<double>(ctx->d_tmp1), n, ptr<double>(ctx->d_tmp2), nullptr));
  else
  {
    // one stopping-table row, exactly as the FP32 engine builds it
    double emax = 0.0;
    for (long long i = 0; i < n; ++i)
      emax = std::max(emax, E[i]);
    const double lo = std::log(STOP_EMIN), hi = std::log(std::max(emax, 1.0) * 1.05);
    const double dl = (hi - lo) / (STOP_N - 1);
    CK(ensure(ctx->d_tmp3, 2 * sizeof(float) * STOP_N + sizeof(int)));
    int zero = 0;
    int * d_rs = reinterpret_cast<int *>(reinterpret_cast<char *>(ctx->d_tmp3.p) + 2 * sizeof(float) * STOP_N);
    CK(cudaMemcpy(d_rs, &zero, sizeof zero, cudaMemcpyHostToDevice));
    CK(launch_build_stop_tables(d_sc, d_mc, nullptr, 1, d_rs, ptr<float>(ctx->d_tmp3), lo, dl, nullptr));
    CK(launch_stopping32(ptr<float>(ctx->d_tmp3), float(lo), float(1.0 / dl), ptr<double>(ctx->d_tmp1), n,
                         ptr<double>(ctx->d_tmp2), nullptr));
  }
  CK(cudaMemcpy(out, ctx->d_tmp2.p, 8 * n, cudaMemcpyDeviceToHost));
  return MTG_OK;
}

mtg_status
mtg_scatter(mtg_ctx * ctx, const double * eps, const double * b, long long n, int precision, double * s2)
{
  return mtg_scatter_potential(ctx, eps, b, n, precision, MTG_POT_UNIVERSAL, s2);
}

mtg_status
mtg_scatter_potential(mtg_ctx * ctx, const double * eps, const double * b, long long n, int precision,
                      int potential, double * s2)
{
  mtg_status st = require_device(ctx);
  if (st != MTG_OK)
    return st;
  if (n < 0 || (n > 0 && (!eps || !b || !s2)))
    return fail(ctx, MTG_ERR_BAD_INPUT, "bad scatter request");
  if (potential < MTG_POT_UNIVERSAL || potential > MTG_POT_CKR ||
      (precision == MTG_PREC_FP32_SURROGATE && potential != MTG_POT_UNIVERSAL))
    return fail(ctx, MTG_ERR_BAD_INPUT, "invalid potential for this precision");
  if (n == 0)
    return MTG_OK;
  CK(ensure(ctx->d_tmp1, 8 * size_t(n)));
  CK(ensure(ctx->d_tmp2, 8 * size_t(n)));
  CK(ensure(ctx->d_tmp3, 8 * size_t(n)));
  CK(cudaMemcpy(ctx->d_tmp1.p, eps, 8 * n, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(ctx->d_tmp2.p, b, 8 * n, cudaMemcpyHostToDevice));
  if (precision == MTG_PREC_FP64)
    CK(launch_scatter64(ptr<double>(ctx->d_tmp1), ptr<double>(ctx->d_tmp2), n, ptr<double>(ctx->d_tmp3), potential,
                        nullptr));
  else if (precision == MTG_PREC_FP32)
    CK(launch_scatter32(ptr<double>(ctx->d_tmp1), ptr<double>(ctx->d_tmp2), n, ptr<double>(ctx->d_tmp3), potential,
                        nullptr));
  else
  {
    if (!ctx->sg_ready)
      return fail(ctx, MTG_ERR_STATE, "no trained surrogate loaded");
    CK(launch_surrogate_eval(ctx->d_sg_net.p, ptr<double>(ctx->d_tmp1), ptr<double>(ctx->d_tmp2), n,
                             ptr<double>(ctx->d_tmp3), nullptr));
  }
  CK(cudaMemcpy(s2, ctx->d_tmp3.p, 8 * n, cudaMemcpyDeviceToHost));
  return MTG_OK;
}

mtg_status
mtg_surrogate_train(mtg_ctx * ctx, const mtg_surrogate_config * cfg, mtg_surrogate_report * rep)
{
  mtg_status st = require_device(ctx);
  if (st != MTG_OK)
    return st;
  if (!cfg || cfg->n_train < 1024 || cfg->batch < 32 || cfg->batch > cfg->n_train || cfg->epochs < 1 ||
      cfg->qat_epochs < 0 || cfg->qat_epochs > cfg->epochs || !(cfg->lr > 0.0f) ||
      (cfg->target != MTG_SURROGATE_TARGET_QUADRATURE && cfg->target != MTG_SURROGATE_TARGET_MAGIC) ||
      (cfg->weighting != MTG_SURROGATE_WEIGHT_UNIFORM && cfg->weighting != MTG_SURROGATE_WEIGHT_TRANSFER))
    return fail(ctx, MTG_ERR_BAD_INPUT, "bad surrogate training configuration");
  CK(ensure(ctx->d_sg_params, 4 * MTG_SURROGATE_NPARAM));
  CK(ensure(ctx->d_sg_net, surrogate_net_bytes()));
  double loss = 0.0, secs = 0.0;
  CK(surrogate_train(cfg->n_train, cfg->batch, cfg->epochs, cfg->qat_epochs, cfg->lr, cfg->seed, cfg->w_tau,
                     cfg->target, cfg->weighting, ptr<float>(ctx->d_sg_params), ctx->d_sg_net.p, &loss, &secs));
  ctx->sg_ready = true;
  if (rep)
  {
    rep->final_loss = loss;
    rep->train_seconds = secs;
    rep->steps = (long long)cfg->epochs * std::max<long long>(1, cfg->n_train / cfg->batch);
  }
  return MTG_OK;
}

mtg_status
mtg_surrogate_get_params(mtg_ctx * ctx, float * params, long long n)
{
  mtg_status st = require_device(ctx);
  if (st != MTG_OK)
    return st;
  if (!params || n != MTG_SURROGATE_NPARAM)
    return fail(ctx, MTG_ERR_BAD_INPUT, "parameter vector must hold MTG_SURROGATE_NPARAM floats");
  if (!ctx->sg_ready)
    return fail(ctx, MTG_ERR_STATE, "no trained surrogate");
  CK(cudaMemcpy(params, ctx->d_sg_params.p, 4 * n, cudaMemcpyDeviceToHost));
  return MTG_OK;
}

mtg_status
mtg_surrogate_set_params(mtg_ctx * ctx, const float * params, long long n)
{
  mtg_status st = require_device(ctx);
  if (st != MTG_OK)
    return st;
  if (!params || n != MTG_SURROGATE_NPARAM)
    return fail(ctx, MTG_ERR_BAD_INPUT, "parameter vector must hold MTG_SURROGATE_NPARAM floats");
  for (long long i = 0; i < n; ++i)
    if (!std::isfinite(params[i]))
      return fail(ctx, MTG_ERR_BAD_INPUT, "non-finite surrogate parameter");
  CK(ensure(ctx->d_sg_params, 4 * MTG_SURROGATE_NPARAM));
  CK(ensure(ctx->d_sg_net, surrogate_net_bytes()));
  CK(cudaMemcpy(ctx->d_sg_params.p, params, 4 * n, cudaMemcpyHostToDevice));
  CK(launch_pack_net(ptr<float>(ctx->d_sg_params), ctx->d_sg_net.p, nullptr));
  CK(cudaDeviceSynchronize());
  ctx->sg_ready = true;
  return MTG_OK;
}

mtg_status
mtg_surrogate_gradients(mtg_ctx * ctx, const float * params, const float * x, const float * y, long long n,
                        float w_tau, float * loss, float * grads)
{
  mtg_status st = require_device(ctx);
  if (st != MTG_OK)
    return st;
  if (!params || !x || !y || !loss || !grads || n < 1 || n > (1 << 22))
    return fail(ctx, MTG_ERR_BAD_INPUT, "bad gradient request");
  CK(surrogate_gradients(params, x, y, n, w_tau, loss, grads));
  return MTG_OK;
}

mtg_status
mtg_surrogate_quadrature(mtg_ctx * ctx, const double * eps, const double * b, long long n, double * s2,
                         double * tau)
{
  mtg_status st = require_device(ctx);
  if (st != MTG_OK)
    return st;
  if (n < 0 || (n > 0 && (!eps || !b || !s2)))
    return fail(ctx, MTG_ERR_BAD_INPUT, "bad quadrature request");
  if (n == 0)
    return MTG_OK;
  for (long long i = 0; i < n; ++i)
    if (!(eps[i] > 0.0) || !(b[i] >= 0.0))
      return fail(ctx, MTG_ERR_BAD_INPUT, "quadrature needs eps > 0 and b >= 0");
  CK(ensure(ctx->d_tmp0, 8 * size_t(n)));
  CK(ensure(ctx->d_tmp1, 8 * size_t(n)));
  CK(ensure(ctx->d_tmp2, 8 * size_t(n)));
  CK(ensure(ctx->d_tmp3, 8 * size_t(n)));
  CK(cudaMemcpy(ctx->d_tmp0.p, eps, 8 * n, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(ctx->d_tmp1.p, b, 8 * n, cudaMemcpyHostToDevice));
  CK(launch_quadrature(ptr<double>(ctx->d_tmp0), ptr<double>(ctx->d_tmp1), n, ptr<double>(ctx->d_tmp2),
                       ptr<double>(ctx->d_tmp3), nullptr));
  CK(cudaMemcpy(s2, ctx->d_tmp2.p, 8 * n, cudaMemcpyDeviceToHost));
  if (tau)
    CK(cudaMemcpy(tau, ctx->d_tmp3.p, 8 * n, cudaMemcpyDeviceToHost));
  return MTG_OK;
}

mtg_status
mtg_get_stats(const mtg_ctx * ctx, mtg_stats * out)
{
  if (!ctx || !out)
    return MTG_ERR_BAD_INPUT;
  *out = ctx->stats;
  return MTG_OK;
}

} // extern "C"
