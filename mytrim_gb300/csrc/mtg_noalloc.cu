// Allocation-free variant of the per-primary tally reduction.
//
// Some programs that embed this engine cannot let it call cudaMalloc: a host code
// that has already handed all device memory to its own pool allocator (as large
// multiphysics applications coupling a cascade code often do), or one that forbids
// libraries to allocate once its time loop runs.  Such a caller keeps the
// per-primary tallies in device buffers it owns and still needs the run totals.
// mtg_reduce_primaries_noalloc gives it those totals with no allocation at all:
// its scratch space (the per-chunk partial sums) is a fixed array in this
// library's own device memory, NOALLOC_MAX_CHUNKS * NQ doubles (120 KiB), which
// every GPU that loads the library holds until the process exits.
//
// The arithmetic is the one mtg_collect uses (mtg_reduce.cuh, shared with
// mtg_reduce.cu): chunks of 65536 primaries, each summed by one block in a fixed
// order, then the chunks in index order with compensated FP64 adds, so the totals
// are the same bits as the ones mtg_collect reports for a single simulation.
#include <cuda.h> // CUcontext / CUresult types only: the driver calls are reached through the runtime
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "mytrim_gpu.h"
#include "mtg_kernels.h"
#include "mtg_reduce.cuh"

namespace
{

constexpr int NOALLOC_BLOCK = mtg::RBLOCK;
constexpr long long NOALLOC_CHUNK = 65536; // primaries per block, as in mtg_collect
constexpr int NOALLOC_MAX_CHUNKS = 1024;   // at most 67,108,864 primaries per call
constexpr int NQ = mtg::NQ;

// The scratch array shared by every call on a device.  Each call writes every
// slot it later reads (one row of NQ partial sums per chunk), so nothing has to
// be cleared between calls; two calls whose kernels overlap on the GPU would
// overwrite each other's partial sums, so calls must be ordered (one stream, or
// synchronised).
static __device__ __align__(256) double g_noalloc_partials[NOALLOC_MAX_CHUNKS * NQ];

__global__ void __launch_bounds__(NOALLOC_BLOCK)
noalloc_chunk_kernel(const unsigned long long * vac, const unsigned long long * coll, const double * eel,
                     const double * enuc, const double * fx, const double * fy, const double * fz,
                     const int * fstate, long long n, double * partials)
{
  const long long begin = (long long)blockIdx.x * NOALLOC_CHUNK;
  const long long end = begin + NOALLOC_CHUNK < n ? begin + NOALLOC_CHUNK : n;
  mtg::block_sum_primaries(vac, coll, eel, enuc, fx, fy, fz, fstate, begin, end, partials + (long long)blockIdx.x * NQ);
}

__global__ void
noalloc_finish_kernel(const double * partials, int nchunks, double * out)
{
  const int k = threadIdx.x;
  if (k >= NQ)
    return;
  mtg::Comp a{0.0, 0.0};
  for (int j = 0; j < nchunks; ++j)
    mtg::comp_add(a, partials[(long long)j * NQ + k]);
  out[k] = a.s + a.c;
}

constexpr int MAX_DEVICES = 64;
std::mutex g_setup_mutex;

// The scratch array's device address is a property of the CUDA context the module
// was loaded into: after cudaDeviceReset (or under another context on the same
// device) the array lives elsewhere.  The address is therefore cached per device
// together with the unique id of the context it was looked up in (cuCtxGetId),
// and looked up again when the current context's id differs.
struct ScratchAddr
{
  unsigned long long ctx_id; // 0: unknown, look up on every call
  double * addr;
};
ScratchAddr g_scratch[MAX_DEVICES] = {};

using CtxGetCurrent = CUresult (*)(CUcontext *);
using CtxGetId = CUresult (*)(CUcontext, unsigned long long *);
CtxGetCurrent g_ctx_get_current = nullptr;
CtxGetId g_ctx_get_id = nullptr;
bool g_entry_points_tried = false;

// unique id of the calling thread's current context, 0 if there is none or the
// driver does not provide the query (caller holds g_setup_mutex)
unsigned long long
current_context_id()
{
  if (!g_entry_points_tried)
  {
    g_entry_points_tried = true;
    void * f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 4000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      g_ctx_get_current = reinterpret_cast<CtxGetCurrent>(f);
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      g_ctx_get_id = reinterpret_cast<CtxGetId>(f);
    cudaGetLastError(); // a failed query leaves no sticky error behind
  }
  if (!g_ctx_get_current || !g_ctx_get_id)
    return 0;
  CUcontext c = nullptr;
  unsigned long long id = 0;
  if (g_ctx_get_current(&c) != CUDA_SUCCESS || !c || g_ctx_get_id(c, &id) != CUDA_SUCCESS)
    return 0;
  return id;
}

void
set_error(char * buf, size_t len, const char * msg)
{
  if (buf && len > 0)
  {
    std::strncpy(buf, msg, len - 1);
    buf[len - 1] = '\0';
  }
}

} // namespace

extern "C" mtg_status
mtg_reduce_primaries_noalloc(const unsigned long long * vacancies, const unsigned long long * collisions,
                             const double * eel, const double * enuc, const double * x, const double * y,
                             const double * z, const int * state, long long n, double * out, void * stream,
                             char * errbuf, size_t errbuf_len)
{
  if (n < 0 || !out || (n > 0 && (!vacancies || !collisions || !eel || !enuc || !x || !y || !z || !state)))
  {
    set_error(errbuf, errbuf_len, "mtg_reduce_primaries_noalloc: null buffer or negative count");
    return MTG_ERR_BAD_INPUT;
  }
  if (n > NOALLOC_CHUNK * NOALLOC_MAX_CHUNKS)
  {
    char msg[160];
    std::snprintf(msg, sizeof msg,
                  "mtg_reduce_primaries_noalloc: %lld primaries exceed the fixed scratch limit of %lld",
                  n, NOALLOC_CHUNK * NOALLOC_MAX_CHUNKS);
    set_error(errbuf, errbuf_len, msg);
    return MTG_ERR_BAD_INPUT;
  }
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess)
  {
    set_error(errbuf, errbuf_len, cudaGetErrorString(e));
    return e == cudaErrorNoDevice ? MTG_ERR_NO_DEVICE : MTG_ERR_CUDA;
  }
  if (dev < 0 || dev >= MAX_DEVICES)
  {
    set_error(errbuf, errbuf_len, "mtg_reduce_primaries_noalloc: device index out of range");
    return MTG_ERR_BAD_INPUT;
  }
  double * scratch = nullptr;
  {
    // once per device (and context), with that device current: the device address
    // of the scratch array (its host-side name is only a stand-in, not an address)
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    unsigned long long id = current_context_id();
    ScratchAddr & c = g_scratch[dev];
    if (!c.addr || id == 0 || c.ctx_id != id)
    {
      void * p = nullptr;
      e = cudaGetSymbolAddress(&p, g_noalloc_partials);
      if (e != cudaSuccess || !p)
      {
        set_error(errbuf, errbuf_len, e != cudaSuccess ? cudaGetErrorString(e) : "null symbol address");
        return MTG_ERR_CUDA;
      }
      // the lookup makes the device's primary context current if none was
      c.addr = static_cast<double *>(p);
      c.ctx_id = id ? id : current_context_id();
    }
    scratch = c.addr;
  }
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  const int nchunks = int((n + NOALLOC_CHUNK - 1) / NOALLOC_CHUNK);
  if (nchunks > 0)
    noalloc_chunk_kernel<<<nchunks, NOALLOC_BLOCK, 0, st>>>(vacancies, collisions, eel, enuc, x, y, z, state, n,
                                                            scratch);
  noalloc_finish_kernel<<<1, 32, 0, st>>>(scratch, nchunks, out);
  e = cudaGetLastError();
  if (e != cudaSuccess)
  {
    set_error(errbuf, errbuf_len, cudaGetErrorString(e));
    return MTG_ERR_CUDA;
  }
  return MTG_OK;
}
