// nnet_burn_noalloc: the burn for callers that cannot allocate device memory.
//
// nnet_burn keeps a workspace per handle (the persistent grid's slot scratch and the work-queue
// and statistics counters) and grows it with cudaMalloc whenever a launch needs a larger grid.
// Some callers cannot let a library allocate in the middle of a time step: hydro codes that
// hand all device memory to their own arena allocator at start-up and run to a fixed budget,
// and codes that keep several streams busy, where a cudaMalloc or cudaFree can synchronise the
// device and stall every stream.  This entry point runs the batched-warp kernel with its slot
// scratch and counters in fixed arrays compiled into the library instead, so a call allocates
// nothing; the caller passes inputs and outputs exactly as to nnet_burn.
//
// Limits and rules:
//   * the arrays hold kSlots particle slots of the largest network (7.2 MiB of scratch) and are
//     reserved on every GPU that loads the library, until the process exits;
//   * scratch does not grow with the number of particles: the persistent grid is capped to the
//     array's slots and the work queue feeds any number of particles through them; a launch whose
//     slots would not fit the array is rejected with NNET_ERR_TOO_LARGE;
//   * the first call on a handle looks up the arrays' device addresses with the handle's device
//     current and keeps them in the handle; make that first call before any stream capture;
//   * every call shares the arrays: the counters are cleared on the caller's stream at the start
//     of each call (the scratch needs no clearing: each slot loads its particle before use), and
//     two calls that overlap on the GPU race on both; nnet_get_stats does not report these calls;
//   * the post-burn steps (normalize_mass, mass_drift, the EOS outputs) are applied by the
//     kernel itself, so they need no extra memory either.
#include <algorithm>
#include <string>

#include "context.hpp"
#include "launch.hpp"

namespace
{
using namespace nnet_gb300;

constexpr size_t kSlots        = 4096;                // particle slots in flight at most
constexpr size_t kSlotDoubles  = kNoallocSlotDoubles; // largest per-slot need of the batched kernels
constexpr size_t kScratch      = kSlots * kSlotDoubles;
constexpr int    kCounterWords = 16; // queue head + statistics (BurnParams::stats)
static_assert(1 + kStatWords <= kCounterWords, "counter array too small");

static __device__ __align__(256) double g_scratch[kScratch];
static __device__ __align__(256) unsigned long long g_counters[kCounterWords];

int cudaFail(cudaError_t e, const char* what)
{
    std::string m = std::string(what) + ": " + cudaGetErrorString(e);
    return setError(NNET_ERR_CUDA, m.c_str());
}

// device addresses of the arrays in the handle's context (the handle's device is current)
int deviceArrays(nnet_context* h)
{
    if (h->noallocScratch) return NNET_SUCCESS;
    void* s = nullptr;
    void* c = nullptr;
    if (cudaError_t e = cudaGetSymbolAddress(&s, g_scratch)) return cudaFail(e, "cudaGetSymbolAddress(scratch)");
    if (cudaError_t e = cudaGetSymbolAddress(&c, g_counters)) return cudaFail(e, "cudaGetSymbolAddress(counters)");
    h->noallocScratch  = static_cast<double*>(s);
    h->noallocCounters = static_cast<unsigned long long*>(c);
    return NNET_SUCCESS;
}
} // namespace

extern "C" int nnet_burn_noalloc(nnet_handle h, const nnet_burn_args* a, void* stream)
{
    if (int rc = validateBurn(h, a)) return rc;
    if (a->solver == NNET_SOLVER_DENSE_FP64)
        return setError(NNET_ERR_INVALID, "nnet_burn_noalloc runs the sparse and mixed solvers only");
    if (a->num_particles == 0) return NNET_SUCCESS;
    if (cudaError_t e = cudaSetDevice(h->device)) return cudaFail(e, "cudaSetDevice");
    if (int rc = deviceArrays(h)) return rc;

    const bool       post = a->normalize_mass || a->mass_drift || a->u;
    const KernelInfo ki   = batchKernel(a->network, a->eos, a->solver == NNET_SOLVER_MIXED, post);
    const int        ni   = a->network == 14 ? 0 : a->network == 86 ? 1 : 2;
    if (ki.maxNnz && h->nets[ni].plan.nnz > ki.maxNnz)
        return setError(NNET_ERR_TOO_LARGE, "sparse factor does not fit the kernel's storage");
    int perSM = 0;
    if (int rc = occupancy(ki, perSM)) return rc;
    if (perSM < 1) return setError(NNET_ERR_TOO_LARGE, "burn kernel does not fit on an SM");
    // the persistent grid: as many blocks as fit the SMs, the particles and the fixed array
    const size_t perBlock = (size_t)ki.block / ki.lanesPerParticle;
    size_t       blocks   = std::min((size_t)h->numSMs * perSM, (a->num_particles + perBlock - 1) / perBlock);
    blocks                = std::min(blocks, kScratch / (ki.perSlot * ki.block));
    const size_t slots    = blocks * ki.block;
    if (blocks == 0 || slots * ki.perSlot > kScratch)
        return setError(NNET_ERR_TOO_LARGE, "nnet_burn_noalloc: one block of this network's slots exceeds the "
                                            "fixed scratch array (7.2 MiB)");

    BurnParams bp;
    fillBurnParams(a, h->noallocCounters, bp);
    bp.laneSlots = h->laneSlots;
    cudaStream_t st = (cudaStream_t)stream;
    if (cudaError_t e = cudaMemsetAsync(h->noallocCounters, 0, sizeof(g_counters), st))
        return cudaFail(e, "cudaMemsetAsync");
    NetView  nv     = h->nets[ni].view;
    HelmView hv     = h->helm;
    double*  sc     = h->noallocScratch;
    size_t   stride = slots;
    void*    args[] = {&bp, &nv, &hv, &sc, &stride};
    if (cudaError_t e = cudaLaunchKernel(ki.func, dim3((unsigned)blocks), dim3(ki.block), args, ki.smem, st))
        return cudaFail(e, "cudaLaunchKernel");
    return NNET_SUCCESS;
}
