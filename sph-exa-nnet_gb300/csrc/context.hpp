// Library context (the object behind nnet_handle) and the internal burn launcher shared by
// the C ABI and the burn server.
#pragma once

#include <algorithm>
#include <cuda_runtime.h>

#include "common.cuh"
#include "launch.hpp"
#include "sparse_plan.hpp"

namespace nnet_gb300
{

// one device allocation per network holding every table of NetView
struct NetBuffer
{
    void*      mem = nullptr;
    NetView    view{};
    SparsePlan plan;
};

// per-launch resources: the persistent grid's slot scratch and the queue / stats counters.
// One launch may be in flight per workspace.
struct Workspace
{
    double*             scratch  = nullptr;
    size_t              doubles  = 0;
    unsigned long long* counters = nullptr; // [0] queue head, [1..] stats (BurnParams::stats)
    int32_t*            status    = nullptr; // per-particle statuses when the caller passes none
    size_t              statusCap = 0;       //   and a post-burn pass needs them
    MigCell*            mig       = nullptr; // hand-off records of the batched layout's rebalancing
    size_t              migCap    = 0;
    int                 ensure(size_t need, cudaStream_t st);
    int                 ensureStatus(size_t P, cudaStream_t st);
    int                 ensureMig(size_t cells, cudaStream_t st);
    void                release();
};

// Post-burn steps (BurnParams::postSteps) of a launch whose kernel does not fuse them: one
// thread per particle after the burn, on `st`; bp.status must hold every particle's status.
int launchPostBurn(const BurnParams& bp, const NetView& nv, const HelmView& hv, int numSMs, cudaStream_t st);

// Launch one burn over args->num_particles particles on `st` with workspace `ws`.
// rs / sliceIters / segFinished enable pausing and resuming (see BurnParams).
int launchBurn(struct ::nnet_context* h, const nnet_burn_args* args, Workspace& ws, cudaStream_t st,
               const ResumeState* rs, long long sliceIters, unsigned long long* segFinished);

// argument checks and kernel parameters of nnet_burn; last-error message of the C ABI
int  validateBurn(struct ::nnet_context* h, const nnet_burn_args* a);
void fillBurnParams(const nnet_burn_args* a, unsigned long long* counters, BurnParams& bp);
int  setError(int code, const char* msg);

// resident blocks per SM of a burn kernel (sets its dynamic shared-memory limit first)
int occupancy(const KernelInfo& ki, int& perSM);

// kernel of (network, eos, solver) under the context's layout
KernelInfo burnKernel(struct ::nnet_context* h, int net, int eos, int solver, bool post = false);

// scratch doubles of the largest persistent grid of any network for `solver`
size_t maxScratchDoubles(struct ::nnet_context* h, int solver);

} // namespace nnet_gb300

struct nnet_context
{
    int                    device = 0, numSMs = 0;
    nnet_gb300::NetBuffer  nets[3];
    void*                  helmMem    = nullptr;
    nnet_gb300::HelmView   helm{};
    bool                   helmLoaded = false;
    nnet_gb300::Workspace  ws;
    cudaStream_t           lastStream = nullptr;
    bool                   lastMulti  = false; // last launch was nnet_burn_batch
    int                    layout     = NNET_LAYOUT_AUTO;
    int                    laneSlots  = 32; // batched layout: particles in flight per warp
    bool                   rebalance  = true; // batched layout: hand particles between warps
    // device addresses of nnet_burn_noalloc's fixed arrays, looked up by its first call on this
    // handle (they live as long as the device context the handle was created in)
    double*                noallocScratch  = nullptr;
    unsigned long long*    noallocCounters = nullptr;
    unsigned long long*    orderCounters   = nullptr; // nnet_cost_order's bucket counters and cursors
};
