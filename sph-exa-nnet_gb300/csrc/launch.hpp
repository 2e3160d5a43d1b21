// Kernel registry shared by the solver translation units and the C ABI.
#pragma once

#include <cstddef>

namespace nnet_gb300
{

struct KernelInfo
{
    const void* func;      // __global__ (BurnParams, NetView, HelmView, double* scratch, size_t stride)
    size_t      perSlot;   // scratch doubles per thread slot
    int         block;     // threads per block
    int         maxNnz;    // sparse forms: capacity of the factor storage (0 = dense)
    size_t      smem = 0;  // warp-cooperative forms: dynamic shared memory per block (bytes)
    int         lanesPerParticle = 1; // 32: one warp per particle in flight
    bool        fusedPost = false;    // the kernel applies the post-burn steps itself
};

// per-slot doubles that nnet_burn_noalloc's fixed scratch array reserves; every batched-layout
// kernel's slot size is checked against it at compile time (burn_batch.cuh)
constexpr size_t kNoallocSlotDoubles = 230;

KernelInfo denseKernel(int net, int eos);
KernelInfo sparseKernel(int net, int eos, int mixed);
KernelInfo warpKernel(int net, int eos, int mixed);  // one warp per particle
// per network / EOS (burn_batch14.cu, burn_batch86.cu, burn_batch87.cu, burn_batch_multi_*.cu)
KernelInfo batchKernel14(int eos, int mixed, bool post);
KernelInfo batchKernel86(int eos, int mixed, bool post);
KernelInfo batchKernel87(int eos, int mixed, bool post);
KernelInfo batchMultiKernel0(int mixed, bool post);
KernelInfo batchMultiKernel1(int mixed, bool post);

// 32 particles per warp in lockstep; `post`: the instantiation that applies the post-burn steps
inline KernelInfo batchKernel(int net, int eos, int mixed, bool post = false)
{
    if (net == 14) return batchKernel14(eos, mixed, post);
    if (net == 86) return batchKernel86(eos, mixed, post);
    return batchKernel87(eos, mixed, post);
}
// the same over net86, net87, net14 sub-batches in one launch
inline KernelInfo batchMultiKernel(int eos, int mixed, bool post = false)
{
    return eos ? batchMultiKernel1(mixed, post) : batchMultiKernel0(mixed, post);
}

} // namespace nnet_gb300
