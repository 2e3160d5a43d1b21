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
};

KernelInfo denseKernel(int net, int eos);
KernelInfo sparseKernel(int net, int eos, int mixed);
KernelInfo warpKernel(int net, int eos, int mixed);  // one warp per particle
KernelInfo batchKernel(int net, int eos, int mixed); // 32 particles per warp in lockstep
KernelInfo batchMultiKernel(int eos, int mixed);     // the same over net86, net87, net14 sub-batches

} // namespace nnet_gb300
