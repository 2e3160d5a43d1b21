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
    size_t      smem = 0;  // warp-per-particle forms: dynamic shared memory per block (bytes)
};

KernelInfo denseKernel(int net, int eos);
KernelInfo sparseKernel(int net, int eos, int mixed);
KernelInfo warpKernel(int net, int eos, int mixed); // one warp per particle (smem != 0)

} // namespace nnet_gb300
