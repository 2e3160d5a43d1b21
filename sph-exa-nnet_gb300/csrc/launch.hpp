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
};

KernelInfo denseKernel(int net, int eos);
KernelInfo sparseKernel(int net, int eos, int mixed);

} // namespace nnet_gb300
