// Plain FP64 form: dense assembly and Gaussian elimination in the reference's operation
// order (DensePolicy in burn_policies.cuh), one thread per particle.
#include "burn_policies.cuh"
#include "launch.hpp"

namespace nnet_gb300
{

template<int NET, int EOS>
__global__ void __launch_bounds__(128) burnDenseKernel(BurnParams bp, NetView nv, HelmView hv, double* scratch,
                                                       size_t stride)
{
    const size_t      slot = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    DensePolicy<NET> pol(scratch, stride, slot);
    burnLoop<NET, EOS>(bp, nv, hv, pol);
}

template<int NET, int EOS>
static KernelInfo denseInfo()
{
    return {(const void*)burnDenseKernel<NET, EOS>, DensePolicy<NET>::perSlot(), 128, 0};
}

KernelInfo denseKernel(int net, int eos)
{
    if (net == 14) return eos ? denseInfo<14, 1>() : denseInfo<14, 0>();
    if (net == 86) return eos ? denseInfo<86, 1>() : denseInfo<86, 0>();
    return eos ? denseInfo<87, 1>() : denseInfo<87, 0>();
}

} // namespace nnet_gb300
