// One launch over sub-batches of different networks (the uneven mixed workload): a
// persistent grid whose threads drain the net86, then net87, then net14 work queues, so
// the most expensive particles start first and the cheap net14 ones fill the tail.  A
// thread moves to the next network only when that network's queue is empty, so lanes of a
// warp diverge only around those transitions.
#include <algorithm>

#include "burn_multi.hpp"
#include "driver.cuh"

// the solver policies
#include "burn_policies.cuh"

namespace nnet_gb300
{

template<int EOS, int FORM>
__global__ void __launch_bounds__(128) burnMultiKernel(MultiParams mp, HelmView hv, double* scratch, size_t stride)
{
    const size_t slot = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (mp.active[1])
    {
        typename PolicyOf<86, FORM>::type pol(scratch, stride, slot);
        if constexpr (FORM == NNET_SOLVER_MIXED) pol.refineStats = mp.bp[1].stats + 7;
        burnLoop<86, EOS>(mp.bp[1], mp.nv[1], hv, pol);
    }
    if (mp.active[2])
    {
        typename PolicyOf<87, FORM>::type pol(scratch, stride, slot);
        if constexpr (FORM == NNET_SOLVER_MIXED) pol.refineStats = mp.bp[2].stats + 7;
        burnLoop<87, EOS>(mp.bp[2], mp.nv[2], hv, pol);
    }
    if (mp.active[0])
    {
        typename PolicyOf<14, FORM>::type pol(scratch, stride, slot);
        if constexpr (FORM == NNET_SOLVER_MIXED) pol.refineStats = mp.bp[0].stats + 7;
        burnLoop<14, EOS>(mp.bp[0], mp.nv[0], hv, pol);
    }
}

template<int EOS, int FORM>
static KernelInfo multiInfo()
{
    const size_t s = std::max({PolicyOf<14, FORM>::type::perSlot(), PolicyOf<86, FORM>::type::perSlot(),
                               PolicyOf<87, FORM>::type::perSlot()});
    return {(const void*)burnMultiKernel<EOS, FORM>, s, 128, PolicyOf<86, FORM>::maxNnz};
}

KernelInfo multiKernel(int eos, int solver)
{
    if (solver == NNET_SOLVER_DENSE_FP64) return eos ? multiInfo<1, 0>() : multiInfo<0, 0>();
    if (solver == NNET_SOLVER_SPARSE_FP64) return eos ? multiInfo<1, 1>() : multiInfo<0, 1>();
    return eos ? multiInfo<1, 2>() : multiInfo<0, 2>();
}

} // namespace nnet_gb300
