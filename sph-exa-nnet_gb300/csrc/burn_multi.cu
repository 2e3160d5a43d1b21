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

// Element index of the FP32 region shared by the three networks' slots (mixed form): above
// the FP64 rows of the largest network, so that no slot's FP32 rows overlap the FP64 rows of
// a slot running another network (see SparsePolicy's constructor).
template<int FORM>
constexpr size_t multiFloatBase()
{
    if constexpr (FORM == NNET_SOLVER_DENSE_FP64)
        return 0;
    else
        return std::max({SparsePolicy<14, true>::doubleElems(), SparsePolicy<86, true>::doubleElems(),
                         SparsePolicy<87, true>::doubleElems()});
}

template<int NET, int FORM>
__device__ __forceinline__ typename PolicyOf<NET, FORM>::type multiPolicy(const BurnParams& bp, double* scratch,
                                                                       size_t stride, size_t slot)
{
    if constexpr (FORM == NNET_SOLVER_DENSE_FP64)
        return typename PolicyOf<NET, FORM>::type(scratch, stride, slot);
    else
    {
        typename PolicyOf<NET, FORM>::type pol(scratch, stride, slot, multiFloatBase<FORM>());
        if constexpr (FORM == NNET_SOLVER_MIXED) pol.refineStats = bp.stats + kStatRefine;
        return pol;
    }
}

template<int EOS, int FORM>
__global__ void __launch_bounds__(128) burnMultiKernel(MultiParams mp, HelmView hv, double* scratch, size_t stride)
{
    const size_t slot = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (mp.active[1])
    {
        auto pol = multiPolicy<86, FORM>(mp.bp[1], scratch, stride, slot);
        burnLoop<86, EOS>(mp.bp[1], mp.nv[1], hv, pol);
    }
    if (mp.active[2])
    {
        auto pol = multiPolicy<87, FORM>(mp.bp[2], scratch, stride, slot);
        burnLoop<87, EOS>(mp.bp[2], mp.nv[2], hv, pol);
    }
    if (mp.active[0])
    {
        auto pol = multiPolicy<14, FORM>(mp.bp[0], scratch, stride, slot);
        burnLoop<14, EOS>(mp.bp[0], mp.nv[0], hv, pol);
    }
}

template<int EOS, int FORM>
static KernelInfo multiInfo()
{
    size_t s = std::max({PolicyOf<14, FORM>::type::perSlot(), PolicyOf<86, FORM>::type::perSlot(),
                         PolicyOf<87, FORM>::type::perSlot()});
    if constexpr (FORM == NNET_SOLVER_MIXED)
        s = multiFloatBase<FORM>() + std::max({SparsePolicy<14, true>::floatElems(), SparsePolicy<86, true>::floatElems(),
                                               SparsePolicy<87, true>::floatElems()});
    return {(const void*)burnMultiKernel<EOS, FORM>, s, 128, PolicyOf<86, FORM>::maxNnz};
}

KernelInfo multiKernel(int eos, int solver)
{
    if (solver == NNET_SOLVER_DENSE_FP64) return eos ? multiInfo<1, 0>() : multiInfo<0, 0>();
    if (solver == NNET_SOLVER_SPARSE_FP64) return eos ? multiInfo<1, 1>() : multiInfo<0, 1>();
    return eos ? multiInfo<1, 2>() : multiInfo<0, 2>();
}

} // namespace nnet_gb300
