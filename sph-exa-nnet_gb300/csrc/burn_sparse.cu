// Sparse FP64 and mixed-precision forms (SparsePolicy in burn_policies.cuh), one thread
// per particle.
#include "burn_policies.cuh"
#include "launch.hpp"

namespace nnet_gb300
{

template<int NET, int EOS, bool MIXED>
__global__ void __launch_bounds__(128) burnSparseKernel(BurnParams bp, NetView nv, HelmView hv, double* scratch,
                                                        size_t stride)
{
    const size_t              slot = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    SparsePolicy<NET, MIXED> pol(scratch, stride, slot);
    pol.refineStats = bp.stats + kStatRefine;
    burnLoop<NET, EOS>(bp, nv, hv, pol);
}

template<int NET, int EOS, bool MIXED>
static KernelInfo sparseInfo()
{
    return {(const void*)burnSparseKernel<NET, EOS, MIXED>, SparsePolicy<NET, MIXED>::perSlot(), 128,
            SparsePolicy<NET, MIXED>::MAXNNZ};
}

template<bool MIXED>
static KernelInfo pick(int net, int eos)
{
    if (net == 14) return eos ? sparseInfo<14, 1, MIXED>() : sparseInfo<14, 0, MIXED>();
    if (net == 86) return eos ? sparseInfo<86, 1, MIXED>() : sparseInfo<86, 0, MIXED>();
    return eos ? sparseInfo<87, 1, MIXED>() : sparseInfo<87, 0, MIXED>();
}

KernelInfo sparseKernel(int net, int eos, int mixed) { return mixed ? pick<true>(net, eos) : pick<false>(net, eos); }

} // namespace nnet_gb300
