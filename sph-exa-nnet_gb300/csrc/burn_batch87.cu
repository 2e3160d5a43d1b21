// Batched-warp burn kernels of net87 (templates in burn_batch.cuh; one translation unit per
// network so that the library's build compiles them in parallel).
#include "burn_batch.cuh"

namespace nnet_gb300
{
KernelInfo batchKernel87(int eos, int mixed, bool post) { return pickBatchNet<87>(eos, mixed, post); }
} // namespace nnet_gb300
