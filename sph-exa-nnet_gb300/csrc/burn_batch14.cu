// Batched-warp burn kernels of net14 (templates in burn_batch.cuh; one translation unit per
// network so that the library's build compiles them in parallel).
#include "burn_batch.cuh"

namespace nnet_gb300
{
KernelInfo batchKernel14(int eos, int mixed, bool post) { return pickBatchNet<14>(eos, mixed, post); }
} // namespace nnet_gb300
