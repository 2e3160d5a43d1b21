// One launch over net86, net87 and net14 sub-batches with the ideal-gas EOS, batched-warp layout
// (templates in burn_batch.cuh).
#include "burn_batch.cuh"

namespace nnet_gb300
{
KernelInfo batchMultiKernel0(int mixed, bool post) { return pickBatchMulti<0>(mixed, post); }
} // namespace nnet_gb300
