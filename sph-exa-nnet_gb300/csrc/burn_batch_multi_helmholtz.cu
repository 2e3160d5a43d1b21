// One launch over net86, net87 and net14 sub-batches with the Helmholtz EOS, batched-warp layout
// (templates in burn_batch.cuh).
#include "burn_batch.cuh"

namespace nnet_gb300
{
KernelInfo batchMultiKernel1(int mixed, bool post) { return pickBatchMulti<1>(mixed, post); }
} // namespace nnet_gb300
