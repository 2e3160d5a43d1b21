// Sparse and mixed-precision forms (not yet built).
#include "launch.hpp"

namespace nnet_gb300
{
KernelInfo sparseKernel(int, int, int) { return {nullptr, 0, 0}; }
} // namespace nnet_gb300
