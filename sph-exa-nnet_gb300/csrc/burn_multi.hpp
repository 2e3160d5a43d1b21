// One persistent launch over sub-batches of different networks (burn_multi.cu).
#pragma once

#include "common.cuh"
#include "launch.hpp"

namespace nnet_gb300
{

// index 0: net14, 1: net86, 2: net87
struct MultiParams
{
    BurnParams bp[3];
    NetView    nv[3];
    int        active[3];
};

KernelInfo multiKernel(int eos, int solver);

} // namespace nnet_gb300
