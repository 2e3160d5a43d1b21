// nnet_cost_order: a work-queue visiting order with the costliest particles first.
//
// Per-particle Newton-iteration counts of a burn differ by more than 100x (c2: median 5, the
// top 1 % above 850).  Given a per-particle cost (for example the previous burn's
// `iterations`), this builds a permutation that hands out the particles in decreasing order
// of floor(log2(cost)): a counting sort over 32 buckets (histogram, exclusive scan, scatter),
// three small kernels on the caller's stream.  The order within a bucket is whatever the
// scatter's atomics give; burn results do not depend on it.
#include <cuda_runtime.h>

#include "context.hpp"

namespace nnet_gb300
{
namespace
{
constexpr int kBuckets = 32;

// bucket of a cost: 0 for the largest costs (2^30 and above), 31 for costs <= 1
__device__ __forceinline__ int bucketOf(int32_t c)
{
    const unsigned u = c > 1 ? (unsigned)c : 1u;
    return __clz(u) - 1; // 31 - floor(log2 u), in [0, 31]
}

__global__ void histogramKernel(const int32_t* cost, size_t P, unsigned long long* count)
{
    __shared__ unsigned int h[kBuckets];
    if (threadIdx.x < kBuckets) h[threadIdx.x] = 0;
    __syncthreads();
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < P; i += (size_t)gridDim.x * blockDim.x)
        atomicAdd(h + bucketOf(cost[i]), 1u);
    __syncthreads();
    if (threadIdx.x < kBuckets && h[threadIdx.x]) atomicAdd(count + threadIdx.x, (unsigned long long)h[threadIdx.x]);
}

// exclusive scan of the bucket counts into the scatter cursors (one warp)
__global__ void scanKernel(const unsigned long long* count, unsigned long long* cursor)
{
    const int          l = threadIdx.x;
    unsigned long long v = count[l], x = v;
    for (int o = 1; o < 32; o <<= 1)
    {
        const unsigned long long y = __shfl_up_sync(0xffffffffu, x, o);
        if (l >= o) x += y;
    }
    cursor[l] = x - v;
}

__global__ void scatterKernel(const int32_t* cost, size_t P, unsigned long long* cursor, uint32_t* order)
{
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < P; i += (size_t)gridDim.x * blockDim.x)
        order[atomicAdd(cursor + bucketOf(cost[i]), 1ull)] = (uint32_t)i;
}
} // namespace
} // namespace nnet_gb300

using namespace nnet_gb300;

extern "C" int nnet_cost_order(nnet_handle h, size_t num_particles, const int32_t* cost, uint32_t* order,
                               void* stream)
{
    if (!h || (num_particles && (!cost || !order))) return setError(NNET_ERR_INVALID, "null argument");
    if (num_particles > 0xffffffffull) return setError(NNET_ERR_TOO_LARGE, "order indices are 32-bit");
    if (num_particles == 0) return NNET_SUCCESS;
    if (cudaSetDevice(h->device) != cudaSuccess) return setError(NNET_ERR_CUDA, "cudaSetDevice failed");
    cudaStream_t st = (cudaStream_t)stream;
    if (!h->orderCounters && cudaMalloc(&h->orderCounters, 2 * kBuckets * sizeof(unsigned long long)) != cudaSuccess)
        return setError(NNET_ERR_CUDA, "cudaMalloc of the order counters failed");
    unsigned long long *count = h->orderCounters, *cursor = count + kBuckets;
    const int    block  = 256;
    const size_t blocks = std::min<size_t>((num_particles + block - 1) / block, (size_t)h->numSMs * 8);
    if (cudaMemsetAsync(count, 0, kBuckets * sizeof(unsigned long long), st) != cudaSuccess)
        return setError(NNET_ERR_CUDA, "cudaMemsetAsync failed");
    histogramKernel<<<(unsigned)blocks, block, 0, st>>>(cost, num_particles, count);
    scanKernel<<<1, kBuckets, 0, st>>>(count, cursor);
    scatterKernel<<<(unsigned)blocks, block, 0, st>>>(cost, num_particles, cursor, order);
    if (cudaGetLastError() != cudaSuccess) return setError(NNET_ERR_CUDA, "nnet_cost_order launch failed");
    return NNET_SUCCESS;
}
