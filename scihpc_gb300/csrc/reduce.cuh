// reduce.cuh -- deterministic block reductions.
//
// Every reduction in this library runs in a fixed order (per-thread contiguous chunks,
// then a fixed tree inside the block, then a fixed tree over block partials), so results
// are bit-reproducible from run to run on the same launch geometry.
#pragma once

#include "common.cuh"

namespace scihpc {

struct SumOp {
    __device__ static double id() { return 0.0; }
    __device__ static double op(double a, double b) { return a + b; }
};
struct MaxOp {
    __device__ static double id() { return 0.0; }   // reductions here are over |x| >= 0
    __device__ static double op(double a, double b) { return fmax(a, b); }
};

// Block-wide ordered tree reduction of one value per thread (blockDim.x a power of two,
// at most 1024).  Thread 0 gets the result.
template <class Op>
__device__ double block_reduce(double v, double *sh) {
    const int t = threadIdx.x;
    sh[t] = v;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (t < w) sh[t] = Op::op(sh[t], sh[t + w]);
        __syncthreads();
    }
    return sh[0];
}

// Final pass over `count` block partials by one block of 1024 threads, same fixed order.
template <class Op>
__global__ void finish_reduce(const double *__restrict__ partial, int count, double *__restrict__ out) {
    __shared__ double sh[1024];
    double v = Op::id();
    const int per = (count + blockDim.x - 1) / blockDim.x;
    const int b = threadIdx.x * per;
    for (int q = b; q < b + per && q < count; ++q) v = Op::op(v, partial[q]);
    v = block_reduce<Op>(v, sh);
    if (threadIdx.x == 0) *out = v;
}

constexpr int RED_THREADS = 256;
constexpr int RED_MAX_BLOCKS = 1024;

inline int red_blocks(long long n) {
    long long b = (n + RED_THREADS * 2 - 1) / (RED_THREADS * 2);   // short chains: these grids are small
    if (b < 1) b = 1;
    if (b > RED_MAX_BLOCKS) b = RED_MAX_BLOCKS;
    return int(b);
}

}  // namespace scihpc
