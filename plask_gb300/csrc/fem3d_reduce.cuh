// Deterministic grid reductions shared by the kernel files: every block writes one
// partial per value, the last block to arrive combines the partials in a fixed order.
#pragma once

#include <cfloat>

#include "fem3d_device.cuh"

namespace plgpu {

struct OpSum {
    __device__ static double init() { return 0.0; }
    __device__ static double op(double a, double b) { return a + b; }
};
struct OpMax {
    __device__ static double init() { return -DBL_MAX; }
    __device__ static double op(double a, double b) { return a > b ? a : b; }
};

__device__ __forceinline__ int linear_tid() {
    return threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
}
__device__ __forceinline__ int block_threads() { return blockDim.x * blockDim.y * blockDim.z; }
__device__ __forceinline__ int linear_bid() { return blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z); }

// Block-wide reduction of NV values; the result is valid in every thread.
template <int NV, typename Op>
__device__ __forceinline__ void block_reduce(double (&v)[NV]) {
    __shared__ double sh[NV][32];
    const int t = linear_tid(), lane = t & 31, warp = t >> 5, nw = (block_threads() + 31) >> 5;
#pragma unroll
    for (int i = 0; i < NV; ++i)
        for (int o = 16; o; o >>= 1) v[i] = Op::op(v[i], __shfl_xor_sync(0xffffffffu, v[i], o));
    if (lane == 0) {
#pragma unroll
        for (int i = 0; i < NV; ++i) sh[i][warp] = v[i];
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < NV; ++i) {
        double w = lane < nw ? sh[i][lane] : Op::init();
        for (int o = 16; o; o >>= 1) w = Op::op(w, __shfl_xor_sync(0xffffffffu, w, o));
        v[i] = w;
    }
    __syncthreads();
}

// Write this block's reduced values to partials[i * kMaxPartialBlocks + slot].
template <int NV, typename Op>
__device__ __forceinline__ void write_partial(double (&v)[NV], double* partials, int slot) {
    block_reduce<NV, Op>(v);
    if (linear_tid() == 0) {
#pragma unroll
        for (int i = 0; i < NV; ++i) partials[(size_t)i * kMaxPartialBlocks + slot] = v[i];
    }
}

// Count this block's arrival; true in the last of `expected` arriving blocks.
__device__ __forceinline__ bool arrive_last(unsigned int* counter, unsigned int expected) {
    __shared__ int last;
    __threadfence();
    __syncthreads();
    if (linear_tid() == 0) {
        unsigned int prev = atomicAdd(counter, 1u);
        last = (prev == expected - 1u);
        if (last) *counter = 0u;  // ready for the next launch
    }
    __syncthreads();
    if (last) __threadfence();
    return last != 0;
}

// Sum partial slots [0, nslots) in a fixed order (valid in every thread).  Each thread
// takes slots t, t + nt, t + 2 nt, ... in increasing order; the loads of 8 of them are
// issued before any is added, so one L2 round trip covers 8 slots.
template <int NV, typename Op>
__device__ __forceinline__ void reduce_partials(double (&v)[NV], const double* partials, int nslots) {
    const int t = linear_tid(), nt = block_threads();
#pragma unroll
    for (int i = 0; i < NV; ++i) {
        const double* src = partials + (size_t)i * kMaxPartialBlocks;
        double a = Op::init();
        for (int s0 = t; s0 < nslots; s0 += 8 * nt) {
            double buf[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                const int s = s0 + u * nt;
                buf[u] = s < nslots ? __ldcg(src + s) : Op::init();
            }
#pragma unroll
            for (int u = 0; u < 8; ++u) a = Op::op(a, buf[u]);
        }
        v[i] = a;
    }
    block_reduce<NV, Op>(v);
}

// The two helpers below keep FP64 arithmetic (a slow pipe on this GPU) to a few
// instructions per block.

// This block's partials of NV FP32 per-thread values: each warp sums its lanes in FP32 (a
// fixed butterfly), thread 0 adds the warps' sums in FP64 in warp order and writes
// partials[i * kMaxPartialBlocks + slot].
template <int NV>
__device__ __forceinline__ void write_partial_f32(float (&v)[NV], double* partials, int slot) {
    __shared__ float sh[NV][32];
    const int t = linear_tid(), lane = t & 31, warp = t >> 5, nw = (block_threads() + 31) >> 5;
#pragma unroll
    for (int i = 0; i < NV; ++i)
        for (int o = 16; o; o >>= 1) v[i] += __shfl_xor_sync(0xffffffffu, v[i], o);
    if (lane == 0) {
#pragma unroll
        for (int i = 0; i < NV; ++i) sh[i][warp] = v[i];
    }
    __syncthreads();
    if (t == 0) {
#pragma unroll
        for (int i = 0; i < NV; ++i) {
            double a = 0.0;
            for (int w = 0; w < nw; ++w) a += (double)sh[i][w];
            partials[(size_t)i * kMaxPartialBlocks + slot] = a;
        }
    }
}

// Sum of partial slots [0, nslots) of NV values, computed by warp 0 alone (lane l takes
// slots l, l + 32, ... in increasing order, then a fixed butterfly), so every block that
// calls it gets the same bits.  The result is valid in warp 0 only; `scalar` (lane 0 of
// warp 0) derives what the block needs from it, and the block synchronises before reading.
template <int NV>
__device__ __forceinline__ void warp0_reduce_partials(double (&v)[NV], const double* partials, int nslots) {
#pragma unroll
    for (int i = 0; i < NV; ++i) {
        const double* src = partials + (size_t)i * kMaxPartialBlocks;
        const int lane = threadIdx.x & 31;
        double a = 0.0;
        for (int s0 = lane; s0 < nslots; s0 += 4 * 32) {
            double buf[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int s = s0 + 32 * u;
                buf[u] = s < nslots ? __ldcg(src + s) : 0.0;
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) a += buf[u];
        }
        for (int o = 16; o; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
        v[i] = a;
    }
}

}  // namespace plgpu
