// Deterministic tile reductions shared by the device translation units (internal linkage in each): a tile of
// TILE_ROWS block rows of one system writes its partial sums, and the block that completes the last tile reduces
// every system's partials in a fixed order.
#pragma once
#include <cuda_runtime.h>

#include "rsg_impl.h"

namespace rsg {
namespace {

constexpr int kTileThreads = 192;           // 64 block rows x 3 per step

// Block reduction of ND <= MAX_DOTS values; result valid in thread 0. Every thread leaves its values in shared
// memory and warp j sums value j (a strided pass, then a shuffle tree), in a fixed order. FP64 runs at 1/64 of
// the FP32 rate on GB300: a shuffle tree in every warp would spend five FP64 adds per thread and value, this
// spends about one per 32 threads. Needs blockDim.x >= 32 * ND.
template <int ND>
__device__ __forceinline__ void block_reduce(double (&v)[MAX_DOTS], double* sh /* [ND][blockDim.x] */) {
    const int nt = blockDim.x, lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int j = 0; j < ND; ++j) sh[j * nt + threadIdx.x] = v[j];
    __syncthreads();
    if (w < ND) {
        const double* q = sh + w * nt;
        double x = 0;
        for (int i = lane; i < nt; i += 32) x += q[i];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        if (lane == 0) sh[w * nt] = x;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int j = 0; j < ND; ++j) v[j] = sh[j * nt];
    }
}

// Last-tile-done: the block that completes the last tile reduces the per-tile partials of every system in a fixed
// order into sysdot[s*MAX_DOTS + j] and returns true (in every thread of that block).
template <int ND>
__device__ bool last_tile_reduce(int ntiles, int nsys, const int* __restrict__ sysTile0, const double* part, unsigned* done,
                                 double* sysdot, double* sh) {
    __shared__ int amLast;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned ticket = atomicAdd(done, 1u);
        amLast = (ticket == unsigned(ntiles) - 1u);
    }
    __syncthreads();
    if (!amLast) return false;
    __threadfence();
    // one warp per system, the same order whatever the batch: a system's inner products do not depend on the
    // systems solved with it (lane-strided partial sums over its tiles, then a shuffle tree)
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int s = w; s < nsys; s += nw) {
        double v[MAX_DOTS] = {0, 0, 0, 0};
        const int t0 = sysTile0[s], t1 = sysTile0[s + 1];
        for (int t = t0 + lane; t < t1; t += 32)
#pragma unroll
            for (int j = 0; j < ND; ++j) v[j] += ((volatile const double*)part)[size_t(t) * MAX_DOTS + j];
#pragma unroll
        for (int j = 0; j < ND; ++j) {
            double x = v[j];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
            if (lane == 0) sysdot[size_t(s) * MAX_DOTS + j] = x;
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) *done = 0u;
    __threadfence();
    return true;
}

}  // namespace
}  // namespace rsg
