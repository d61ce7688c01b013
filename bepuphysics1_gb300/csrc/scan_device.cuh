// Block-wide prefix sums shared by the island and pair kernels.
#pragma once

#include <cuda_runtime.h>

namespace bepugpu {

// Inclusive sum over the block (blockDim.x a multiple of 32, at most 1,024);
// warpSums holds 32 ints of shared memory.
__device__ __forceinline__ int BlockInclusiveSum(int v, int* warpSums) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, warps = blockDim.x >> 5;
    for (int o = 1; o < 32; o <<= 1) {
        const int u = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += u;
    }
    if (lane == 31) warpSums[warp] = v;
    __syncthreads();
    if (warp == 0) {
        int w = lane < warps ? warpSums[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            const int u = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += u;
        }
        if (lane < warps) warpSums[lane] = w;
    }
    __syncthreads();
    const int before = warp ? warpSums[warp - 1] : 0;
    __syncthreads();
    return v + before;
}

}  // namespace bepugpu
