// reduce.cuh - deterministic block and grid reductions used by the kernels.
//
// Grid-wide sums use the "last block finishes" pattern: every block writes
// its partial to a slot indexed by blockIdx, the block that takes the final
// ticket sums the slots in a fixed order and resets the ticket counter.  The
// result therefore does not depend on block scheduling.
#pragma once

#include <cuda_runtime.h>

namespace iptgb {

// Block-wide sum of two doubles; the result is valid in thread 0.  Must be
// called by every thread of the block (it synchronises).
__device__ __forceinline__ double2 block_sum2(double a, double b)
{
    __shared__ double sa[32];
    __shared__ double sb[32];
    for (int off = 16; off > 0; off >>= 1) {
        a += __shfl_down_sync(0xffffffffu, a, off);
        b += __shfl_down_sync(0xffffffffu, b, off);
    }
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) {
        sa[warp] = a;
        sb[warp] = b;
    }
    __syncthreads();
    const int nw = (blockDim.x + 31) >> 5;
    if (warp == 0) {
        a = lane < nw ? sa[lane] : 0.0;
        b = lane < nw ? sb[lane] : 0.0;
        for (int off = 16; off > 0; off >>= 1) {
            a += __shfl_down_sync(0xffffffffu, a, off);
            b += __shfl_down_sync(0xffffffffu, b, off);
        }
    }
    __syncthreads();
    return make_double2(a, b);
}

// Warp-wide sum; every lane receives the total.
__device__ __forceinline__ double warp_sum(double v)
{
    for (int off = 16; off > 0; off >>= 1) {
        v += __shfl_xor_sync(0xffffffffu, v, off);
    }
    return v;
}

// Deterministic grid-wide finish of per-block (a, b) sums.  `mine` must be
// valid in thread 0.  The last block writes out[0] = sqrt(sum a) and
// out[1] = sqrt(sum b) and re-arms *counter for the next launch.
__device__ __forceinline__ void grid_finish_norms2(double2 mine, double2 *partials,
                                                   unsigned int *counter, double *out)
{
    __shared__ bool last;
    if (threadIdx.x == 0) {
        partials[blockIdx.x] = mine;
        __threadfence();
        const unsigned int done = atomicAdd(counter, 1u);
        last = (done == gridDim.x - 1);
    }
    __syncthreads();
    if (!last) {
        return;
    }
    __threadfence();
    double a = 0.0, b = 0.0;
    for (unsigned int i = threadIdx.x; i < gridDim.x; i += blockDim.x) {
        const double2 p = __ldcg(&partials[i]);
        a += p.x;
        b += p.y;
    }
    const double2 t = block_sum2(a, b);
    if (threadIdx.x == 0) {
        out[0] = sqrt(t.x);
        out[1] = sqrt(t.y);
        *counter = 0u;
    }
}

}  // namespace iptgb
