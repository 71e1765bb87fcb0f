// Deterministic warp / block reductions (fixed shuffle trees, no atomics on results).
#pragma once

#include <cuda_runtime.h>

namespace lbm {

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Block sum of N doubles; thread 0 writes out[0..N-1].  blockDim.x: multiple of 32, <= 1024.
template <int N>
__device__ __forceinline__ void block_sum(double (&v)[N], double *out) {
    __shared__ double sm[N][32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < N; ++k) v[k] = warp_sum_d(v[k]);
    if (lane == 0) {
#pragma unroll
        for (int k = 0; k < N; ++k) sm[k][wid] = v[k];
    }
    __syncthreads();
    if (wid == 0) {
#pragma unroll
        for (int k = 0; k < N; ++k) {
            double t = lane < nw ? sm[k][lane] : 0.0;
            t = warp_sum_d(t);
            if (lane == 0) out[k] = t;
        }
    }
}

}  // namespace lbm
