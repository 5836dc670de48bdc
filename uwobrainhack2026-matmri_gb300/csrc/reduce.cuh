// FP64 block reductions shared by the device-resident solvers.
#pragma once

#include <cuda_runtime.h>

namespace mmr {

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Block-reduces NV doubles; thread 0 atomically adds them to dst[0..NV-1]
// (a NULL destination is skipped).
template <int NV>
__device__ __forceinline__ void block_accumulate(double (&v)[NV], double* const (&dst)[NV]) {
    __shared__ double red[NV][32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        const double s = warp_sum(v[k]);
        if (lane == 0) red[k][warp] = s;
    }
    __syncthreads();
    if (warp == 0) {
        const int nw = blockDim.x >> 5;
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            double s = lane < nw ? red[k][lane] : 0.0;
            s = warp_sum(s);
            if (lane == 0 && dst[k]) atomicAdd(dst[k], s);
        }
    }
}

// True in exactly one thread: thread 0 of the last block to arrive at the
// counter (which the caller resets for the next use).
__device__ __forceinline__ bool last_block_of(unsigned int* counter) {
    __shared__ bool last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(counter, 1u) == gridDim.x - 1;
    __syncthreads();
    if (last && threadIdx.x == 0) {
        __threadfence();
        return true;
    }
    return false;
}

// Copies a device state struct (a whole number of 8-byte words, updated by other
// blocks' atomics) into registers with independent L2 loads, and back.  For the
// one thread that finalises an iteration: one round trip instead of one per field.
template <class S>
__device__ __forceinline__ void state_copy_in(S& s, const S* g) {
    static_assert(sizeof(S) % 8 == 0, "state must be a whole number of 8-byte words");
    const unsigned long long* src = reinterpret_cast<const unsigned long long*>(g);
    unsigned long long* dst = reinterpret_cast<unsigned long long*>(&s);
#pragma unroll
    for (int i = 0; i < (int)(sizeof(S) / 8); ++i) dst[i] = __ldcg(src + i);
}

template <class S>
__device__ __forceinline__ void state_copy_out(S* g, const S& s) {
    unsigned long long* dst = reinterpret_cast<unsigned long long*>(g);
    const unsigned long long* src = reinterpret_cast<const unsigned long long*>(&s);
#pragma unroll
    for (int i = 0; i < (int)(sizeof(S) / 8); ++i) __stcg(dst + i, src[i]);
    __threadfence();
}

}  // namespace mmr
