// FP64 block reductions shared by the device-resident solvers.
#pragma once

#include <cuda_runtime.h>

namespace mmr {

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Warp reduce-scatter of NV doubles per lane (NV a power of two, <= 32): at each of the first
// log2(NV) butterfly levels a lane keeps half of its values and adds the partner's copies of
// them, so a lane ends with one value; the remaining levels are plain butterflies.  Afterwards
// lane l holds the warp sum of value l >> (5 - log2 NV).  NV - 1 + 5 - log2(NV) additions per
// lane instead of 5 NV (FP64 arithmetic is scarce on this part).
template <int NV>
__device__ __forceinline__ double warp_reduce_scatter(double (&v)[NV]) {
    static_assert(NV >= 1 && NV <= 32 && (NV & (NV - 1)) == 0, "NV must be a power of two <= 32");
    const int lane = threadIdx.x & 31;
    int c = NV;
    int o = 16;
#pragma unroll
    for (int lvl = 0; (1 << lvl) < NV; ++lvl) {
        const int h = c >> 1;
        const bool up = (lane & o) != 0;      // this lane keeps the upper half
#pragma unroll
        for (int i = 0; i < NV / 2; ++i) {
            if (i < h) {
                const double send = up ? v[i] : v[i + h];
                const double keep = up ? v[i + h] : v[i];
                v[i] = keep + __shfl_xor_sync(0xffffffffu, send, o);
            }
        }
        c = h;
        o >>= 1;
    }
    double s = v[0];
    for (; o >= 1; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    return s;
}

// Block-reduces NV doubles; NV threads atomically add them to dst[0..NV-1] (a NULL destination is
// skipped).  Power-of-two NV use the warp reduce-scatter above.
template <int NV>
__device__ __forceinline__ void block_accumulate(double (&v)[NV], double* const (&dst)[NV]) {
    __shared__ double red[NV][32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nw = blockDim.x >> 5;
    if constexpr ((NV & (NV - 1)) == 0 && NV <= 32) {
        constexpr int SHIFT = 5 - (NV >= 32 ? 5 : NV >= 16 ? 4 : NV >= 8 ? 3 : NV >= 4 ? 2 : NV >= 2 ? 1 : 0);
        const double s = warp_reduce_scatter<NV>(v);
        if ((lane & ((1 << SHIFT) - 1)) == 0) red[lane >> SHIFT][warp] = s;
        __syncthreads();
        if (threadIdx.x < NV) {
            double t = 0.0;
            for (int w = 0; w < nw; ++w) t += red[threadIdx.x][w];
            if (dst[threadIdx.x]) atomicAdd(dst[threadIdx.x], t);
        }
    } else {
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            const double s = warp_sum(v[k]);
            if (lane == 0) red[k][warp] = s;
        }
        __syncthreads();
        if (warp == 0) {
#pragma unroll
            for (int k = 0; k < NV; ++k) {
                double s = lane < nw ? red[k][lane] : 0.0;
                s = warp_sum(s);
                if (lane == 0 && dst[k]) atomicAdd(dst[k], s);
            }
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
