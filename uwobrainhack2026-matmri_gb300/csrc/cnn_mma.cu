// Tensor-core inference path of the preconditioner network (FP16 activations,
// FP16 copies of the FP32 weights in the hidden layers, FP32 accumulation).
//
// Activations are FP16 rather than BF16 here: the network is used as a
// preconditioner inside flexible CG, where the operator has to be (nearly) the
// same for every residual, and BF16's 8-bit mantissa makes it noisy enough to
// cost up to twice the iterations of FP32 activations on held-out cases; FP16's
// 11 bits do not.  Inputs are normalised to unit RMS, so the FP16 range holds.
// Rounding the weights, by contrast, only changes which fixed operator is
// applied (by ~1e-4), which CG does not notice.
//
// Hidden 32 -> 32 layers: implicit GEMM [pixels x 288] x [288 x 32] with K
// ordered tap-major (k = tap * 32 + ci), so one 16-wide K step is 16 channels
// of one tap and the A fragments are 32-bit loads of channel pairs from an
// NHWC tile in shared memory.  CTA: 256 threads, 16 x 16 output pixels; warp
// w computes image rows 2w and 2w + 1 of the tile (two m16 tiles) x all 32
// output channels (four n8 tiles): 8 mma.sync per K step, 18 K steps.
// First (2 -> 32) and last (32 -> 2) layers: one pixel per thread, weights
// broadcast from shared memory, taps read through L1.
#include <algorithm>

#include <cuda_fp16.h>

#include "cnn.cuh"

namespace mmr {

constexpr int MT = 16;                  // tile side
constexpr int MH = MT + 2;              // with halo
constexpr int PIX_STRIDE = 40;          // halves per pixel in shared (32 + 8 pad: conflict-free A loads)
constexpr int KDIM = 9 * CNN_HIDDEN;    // 288
constexpr int KSTRIDE = KDIM + 8;       // 296 halves per output channel (conflict-free B loads)
constexpr size_t MMA_WEIGHTS = (size_t)CNN_HIDDEN * KSTRIDE;   // halves per hidden layer
constexpr size_t MMA_SMEM = (size_t)MH * MH * PIX_STRIDE * 2 + MMA_WEIGHTS * 2;

__device__ __forceinline__ void mma_f16(float (&c)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3,
                                        uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

__global__ void __launch_bounds__(256) conv3x3_mma_kernel(const __half* __restrict__ in, __half* __restrict__ out,
                                                          const __half* __restrict__ wmma, int X, int Y, int relu) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __half* s_in = reinterpret_cast<__half*>(smem_raw);
    __half* s_w = s_in + MH * MH * PIX_STRIDE;       // [32][KSTRIDE]
    const int b = blockIdx.z;
    const int x0 = blockIdx.x * MT, y0 = blockIdx.y * MT;
    const long long P = (long long)X * Y;
    // weights, already padded to KSTRIDE
    {
        const uint4* src = reinterpret_cast<const uint4*>(wmma);
        uint4* dst = reinterpret_cast<uint4*>(s_w);
        constexpr int NV = (int)(MMA_WEIGHTS * 2 / 16);
        for (int i = threadIdx.x; i < NV; i += 256) dst[i] = src[i];
    }
    // input tile with halo: 4 x 16 B per pixel
    for (int i = threadIdx.x; i < MH * MH * 4; i += 256) {
        const int q = i & 3, pix = i >> 2, hx = pix % MH, hy = pix / MH;
        const int gx = x0 + hx - 1, gy = y0 + hy - 1;
        uint4 v = make_uint4(0, 0, 0, 0);
        if (gx >= 0 && gx < X && gy >= 0 && gy < Y)
            v = reinterpret_cast<const uint4*>(in + ((long long)b * P + (long long)gy * X + gx) * CNN_HIDDEN)[q];
        *reinterpret_cast<uint4*>(s_in + pix * PIX_STRIDE + q * 8) = v;
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int gid = lane >> 2, tig = lane & 3;
    float acc[2][4][4];
#pragma unroll
    for (int m = 0; m < 2; ++m)
#pragma unroll
        for (int n = 0; n < 4; ++n)
#pragma unroll
            for (int j = 0; j < 4; ++j) acc[m][n][j] = 0.f;
#pragma unroll 2
    for (int ks = 0; ks < 18; ++ks) {
        const int tap = ks >> 1, c0 = (ks & 1) * 16;
        const int ky = tap / 3, kx = tap % 3;
        uint32_t a[2][4];
#pragma unroll
        for (int m = 0; m < 2; ++m) {
            const int yl = warp * 2 + m + ky;
            const __half* r0 = s_in + (yl * MH + gid + kx) * PIX_STRIDE + c0 + 2 * tig;
            const __half* r1 = r0 + 8 * PIX_STRIDE;
            a[m][0] = *reinterpret_cast<const uint32_t*>(r0);
            a[m][1] = *reinterpret_cast<const uint32_t*>(r1);
            a[m][2] = *reinterpret_cast<const uint32_t*>(r0 + 8);
            a[m][3] = *reinterpret_cast<const uint32_t*>(r1 + 8);
        }
        const int k0 = ks * 16 + 2 * tig;
#pragma unroll
        for (int n = 0; n < 4; ++n) {
            const __half* wr = s_w + (n * 8 + gid) * KSTRIDE + k0;
            const uint32_t b0 = *reinterpret_cast<const uint32_t*>(wr);
            const uint32_t b1 = *reinterpret_cast<const uint32_t*>(wr + 8);
#pragma unroll
            for (int m = 0; m < 2; ++m) mma_f16(acc[m][n], a[m][0], a[m][1], a[m][2], a[m][3], b0, b1);
        }
    }
    // epilogue: ReLU (unless the network is linear), FP16, NHWC
    auto act = [relu](float v) { return relu ? fmaxf(v, 0.f) : v; };
#pragma unroll
    for (int m = 0; m < 2; ++m) {
        const int y = y0 + warp * 2 + m;
        if (y >= Y) continue;
#pragma unroll
        for (int hh = 0; hh < 2; ++hh) {
            const int x = x0 + gid + 8 * hh;
            if (x >= X) continue;
            __half* o = out + ((long long)b * P + (long long)y * X + x) * CNN_HIDDEN;
#pragma unroll
            for (int n = 0; n < 4; ++n) {
                const __half2 v = __floats2half2_rn(act(acc[m][n][2 * hh]), act(acc[m][n][2 * hh + 1]));
                *reinterpret_cast<__half2*>(o + n * 8 + 2 * tig) = v;
            }
        }
    }
}

// First layer: a1[p][co] = act(sum_{ci,t} w[(ci*9+t)*32+co] * (r/s)[p+off(t)][ci]), r complex.
__global__ void __launch_bounds__(256) conv_first_f16_kernel(const float2* __restrict__ r, __half* __restrict__ out,
                                                             const float* __restrict__ wpk,
                                                             const double* __restrict__ sumsq, int X, int Y,
                                                             int relu) {
    __shared__ float4 s_w[2 * 9 * CNN_HIDDEN / 4];
    for (int i = threadIdx.x; i < 2 * 9 * CNN_HIDDEN / 4; i += blockDim.x)
        s_w[i] = reinterpret_cast<const float4*>(wpk)[i];
    __syncthreads();
    const int b = blockIdx.y;
    const long long P = (long long)X * Y;
    const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P) return;
    const double sd = sqrt(sumsq[b] / (double)P);
    const float inv_s = sd > 0 ? (float)(1.0 / sd) : 0.f;
    const int x = (int)(p % X), y = (int)(p / X);
    float acc[CNN_HIDDEN];
#pragma unroll
    for (int c = 0; c < CNN_HIDDEN; ++c) acc[c] = 0.f;
#pragma unroll
    for (int t = 0; t < 9; ++t) {
        const int nx = x + t % 3 - 1, ny = y + t / 3 - 1;
        if (nx < 0 || nx >= X || ny < 0 || ny >= Y) continue;
        const float2 rv = r[(long long)b * P + (long long)ny * X + nx];
        const float re = rv.x * inv_s, im = rv.y * inv_s;
#pragma unroll
        for (int j = 0; j < CNN_HIDDEN / 4; ++j) {
            const float4 w0 = s_w[(0 * 9 + t) * (CNN_HIDDEN / 4) + j];
            const float4 w1 = s_w[(1 * 9 + t) * (CNN_HIDDEN / 4) + j];
            acc[4 * j] += w0.x * re + w1.x * im;
            acc[4 * j + 1] += w0.y * re + w1.y * im;
            acc[4 * j + 2] += w0.z * re + w1.z * im;
            acc[4 * j + 3] += w0.w * re + w1.w * im;
        }
    }
    uint4* o = reinterpret_cast<uint4*>(out + ((long long)b * P + p) * CNN_HIDDEN);
#pragma unroll
    for (int q = 0; q < CNN_HIDDEN / 8; ++q) {
        __half2 h[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            float v0 = acc[8 * q + 2 * k], v1 = acc[8 * q + 2 * k + 1];
            if (relu) {
                v0 = fmaxf(v0, 0.f);
                v1 = fmaxf(v1, 0.f);
            }
            h[k] = __floats2half2_rn(v0, v1);
        }
        o[q] = *reinterpret_cast<const uint4*>(h);
    }
}

// Last layer: z[p] = s * sum_{ci,t} w[(ci*9+t)*2+co] a[p+off(t)][ci] + skip * r[p]  (complex out)
__global__ void __launch_bounds__(256) conv_last_f16_kernel(const __half* __restrict__ in, float2* __restrict__ z,
                                                            const float* __restrict__ wpk,
                                                            const float2* __restrict__ r,
                                                            const double* __restrict__ sumsq,
                                                            const float* __restrict__ skip, int X, int Y) {
    __shared__ float2 s_w[CNN_HIDDEN * 9];
    for (int i = threadIdx.x; i < CNN_HIDDEN * 9; i += blockDim.x) s_w[i] = reinterpret_cast<const float2*>(wpk)[i];
    __syncthreads();
    const int b = blockIdx.y;
    const long long P = (long long)X * Y;
    const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P) return;
    const float s = (float)sqrt(sumsq[b] / (double)P);
    const int x = (int)(p % X), y = (int)(p / X);
    float a0 = 0.f, a1 = 0.f;
#pragma unroll
    for (int t = 0; t < 9; ++t) {
        const int nx = x + t % 3 - 1, ny = y + t / 3 - 1;
        if (nx < 0 || nx >= X || ny < 0 || ny >= Y) continue;
        const uint4* src = reinterpret_cast<const uint4*>(in + ((long long)b * P + (long long)ny * X + nx) * CNN_HIDDEN);
#pragma unroll
        for (int q = 0; q < CNN_HIDDEN / 8; ++q) {
            const uint4 u = src[q];
            const __half2* h = reinterpret_cast<const __half2*>(&u);
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const float2 v = __half22float2(h[k]);
                const int ci = 8 * q + 2 * k;
                const float2 w0 = s_w[ci * 9 + t], w1 = s_w[(ci + 1) * 9 + t];
                a0 += w0.x * v.x + w1.x * v.y;
                a1 += w0.y * v.x + w1.y * v.y;
            }
        }
    }
    const float2 rv = r[(long long)b * P + p];
    const float sk = *skip;
    z[(long long)b * P + p] = make_float2(s * a0 + sk * rv.x, s * a1 + sk * rv.y);
}

// wmma[l][n][k] (k = tap * 32 + ci, padded to KSTRIDE) for hidden layers l = 1 .. L-2
__global__ void cnn_pack_mma_kernel(const float* __restrict__ W, __half* __restrict__ dst) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= CNN_HIDDEN * KSTRIDE) return;
    const int n = i / KSTRIDE, k = i % KSTRIDE;
    float w = 0.f;
    if (k < KDIM) {
        const int tap = k / CNN_HIDDEN, ci = k % CNN_HIDDEN;
        w = W[(n * CNN_HIDDEN + ci) * 9 + tap];
    }
    dst[i] = __float2half_rn(w);
}

void cnn_pack_mma(CnnNet& n, cudaStream_t st) {
    const size_t per = MMA_WEIGHTS;
    n.wmma.ensure(per * 2 * std::max(1, n.L - 2));
    for (int l = 1; l < n.L - 1; ++l) {
        cnn_pack_mma_kernel<<<(unsigned)cdiv(CNN_HIDDEN * KSTRIDE, 256), 256, 0, st>>>(
            n.theta.as<float>() + n.woff[l], n.wmma.as<__half>() + (size_t)(l - 1) * per);
        check_launch("cnn_pack_mma");
    }
}

// The whole network on the tensor path: z = net(r) for `batch` images of nx x ny.
void cnn_forward_tensor(CnnNet& n, const float2* r, float2* z, int nx, int ny, int batch, bool relu,
                        cudaStream_t st) {
    static bool attr = false;
    if (!attr) {
        MMR_CUDA(cudaFuncSetAttribute(conv3x3_mma_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)MMA_SMEM));
        attr = true;
    }
    const long long P = (long long)nx * ny;
    const size_t per_act = (size_t)P * batch * CNN_HIDDEN;
    __half* acts = n.act.as<__half>();
    const float* wpk = n.wpk.as<float>();
    const dim3 pg((unsigned)cdiv(P, 256), (unsigned)batch);
    conv_first_f16_kernel<<<pg, 256, 0, st>>>(r, acts, wpk + n.woff[0], n.sumsq.as<double>(), nx, ny, relu ? 1 : 0);
    check_launch("conv_first_f16");
    const size_t per_w = MMA_WEIGHTS;
    const dim3 grid((unsigned)cdiv(nx, MT), (unsigned)cdiv(ny, MT), (unsigned)batch);
    int cur = 0;
    for (int l = 1; l < n.L - 1; ++l) {
        conv3x3_mma_kernel<<<grid, 256, MMA_SMEM, st>>>(acts + cur * per_act, acts + (cur ^ 1) * per_act,
                                                       n.wmma.as<__half>() + (size_t)(l - 1) * per_w, nx, ny,
                                                       relu ? 1 : 0);
        check_launch("conv3x3_mma");
        cur ^= 1;
    }
    conv_last_f16_kernel<<<pg, 256, 0, st>>>(acts + cur * per_act, z, wpk + n.woff[n.L - 1], r, n.sumsq.as<double>(),
                                             n.theta.as<float>() + n.nparam - 1, nx, ny);
    check_launch("conv_last_f16");
}

}  // namespace mmr
