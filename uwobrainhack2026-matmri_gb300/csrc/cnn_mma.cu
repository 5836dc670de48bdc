// Tensor-core forward of the hidden 32 -> 32 layers of the preconditioner
// network (BF16 activations, FP32 weights as a BF16 hi + lo pair, FP32
// accumulation): an implicit GEMM [pixels x 288] x [288 x 32] per layer with
// K ordered tap-major (k = tap * 32 + ci), so one 16-wide K step is 16
// channels of one tap and the A fragments are 32-bit loads of channel pairs
// from an NHWC tile in shared memory.
//
// CTA: 256 threads, 16 x 16 output pixels; warp w computes image rows 2w and
// 2w + 1 of the tile (two m16 tiles) x all 32 output channels (four n8
// tiles), i.e. 16 mma.sync per K step over 18 K steps, twice (hi, lo).
#include <algorithm>

#include "cnn.cuh"

namespace mmr {

constexpr int MT = 16;                  // tile side
constexpr int MH = MT + 2;              // with halo
constexpr int PIX_STRIDE = 40;          // bf16 per pixel in shared (32 + 8 pad: conflict-free A loads)
constexpr int KDIM = 9 * CNN_HIDDEN;    // 288
constexpr int KSTRIDE = KDIM + 8;       // 296 bf16 per output channel (conflict-free B loads)
constexpr size_t MMA_SMEM = (size_t)MH * MH * PIX_STRIDE * 2 + (size_t)2 * CNN_HIDDEN * KSTRIDE * 2;

__device__ __forceinline__ void mma_bf16(float (&c)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3,
                                         uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

__global__ void __launch_bounds__(256) conv3x3_mma_kernel(const __nv_bfloat16* __restrict__ in,
                                                          __nv_bfloat16* __restrict__ out,
                                                          const __nv_bfloat16* __restrict__ wmma, int X, int Y,
                                                          int relu) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __nv_bfloat16* s_in = reinterpret_cast<__nv_bfloat16*>(smem_raw);
    __nv_bfloat16* s_w = s_in + MH * MH * PIX_STRIDE;       // [2][32][KSTRIDE]
    const int b = blockIdx.z;
    const int x0 = blockIdx.x * MT, y0 = blockIdx.y * MT;
    const long long P = (long long)X * Y;
    // weights (hi, lo), already padded to KSTRIDE
    {
        const uint4* src = reinterpret_cast<const uint4*>(wmma);
        uint4* dst = reinterpret_cast<uint4*>(s_w);
        constexpr int NV = 2 * CNN_HIDDEN * KSTRIDE * 2 / 16;
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
            const __nv_bfloat16* r0 = s_in + (yl * MH + gid + kx) * PIX_STRIDE + c0 + 2 * tig;
            const __nv_bfloat16* r1 = r0 + 8 * PIX_STRIDE;
            a[m][0] = *reinterpret_cast<const uint32_t*>(r0);
            a[m][1] = *reinterpret_cast<const uint32_t*>(r1);
            a[m][2] = *reinterpret_cast<const uint32_t*>(r0 + 8);
            a[m][3] = *reinterpret_cast<const uint32_t*>(r1 + 8);
        }
        const int k0 = ks * 16 + 2 * tig;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
#pragma unroll
            for (int n = 0; n < 4; ++n) {
                const __nv_bfloat16* wr = s_w + (h * CNN_HIDDEN + n * 8 + gid) * KSTRIDE + k0;
                const uint32_t b0 = *reinterpret_cast<const uint32_t*>(wr);
                const uint32_t b1 = *reinterpret_cast<const uint32_t*>(wr + 8);
#pragma unroll
                for (int m = 0; m < 2; ++m) mma_bf16(acc[m][n], a[m][0], a[m][1], a[m][2], a[m][3], b0, b1);
            }
        }
    }
    // epilogue: ReLU (unless the network is linear), BF16, NHWC
    auto act = [relu](float v) { return relu ? fmaxf(v, 0.f) : v; };
#pragma unroll
    for (int m = 0; m < 2; ++m) {
        const int y = y0 + warp * 2 + m;
        if (y >= Y) continue;
#pragma unroll
        for (int hh = 0; hh < 2; ++hh) {
            const int x = x0 + gid + 8 * hh;
            if (x >= X) continue;
            __nv_bfloat16* o = out + ((long long)b * P + (long long)y * X + x) * CNN_HIDDEN;
#pragma unroll
            for (int n = 0; n < 4; ++n) {
                const __nv_bfloat162 v = __floats2bfloat162_rn(act(acc[m][n][2 * hh]), act(acc[m][n][2 * hh + 1]));
                *reinterpret_cast<__nv_bfloat162*>(o + n * 8 + 2 * tig) = v;
            }
        }
    }
}

// wmma[l][h][n][k] (h = 0 hi, 1 lo; k = tap * 32 + ci, padded to KSTRIDE) for hidden layers l = 1 .. L-2
__global__ void cnn_pack_mma_kernel(const float* __restrict__ W, __nv_bfloat16* __restrict__ dst) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= CNN_HIDDEN * KSTRIDE) return;
    const int n = i / KSTRIDE, k = i % KSTRIDE;
    float w = 0.f;
    if (k < KDIM) {
        const int tap = k / CNN_HIDDEN, ci = k % CNN_HIDDEN;
        w = W[(n * CNN_HIDDEN + ci) * 9 + tap];
    }
    const __nv_bfloat16 hi = __float2bfloat16_rn(w);
    const __nv_bfloat16 lo = __float2bfloat16_rn(w - __bfloat162float(hi));
    dst[i] = hi;
    dst[CNN_HIDDEN * KSTRIDE + i] = lo;
}

void cnn_pack_mma(CnnNet& n, cudaStream_t st) {
    const size_t per = (size_t)2 * CNN_HIDDEN * KSTRIDE;
    n.wmma.ensure(per * 2 * std::max(1, n.L - 2));
    for (int l = 1; l < n.L - 1; ++l) {
        cnn_pack_mma_kernel<<<(unsigned)cdiv(CNN_HIDDEN * KSTRIDE, 256), 256, 0, st>>>(
            n.theta.as<float>() + n.woff[l], n.wmma.as<__nv_bfloat16>() + (size_t)(l - 1) * per);
        check_launch("cnn_pack_mma");
    }
}

void cnn_forward_mma(CnnNet& n, int layer, const __nv_bfloat16* in, __nv_bfloat16* out, int nx, int ny, int batch,
                     bool relu, cudaStream_t st) {
    static bool attr = false;
    if (!attr) {
        MMR_CUDA(cudaFuncSetAttribute(conv3x3_mma_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)MMA_SMEM));
        attr = true;
    }
    const size_t per = (size_t)2 * CNN_HIDDEN * KSTRIDE;
    dim3 grid((unsigned)cdiv(nx, MT), (unsigned)cdiv(ny, MT), (unsigned)batch);
    conv3x3_mma_kernel<<<grid, 256, MMA_SMEM, st>>>(in, out, n.wmma.as<__nv_bfloat16>() + (size_t)(layer - 1) * per,
                                                   nx, ny, relu ? 1 : 0);
    check_launch("conv3x3_mma");
}

}  // namespace mmr
