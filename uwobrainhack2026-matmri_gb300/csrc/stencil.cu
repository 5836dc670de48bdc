// The gridding normal operator C^H diag(w) C as a per-cell stencil.
//
// With convMat C (nufftOp.m:257) the normal operator of the gridding step is
//   (C^H D C)[o, i] = sum_s w_s C[s, o] C[s, i],
// non-zero only for |o - i| <= W - 1 in each dimension.  The plan evaluates it
// once in FP64 on the host for every output cell o and offset d = i - o
// ((2W-1)^2 values per cell, stored as FP32 [(2W-1)^2][G1*G2]).  Applying it
// is then a regular, atomic-free stencil over a shared-memory tile with halo,
// reused across the coils of a CTA: the same sums as interp -> weight ->
// spread (nufftOp.m:389, 392/357, 359) in a different association order.
#include <algorithm>
#include <cmath>

#include "nufft.cuh"

namespace mmr {

bool nufft_stencil_supported(const NufftPlan& p) {
    return p.nd == 2 && p.W <= 8 && p.G[0] >= 2 * p.W && p.G[1] >= 2 * p.W;
}

void nufft_build_stencil(NufftPlan& p, const float* w, long long key) {
    MMR_REQUIRE(nufft_stencil_supported(p), "stencil normal operator needs a 2D plan with kwidth <= 8");
    if (p.stencil_key == key && p.d_stencil.p) return;
    const int W = p.W, D = 2 * W - 1, H = W - 1, off0 = -W / 2 + 1;
    const int G1 = p.G[0], G2 = p.G[1];
    const size_t GG = (size_t)G1 * G2;
    std::vector<int> base((size_t)2 * p.M);
    std::vector<float> wts((size_t)p.M * 2 * W);
    MMR_CUDA(cudaMemcpy(base.data(), p.d_base.p, base.size() * sizeof(int), cudaMemcpyDeviceToHost));
    MMR_CUDA(cudaMemcpy(wts.data(), p.d_w.p, wts.size() * sizeof(float), cudaMemcpyDeviceToHost));
    std::vector<double> acc((size_t)D * D * GG, 0.0);
    for (long long s = 0; s < p.M; ++s) {
        const double ws = w ? (double)w[s] : 1.0;
        if (ws == 0.0) continue;
        const int c1 = base[s], c2 = base[p.M + s];
        const float* w1 = &wts[(size_t)s * 2 * W];
        const float* w2 = w1 + W;
        for (int a2 = 0; a2 < W; ++a2) {
            int o2 = c2 + off0 + a2;
            o2 += o2 < 0 ? G2 : 0;
            o2 -= o2 >= G2 ? G2 : 0;
            for (int a1 = 0; a1 < W; ++a1) {
                int o1 = c1 + off0 + a1;
                o1 += o1 < 0 ? G1 : 0;
                o1 -= o1 >= G1 ? G1 : 0;
                const double wo = ws * (double)w1[a1] * (double)w2[a2];
                const size_t cell = (size_t)o1 + (size_t)G1 * o2;
                for (int b2 = 0; b2 < W; ++b2) {
                    const double wb2 = wo * (double)w2[b2];
                    const size_t row = (size_t)D * (b2 - a2 + H);
                    for (int b1 = 0; b1 < W; ++b1)
                        acc[(row + (b1 - a1 + H)) * GG + cell] += wb2 * (double)w1[b1];
                }
            }
        }
    }
    std::vector<float> f(acc.size());
    for (size_t i = 0; i < acc.size(); ++i) f[i] = (float)acc[i];
    p.d_stencil.upload(f);
    p.stencil_key = key;
}

// Thread: CPT consecutive cells along axis 0 for CGS coils.  CTA: TX x TY cells.
template <int W, int CGS>
__global__ void __launch_bounds__(256) stencil2d_kernel(const float2* __restrict__ gin, float2* __restrict__ gout,
                                                        const float* __restrict__ sw, int G1, int G2, long long nb,
                                                        const int* active) {
    constexpr int D = 2 * W - 1, H = W - 1;
    constexpr int CPT = 4, TX = 64, TY = 16;
    constexpr int RX = TX + 2 * H, RY = TY + 2 * H;
    extern __shared__ float4 sm4[];
    float2* reg = reinterpret_cast<float2*>(sm4);   // [CGS][RY][RX]
    pdl_wait();
    pdl_trigger();
    if (active && *active) return;
    const int u0 = blockIdx.x * TX, v0 = blockIdx.y * TY, c0 = blockIdx.z * CGS;
    // stage the tile + halo (periodic wrap), one warp per (coil, row)
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
    for (int cr = warp; cr < CGS * RY; cr += nwarp) {
        const int c = cr / RY, ry = cr - c * RY;
        int v = v0 - H + ry;
        v += v < 0 ? G2 : 0;
        v -= v >= G2 ? G2 : 0;
        const bool cv = c0 + c < nb;
        const float2* src = gin + (long long)G1 * (v + (long long)G2 * (c0 + c));
        float2* dst = reg + (size_t)cr * RX;
        for (int rx = lane; rx < RX; rx += 32) {
            int u = u0 - H + rx;
            u += u < 0 ? G1 : 0;
            u -= u >= G1 ? G1 : 0;
            dst[rx] = cv ? src[u] : make_float2(0.f, 0.f);
        }
    }
    __syncthreads();
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const int u = u0 + tx * CPT, v = v0 + ty;
    const size_t GG = (size_t)G1 * G2;
    float2 acc[CPT][CGS];
#pragma unroll
    for (int i = 0; i < CPT; ++i)
#pragma unroll
        for (int c = 0; c < CGS; ++c) acc[i][c] = make_float2(0.f, 0.f);
    if (v < G2) {
        for (int dy = 0; dy < D; ++dy) {
            float wr[CPT][D];
#pragma unroll
            for (int dx = 0; dx < D; ++dx)
#pragma unroll
                for (int i = 0; i < CPT; ++i)
                    wr[i][dx] = (u + i < G1) ? __ldg(sw + (size_t)(dx + D * dy) * GG + (u + i) + (size_t)G1 * v) : 0.f;
#pragma unroll
            for (int c = 0; c < CGS; ++c) {
                const float2* row = reg + ((size_t)c * RY + ty + dy) * RX + tx * CPT;
                float2 in[CPT + D - 1];
#pragma unroll
                for (int j = 0; j < CPT + D - 1; ++j) in[j] = row[j];
#pragma unroll
                for (int i = 0; i < CPT; ++i)
#pragma unroll
                    for (int dx = 0; dx < D; ++dx) {
                        acc[i][c].x += wr[i][dx] * in[i + dx].x;
                        acc[i][c].y += wr[i][dx] * in[i + dx].y;
                    }
            }
        }
#pragma unroll
        for (int c = 0; c < CGS; ++c) {
            if (c0 + c >= nb) continue;
            float2* o = gout + (size_t)G1 * (v + (size_t)G2 * (c0 + c));
#pragma unroll
            for (int i = 0; i < CPT; ++i)
                if (u + i < G1) o[u + i] = acc[i][c];
        }
    }
}

template <int W, int CGS>
static void launch_stencil(const NufftPlan& p, const float2* gin, float2* gout, long long nb, cudaStream_t st,
                           const int* active) {
    constexpr int H = W - 1, RX = 64 + 2 * H, RY = 16 + 2 * H;
    const size_t smem = (size_t)CGS * RX * RY * sizeof(float2);
    MMR_CUDA(cudaFuncSetAttribute(stencil2d_kernel<W, CGS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    dim3 grid((unsigned)cdiv(p.G[0], 64), (unsigned)cdiv(p.G[1], 16), (unsigned)cdiv(nb, CGS));
    launch_dependent(stencil2d_kernel<W, CGS>, grid, dim3(256), smem, st, gin, gout, p.d_stencil.as<float>(), p.G[0],
                     p.G[1], nb, active);
}

template <int W>
static void launch_stencil_w(const NufftPlan& p, const float2* gin, float2* gout, long long nb, cudaStream_t st,
                             const int* active) {
    const int cg = std::max(1, std::min(p.cg_pref, 8));
    if (cg >= 8 && nb >= 8) launch_stencil<W, 8>(p, gin, gout, nb, st, active);
    else if (cg >= 4 && nb >= 4) launch_stencil<W, 4>(p, gin, gout, nb, st, active);
    else if (cg >= 2 && nb >= 2) launch_stencil<W, 2>(p, gin, gout, nb, st, active);
    else launch_stencil<W, 1>(p, gin, gout, nb, st, active);
}

void nufft_grid_normal_stencil(NufftPlan& p, const float2* gin, float2* gout, long long nb, cudaStream_t st,
                               const int* active) {
    MMR_REQUIRE(p.d_stencil.p, "stencil not built");
    switch (p.W) {
        case 2: launch_stencil_w<2>(p, gin, gout, nb, st, active); break;
        case 4: launch_stencil_w<4>(p, gin, gout, nb, st, active); break;
        case 6: launch_stencil_w<6>(p, gin, gout, nb, st, active); break;
        case 8: launch_stencil_w<8>(p, gin, gout, nb, st, active); break;
        default: MMR_THROW(MMR_ERR_UNSUPPORTED, "kwidth %d", p.W);
    }
}

}  // namespace mmr
