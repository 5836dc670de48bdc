// Learned preconditioner network (see cnn.cuh): training and inference kernels.
//
// Training (SIMT, FP32 arithmetic):
//   forward      conv3x3_simt, one CTA per 32 x 16 pixel tile, all output
//                channels per thread (two pixels per thread, weights broadcast
//                from shared memory as float4, input tile planar in shared)
//   data grad    the same kernel with the transposed, flipped kernel and the
//                ReLU mask of the layer input
//   weight grad  conv3x3_wgrad: per-CTA partial sums over a grid-stride loop of
//                16 x 16 tiles, then a fixed-order reduction (deterministic)
//   loss         per image over the interior mask, FP64 reductions: relative L2,
//                or 1 - cosine^2 between output and target (scale invariant)
//   optimiser    Adam on the FP32 parameter vector
// Inference: the same forward, or the tensor-core path (cnn_mma.cu, FP16
// activations).
#include <algorithm>
#include <cmath>

#include "cnn.cuh"

namespace mmr {

void cnn_forward_tensor(CnnNet& n, const float2* r, float2* z, int nx, int ny, int batch, bool relu,
                        cudaStream_t st);
void cnn_pack_mma(CnnNet& n, cudaStream_t st);

// ------------------------------------------------------------ load / store ----
__device__ __forceinline__ float ldf(const float* p) { return *p; }
__device__ __forceinline__ float ldf(const __nv_bfloat16* p) { return __bfloat162float(*p); }
__device__ __forceinline__ void stf(float* p, float v) { *p = v; }
__device__ __forceinline__ void stf(__nv_bfloat16* p, float v) { *p = __float2bfloat16_rn(v); }

enum ConvMode { IN_CPLX = 1, OUT_RELU = 2, OUT_FINAL = 4, OUT_MASK = 8 };

struct ConvArgs {
    int X, Y;
    const double* sumsq;     // IN_CPLX / OUT_FINAL: per-image sum |r|^2
    const void* mask;        // OUT_MASK: activation [B][P][COUT] (ReLU output of the layer input)
    const float2* r;         // OUT_FINAL: network input for the skip path
    const float* skip;       // OUT_FINAL: device scalar
    int relu;                // 0: identity activations (a linear network)
};

__device__ __forceinline__ float image_scale(const double* sumsq, int b, long long P, float* inv) {
    const double s = sqrt(sumsq[b] / (double)P);
    *inv = s > 0 ? (float)(1.0 / s) : 0.f;
    return (float)s;
}

constexpr int CV_TX = 32, CV_TY = 16, CV_HX = CV_TX + 2, CV_HY = CV_TY + 2;

template <int CIN, int COUT>
constexpr size_t conv_smem_bytes() {
    return sizeof(float) * ((size_t)CIN * 9 * COUT + (size_t)(CIN < 8 ? CIN : 8) * CV_HY * CV_HX);
}

// out[b][p][co] = sum_ci,tap w[(ci*9+tap)*COUT + co] * in[b][p+off(tap)][ci]   (zero padding)
template <int CIN, int COUT, class TIn, class TOut, class TMask, int MODE>
__global__ void __launch_bounds__(256, 2) conv3x3_simt(const TIn* __restrict__ in, TOut* __restrict__ out,
                                                    const float* __restrict__ wpk, ConvArgs a) {
    constexpr int CCH = CIN < 8 ? CIN : 8;
    extern __shared__ float smem[];
    float* s_w = smem;
    float* s_in = smem + CIN * 9 * COUT;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int b = blockIdx.z;
    const int x0 = blockIdx.x * CV_TX, y0 = blockIdx.y * CV_TY;
    const int X = a.X, Y = a.Y;
    const long long P = (long long)X * Y;
    float inv_s = 1.f, sval = 1.f;
    if (MODE & (IN_CPLX | OUT_FINAL)) sval = image_scale(a.sumsq, b, P, &inv_s);
    for (int i = threadIdx.x; i < CIN * 9 * COUT; i += 256) s_w[i] = wpk[i];
    float acc0[COUT], acc1[COUT];
#pragma unroll
    for (int c = 0; c < COUT; ++c) acc0[c] = acc1[c] = 0.f;
    for (int c0 = 0; c0 < CIN; c0 += CCH) {
        __syncthreads();
        for (int i = threadIdx.x; i < CV_HY * CV_HX * CCH; i += 256) {
            const int c = i % CCH, pix = i / CCH, hx = pix % CV_HX, hy = pix / CV_HX;
            const int gx = x0 + hx - 1, gy = y0 + hy - 1;
            float v = 0.f;
            if (gx >= 0 && gx < X && gy >= 0 && gy < Y) {
                const long long gp = (long long)b * P + (long long)gy * X + gx;
                if constexpr ((MODE & IN_CPLX) != 0) {
                    const float2 rv = reinterpret_cast<const float2*>(in)[gp];
                    v = (c == 0 ? rv.x : rv.y) * inv_s;
                } else {
                    v = ldf(in + gp * CIN + c0 + c);
                }
            }
            s_in[(c * CV_HY + hy) * CV_HX + hx] = v;
        }
        __syncthreads();
#pragma unroll 1
        for (int c = 0; c < CCH; ++c) {
#pragma unroll
            for (int t = 0; t < 9; ++t) {
                const int ky = t / 3, kx = t % 3;
                const float i0 = s_in[(c * CV_HY + ty + ky) * CV_HX + tx + kx];
                const float i1 = s_in[(c * CV_HY + ty + 8 + ky) * CV_HX + tx + kx];
                const float* wr = s_w + ((c0 + c) * 9 + t) * COUT;
                if constexpr (COUT % 4 == 0) {
#pragma unroll
                    for (int j = 0; j < COUT / 4; ++j) {
                        const float4 w = reinterpret_cast<const float4*>(wr)[j];
                        acc0[4 * j] += w.x * i0; acc0[4 * j + 1] += w.y * i0;
                        acc0[4 * j + 2] += w.z * i0; acc0[4 * j + 3] += w.w * i0;
                        acc1[4 * j] += w.x * i1; acc1[4 * j + 1] += w.y * i1;
                        acc1[4 * j + 2] += w.z * i1; acc1[4 * j + 3] += w.w * i1;
                    }
                } else {
#pragma unroll
                    for (int j = 0; j < COUT; ++j) {
                        acc0[j] += wr[j] * i0;
                        acc1[j] += wr[j] * i1;
                    }
                }
            }
        }
    }
    const int x = x0 + tx;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const int y = y0 + ty + 8 * h;
        if (x >= X || y >= Y) continue;
        const float* acc = h ? acc1 : acc0;
        const long long gp = (long long)b * P + (long long)y * X + x;
        if constexpr ((MODE & OUT_FINAL) != 0) {
            static_assert(COUT == 2, "final layer writes a complex image");
            const float2 rv = a.r[gp];
            const float sk = *a.skip;
            reinterpret_cast<float2*>(out)[gp] = make_float2(sval * acc[0] + sk * rv.x, sval * acc[1] + sk * rv.y);
        } else {
#pragma unroll
            for (int co = 0; co < COUT; ++co) {
                float v = acc[co];
                if ((MODE & OUT_RELU) && a.relu) v = fmaxf(v, 0.f);
                if ((MODE & OUT_MASK) && a.relu) {
                    if (!(ldf(static_cast<const TMask*>(a.mask) + gp * COUT + co) > 0.f)) v = 0.f;
                }
                stf(out + gp * COUT + co, v);
            }
        }
    }
}

// ------------------------------------------------------------- weight grad ----
constexpr int WG_T = 16, WG_H = WG_T + 2, WG_PLANE = WG_H * WG_H + 1, WG_GSTRIDE = WG_T * WG_T + 1;

template <int CIN, int COUT>
constexpr size_t wgrad_smem_bytes() {
    return sizeof(float) * ((size_t)CIN * WG_PLANE + (size_t)COUT * WG_GSTRIDE);
}

// partial[blockIdx.x][(co*CIN + ci)*9 + tap] = sum over this CTA's tiles of g[co][p] a[ci][p+off(tap)]
template <int CIN, int COUT, class TAct, bool CPLX>
__global__ void __launch_bounds__(256) conv3x3_wgrad(const TAct* __restrict__ act, const float* __restrict__ g,
                                                     float* __restrict__ partial, int X, int Y, int B,
                                                     const double* __restrict__ sumsq) {
    constexpr int NPAIR = CIN * COUT;
    constexpr int KP = (NPAIR + 255) / 256;
    extern __shared__ float smem[];
    float* s_a = smem;                       // [CIN][WG_PLANE]
    float* s_g = smem + CIN * WG_PLANE;      // [COUT][WG_GSTRIDE]
    const long long P = (long long)X * Y;
    const int tilesX = (X + WG_T - 1) / WG_T, tilesY = (Y + WG_T - 1) / WG_T;
    const long long ntiles = (long long)tilesX * tilesY * B;
    float acc[KP][9];
#pragma unroll
    for (int k = 0; k < KP; ++k)
#pragma unroll
        for (int t = 0; t < 9; ++t) acc[k][t] = 0.f;
    for (long long T = blockIdx.x; T < ntiles; T += gridDim.x) {
        const int b = (int)(T / ((long long)tilesX * tilesY));
        const int rem = (int)(T % ((long long)tilesX * tilesY));
        const int x0 = (rem % tilesX) * WG_T, y0 = (rem / tilesX) * WG_T;
        float inv_s = 1.f;
        if (CPLX) image_scale(sumsq, b, P, &inv_s);
        __syncthreads();
        for (int i = threadIdx.x; i < WG_H * WG_H * CIN; i += 256) {
            const int c = i % CIN, pix = i / CIN, hx = pix % WG_H, hy = pix / WG_H;
            const int gx = x0 + hx - 1, gy = y0 + hy - 1;
            float v = 0.f;
            if (gx >= 0 && gx < X && gy >= 0 && gy < Y) {
                const long long gp = (long long)b * P + (long long)gy * X + gx;
                if constexpr (CPLX) {
                    const float2 rv = reinterpret_cast<const float2*>(act)[gp];
                    v = (c == 0 ? rv.x : rv.y) * inv_s;
                } else {
                    v = ldf(act + gp * CIN + c);
                }
            }
            s_a[c * WG_PLANE + hy * WG_H + hx] = v;
        }
        for (int i = threadIdx.x; i < WG_T * WG_T * COUT; i += 256) {
            const int c = i % COUT, pix = i / COUT, px = pix % WG_T, py = pix / WG_T;
            const int gx = x0 + px, gy = y0 + py;
            float v = 0.f;
            if (gx < X && gy < Y) v = g[((long long)b * P + (long long)gy * X + gx) * COUT + c];
            s_g[c * WG_GSTRIDE + pix] = v;
        }
        __syncthreads();
#pragma unroll 1
        for (int p = 0; p < WG_T * WG_T; ++p) {
            const int py = p / WG_T, px = p % WG_T;
#pragma unroll
            for (int k = 0; k < KP; ++k) {
                const int q = threadIdx.x + 256 * k;
                if (q < NPAIR) {
                    const int co = q / CIN, ci = q % CIN;
                    const float gv = s_g[co * WG_GSTRIDE + p];
                    const float* ap = s_a + ci * WG_PLANE + py * WG_H + px;
#pragma unroll
                    for (int t = 0; t < 9; ++t) acc[k][t] += gv * ap[(t / 3) * WG_H + (t % 3)];
                }
            }
        }
    }
    float* dst = partial + (size_t)blockIdx.x * NPAIR * 9;
#pragma unroll
    for (int k = 0; k < KP; ++k) {
        const int q = threadIdx.x + 256 * k;
        if (q < NPAIR)
#pragma unroll
            for (int t = 0; t < 9; ++t) dst[q * 9 + t] = acc[k][t];
    }
}

// grad[i] = sum_b partial[b][i]   (fixed order)
__global__ void reduce_partials_kernel(const float* __restrict__ partial, int nblk, int n, float* __restrict__ grad) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double s = 0;
    for (int k = 0; k < nblk; ++k) s += partial[(size_t)k * n + i];
    grad[i] = (float)s;
}

// ------------------------------------------------------------ misc kernels ----
// sumsq[b] += sum_p |r[b][p]|^2   (sumsq zeroed by the caller)
__global__ void cnn_sumsq_kernel(const float2* __restrict__ r, long long P, double* __restrict__ sumsq) {
    const int b = blockIdx.y;
    double s = 0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < P; i += (long long)gridDim.x * blockDim.x) {
        const float2 v = r[(long long)b * P + i];
        s += (double)v.x * v.x + (double)v.y * v.y;
    }
    for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    __shared__ double red[8];
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
        atomicAdd(sumsq + b, t);
    }
}

// wpk[(ci*9+t)*COUT + co] = W[co][ci][t];  wpkT[(co*9+t)*CIN + ci] = W[co][ci][8-t]
__global__ void cnn_pack_kernel(const float* __restrict__ W, int cin, int cout, float* __restrict__ wpk,
                                float* __restrict__ wpkT) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = cin * cout * 9;
    if (i >= n) return;
    const int t = i % 9, ci = (i / 9) % cin, co = i / (9 * cin);
    const float w = W[i];
    wpk[(ci * 9 + t) * cout + co] = w;
    wpkT[(co * 9 + (8 - t)) * cin + ci] = w;
}

// Per image over the interior mask m, LOSS_ACC values: sum |z-e|^2, sum |e|^2, sum |z|^2,
// re and im of sum conj(z) e.
constexpr int LOSS_ACC = 5;

__global__ void cnn_loss_reduce_kernel(const float2* __restrict__ z, const float2* __restrict__ e, int X, int Y,
                                       int margin, double* __restrict__ acc) {
    const int b = blockIdx.y;
    const long long P = (long long)X * Y;
    double v[LOSS_ACC] = {0, 0, 0, 0, 0};
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < P; i += (long long)gridDim.x * blockDim.x) {
        const int x = (int)(i % X), y = (int)(i / X);
        if (x < margin || x >= X - margin || y < margin || y >= Y - margin) continue;
        const float2 zv = z[(long long)b * P + i], ev = e[(long long)b * P + i];
        const double dx = (double)zv.x - ev.x, dy = (double)zv.y - ev.y;
        v[0] += dx * dx + dy * dy;
        v[1] += (double)ev.x * ev.x + (double)ev.y * ev.y;
        v[2] += (double)zv.x * zv.x + (double)zv.y * zv.y;
        v[3] += (double)zv.x * ev.x + (double)zv.y * ev.y;
        v[4] += (double)zv.x * ev.y - (double)zv.y * ev.x;
    }
    __shared__ double red[LOSS_ACC][8];
#pragma unroll
    for (int k = 0; k < LOSS_ACC; ++k) {
        double s = v[k];
        for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if ((threadIdx.x & 31) == 0) red[k][threadIdx.x >> 5] = s;
    }
    __syncthreads();
    if (threadIdx.x < LOSS_ACC) {
        double t = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[threadIdx.x][w];
        atomicAdd(acc + LOSS_ACC * b + threadIdx.x, t);
    }
}

// gv = s * dL/dz (the gradient w.r.t. the last conv output); dskip += sum gv * r / s.
//   relative L2:  dL/dz = 2 m (z - e) / E / B
//   cosine:       dL/dz = m (-2 conj(c) e / (Z E) + 2 |c|^2 z / (Z^2 E)) / B,  c = sum conj(z) e
__global__ void cnn_loss_grad_kernel(const float2* __restrict__ z, const float2* __restrict__ e,
                                     const float2* __restrict__ r, const double* __restrict__ sumsq,
                                     const double* __restrict__ acc, int X, int Y, int B, int margin, int cosine,
                                     float2* __restrict__ gv, double* __restrict__ dskip) {
    const int b = blockIdx.y;
    const long long P = (long long)X * Y;
    float inv_s;
    const float s = image_scale(sumsq, b, P, &inv_s);
    const double* a = acc + LOSS_ACC * b;
    const double E = a[1] > 0 ? a[1] : 1.0;
    // g = ce * e + cz * z with complex ce, real cz
    double cer = 0, cei = 0, cz = 0;
    if (!cosine) {
        cz = 2.0 / E / B;
        cer = -cz;
    } else if (a[2] > 0) {
        const double Z = a[2], c2 = a[3] * a[3] + a[4] * a[4];
        cer = -2.0 * a[3] / (Z * E) / B;          // -2 conj(c) / (Z E) / B
        cei = 2.0 * a[4] / (Z * E) / B;
        cz = 2.0 * c2 / (Z * Z * E) / B;
    }
    double ds = 0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < P; i += (long long)gridDim.x * blockDim.x) {
        const int x = (int)(i % X), y = (int)(i / X);
        const long long gp = (long long)b * P + i;
        float2 g = make_float2(0.f, 0.f);
        if (!(x < margin || x >= X - margin || y < margin || y >= Y - margin)) {
            const float2 zv = z[gp], ev = e[gp];
            g = make_float2((float)(s * (cer * ev.x - cei * ev.y + cz * zv.x)),
                            (float)(s * (cer * ev.y + cei * ev.x + cz * zv.y)));
        }
        gv[gp] = g;
        const float2 rv = r[gp];
        ds += (double)g.x * rv.x * inv_s + (double)g.y * rv.y * inv_s;
    }
    for (int o = 16; o; o >>= 1) ds += __shfl_xor_sync(0xffffffffu, ds, o);
    __shared__ double red[8];
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = ds;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
        atomicAdd(dskip, t);
    }
}

__global__ void cnn_set_skip_grad_kernel(const double* __restrict__ dskip, float* __restrict__ g) { *g = (float)*dskip; }

__global__ void cnn_adam_kernel(float* __restrict__ th, const float* __restrict__ g, float* __restrict__ m,
                                float* __restrict__ v, long long n, float lr, float b1, float b2, float eps, float c1,
                                float c2) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    th[i] -= lr * (mi * c1) / (sqrtf(vi * c2) + eps);
}

// ------------------------------------------------------------------- host ----
template <class K>
static void set_smem(K kernel, size_t bytes) {
    static_assert(sizeof(K) > 0, "");
    MMR_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
}

template <int CIN, int COUT, class TIn, class TOut, class TMask, int MODE>
static void launch_conv(const TIn* in, TOut* out, const float* wpk, const ConvArgs& a, int B, cudaStream_t st) {
    auto k = conv3x3_simt<CIN, COUT, TIn, TOut, TMask, MODE>;
    const size_t sm = conv_smem_bytes<CIN, COUT>();
    static bool attr = false;
    if (!attr) {
        set_smem(k, sm);
        attr = true;
    }
    dim3 grid((unsigned)cdiv(a.X, CV_TX), (unsigned)cdiv(a.Y, CV_TY), (unsigned)B);
    k<<<grid, 256, sm, st>>>(in, out, wpk, a);
    check_launch("conv3x3_simt");
}

template <int CIN, int COUT, class TAct, bool CPLX>
static void launch_wgrad(const TAct* act, const float* g, CnnNet& n, int layer, int X, int Y, int B,
                         cudaStream_t st) {
    auto k = conv3x3_wgrad<CIN, COUT, TAct, CPLX>;
    const size_t sm = wgrad_smem_bytes<CIN, COUT>();
    static bool attr = false;
    if (!attr) {
        set_smem(k, sm);
        attr = true;
    }
    const long long ntiles = cdiv(X, WG_T) * cdiv(Y, WG_T) * B;
    const int nblk = (int)std::min<long long>(ntiles, 2LL * device_sm_count());
    const int nw = CIN * COUT * 9;
    n.partial.ensure((size_t)nblk * nw * sizeof(float));
    k<<<nblk, 256, sm, st>>>(act, g, n.partial.as<float>(), X, Y, B, n.sumsq.as<double>());
    check_launch("conv3x3_wgrad");
    reduce_partials_kernel<<<(unsigned)cdiv(nw, 256), 256, 0, st>>>(n.partial.as<float>(), nblk, nw,
                                                                      n.grad.as<float>() + n.woff[layer]);
    check_launch("reduce_partials");
}

void cnn_pack(CnnNet& n, cudaStream_t st) {
    if (n.packed_version == n.version) return;
    for (int l = 0; l < n.L; ++l) {
        const int nw = n.ch[l] * n.ch[l + 1] * 9;
        cnn_pack_kernel<<<(unsigned)cdiv(nw, 256), 256, 0, st>>>(n.theta.as<float>() + n.woff[l], n.ch[l], n.ch[l + 1],
                                                                 n.wpk.as<float>() + n.woff[l],
                                                                 n.wpkT.as<float>() + n.woff[l]);
        check_launch("cnn_pack");
    }
    cnn_pack_mma(n, st);
    n.packed_version = n.version;
}

static void ensure_scratch(CnnNet& n, long long P, int B, bool training, bool fp32) {
    const size_t per = (size_t)P * B * CNN_HIDDEN;
    const size_t esz = fp32 ? 4 : 2;
    const int nact = training ? (n.L - 1) : 2;
    n.act.ensure(per * esz * nact);
    if (training) {
        n.gbuf.ensure(per * 4 * 2);
        n.gv.ensure((size_t)P * B * 8);
    }
    n.z.ensure((size_t)P * B * 8);
    n.sumsq.ensure((size_t)B * 8);
    n.lossacc.ensure((size_t)B * LOSS_ACC * 8);
    n.dskip.ensure(8);
}

template <class TAct>
static void forward_simt(CnnNet& n, const float2* r, float2* z, int X, int Y, int B, bool keep, bool relu,
                         cudaStream_t st) {
    const long long P = (long long)X * Y;
    const size_t per = (size_t)P * B * CNN_HIDDEN;
    TAct* acts = n.act.as<TAct>();
    auto act = [&](int i) { return acts + (keep ? (size_t)i : (size_t)(i & 1)) * per; };   // a_{i+1}
    const float* wpk = n.wpk.as<float>();
    ConvArgs a{X, Y, n.sumsq.as<double>(), nullptr, r, n.theta.as<float>() + n.nparam - 1, relu ? 1 : 0};
    launch_conv<2, CNN_HIDDEN, float2, TAct, TAct, IN_CPLX | OUT_RELU>(r, act(0), wpk + n.woff[0], a, B, st);
    for (int l = 1; l < n.L - 1; ++l)
        launch_conv<CNN_HIDDEN, CNN_HIDDEN, TAct, TAct, TAct, OUT_RELU>(act(l - 1), act(l), wpk + n.woff[l], a, B, st);
    launch_conv<CNN_HIDDEN, 2, TAct, float2, TAct, OUT_FINAL>(act(n.L - 2), z, wpk + n.woff[n.L - 1], a, B, st);
}

static void compute_sumsq(CnnNet& n, const float2* r, long long P, int B, cudaStream_t st) {
    MMR_CUDA(cudaMemsetAsync(n.sumsq.p, 0, (size_t)B * 8, st));
    cnn_sumsq_kernel<<<dim3((unsigned)std::min<long long>(cdiv(P, 256), 64), (unsigned)B), 256, 0, st>>>(
        r, P, n.sumsq.as<double>());
    check_launch("cnn_sumsq");
}

// ------------------------------------------------------------ folded linear network ----
// A linear network (identity activations) is one linear operator: composing the 3x3
// layers (cross-correlations: offsets add) gives a single (2L+1)^2 filter with a real
// 2x2 matrix per tap, z[p] = sum_d K[d] r[p + d] + skip r[p]; the input scale s cancels.
// It is the operator the network computes on the zero-extended image (no intermediate
// zero padding), which is what crop training past the image edge optimises.  Composed
// on the host in FP64 whenever the weights change.
static void cnn_fold(CnnNet& n, cudaStream_t st) {
    if (n.folded_version == n.version) return;
    std::vector<float> th((size_t)n.nparam);
    MMR_CUDA(cudaMemcpyAsync(th.data(), n.theta.p, th.size() * 4, cudaMemcpyDeviceToHost, st));
    MMR_CUDA(cudaStreamSynchronize(st));
    // T[(dy+R)*(2R+1) + dx+R][co][ci], R grows by 1 per layer
    int R = 1, cout = n.ch[1];
    const int cin0 = n.ch[0];
    std::vector<double> T((size_t)9 * cout * cin0);
    for (int co = 0; co < cout; ++co)
        for (int ci = 0; ci < cin0; ++ci)
            for (int t = 0; t < 9; ++t)
                T[((size_t)t * cout + co) * cin0 + ci] = th[n.woff[0] + ((size_t)co * cin0 + ci) * 9 + t];
    for (int l = 1; l < n.L; ++l) {
        const int cmid = n.ch[l], co2 = n.ch[l + 1], R2 = R + 1, S = 2 * R + 1, S2 = 2 * R2 + 1;
        std::vector<double> U((size_t)S2 * S2 * co2 * cin0, 0.0);
        const float* W = th.data() + n.woff[l];
        for (int t = 0; t < 9; ++t) {
            const int oy = t / 3 - 1, ox = t % 3 - 1;
            for (int dy = -R; dy <= R; ++dy)
                for (int dx = -R; dx <= R; ++dx) {
                    const double* Tin = &T[((size_t)((dy + R) * S + dx + R) * cmid) * cin0];
                    double* Uo = &U[((size_t)((dy + oy + R2) * S2 + dx + ox + R2) * co2) * cin0];
                    for (int o = 0; o < co2; ++o)
                        for (int c = 0; c < cmid; ++c) {
                            const double w = W[((size_t)o * cmid + c) * 9 + t];
                            if (w == 0.0) continue;
                            for (int ci = 0; ci < cin0; ++ci) Uo[(size_t)o * cin0 + ci] += w * Tin[(size_t)c * cin0 + ci];
                        }
                }
        }
        T.swap(U);
        R = R2;
        cout = co2;
    }
    MMR_REQUIRE(cout == 2 && cin0 == 2, "folding needs a complex-in, complex-out network");
    const int S = 2 * R + 1;
    const double skip = th[n.nparam - 1];
    std::vector<float4> K((size_t)S * S);
    for (int d = 0; d < S * S; ++d) {
        const double* m = &T[(size_t)d * 4];   // [co][ci]
        const bool centre = d == R * S + R;
        K[d] = make_float4((float)(m[0] + (centre ? skip : 0.0)), (float)m[1], (float)m[2],
                           (float)(m[3] + (centre ? skip : 0.0)));
    }
    n.fold.ensure(K.size() * sizeof(float4));
    MMR_CUDA(cudaMemcpyAsync(n.fold.p, K.data(), K.size() * sizeof(float4), cudaMemcpyHostToDevice, st));
    MMR_CUDA(cudaStreamSynchronize(st));
    n.fold_radius = R;
    n.folded_version = n.version;
}

constexpr int FD_TX = 32, FD_TY = 16, FD_MAXR = 8;

// z[p] = sum_d K[d] r[p+d]  (K: 2x2 real per tap as float4 {k00, k01, k10, k11}, zero outside the image)
template <int R>
__global__ void __launch_bounds__(256) conv_folded_kernel(const float2* __restrict__ r, float2* __restrict__ z,
                                                          const float4* __restrict__ K, int X, int Y) {
    constexpr int S = 2 * R + 1, HX = FD_TX + 2 * R, HY = FD_TY + 2 * R;
    __shared__ float4 s_k[S * S];
    __shared__ float2 s_r[HY][HX + 1];
    const int b = blockIdx.z;
    const long long P = (long long)X * Y;
    const int x0 = blockIdx.x * FD_TX, y0 = blockIdx.y * FD_TY;
    for (int i = threadIdx.x; i < S * S; i += blockDim.x) s_k[i] = K[i];
    for (int i = threadIdx.x; i < HX * HY; i += blockDim.x) {
        const int hx = i % HX, hy = i / HX, gx = x0 + hx - R, gy = y0 + hy - R;
        s_r[hy][hx] = (gx >= 0 && gx < X && gy >= 0 && gy < Y) ? r[(long long)b * P + (long long)gy * X + gx]
                                                                : make_float2(0.f, 0.f);
    }
    __syncthreads();
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    float a[2][2] = {{0.f, 0.f}, {0.f, 0.f}};
#pragma unroll 1
    for (int dy = 0; dy < S; ++dy) {
#pragma unroll
        for (int dx = 0; dx < S; ++dx) {
            const float4 k = s_k[dy * S + dx];
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const float2 v = s_r[ty + 8 * h + dy][tx + dx];
                a[h][0] += k.x * v.x + k.y * v.y;
                a[h][1] += k.z * v.x + k.w * v.y;
            }
        }
    }
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const int x = x0 + tx, y = y0 + ty + 8 * h;
        if (x < X && y < Y) z[(long long)b * P + (long long)y * X + x] = make_float2(a[h][0], a[h][1]);
    }
}

static void forward_folded(CnnNet& n, const float2* r, float2* z, int X, int Y, int B, cudaStream_t st) {
    cnn_fold(n, st);
    const dim3 grid((unsigned)cdiv(X, FD_TX), (unsigned)cdiv(Y, FD_TY), (unsigned)B);
    MMR_REQUIRE(n.fold_radius <= FD_MAXR, "folded filter radius %d above %d", n.fold_radius, FD_MAXR);
    switch (n.fold_radius) {
        case 2: conv_folded_kernel<2><<<grid, 256, 0, st>>>(r, z, n.fold.as<float4>(), X, Y); break;
        case 3: conv_folded_kernel<3><<<grid, 256, 0, st>>>(r, z, n.fold.as<float4>(), X, Y); break;
        case 4: conv_folded_kernel<4><<<grid, 256, 0, st>>>(r, z, n.fold.as<float4>(), X, Y); break;
        case 5: conv_folded_kernel<5><<<grid, 256, 0, st>>>(r, z, n.fold.as<float4>(), X, Y); break;
        case 6: conv_folded_kernel<6><<<grid, 256, 0, st>>>(r, z, n.fold.as<float4>(), X, Y); break;
        case 7: conv_folded_kernel<7><<<grid, 256, 0, st>>>(r, z, n.fold.as<float4>(), X, Y); break;
        case 8: conv_folded_kernel<8><<<grid, 256, 0, st>>>(r, z, n.fold.as<float4>(), X, Y); break;
        default: MMR_THROW(MMR_ERR_UNSUPPORTED, "folded filter radius %d", n.fold_radius);
    }
    check_launch("conv_folded");
}

void cnn_forward(CnnNet& n, const float2* r, float2* z, int X, int Y, int B, const double* sumsq, int flags,
                 cudaStream_t st) {
    const long long P = (long long)X * Y;
    if ((flags & CNN_FOLDED) && (flags & CNN_LINEAR)) {
        forward_folded(n, r, z, X, Y, B, st);
        return;
    }
    const bool fp32 = flags & CNN_FP32_ACT;
    const bool tc = (flags & CNN_TENSOR) && !fp32;
    ensure_scratch(n, P, B, false, fp32);
    cnn_pack(n, st);
    if (sumsq) {
        MMR_CUDA(cudaMemcpyAsync(n.sumsq.p, sumsq, (size_t)B * 8, cudaMemcpyDeviceToDevice, st));
    } else {
        compute_sumsq(n, r, P, B, st);
    }
    const bool relu = !(flags & CNN_LINEAR);
    if (tc) cnn_forward_tensor(n, r, z, X, Y, B, relu, st);
    else if (fp32) forward_simt<float>(n, r, z, X, Y, B, false, relu, st);
    else forward_simt<__nv_bfloat16>(n, r, z, X, Y, B, false, relu, st);
}

// Loss, gradient (into n.grad) of a batch; returns the loss on the host.
template <class TAct>
static double loss_grad(CnnNet& n, const float2* r, const float2* e, int X, int Y, int B, int margin, bool cosine,
                        bool relu, cudaStream_t st) {
    const long long P = (long long)X * Y;
    const size_t per = (size_t)P * B * CNN_HIDDEN;
    ensure_scratch(n, P, B, true, sizeof(TAct) == 4);
    cnn_pack(n, st);
    compute_sumsq(n, r, P, B, st);
    float2* z = n.z.as<float2>();
    forward_simt<TAct>(n, r, z, X, Y, B, true, relu, st);
    TAct* acts = n.act.as<TAct>();
    auto act = [&](int i) { return acts + (size_t)i * per; };   // a_{i+1}
    MMR_CUDA(cudaMemsetAsync(n.lossacc.p, 0, (size_t)B * LOSS_ACC * 8, st));
    MMR_CUDA(cudaMemsetAsync(n.dskip.p, 0, 8, st));
    const dim3 rg((unsigned)std::min<long long>(cdiv(P, 256), 64), (unsigned)B);
    cnn_loss_reduce_kernel<<<rg, 256, 0, st>>>(z, e, X, Y, margin, n.lossacc.as<double>());
    check_launch("cnn_loss_reduce");
    float2* gv = n.gv.as<float2>();
    cnn_loss_grad_kernel<<<rg, 256, 0, st>>>(z, e, r, n.sumsq.as<double>(), n.lossacc.as<double>(), X, Y, B, margin,
                                             cosine ? 1 : 0, gv, n.dskip.as<double>());
    check_launch("cnn_loss_grad");
    cnn_set_skip_grad_kernel<<<1, 1, 0, st>>>(n.dskip.as<double>(), n.grad.as<float>() + n.nparam - 1);
    check_launch("cnn_skip_grad");
    // last layer: g = gv (2 channels)
    const int Lm = n.L - 1;
    launch_wgrad<CNN_HIDDEN, 2, TAct, false>(act(Lm - 1), reinterpret_cast<const float*>(gv), n, Lm, X, Y, B, st);
    float* gb = n.gbuf.as<float>();
    ConvArgs a{X, Y, n.sumsq.as<double>(), nullptr, nullptr, nullptr, relu ? 1 : 0};
    a.mask = act(Lm - 1);
    launch_conv<2, CNN_HIDDEN, float, float, TAct, OUT_MASK>(reinterpret_cast<const float*>(gv), gb,
                                                             n.wpkT.as<float>() + n.woff[Lm], a, B, st);
    int cur = 0;
    for (int l = Lm - 1; l >= 1; --l) {
        float* g = gb + (size_t)cur * per;
        launch_wgrad<CNN_HIDDEN, CNN_HIDDEN, TAct, false>(act(l - 1), g, n, l, X, Y, B, st);
        a.mask = act(l - 1);
        launch_conv<CNN_HIDDEN, CNN_HIDDEN, float, float, TAct, OUT_MASK>(g, gb + (size_t)(cur ^ 1) * per,
                                                                          n.wpkT.as<float>() + n.woff[l], a, B, st);
        cur ^= 1;
    }
    launch_wgrad<2, CNN_HIDDEN, float2, true>(r, gb + (size_t)cur * per, n, 0, X, Y, B, st);
    std::vector<double> h((size_t)LOSS_ACC * B);
    MMR_CUDA(cudaMemcpyAsync(h.data(), n.lossacc.p, h.size() * 8, cudaMemcpyDeviceToHost, st));
    MMR_CUDA(cudaStreamSynchronize(st));
    double L = 0;
    for (int b = 0; b < B; ++b) {
        const double* a = h.data() + (size_t)LOSS_ACC * b;
        const double E = a[1] > 0 ? a[1] : 1.0;
        if (!cosine) L += a[0] / E;
        else L += a[2] > 0 ? 1.0 - (a[3] * a[3] + a[4] * a[4]) / (a[2] * E) : 1.0;
    }
    return L / B;
}

static void cnn_init(CnnNet& n, int L, const int* ch) {
    MMR_REQUIRE(L >= 2 && L <= 16, "layers must be 2..16");
    MMR_REQUIRE(ch[0] == 2 && ch[L] == 2, "input and output channels must be 2 (complex)");
    for (int l = 1; l < L; ++l) MMR_REQUIRE(ch[l] == CNN_HIDDEN, "hidden channels must be %d", CNN_HIDDEN);
    n.L = L;
    n.ch.assign(ch, ch + L + 1);
    n.woff.resize(L);
    long long o = 0;
    for (int l = 0; l < L; ++l) {
        n.woff[l] = o;
        o += (long long)ch[l] * ch[l + 1] * 9;
    }
    n.nparam = o + 1;
    for (DevBuf* b : {&n.theta, &n.grad, &n.adam_m, &n.adam_v, &n.wpk, &n.wpkT}) {
        b->ensure((size_t)n.nparam * 4);
        MMR_CUDA(cudaMemset(b->p, 0, (size_t)n.nparam * 4));
    }
}

}  // namespace mmr

using namespace mmr;

extern "C" int mmr_cnn_create(int32_t nlayers, const int32_t* channels, mmr_cnn** out) {
    return guarded([&] {
        MMR_REQUIRE(channels && out, "NULL argument");
        auto* h = new mmr_cnn();
        try {
            cnn_init(h->n, nlayers, channels);
        } catch (...) {
            delete h;
            throw;
        }
        *out = h;
    });
}

extern "C" int mmr_cnn_num_params(const mmr_cnn* net, int64_t* n) {
    return guarded([&] {
        MMR_REQUIRE(net && n, "NULL argument");
        *n = net->n.nparam;
    });
}

extern "C" int mmr_cnn_set_params(mmr_cnn* net, const float* theta) {
    return guarded([&] {
        MMR_REQUIRE(net && theta, "NULL argument");
        MMR_CUDA(cudaMemcpy(net->n.theta.p, theta, (size_t)net->n.nparam * 4, cudaMemcpyDefault));
        MMR_CUDA(cudaMemset(net->n.adam_m.p, 0, (size_t)net->n.nparam * 4));
        MMR_CUDA(cudaMemset(net->n.adam_v.p, 0, (size_t)net->n.nparam * 4));
        net->n.adam_t = 0;
        ++net->n.version;
    });
}

extern "C" int mmr_cnn_get_params(const mmr_cnn* net, float* theta) {
    return guarded([&] {
        MMR_REQUIRE(net && theta, "NULL argument");
        MMR_CUDA(cudaMemcpy(theta, net->n.theta.p, (size_t)net->n.nparam * 4, cudaMemcpyDefault));
    });
}

extern "C" int mmr_cnn_forward(mmr_cnn* net, const void* r, void* z, int64_t nx, int64_t ny, int64_t batch,
                               int32_t flags, void* stream) {
    return guarded([&] {
        MMR_REQUIRE(net && r && z, "NULL argument");
        MMR_REQUIRE(nx > 0 && ny > 0 && batch > 0 && batch <= 65535, "bad shape");
        CnnNet& n = net->n;
        cudaStream_t st = as_stream(stream);
        const size_t bytes = (size_t)nx * ny * batch * 8;
        const float2* rin = (const float2*)stage_in(n.st_in, r, bytes, st);
        float2* zo = (float2*)stage_out(n.st_out, z, bytes);
        cnn_forward(n, rin, zo, (int)nx, (int)ny, (int)batch, nullptr, flags, st);
        finish_out(n.st_out, bytes, st);
        MMR_CUDA(cudaStreamSynchronize(st));
    });
}

extern "C" int mmr_cnn_loss_grad(mmr_cnn* net, const void* r, const void* e, int64_t nx, int64_t ny, int64_t batch,
                                 int32_t margin, int32_t flags, double* loss, float* grad, void* stream) {
    return guarded([&] {
        MMR_REQUIRE(net && r && e, "NULL argument");
        MMR_REQUIRE(nx > 2 * margin && ny > 2 * margin && batch > 0 && batch <= 65535 && margin >= 0, "bad shape");
        CnnNet& n = net->n;
        cudaStream_t st = as_stream(stream);
        const size_t bytes = (size_t)nx * ny * batch * 8;
        const float2* rin = (const float2*)stage_in(n.st_in, r, bytes, st);
        const float2* ein = (const float2*)stage_in(n.st_tgt, e, bytes, st);
        const bool cosine = flags & CNN_LOSS_COS;
        const bool relu = !(flags & CNN_LINEAR);
        const double L =
            (flags & CNN_FP32_ACT)
                ? loss_grad<float>(n, rin, ein, (int)nx, (int)ny, (int)batch, margin, cosine, relu, st)
                : loss_grad<__nv_bfloat16>(n, rin, ein, (int)nx, (int)ny, (int)batch, margin, cosine, relu, st);
        if (loss) *loss = L;
        if (grad) MMR_CUDA(cudaMemcpy(grad, n.grad.p, (size_t)n.nparam * 4, cudaMemcpyDeviceToHost));
    });
}

extern "C" int mmr_cnn_adam_step(mmr_cnn* net, float lr, void* stream) {
    return guarded([&] {
        MMR_REQUIRE(net && lr > 0, "bad argument");
        CnnNet& n = net->n;
        cudaStream_t st = as_stream(stream);
        ++n.adam_t;
        const float b1 = 0.9f, b2 = 0.999f;
        const float c1 = (float)(1.0 / (1.0 - std::pow(0.9, (double)n.adam_t)));
        const float c2 = (float)(1.0 / (1.0 - std::pow(0.999, (double)n.adam_t)));
        cnn_adam_kernel<<<(unsigned)cdiv(n.nparam, 256), 256, 0, st>>>(n.theta.as<float>(), n.grad.as<float>(),
                                                                        n.adam_m.as<float>(), n.adam_v.as<float>(),
                                                                        n.nparam, lr, b1, b2, 1e-8f, c1, c2);
        check_launch("cnn_adam");
        ++n.version;
    });
}

extern "C" int mmr_cnn_destroy(mmr_cnn* net) {
    return guarded([&] { delete net; });
}
