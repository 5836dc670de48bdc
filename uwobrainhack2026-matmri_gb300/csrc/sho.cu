// @sampHighOrder direct encoding on GB300.
//
// Phase (sampHighOrder.m:496-588, prepForDirect):
//   kbase[v, m] = sum_n SH_n(r_v) phs_spha[n, m]      (b0mask on n > 4, 564-566)
//               + sum_n conc_n(r_v) phs_conc[n, m]    (b0mask, 570-579)
//               + b0[v] b0mask[v] t[m]                (580-586)
// i.e. a real rank-K product B[V x K] P[K x M].  The plan forms B and P in
// FP64 (basisFuncHarm.m:24-96, basisFuncConc.m:13-23), evaluates kbase once
// on the device in FP64 and stores it reduced modulo 2*pi as FP32 "turns" in
// [-1/2, 1/2) (absolute phase error ~2e-7 rad even where |kbase| ~ 1e3 rad).
// Forward  y = exp(+i kbase.') x / sqrt(V)  (sampHighOrder.m:376, 387)
// adjoint  x = exp(-i kbase)   y / sqrt(V)  (sampHighOrder.m:371, 387)
// evaluate sincospi of the stored turns and accumulate in FP32.  Without room
// for the table the kernels evaluate kbase per element in FP64 (the
// no-precompute segmented approach 3, sampHighOrder.m:413-431).
#include <algorithm>
#include <cmath>

#include "sense.cuh"
#include "sho_interp.cuh"
#include "sho_tc.cuh"

namespace mmr {

struct ShoPlan {
    int nd = 0;
    long long imN[3] = {1, 1, 1};
    long long V = 0, M = 0;
    int K = 0;
    DevBuf d_B;     // double [K][V]
    DevBuf d_P;     // double [K][M]
    DevBuf d_turn;  // float  [V][M] (empty: on-the-fly FP64 phase)
    bool table = false;
    // with the table: 1 the tcgen05 contraction (sho_umma.cu), 2 the mma.sync contraction (sho_tc.cu),
    // 0 the SIMT kernels
    int tensor = 1;
    ShoTcScratch tc;
    ShoUmma umma;
    std::shared_ptr<ShoInterp> interp;   // approach 1 (sho_interp.cu); the fields above stay empty
    int nspha = 0, nconc = 0;
    // setPhiDiv (sampHighOrder.m:590-622): a derived plan that refers to `base` (not owned) and
    // holds the derivative phase d[v, m] = sum_j Bd[j][v] Pd[j][m] (prepForDirect with
    // sampTimes = 1, i.e. no B0 term; sampHighOrder.m:376-380)
    ShoPlan* base = nullptr;
    int Kd = 0;
    DevBuf d_Bd, d_Pd;      // double [Kd][V], [Kd][M]
    DevBuf s_X, s_T;        // scratch: [V, Kd * chunk], [M, Kd * chunk]
    Staged st_in, st_out;
};

long long sho_nvox(const ShoPlan& s) { return s.V; }
long long sho_nsamp(const ShoPlan& s) { return s.M; }

static double harm(int n, double x, double y, double z) {
    const double r2 = x * x + y * y + z * z;
    switch (n) {
        case 1: return 1.0;
        case 2: return x;
        case 3: return y;
        case 4: return z;
        case 5: return x * y;
        case 6: return z * y;
        case 7: return 3 * z * z - r2;
        case 8: return x * z;
        case 9: return x * x - y * y;
        case 10: return 3 * y * x * x - y * y * y;
        case 11: return x * z * y;
        case 12: return (5 * z * z - r2) * y;
        case 13: return 5 * z * z * z - 3 * z * r2;
        case 14: return (5 * z * z - r2) * x;
        case 15: return x * x * z - y * y * z;
        case 16: return x * x * x - 3 * x * y * y;
        case 17: return (x * y) * (x * x - y * y);
        case 18: return (y * z) * (3 * x * x - y * y);
        case 19: return (x * y) * (7 * z * z - r2);
        case 20: return y * (7 * z * z * z - 3 * z * r2);
        case 21: return 35 * z * z * z * z - 30 * z * z * r2 + 3 * r2 * r2;
        case 22: return x * (7 * z * z * z - 3 * z * r2);
        case 23: return (x * x - y * y) * (7 * z * z - r2);
        case 24: return x * (x * x - 3 * y * y) * z;
        case 25: return x * x * (x * x - 3 * y * y) - y * y * (3 * x * x - y * y);
        case 26: return y * (5 * x * x * x * x - 10 * x * x * y * y + y * y * y * y);
        case 27: return x * y * z * (x * x - y * y);
        case 28: return y * (r2 - 9 * z * z) * (y * y - 3 * x * x);
        case 29: return x * y * z * (3 * z * z - r2);
        case 30: return y * (r2 * r2 - 14 * r2 * z * z + 21 * z * z * z * z);
        case 31: return 63 * z * z * z * z * z - 70 * z * z * z * r2 + 15 * z * r2 * r2;
        case 32: return x * (r2 * r2 - 14 * r2 * z * z + 21 * z * z * z * z);
        case 33: return z * (3 * z * z - r2) * (x * x - y * y);
        case 34: return x * (r2 - 9 * z * z) * (3 * y * y - x * x);
        case 35: return z * (x * x * x * x - 6 * x * x * y * y + y * y * y * y);
        case 36: return x * x * x * x * x - 10 * x * x * x * y * y + 5 * x * y * y * y * y;
        default: return 0.0;
    }
}

static double conc(int n, double x, double y, double z) {
    switch (n) {
        case 1: return z * z;
        case 2: return x * x + y * y;
        case 3: return x * z;
        case 4: return y * z;
        default: return 0.0;
    }
}

__device__ __forceinline__ double sho_phase(const double* __restrict__ B, const double* __restrict__ P, int K,
                                            long long V, long long M, long long v, long long m) {
    double ph = 0.0;
    for (int k = 0; k < K; ++k) ph = fma(B[k * V + v], P[k * M + m], ph);
    return ph;
}

__device__ __forceinline__ float phase_turn(double ph) {
    double t = ph * 0.15915494309189533577;   // 1 / (2 pi)
    t -= rint(t);
    return (float)t;
}

__global__ void sho_table_kernel(const double* __restrict__ B, const double* __restrict__ P, int K, long long V,
                                 long long M, float* __restrict__ turn) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= V * M) return;
    const long long v = i / M, m = i - v * M;
    turn[i] = phase_turn(sho_phase(B, P, K, V, M, v, m));
}

// kbase[v + V (m - m0)] for samples m0 .. m0 + nm - 1, FP64 (the public kbase of prepForDirect).
__global__ void sho_kbase_kernel(const double* __restrict__ B, const double* __restrict__ P, int K, long long V,
                                 long long M, long long m0, long long nm, double* __restrict__ out) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= V * nm) return;
    const long long ml = i / V, v = i - ml * V;
    out[i] = sho_phase(B, P, K, V, M, v, m0 + ml);
}

// Forward: thread per sample m, CPT coils per thread, loop over voxels.
template <int CPT>
__global__ void __launch_bounds__(256) sho_fwd_kernel(const float* __restrict__ turn, const double* __restrict__ B,
                                                      const double* __restrict__ P, int K, long long V, long long M,
                                                      const float2* __restrict__ x, float2* __restrict__ y,
                                                      long long nb, float scale, const int* active) {
    if (active && *active) return;
    constexpr int VC = 32;
    __shared__ float2 xs[VC][CPT];
    const long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int c0 = blockIdx.y * CPT;
    float2 acc[CPT];
#pragma unroll
    for (int c = 0; c < CPT; ++c) acc[c] = make_float2(0.f, 0.f);
    for (long long v0 = 0; v0 < V; v0 += VC) {
        __syncthreads();
        for (int i = threadIdx.x; i < VC * CPT; i += blockDim.x) {
            const int vv = i / CPT, c = i - vv * CPT;
            const long long v = v0 + vv;
            xs[vv][c] = (v < V && c0 + c < nb) ? x[v + V * (c0 + c)] : make_float2(0.f, 0.f);
        }
        __syncthreads();
        if (m < M) {
            const int nv = (int)(V - v0 < VC ? V - v0 : VC);
            for (int vv = 0; vv < nv; ++vv) {
                const float t = turn ? turn[(v0 + vv) * M + m] : phase_turn(sho_phase(B, P, K, V, M, v0 + vv, m));
                float s, c;
                sincospif(2.f * t, &s, &c);
#pragma unroll
                for (int q = 0; q < CPT; ++q) {
                    const float2 xv = xs[vv][q];
                    acc[q].x += c * xv.x - s * xv.y;
                    acc[q].y += c * xv.y + s * xv.x;
                }
            }
        }
    }
    if (m < M) {
#pragma unroll
        for (int q = 0; q < CPT; ++q)
            if (c0 + q < nb) y[m + M * (c0 + q)] = make_float2(acc[q].x * scale, acc[q].y * scale);
    }
}

// Adjoint: thread per voxel v; the [256 v x 32 m] phase tile is staged through smem
// so that the table is read along m (coalesced).
template <int CPT>
__global__ void __launch_bounds__(256) sho_adj_kernel(const float* __restrict__ turn, const double* __restrict__ B,
                                                      const double* __restrict__ P, int K, long long V, long long M,
                                                      const float2* __restrict__ y, float2* __restrict__ x,
                                                      long long nb, float scale, const int* active) {
    if (active && *active) return;
    constexpr int MC = 32, VT = 256;
    __shared__ float tt[VT][MC + 1];
    __shared__ float2 ys[MC][CPT];
    const long long v0 = (long long)blockIdx.x * VT;
    const long long v = v0 + threadIdx.x;
    const int c0 = blockIdx.y * CPT;
    float2 acc[CPT];
#pragma unroll
    for (int c = 0; c < CPT; ++c) acc[c] = make_float2(0.f, 0.f);
    for (long long m0 = 0; m0 < M; m0 += MC) {
        __syncthreads();
        for (int i = threadIdx.x; i < VT * MC; i += blockDim.x) {
            const int vv = i / MC, mm = i - vv * MC;
            const long long vg = v0 + vv, mg = m0 + mm;
            float t = 0.f;
            if (vg < V && mg < M) t = turn ? turn[vg * M + mg] : phase_turn(sho_phase(B, P, K, V, M, vg, mg));
            tt[vv][mm] = t;
        }
        for (int i = threadIdx.x; i < MC * CPT; i += blockDim.x) {
            const int mm = i / CPT, c = i - mm * CPT;
            const long long mg = m0 + mm;
            ys[mm][c] = (mg < M && c0 + c < nb) ? y[mg + M * (c0 + c)] : make_float2(0.f, 0.f);
        }
        __syncthreads();
        if (v < V) {
            const int nm = (int)(M - m0 < MC ? M - m0 : MC);
            for (int mm = 0; mm < nm; ++mm) {
                float s, c;
                sincospif(2.f * tt[threadIdx.x][mm], &s, &c);
#pragma unroll
                for (int q = 0; q < CPT; ++q) {
                    const float2 yv = ys[mm][q];
                    acc[q].x += c * yv.x + s * yv.y;
                    acc[q].y += c * yv.y - s * yv.x;
                }
            }
        }
    }
    if (v < V) {
#pragma unroll
        for (int q = 0; q < CPT; ++q)
            if (c0 + q < nb) x[v + V * (c0 + q)] = make_float2(acc[q].x * scale, acc[q].y * scale);
    }
}

// X[:, j + Kd b] = Bd[j] .* x[:, b]
__global__ void phidiv_expand_kernel(const float2* __restrict__ x, const double* __restrict__ Bd,
                                     float2* __restrict__ X, long long V, int Kd, long long nb, const int* active) {
    if (active && *active) return;
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= V * Kd * nb) return;
    const long long v = i % V, col = i / V;
    const int j = (int)(col % Kd);
    const long long b = col / Kd;
    X[i] = cscale(x[v + V * b], (float)Bd[(size_t)j * V + v]);
}

// y[m, b] = i sum_j Pd[j][m] T[m, j + Kd b]   (sampHighOrder.m:377-380)
__global__ void phidiv_combine_kernel(const float2* __restrict__ T, const double* __restrict__ Pd,
                                      float2* __restrict__ y, long long M, int Kd, long long nb, const int* active) {
    if (active && *active) return;
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= M * nb) return;
    const long long m = i % M, b = i / M;
    float re = 0.f, im = 0.f;
    for (int j = 0; j < Kd; ++j) {
        const float p = (float)Pd[(size_t)j * M + m];
        const float2 t = T[m + M * (j + (long long)Kd * b)];
        re += p * t.x;
        im += p * t.y;
    }
    y[i] = make_float2(-im, re);
}

static void phidiv_forward(ShoPlan& s, const float2* x, float2* y, long long nb, cudaStream_t st,
                           const int* active) {
    const long long chunk = std::max<long long>(1, 256 / s.Kd);
    s.s_X.ensure((size_t)s.V * s.Kd * chunk * sizeof(float2));
    s.s_T.ensure((size_t)s.M * s.Kd * chunk * sizeof(float2));
    for (long long b0 = 0; b0 < nb; b0 += chunk) {
        const long long n = std::min(chunk, nb - b0);
        phidiv_expand_kernel<<<(unsigned)cdiv(s.V * s.Kd * n, 256), 256, 0, st>>>(
            x + s.V * b0, s.d_Bd.as<double>(), s.s_X.as<float2>(), s.V, s.Kd, n, active);
        check_launch("phidiv_expand");
        sho_forward(*s.base, s.s_X.as<float2>(), s.s_T.as<float2>(), s.Kd * n, st, active);
        phidiv_combine_kernel<<<(unsigned)cdiv(s.M * n, 256), 256, 0, st>>>(
            s.s_T.as<float2>(), s.d_Pd.as<double>(), y + s.M * b0, s.M, s.Kd, n, active);
        check_launch("phidiv_combine");
    }
}

void sho_forward(ShoPlan& s, const float2* x, float2* y, long long nb, cudaStream_t st, const int* active) {
    if (s.base) {
        phidiv_forward(s, x, y, nb, st, active);
        return;
    }
    if (s.interp) {
        sho_interp_forward(*s.interp, x, y, nb, st, active);
        return;
    }
    if (s.table && s.tensor == 1 && s.umma.ok && nb <= SHO_TC_MAX_COILS) {
        sho_umma_forward(s.umma, s.V, s.M, x, y, nb, st, active);
        return;
    }
    if (s.table && s.tensor && nb <= SHO_TC_MAX_COILS) {
        sho_tc_forward(s.tc, s.d_turn.as<float>(), s.V, s.M, x, y, nb, st, active);
        return;
    }
    const float scale = (float)(1.0 / std::sqrt((double)s.V));
    const float* tb = s.table ? s.d_turn.as<float>() : nullptr;
    const unsigned gx = (unsigned)cdiv(s.M, 256);
    if (nb > 4) {
        sho_fwd_kernel<16><<<dim3(gx, (unsigned)cdiv(nb, 16)), 256, 0, st>>>(
            tb, s.d_B.as<double>(), s.d_P.as<double>(), s.K, s.V, s.M, x, y, nb, scale, active);
    } else if (nb > 1) {
        sho_fwd_kernel<4><<<dim3(gx, (unsigned)cdiv(nb, 4)), 256, 0, st>>>(
            tb, s.d_B.as<double>(), s.d_P.as<double>(), s.K, s.V, s.M, x, y, nb, scale, active);
    } else {
        sho_fwd_kernel<1><<<dim3(gx, 1), 256, 0, st>>>(tb, s.d_B.as<double>(), s.d_P.as<double>(), s.K, s.V, s.M, x,
                                                       y, nb, scale, active);
    }
    check_launch("sho_fwd");
}

void sho_adjoint(ShoPlan& s, const float2* y, float2* x, long long nb, cudaStream_t st, const int* active) {
    if (s.base) {   // the adjoint ignores phiDiv (sampHighOrder.m:369-372)
        sho_adjoint(*s.base, y, x, nb, st, active);
        return;
    }
    if (s.interp) {
        sho_interp_adjoint(*s.interp, y, x, nb, st, active);
        return;
    }
    if (s.table && s.tensor == 1 && s.umma.ok && nb <= SHO_TC_MAX_COILS) {
        sho_umma_adjoint(s.umma, s.V, s.M, y, x, nb, st, active);
        return;
    }
    if (s.table && s.tensor && nb <= SHO_TC_MAX_COILS) {
        sho_tc_adjoint(s.tc, s.d_turn.as<float>(), s.V, s.M, y, x, nb, st, active);
        return;
    }
    const float scale = (float)(1.0 / std::sqrt((double)s.V));
    const float* tb = s.table ? s.d_turn.as<float>() : nullptr;
    const unsigned gx = (unsigned)cdiv(s.V, 256);
    if (nb > 4) {
        sho_adj_kernel<16><<<dim3(gx, (unsigned)cdiv(nb, 16)), 256, 0, st>>>(
            tb, s.d_B.as<double>(), s.d_P.as<double>(), s.K, s.V, s.M, y, x, nb, scale, active);
    } else if (nb > 1) {
        sho_adj_kernel<4><<<dim3(gx, (unsigned)cdiv(nb, 4)), 256, 0, st>>>(
            tb, s.d_B.as<double>(), s.d_P.as<double>(), s.K, s.V, s.M, y, x, nb, scale, active);
    } else {
        sho_adj_kernel<1><<<dim3(gx, 1), 256, 0, st>>>(tb, s.d_B.as<double>(), s.d_P.as<double>(), s.K, s.V, s.M, y,
                                                       x, nb, scale, active);
    }
    check_launch("sho_adj");
}

// E[m + M j] = exp(i kbase[vox[j], m])   (mrSampFuncMat.m:35-37 before the 1/sqrt scaling)
__global__ void sho_emat_kernel(const float* __restrict__ turn, const double* __restrict__ B,
                                const double* __restrict__ P, int K, long long V, long long M,
                                const long long* __restrict__ vox, long long nvox, float2* __restrict__ E) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= M * nvox) return;
    const long long m = i % M, v = vox[i / M];
    const float t = turn ? turn[v * M + m] : phase_turn(sho_phase(B, P, K, V, M, v, m));
    float sn, cs;
    sincospif(2.f * t, &sn, &cs);
    E[i] = make_float2(cs, sn);
}

void sho_encoding_matrix(ShoPlan& s, const long long* vox, long long nvox, float2* E, cudaStream_t st) {
    MMR_REQUIRE(!s.base && !s.interp, "the dense encoding needs a direct sampHighOrder plan");
    sho_emat_kernel<<<(unsigned)cdiv(s.M * nvox, 256), 256, 0, st>>>(s.table ? s.d_turn.as<float>() : nullptr,
                                                                     s.d_B.as<double>(), s.d_P.as<double>(), s.K,
                                                                     s.V, s.M, vox, nvox, E);
    check_launch("sho_emat");
}

// Operands of the dense Gram on the tensor cores: for mask voxel r (row) and sample k,
// op[p][r][k] (FP16) with p = cos hi, cos lo, sin hi, sin lo of exp(i kbase[vox[r], k]): hi =
// round(2^11 v), exact in FP16, lo = 2^11 v - hi.  Rows past nvox and samples past M are zero.
__global__ void sho_gram_operands_kernel(const float* __restrict__ turn, const double* __restrict__ B,
                                         const double* __restrict__ P, int K, long long V, long long M,
                                         const long long* __restrict__ vox, long long nvox, long long rows,
                                         long long kpad, __half* __restrict__ op) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= rows * kpad) return;
    const long long r = i / kpad, k = i - r * kpad;
    float ch = 0.f, cl = 0.f, sh = 0.f, sl = 0.f;
    if (r < nvox && k < M) {
        const long long v = vox[r];
        const float t = turn ? turn[v * M + k] : phase_turn(sho_phase(B, P, K, V, M, v, k));
        float sn, cs;
        sincospif(2.f * t, &sn, &cs);
        ch = rintf(cs * 2048.f);
        cl = fmaf(cs, 2048.f, -ch);
        sh = rintf(sn * 2048.f);
        sl = fmaf(sn, 2048.f, -sh);
    }
    const size_t plane = (size_t)rows * kpad;
    op[i] = __float2half_rn(ch);
    op[i + plane] = __float2half_rn(cl);
    op[i + 2 * plane] = __float2half_rn(sh);
    op[i + 3 * plane] = __float2half_rn(sl);
}

void sho_gram_operands(ShoPlan& s, const long long* vox, long long nvox, long long rows, long long kpad, __half* op,
                       cudaStream_t st) {
    MMR_REQUIRE(!s.base && !s.interp, "the dense encoding needs a direct sampHighOrder plan");
    sho_gram_operands_kernel<<<(unsigned)cdiv(rows * kpad, 256), 256, 0, st>>>(
        s.table ? s.d_turn.as<float>() : nullptr, s.d_B.as<double>(), s.d_P.as<double>(), s.K, s.V, s.M, vox, nvox,
        rows, kpad, op);
    check_launch("sho_gram_operands");
}

static void sho_build(ShoPlan& s, const mmr_sho_desc& d) {
    MMR_REQUIRE(d.ndim >= 1 && d.ndim <= 3, "ndim must be 1..3");
    MMR_REQUIRE(d.nsamp >= 1 && d.t && d.spha && d.gx && d.gy && d.gz, "missing sampHighOrder input");
    MMR_REQUIRE(d.nspha >= 0 && d.nspha <= 36 && d.nconc >= 0 && d.nconc <= 4, "nspha <= 36, nconc <= 4");
    MMR_REQUIRE(d.nconc == 0 || d.conc, "conc is NULL");
    s.nd = d.ndim;
    s.V = 1;
    for (int k = 0; k < d.ndim; ++k) {
        MMR_REQUIRE(d.imN[k] >= 1, "bad image size");
        s.imN[k] = d.imN[k];
        s.V *= d.imN[k];
    }
    s.M = d.nsamp;
    s.nspha = d.nspha;
    s.nconc = d.nconc;
    const bool with_b0 = s.M > 1;                                          // 580
    s.K = d.nspha + d.nconc + (with_b0 ? 1 : 0);
    MMR_REQUIRE(s.K >= 1, "no phase terms");
    std::vector<double> B((size_t)s.K * s.V), P((size_t)s.K * s.M);
    int k = 0;
    for (int n = 1; n <= d.nspha; ++n, ++k) {                              // 560-569
        for (long long v = 0; v < s.V; ++v) {
            double b = harm(n, d.gx[v], d.gy[v], d.gz[v]);
            if (n > 4 && d.mask) b *= d.mask[v];
            B[(size_t)k * s.V + v] = b;
        }
        for (long long m = 0; m < s.M; ++m) P[(size_t)k * s.M + m] = d.spha[(n - 1) + (size_t)d.nspha * m];
    }
    for (int n = 1; n <= d.nconc; ++n, ++k) {                              // 570-579
        for (long long v = 0; v < s.V; ++v) {
            double b = conc(n, d.gx[v], d.gy[v], d.gz[v]);
            if (d.mask) b *= d.mask[v];
            B[(size_t)k * s.V + v] = b;
        }
        for (long long m = 0; m < s.M; ++m) P[(size_t)k * s.M + m] = d.conc[(n - 1) + (size_t)d.nconc * m];
    }
    if (with_b0) {                                                          // 580-586
        for (long long v = 0; v < s.V; ++v) {
            double b = d.b0 ? d.b0[v] : 0.0;
            if (d.mask) b *= d.mask[v];
            B[(size_t)k * s.V + v] = b;
        }
        for (long long m = 0; m < s.M; ++m) P[(size_t)k * s.M + m] = d.t[m];
        ++k;
    }
    for (double v : B) MMR_REQUIRE(std::isfinite(v), "non-finite basis value (check grid / b0 / mask)");
    for (double v : P) MMR_REQUIRE(std::isfinite(v), "non-finite phase coefficient");
    s.d_B.upload(B);
    s.d_P.upload(P);
    // Phase table: up to 8 GiB, and at most a quarter of the free memory.
    size_t fr = 0, tot = 0;
    MMR_CUDA(cudaMemGetInfo(&fr, &tot));
    const size_t bytes = (size_t)s.V * s.M * sizeof(float);
    s.table = bytes <= (8ull << 30) && bytes <= fr / 4;
    if (s.table) {
        s.d_turn.ensure(bytes);
        const long long n = s.V * s.M;
        sho_table_kernel<<<(unsigned)cdiv(n, 256), 256>>>(s.d_B.as<double>(), s.d_P.as<double>(), s.K, s.V, s.M,
                                                          s.d_turn.as<float>());
        check_launch("sho_table");
        MMR_CUDA(cudaDeviceSynchronize());
        sho_tc_alloc(s.tc, s.V, s.M);
        sho_umma_prepare(s.umma, s.d_turn.as<float>(), s.V, s.M);
    }
}

}  // namespace mmr

using namespace mmr;

extern "C" int mmr_sho_create(const mmr_sho_desc* desc, mmr_sho** out) {
    return guarded([&] {
        MMR_REQUIRE(desc && out, "NULL argument");
        *out = nullptr;
        auto* s = new ShoPlan();
        try {
            sho_build(*s, *desc);
        } catch (...) {
            delete s;
            throw;
        }
        *out = reinterpret_cast<mmr_sho*>(s);
    });
}

extern "C" int mmr_sho_interp_create(const mmr_sho_interp_desc* desc, mmr_sho** out) {
    return guarded([&] {
        MMR_REQUIRE(desc && out, "NULL argument");
        *out = nullptr;
        auto* s = new ShoPlan();
        try {
            s->interp = sho_interp_build(*desc);
            s->nd = 2;
            s->imN[0] = desc->imN[0];
            s->imN[1] = desc->imN[1];
            s->V = sho_interp_nvox(*s->interp);
            s->M = sho_interp_nsamp(*s->interp);
            s->tensor = 0;
        } catch (...) {
            delete s;
            throw;
        }
        *out = reinterpret_cast<mmr_sho*>(s);
    });
}

extern "C" int mmr_sho_kbase(const mmr_sho* h, double* kbase) {
    return guarded([&] {
        MMR_REQUIRE(h && kbase, "NULL argument");
        const ShoPlan* s = reinterpret_cast<const ShoPlan*>(h);
        if (s->base) s = s->base;   // setPhiDiv keeps the base encoding's kbase (sampHighOrder.m:590-622)
        MMR_REQUIRE(!s->interp, "kbase is not formed by the interpolated approach");
        const long long V = s->V, M = s->M;
        // sample chunks of at most 32 Mi values (256 MiB) through one device buffer
        const long long nm_max = std::max<long long>(1, std::min<long long>(M, (32LL << 20) / std::max<long long>(V, 1)));
        DevBuf buf;
        buf.ensure((size_t)V * nm_max * sizeof(double));
        for (long long m0 = 0; m0 < M; m0 += nm_max) {
            const long long nm = std::min(nm_max, M - m0);
            sho_kbase_kernel<<<(unsigned)cdiv(V * nm, 256), 256>>>(s->d_B.as<double>(), s->d_P.as<double>(), s->K, V, M,
                                                                   m0, nm, buf.as<double>());
            check_launch("sho_kbase");
            MMR_CUDA(cudaMemcpy(kbase + (size_t)V * m0, buf.p, (size_t)V * nm * sizeof(double), cudaMemcpyDeviceToHost));
        }
    });
}

extern "C" int mmr_sho_phidiv_create(mmr_sho* base_h, int32_t nspha, int32_t nconc, const double* kspha_div,
                                     const double* kconc_div, mmr_sho** out) {
    return guarded([&] {
        MMR_REQUIRE(base_h && out, "NULL argument");
        *out = nullptr;
        ShoPlan& b = *reinterpret_cast<ShoPlan*>(base_h);
        MMR_REQUIRE(!b.base, "the base plan already carries phiDiv");
        MMR_REQUIRE(!b.interp, "phiDiv not yet implemented for interpolated approach");   // sampHighOrder.m:340-342
        MMR_REQUIRE(nspha >= 0 && nconc >= 0 && nspha + nconc >= 1, "no phiDiv terms");
        MMR_REQUIRE(nspha <= b.nspha && nconc <= b.nconc,
                    "phiDiv has more terms than the plan's phs_spha / phs_conc");
        MMR_REQUIRE((nspha == 0 || kspha_div) && (nconc == 0 || kconc_div), "missing phiDiv coefficients");
        auto* s = new ShoPlan();
        try {
            s->base = &b;
            s->nd = b.nd;
            for (int k = 0; k < 3; ++k) s->imN[k] = b.imN[k];
            s->V = b.V;
            s->M = b.M;
            s->Kd = nspha + nconc;
            std::vector<double> Pd((size_t)s->Kd * s->M);
            for (int j = 0; j < nspha; ++j)
                for (long long m = 0; m < s->M; ++m) Pd[(size_t)j * s->M + m] = kspha_div[j + (size_t)nspha * m];
            for (int j = 0; j < nconc; ++j)
                for (long long m = 0; m < s->M; ++m)
                    Pd[(size_t)(nspha + j) * s->M + m] = kconc_div[j + (size_t)nconc * m];
            for (double v : Pd) MMR_REQUIRE(std::isfinite(v), "non-finite phiDiv coefficient");
            s->d_Pd.upload(Pd);
            // basis columns of the base plan: spherical harmonics 1..nspha, concomitant 1..nconc
            s->d_Bd.ensure((size_t)s->Kd * s->V * sizeof(double));
            const size_t col = (size_t)s->V * sizeof(double);
            if (nspha)
                MMR_CUDA(cudaMemcpy(s->d_Bd.p, b.d_B.p, (size_t)nspha * col, cudaMemcpyDeviceToDevice));
            if (nconc)
                MMR_CUDA(cudaMemcpy((char*)s->d_Bd.p + (size_t)nspha * col, (char*)b.d_B.p + (size_t)b.nspha * col,
                                    (size_t)nconc * col, cudaMemcpyDeviceToDevice));
        } catch (...) {
            delete s;
            throw;
        }
        *out = reinterpret_cast<mmr_sho*>(s);
    });
}

extern "C" int mmr_sho_apply(mmr_sho* h, int adjoint, const void* in, void* out, int64_t nbatch, void* stream) {
    return guarded([&] {
        MMR_REQUIRE(h && in && out && nbatch >= 1, "bad argument");
        ShoPlan& s = *reinterpret_cast<ShoPlan*>(h);
        cudaStream_t st = as_stream(stream);
        const size_t bv = (size_t)s.V * nbatch * 8, bm = (size_t)s.M * nbatch * 8;
        const float2* din = (const float2*)stage_in(s.st_in, in, adjoint ? bm : bv, st);
        float2* dout = (float2*)stage_out(s.st_out, out, adjoint ? bv : bm);
        if (adjoint) sho_adjoint(s, din, dout, nbatch, st, nullptr);
        else sho_forward(s, din, dout, nbatch, st, nullptr);
        finish_out(s.st_out, adjoint ? bv : bm, st);
        if (s.interp && s.st_out.host && device_error_word(st))
            MMR_THROW(MMR_ERR_TIMEOUT, "a bounded device wait ran out");
    });
}

extern "C" int mmr_sho_set_tensor(mmr_sho* h, int on) {
    return guarded([&] {
        MMR_REQUIRE(h, "NULL argument");
        MMR_REQUIRE(on >= 0 && on <= 2, "tensor mode must be 0 (SIMT), 1 (tcgen05) or 2 (mma.sync)");
        reinterpret_cast<ShoPlan*>(h)->tensor = on;
    });
}

extern "C" int mmr_sho_destroy(mmr_sho* h) {
    return guarded([&] { delete reinterpret_cast<ShoPlan*>(h); });
}
