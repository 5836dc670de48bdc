// sampHighOrder encoding on the tensor cores (mma.sync m16n8k16, FP16 split
// operands, FP32 accumulation).
//
// Forward  y[m, c] = sum_v exp(+i 2 pi t[v, m]) x[v, c]   (sampHighOrder.m:376)
// adjoint  x[v, c] = sum_m exp(-i 2 pi t[v, m]) y[m, c]   (sampHighOrder.m:371)
// with t the stored phase in turns and the 1/sqrt(V) of sampHighOrder.m:387.
// As a real GEMM: rows = outputs (samples / voxels), K = 2 x inputs (cos and
// sin of each input element, interleaved), N = 2 x coils (real parts, then
// imaginary parts):
//   forward  A[m, 2v..2v+1] = (cos, sin)   B[2v, c] = x_r    B[2v+1, c] = -x_i
//                                          B[2v, C+c] = x_i  B[2v+1, C+c] = x_r
//   adjoint  A[v, 2m..2m+1] = (cos, sin)   B[2m, c] = y_r    B[2m+1, c] = y_i
//                                          B[2m, C+c] = y_i  B[2m+1, C+c] = -y_r
// The A fragments are generated in registers (table read, sincospif, split)
// and never stored.  Precision: every operand is split into an FP16 high part
// and a low part scaled by 2^11 (the input columns first normalised to max 1),
// and three products hi*hi + (hi*lo' + lo'*hi) / 2^11 are accumulated in FP32,
// i.e. ~22-bit operands, FP32-level results (error vs FP64 in the tests).
// Work split: a warp owns 16 TC_MTW output rows x 8 NT columns and loads the
// phases of the next K step while it works on the current one; the K range is
// split over gridDim.y CTAs whose partial sums a second kernel adds in a fixed
// order.  The tensor-core accumulators are promoted into FP32 register sums
// every TC_PROMOTE K steps.
#include <algorithm>
#include <cmath>

#include <cuda_fp16.h>

#include "sho_tc.cuh"

namespace mmr {

constexpr int TC_WARPS = 4;            // warps per CTA
constexpr int TC_MTW = 1;              // m16 tiles per warp (one keeps registers low, occupancy high)
constexpr int TC_ROWS = 16 * TC_MTW * TC_WARPS; // output rows per CTA
constexpr float TC_LO = 2048.f;        // scale of the low parts
constexpr int TC_PROMOTE = 8;          // K steps (of 8 inputs) per tensor-core accumulation

__device__ __forceinline__ void mma16816(float (&c)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3,
                                         uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

__device__ __forceinline__ uint32_t pack_h2(__half a, __half b) {
    __half2 h = __halves2half2(a, b);
    return *reinterpret_cast<uint32_t*>(&h);
}

// (cos, sin) of one phase as the hi and lo' halves of an A register pair.
__device__ __forceinline__ void cs_split(float turn, uint32_t& hi, uint32_t& lo) {
    float s, c;
    sincospif(2.f * turn, &s, &c);
    const __half ch = __float2half_rn(c), sh = __float2half_rn(s);
    const __half cl = __float2half_rn((c - __half2float(ch)) * TC_LO);
    const __half sl = __float2half_rn((s - __half2float(sh)) * TC_LO);
    hi = pack_h2(ch, sh);
    lo = pack_h2(cl, sl);
}

// Per-column max |re|, |im| of in[L, nb] (complex), as float bits (non-negative floats
// order like their bit patterns); cmax zeroed by the caller.
__global__ void sho_tc_colmax_kernel(const float2* __restrict__ in, long long L, int nb, unsigned* __restrict__ cmax,
                                     const int* active) {
    if (active && *active) return;
    const int c = blockIdx.y;
    float m = 0.f;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < L; i += (long long)gridDim.x * blockDim.x) {
        const float2 v = in[i + L * c];
        m = fmaxf(m, fmaxf(fabsf(v.x), fabsf(v.y)));
    }
    for (int o = 16; o; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(cmax + c, __float_as_uint(m));
}

// Bt_hi / Bt_lo [N = 8 NT][K] (halves, k contiguous, row stride K) for coils c0 .. c0 + 4 NT - 1 of
// in[L, nb]; entries k >= 2 L stay zero.
template <bool ADJ>
__global__ void sho_tc_prep_kernel(const float2* __restrict__ in, long long L, long long K, int nb, int c0, int ncg,
                                   const unsigned* __restrict__ cmax, __half* __restrict__ bhi,
                                   __half* __restrict__ blo, const int* active) {
    if (active && *active) return;
    const int cl = blockIdx.y;        // coil within the group
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (2 * i >= K) return;
    const int c = c0 + cl;
    float2 v = make_float2(0.f, 0.f);
    float inv = 0.f;
    if (c < nb && i < L) {   // the padding up to K is rewritten with zeros
        const float mx = __uint_as_float(cmax[c]);
        inv = mx > 0.f ? 1.f / mx : 0.f;
        v = in[i + L * c];
    }
    const float re = v.x * inv, im = v.y * inv;
    // rows c (real part of the output) and ncg + c (imaginary part), at k = 2i, 2i+1
    const float r0a = re, r0b = ADJ ? im : -im;      // B[2i, c], B[2i+1, c]
    const float r1a = im, r1b = ADJ ? -re : re;      // B[2i, C+c], B[2i+1, C+c]
    auto put = [&](int row, float a, float b) {
        const __half ah = __float2half_rn(a), bh = __float2half_rn(b);
        const __half al = __float2half_rn((a - __half2float(ah)) * TC_LO);
        const __half bl = __float2half_rn((b - __half2float(bh)) * TC_LO);
        *reinterpret_cast<__half2*>(bhi + row * K + 2 * i) = __halves2half2(ah, bh);
        *reinterpret_cast<__half2*>(blo + row * K + 2 * i) = __halves2half2(al, bl);
    };
    put(cl, r0a, r0b);
    put(ncg + cl, r1a, r1b);
}

// partial[split][row][8 NT] = sum over this split's K range of A[row, k] B[k, n]
// (hi*hi + (hi*lo' + lo'*hi) / 2^11).  turn is the [V][M] phase table; B rows have stride K,
// zero beyond 2 L, so the reads of the last (partial) K step stay in the buffer.
template <bool ADJ, int NT>
__global__ void __launch_bounds__(TC_WARPS * 32) sho_tc_kernel(const float* __restrict__ turn,
                                                               const __half* __restrict__ bhi,
                                                               const __half* __restrict__ blo,
                                                               float* __restrict__ partial, long long R, long long L,
                                                               long long K, long long M, long long kchunk,
                                                               const int* active) {
    if (active && *active) return;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int gid = lane >> 2, tig = lane & 3;
    const long long row0 = (long long)blockIdx.x * TC_ROWS + warp * (16 * TC_MTW);
    const long long i0 = (long long)blockIdx.y * kchunk;             // first input element of this split
    const long long i1 = i0 + kchunk < L ? i0 + kchunk : L;
    // acc0 / acc1: the tensor-core accumulators of the current TC_PROMOTE K steps; tot: their sum,
    // added on the FP32 pipe, so that no tensor-core accumulation runs over more than
    // TC_PROMOTE x 16 products (its internal alignment of the addends costs accuracy as the
    // accumulator grows)
    float acc0[TC_MTW][NT][4], acc1[TC_MTW][NT][4], tot[TC_MTW][NT][4];
#pragma unroll
    for (int m = 0; m < TC_MTW; ++m)
#pragma unroll
        for (int n = 0; n < NT; ++n)
#pragma unroll
            for (int j = 0; j < 4; ++j) acc0[m][n][j] = acc1[m][n][j] = tot[m][n][j] = 0.f;
    int steps = 0;
    // rows handled by this thread: row0 + 16 m + gid (+8)
    long long rows[TC_MTW][2];
#pragma unroll
    for (int m = 0; m < TC_MTW; ++m) {
        rows[m][0] = row0 + 16 * m + gid;
        rows[m][1] = rows[m][0] + 8;
    }
    // phases of the next K step, loaded one step ahead to hide the table latency
    auto load_turns = [&](long long ib, float (&t)[TC_MTW][4]) {
#pragma unroll
        for (int m = 0; m < TC_MTW; ++m)
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const long long rr = rows[m][q & 1];
                const long long ii = ib + tig + (q >> 1) * 4;
                t[m][q] = (rr < R && ii < i1) ? (ADJ ? turn[rr * M + ii] : turn[ii * M + rr]) : 0.f;
            }
    };
    float tnext[TC_MTW][4];
    load_turns(i0, tnext);
    for (long long ib = i0; ib < i1; ib += 8) {
        float tcur[TC_MTW][4];
#pragma unroll
        for (int m = 0; m < TC_MTW; ++m)
#pragma unroll
            for (int q = 0; q < 4; ++q) tcur[m][q] = tnext[m][q];
        if (ib + 8 < i1) load_turns(ib + 8, tnext);
        // A fragments: inputs ib + tig (k = 2 tig, 2 tig + 1) and ib + tig + 4 (k + 8)
        uint32_t ah[TC_MTW][4], al[TC_MTW][4];
#pragma unroll
        for (int m = 0; m < TC_MTW; ++m) {
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const long long rr = rows[m][q & 1];
                const long long ii = ib + tig + (q >> 1) * 4;
                uint32_t h, l;
                cs_split(tcur[m][q], h, l);
                if (!(rr < R && ii < i1)) h = l = 0u;
                ah[m][q] = h;
                al[m][q] = l;
            }
        }
        const long long k0 = 2 * ib + 2 * tig;
#pragma unroll
        for (int n = 0; n < NT; ++n) {
            const long long boff = (long long)(n * 8 + gid) * K + k0;
            const uint32_t bh0 = *reinterpret_cast<const uint32_t*>(bhi + boff);
            const uint32_t bh1 = *reinterpret_cast<const uint32_t*>(bhi + boff + 8);
            const uint32_t bl0 = *reinterpret_cast<const uint32_t*>(blo + boff);
            const uint32_t bl1 = *reinterpret_cast<const uint32_t*>(blo + boff + 8);
#pragma unroll
            for (int m = 0; m < TC_MTW; ++m) {
                mma16816(acc0[m][n], ah[m][0], ah[m][1], ah[m][2], ah[m][3], bh0, bh1);
                mma16816(acc1[m][n], ah[m][0], ah[m][1], ah[m][2], ah[m][3], bl0, bl1);
                mma16816(acc1[m][n], al[m][0], al[m][1], al[m][2], al[m][3], bh0, bh1);
            }
        }
        if (++steps == TC_PROMOTE || ib + 8 >= i1) {
            steps = 0;
#pragma unroll
            for (int m = 0; m < TC_MTW; ++m)
#pragma unroll
                for (int n = 0; n < NT; ++n)
#pragma unroll
                    for (int j = 0; j < 4; ++j) {
                        tot[m][n][j] += acc0[m][n][j] + acc1[m][n][j] * (1.f / TC_LO);
                        acc0[m][n][j] = acc1[m][n][j] = 0.f;
                    }
        }
    }
    float* out = partial + (long long)blockIdx.y * R * (8 * NT);
#pragma unroll
    for (int m = 0; m < TC_MTW; ++m)
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const long long rr = rows[m][h];
            if (rr >= R) continue;
#pragma unroll
            for (int n = 0; n < NT; ++n)
                *reinterpret_cast<float2*>(out + rr * (8 * NT) + n * 8 + 2 * tig) =
                    make_float2(tot[m][n][2 * h], tot[m][n][2 * h + 1]);
        }
}

// out[row + R c] = scale * max|in_c| * (sum_split partial[row][c] + i partial[row][ncg + c])
template <int NT>
__global__ void sho_tc_reduce_kernel(const float* __restrict__ partial, int nsplit, long long R, int nb, int c0,
                                     const unsigned* __restrict__ cmax, float scale, float2* __restrict__ out,
                                     const int* active) {
    if (active && *active) return;
    constexpr int NCG = 4 * NT;
    const long long row = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int cl = blockIdx.y;
    const int c = c0 + cl;
    if (row >= R || c >= nb) return;
    double re = 0, im = 0;
    for (int s = 0; s < nsplit; ++s) {
        const float* p = partial + ((long long)s * R + row) * (8 * NT);
        re += p[cl];
        im += p[NCG + cl];
    }
    const float f = scale * __uint_as_float(cmax[c]);
    out[row + R * c] = make_float2((float)re * f, (float)im * f);
}

static int tc_nsplit(long long R, long long L) {
    const long long rblocks = cdiv(R, TC_ROWS);
    const long long want = cdiv(4LL * device_sm_count(), rblocks);     // about four CTAs per SM
    return (int)std::max<long long>(1, std::min<long long>(want, cdiv(L, 512)));
}

void sho_tc_alloc(ShoTcScratch& s, long long V, long long M) {
    s.kpad = 2 * cdiv(std::max(V, M), 8) * 8;
    const size_t bbytes = (size_t)32 * s.kpad * sizeof(__half);
    s.bhi.ensure(bbytes);
    s.blo.ensure(bbytes);
    MMR_CUDA(cudaMemset(s.bhi.p, 0, bbytes));
    MMR_CUDA(cudaMemset(s.blo.p, 0, bbytes));
    s.nsplit[0] = tc_nsplit(M, V);
    s.nsplit[1] = tc_nsplit(V, M);
    const size_t pf = (size_t)s.nsplit[0] * M, pa = (size_t)s.nsplit[1] * V;
    s.partial.ensure(std::max(pf, pa) * 32 * sizeof(float));
    s.cmax.ensure((size_t)SHO_TC_MAX_COILS * sizeof(unsigned));
}

// y (adjoint = false: [M, nb]) or x (adjoint = true: [V, nb]) from the phase table.
template <bool ADJ>
static void sho_tc_apply(ShoTcScratch& s, const float* turn, long long V, long long M, const float2* in,
                         float2* out, long long nb, cudaStream_t st, const int* active) {
    MMR_REQUIRE(nb >= 1 && nb <= SHO_TC_MAX_COILS, "tensor-core encoding handles 1..%lld columns", SHO_TC_MAX_COILS);
    const long long R = ADJ ? V : M;     // output rows
    const long long L = ADJ ? M : V;     // inputs (K = 2 L, stored with the padded stride kpad)
    const long long K = s.kpad;
    MMR_CUDA(cudaMemsetAsync(s.cmax.p, 0, (size_t)nb * sizeof(unsigned), st));
    sho_tc_colmax_kernel<<<dim3((unsigned)std::min<long long>(cdiv(L, 256), 256), (unsigned)nb), 256, 0, st>>>(
        in, L, (int)nb, s.cmax.as<unsigned>(), active);
    check_launch("sho_tc_colmax");
    const int NT = nb <= 4 ? 1 : (nb <= 8 ? 2 : 4);
    const int ncg = 4 * NT;
    const int nsplit = s.nsplit[ADJ ? 1 : 0];
    const long long kchunk = cdiv(cdiv(L, nsplit), 8) * 8;
    const float scale = (float)(1.0 / std::sqrt((double)V));
    __half* bh = s.bhi.as<__half>();
    __half* bl = s.blo.as<__half>();
    float* part = s.partial.as<float>();
    const unsigned* cm = s.cmax.as<unsigned>();
    for (long long c0 = 0; c0 < nb; c0 += ncg) {
        sho_tc_prep_kernel<ADJ><<<dim3((unsigned)cdiv(K / 2, 256), (unsigned)ncg), 256, 0, st>>>(
            in, L, K, (int)nb, (int)c0, ncg, cm, bh, bl, active);
        check_launch("sho_tc_prep");
        const dim3 grid((unsigned)cdiv(R, TC_ROWS), (unsigned)nsplit);
        const dim3 rg((unsigned)cdiv(R, 256), (unsigned)ncg);
        if (NT == 1) {
            sho_tc_kernel<ADJ, 1><<<grid, TC_WARPS * 32, 0, st>>>(turn, bh, bl, part, R, L, K, M, kchunk, active);
            check_launch("sho_tc");
            sho_tc_reduce_kernel<1><<<rg, 256, 0, st>>>(part, nsplit, R, (int)nb, (int)c0, cm, scale, out, active);
        } else if (NT == 2) {
            sho_tc_kernel<ADJ, 2><<<grid, TC_WARPS * 32, 0, st>>>(turn, bh, bl, part, R, L, K, M, kchunk, active);
            check_launch("sho_tc");
            sho_tc_reduce_kernel<2><<<rg, 256, 0, st>>>(part, nsplit, R, (int)nb, (int)c0, cm, scale, out, active);
        } else {
            sho_tc_kernel<ADJ, 4><<<grid, TC_WARPS * 32, 0, st>>>(turn, bh, bl, part, R, L, K, M, kchunk, active);
            check_launch("sho_tc");
            sho_tc_reduce_kernel<4><<<rg, 256, 0, st>>>(part, nsplit, R, (int)nb, (int)c0, cm, scale, out, active);
        }
        check_launch("sho_tc_reduce");
    }
}

void sho_tc_forward(ShoTcScratch& s, const float* turn, long long V, long long M, const float2* x, float2* y,
                    long long nb, cudaStream_t st, const int* active) {
    sho_tc_apply<false>(s, turn, V, M, x, y, nb, st, active);
}

void sho_tc_adjoint(ShoTcScratch& s, const float* turn, long long V, long long M, const float2* y, float2* x,
                    long long nb, cudaStream_t st, const int* active) {
    sho_tc_apply<true>(s, turn, V, M, y, x, nb, st, active);
}

}  // namespace mmr
