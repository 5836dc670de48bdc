// Hand-written mixed-radix Stockham FFT passes in shared memory (sm_103a).
//
// A "pass" transforms every line of an array along one axis.  The array is
// viewed as [inner, n_axis, outer] (column-major: `inner` is the product of
// the dims before the axis, `outer` the product after it).  Input position
// t < nin holds natural index (in_start + t) mod L; output position t < nout
// takes natural index (out_start + t) mod L.  This expresses, without data
// movement, the zero padding "at the end" of ifftnc(..., sz) (general/ifftnc.m:102-104),
// the crop 1:imN of nufftOp.m:366-372, the image-centering phase ramp
// fftShiftArray (nufftOp.m:258-272, a pure index shift of N/2 plus the
// constant exp(i*pi*N/2)), and the fft-shifted ("centered") storage of the
// oversampled grid used by the gridding kernels.
#pragma once

#include <cuda_runtime.h>

#include "common.h"

namespace mmr {

constexpr int FFT_MAX_STAGES = 12;

struct FftFactors {
    int L = 0;
    int nstage = 0;
    int radix[FFT_MAX_STAGES] = {0};
};

FftFactors fft_factorize(int L);            // radices from {8,4,2,3,5,7}
const float2* fft_twiddles(int L);          // device table e^{-2 pi i m / L}, m < L (cached)

enum PassMode : int {
    PASS_PLAIN = 0,     // value = in[...] * in_fac[t]
    PASS_FWD_IMG = 1    // value = img[t, line % lpc] * maps[t, c0*lpc + line] * in_fac[t]
};

struct PassArgs {
    const float2* in = nullptr;
    float2* out = nullptr;
    const float2* maps = nullptr;   // FWD_IMG
    const float2* in_fac = nullptr; // per input position (nullable)
    const float2* out_fac = nullptr;// per output position (nullable)
    const float2* in_line = nullptr;  // per input line, indexed by line % lpc (contiguous passes; nullable)
    const float2* out_line = nullptr; // per output line, indexed by the inner index (strided passes; nullable)
    const float2* tw = nullptr;
    const int* active = nullptr;    // solver "finished" flag: skip when *active != 0
    long long inner = 1;            // product of dims before the axis
    long long outer = 1;            // product of dims after the axis (lines = inner*outer)
    long long lpc = 1;              // FWD_IMG / in_line: lines per coil (image lines)
    int L = 0;
    int nin = 0, in_start = 0;
    int nout = 0, out_start = 0;
    int sign = -1;                  // -1: e^{-i} (fft), +1: e^{+i} (ifft)
    float scale = 1.f;
    int B = 1;                      // lines per block (power of two)
    FftFactors f;
};

// ------------------------------------------------------------ complex math ----
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cmulc(float2 a, float2 b) {   // a * conj(b)
    return make_float2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
// multiply by sign*i  (sign = -1 -> -i, +1 -> +i)
__device__ __forceinline__ float2 cmul_si(float2 a, int sign) {
    return sign < 0 ? make_float2(a.y, -a.x) : make_float2(-a.y, a.x);
}

// ------------------------------------------------------------- butterflies ----
template <int SIGN>
__device__ __forceinline__ void dft2(float2& a, float2& b) {
    float2 t = a;
    a = cadd(t, b);
    b = csub(t, b);
}

template <int SIGN>
__device__ __forceinline__ void dft4(float2* v) {
    float2 a0 = cadd(v[0], v[2]), a1 = csub(v[0], v[2]);
    float2 a2 = cadd(v[1], v[3]), a3 = cmul_si(csub(v[1], v[3]), SIGN);
    v[0] = cadd(a0, a2);
    v[2] = csub(a0, a2);
    v[1] = cadd(a1, a3);
    v[3] = csub(a1, a3);
}

template <int SIGN>
__device__ __forceinline__ void dft8(float2* v) {
    const float h = 0.70710678118654752440f;
    float2 e[4] = {v[0], v[2], v[4], v[6]};
    float2 o[4] = {v[1], v[3], v[5], v[7]};
    dft4<SIGN>(e);
    dft4<SIGN>(o);
    // twiddles w8^k, k = 0..3, w8 = e^{SIGN i pi/4}
    float2 t1 = make_float2(h * (o[1].x - SIGN * o[1].y), h * (o[1].y + SIGN * o[1].x));
    float2 t2 = cmul_si(o[2], SIGN);
    float2 t3 = make_float2(h * (-o[3].x - SIGN * o[3].y), h * (-o[3].y + SIGN * o[3].x));
    v[0] = cadd(e[0], o[0]);
    v[4] = csub(e[0], o[0]);
    v[1] = cadd(e[1], t1);
    v[5] = csub(e[1], t1);
    v[2] = cadd(e[2], t2);
    v[6] = csub(e[2], t2);
    v[3] = cadd(e[3], t3);
    v[7] = csub(e[3], t3);
}

// Direct DFT for the odd radices 3, 5, 7 (constants from cospi/sinpi).
template <int R, int SIGN>
__device__ __forceinline__ void dft_odd(float2* v) {
    float2 outv[R];
#pragma unroll
    for (int k = 0; k < R; ++k) {
        float2 acc = v[0];
#pragma unroll
        for (int r = 1; r < R; ++r) {
            const int m = (r * k) % R;
            const float c = cospif(2.0f * m / R);
            const float s = SIGN * sinpif(2.0f * m / R);
            acc.x += v[r].x * c - v[r].y * s;
            acc.y += v[r].x * s + v[r].y * c;
        }
        outv[k] = acc;
    }
#pragma unroll
    for (int k = 0; k < R; ++k) v[k] = outv[k];
}

template <int R, int SIGN>
__device__ __forceinline__ void dftR(float2* v) {
    if constexpr (R == 2) dft2<SIGN>(v[0], v[1]);
    else if constexpr (R == 4) dft4<SIGN>(v);
    else if constexpr (R == 8) dft8<SIGN>(v);
    else dft_odd<R, SIGN>(v);
}

// Twiddles w^r (r = 1..R-1, w = e^{SIGN 2 pi i m / L}, m = k * tws) for one
// butterfly: w and w^4 are read from the table, the others are products at
// most two deep (relative error a few ulp), instead of R - 1 table reads.
template <int R, int SIGN>
__device__ __forceinline__ void apply_twiddles(float2* v, const float2* __restrict__ tw, int m) {
    if constexpr (R == 8 || R == 4 || R == 2 || R == 3) {
        float2 w1 = __ldg(tw + m);
        if (SIGN > 0) w1.y = -w1.y;
        v[1] = cmul(v[1], w1);
        if constexpr (R >= 3) {
            const float2 w2 = cmul(w1, w1);
            v[2] = cmul(v[2], w2);
            if constexpr (R >= 4) {
                const float2 w3 = cmul(w1, w2);
                v[3] = cmul(v[3], w3);
                if constexpr (R == 8) {
                    float2 w4 = __ldg(tw + 4 * m);
                    if (SIGN > 0) w4.y = -w4.y;
                    v[4] = cmul(v[4], w4);
                    v[5] = cmul(v[5], cmul(w4, w1));
                    v[6] = cmul(v[6], cmul(w4, w2));
                    v[7] = cmul(v[7], cmul(w4, w3));
                }
            }
        }
    } else {
#pragma unroll
        for (int r = 1; r < R; ++r) {
            float2 t = __ldg(tw + r * m);
            if (SIGN > 0) t.y = -t.y;
            v[r] = cmul(v[r], t);
        }
    }
}

// Shared-memory layouts of the B lines a block transforms (B * padded_len(L) float2
// per buffer either way; one pad slot per 16 entries).
//  * line-major (contiguous axes; consecutive threads take consecutive butterflies of
//    one line): element n of line b at b * ls + n + n / 16, ls = padded_len(L).  The
//    pad slots break the stride-R bank conflicts of the Stockham scatter.
//  * interleaved (strided axes; consecutive threads take consecutive lines): element n
//    of line b at (n + n / 16) * B + b.  A half-warp (16 threads, one 8-byte access each)
//    covers 16 / B consecutive butterflies of B lines: the stage reads and the later
//    scatters fall on 16 distinct bank pairs, the radix-8 first-stage scatter on 8.  The
//    line-major layout put up to 3 threads of a half-warp on one bank pair there.
__device__ __forceinline__ int pidx(int i) { return i + (i >> 4); }
__host__ __device__ __forceinline__ int padded_len(int L) { return L + (L >> 4) + 1; }
// float2 words of one of the two ping-pong buffers
__host__ __device__ __forceinline__ int fft_buf_words(int L, int B) { return B * padded_len(L); }
template <bool TR>
__device__ __forceinline__ int sidx(int b, int n, int ls, int B) {
    return TR ? pidx(n) * B + b : b * ls + pidx(n);
}

// One Stockham stage over B lines.  FIRST reads its inputs through `ld(b, n)`
// (natural index n, straight from global memory); LAST hands its outputs to
// `stf(b, n, v)`; the stages in between read `src` and write `dst` (shared
// memory, layout sidx<TR>).  TR: consecutive threads take consecutive lines
// (strided axes, interleaved layout), else consecutive butterflies (line-major).
template <int R, int SIGN, bool FIRST, bool LAST, bool TR, class Ld, class St>
__device__ __forceinline__ void stockham_stage(const float2* __restrict__ src, float2* __restrict__ dst,
                                               const float2* __restrict__ tw, int L, int Ns, int B, int lgB, int ls,
                                               const Ld& ld, const St& stf) {
    const int nbf = L / R;
    const int tws = L / (Ns * R);
    for (int w = threadIdx.x; w < nbf * B; w += blockDim.x) {
        int b, j;
        if (TR) { b = w & (B - 1); j = w >> lgB; }
        else { b = w / nbf; j = w - b * nbf; }
        const int k = j % Ns;
        float2 v[R];
        if (FIRST) {
#pragma unroll
            for (int r = 0; r < R; ++r) v[r] = ld(b, j + r * nbf);
        } else {
#pragma unroll
            for (int r = 0; r < R; ++r) v[r] = src[sidx<TR>(b, j + r * nbf, ls, B)];
        }
        if (!FIRST && Ns > 1) apply_twiddles<R, SIGN>(v, tw, k * tws);
        dftR<R, SIGN>(v);
        const int base = (j / Ns) * Ns * R + k;
        if (LAST) {
#pragma unroll
            for (int r = 0; r < R; ++r) stf(b, base + r * Ns, v[r]);
        } else {
#pragma unroll
            for (int r = 0; r < R; ++r) dst[sidx<TR>(b, base + r * Ns, ls, B)] = v[r];
        }
    }
}

template <int R, int SIGN, bool TR, class Ld, class St>
__device__ __forceinline__ void run_stage(int s, int nstage, const float2* src, float2* dst, const float2* tw, int L,
                                          int Ns, int B, int lgB, int ls, const Ld& ld, const St& stf) {
    const bool first = s == 0, last = s == nstage - 1;
    if (first && last) stockham_stage<R, SIGN, true, true, TR>(src, dst, tw, L, Ns, B, lgB, ls, ld, stf);
    else if (first) stockham_stage<R, SIGN, true, false, TR>(src, dst, tw, L, Ns, B, lgB, ls, ld, stf);
    else if (last) stockham_stage<R, SIGN, false, true, TR>(src, dst, tw, L, Ns, B, lgB, ls, ld, stf);
    else stockham_stage<R, SIGN, false, false, TR>(src, dst, tw, L, Ns, B, lgB, ls, ld, stf);
}

// Runs all stages of B length-L transforms: input from ld, output to stf,
// intermediates ping-pong between a and b (each fft_buf_words(L, B, TR) float2).
template <int SIGN, bool TR, class Ld, class St>
__device__ void fft_lines(float2* a, float2* b, const float2* tw, const FftFactors& f, int B, int lgB, int ls,
                          const Ld& ld, const St& stf) {
    int Ns = 1;
    for (int s = 0; s < f.nstage; ++s) {
        const int R = f.radix[s];
        switch (R) {
            case 8: run_stage<8, SIGN, TR>(s, f.nstage, a, b, tw, f.L, Ns, B, lgB, ls, ld, stf); break;
            case 4: run_stage<4, SIGN, TR>(s, f.nstage, a, b, tw, f.L, Ns, B, lgB, ls, ld, stf); break;
            case 2: run_stage<2, SIGN, TR>(s, f.nstage, a, b, tw, f.L, Ns, B, lgB, ls, ld, stf); break;
            case 3: run_stage<3, SIGN, TR>(s, f.nstage, a, b, tw, f.L, Ns, B, lgB, ls, ld, stf); break;
            case 5: run_stage<5, SIGN, TR>(s, f.nstage, a, b, tw, f.L, Ns, B, lgB, ls, ld, stf); break;
            case 7: run_stage<7, SIGN, TR>(s, f.nstage, a, b, tw, f.L, Ns, B, lgB, ls, ld, stf); break;
            default: break;
        }
        __syncthreads();
        float2* t = a;
        a = b;
        b = t;
        Ns *= R;
    }
}

// ---- compile-time radix plans for the oversampled grid lengths of the workloads
// (2 x {64, 96, 128, 192, 256}); other lengths use the runtime path above.
__host__ __device__ constexpr int cnstage(int L) {
    return (L == 512 || L == 256 || L == 192 || L == 128) ? 3 : (L == 384 ? 4 : 0);
}
__host__ __device__ constexpr int cradix(int L, int s) {
    return L == 512 ? 8
         : L == 256 ? (s < 2 ? 8 : 4)
         : L == 384 ? (s < 2 ? 8 : (s == 2 ? 2 : 3))
         : L == 192 ? (s < 2 ? 8 : 3)
         : L == 128 ? (s < 1 ? 8 : 4)
         : 1;
}
__host__ __device__ constexpr int cns(int L, int s) { return s == 0 ? 1 : cns(L, s - 1) * cradix(L, s - 1); }
__host__ __device__ constexpr bool fft_has_cplan(int L) { return cnstage(L) > 0; }

// Offset (in float2, before the factor B of the interleaved layout) of element r of a
// butterfly's reads (n = j + r * nbf) and writes (n = base + r * Ns) from its element 0,
// when the pad slots make it a compile-time constant; -1 otherwise.  It holds for every
// line, butterfly and r of the compile-time plans where it is not -1: a stride that is
// a multiple of 16 shifts the pad count by a constant; a first-stage radix dividing 16
// keeps the R outputs of a butterfly inside one 16-entry group; a write stride of 8
// with an even radix starts every butterfly's group in the lower half of a 16-entry block.
__host__ __device__ constexpr int rd_off(int nbf, int r) { return nbf % 16 == 0 ? r * nbf + r * nbf / 16 : -1; }
__host__ __device__ constexpr int wr_off(int R, int Ns, int r) {
    return Ns == 1 ? (16 % R == 0 ? r : -1)
         : Ns % 16 == 0 ? r * Ns + r * Ns / 16
         : (Ns == 8 && R % 2 == 0) ? 8 * r + r / 2
         : -1;
}

template <int L, int S, int SIGN, bool TR, class Ld, class St>
__device__ __forceinline__ void cstage(const float2* __restrict__ src, float2* __restrict__ dst,
                                       const float2* __restrict__ tw, int B, int lgB, int ls, const Ld& ld,
                                       const St& stf) {
    constexpr int R = cradix(L, S);
    constexpr int Ns = cns(L, S);
    constexpr bool FIRST = S == 0, LAST = S == cnstage(L) - 1;
    constexpr int nbf = L / R;
    constexpr int tws = L / (Ns * R);
    constexpr bool RDC = rd_off(nbf, 1) >= 0, WRC = wr_off(R, Ns, 1) >= 0;
    const int m = TR ? B : 1;   // offset multiplier of the layout
    for (int w = threadIdx.x; w < nbf * B; w += blockDim.x) {
        int b, j;
        if (TR) { b = w & (B - 1); j = w >> lgB; }
        else { b = w / nbf; j = w - b * nbf; }
        const int k = j % Ns;
        float2 v[R];
        if (FIRST) {
#pragma unroll
            for (int r = 0; r < R; ++r) v[r] = ld(b, j + r * nbf);
        } else {
            if constexpr (RDC) {
                const float2* s0 = src + sidx<TR>(b, j, ls, B);
#pragma unroll
                for (int r = 0; r < R; ++r) v[r] = s0[rd_off(nbf, r) * m];
            } else {
#pragma unroll
                for (int r = 0; r < R; ++r) v[r] = src[sidx<TR>(b, j + r * nbf, ls, B)];
            }
            if constexpr (Ns > 1) apply_twiddles<R, SIGN>(v, tw, k * tws);
        }
        dftR<R, SIGN>(v);
        const int base = (j / Ns) * Ns * R + k;
        if (LAST) {
#pragma unroll
            for (int r = 0; r < R; ++r) stf(b, base + r * Ns, v[r]);
        } else if constexpr (WRC) {
            float2* d0 = dst + sidx<TR>(b, base, ls, B);
#pragma unroll
            for (int r = 0; r < R; ++r) d0[wr_off(R, Ns, r) * m] = v[r];
        } else {
#pragma unroll
            for (int r = 0; r < R; ++r) dst[sidx<TR>(b, base + r * Ns, ls, B)] = v[r];
        }
    }
}

template <int L, int S, int SIGN, bool TR, class Ld, class St>
__device__ __forceinline__ void cstages(float2* a, float2* b, const float2* tw, int B, int lgB, int ls,
                                        const Ld& ld, const St& stf) {
    if constexpr (S < cnstage(L)) {
        cstage<L, S, SIGN, TR>(a, b, tw, B, lgB, ls, ld, stf);
        __syncthreads();
        cstages<L, S + 1, SIGN, TR>(b, a, tw, B, lgB, ls, ld, stf);
    }
}

// LC = compile-time length (0: runtime plan f).  TR: interleaved layout, consecutive
// threads on consecutive lines (strided axes).
template <int LC, int SIGN, bool TR, class Ld, class St>
__device__ __forceinline__ void run_fft(float2* a, float2* b, const float2* tw, const FftFactors& f, int B, int lgB,
                                        int ls, const Ld& ld, const St& stf) {
    if constexpr (LC == 0) fft_lines<SIGN, TR>(a, b, tw, f, B, lgB, ls, ld, stf);
    else cstages<LC, 0, SIGN, TR>(a, b, tw, B, lgB, ls, ld, stf);
}

// Launch a pass (host).
void launch_fft_pass(int mode, const PassArgs& a, cudaStream_t st);

}  // namespace mmr
