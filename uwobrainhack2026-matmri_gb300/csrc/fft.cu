// FFT pass kernels: Stockham radix stages in shared memory with fused
// prologue (deapodisation, coil-map multiply, zero padding) and epilogue
// (crop, deapodisation, scaling).
#include <cmath>
#include <map>
#include <mutex>

#include "fft.cuh"

namespace mmr {

FftFactors fft_factorize(int L) {
    FftFactors f;
    f.L = L;
    int n = L;
    std::vector<int> r;
    while (n % 8 == 0) { r.push_back(8); n /= 8; }
    while (n % 4 == 0) { r.push_back(4); n /= 4; }
    while (n % 2 == 0) { r.push_back(2); n /= 2; }
    while (n % 3 == 0) { r.push_back(3); n /= 3; }
    while (n % 5 == 0) { r.push_back(5); n /= 5; }
    while (n % 7 == 0) { r.push_back(7); n /= 7; }
    MMR_REQUIRE(n == 1, "FFT length %d has a prime factor > 7", L);
    MMR_REQUIRE((int)r.size() <= FFT_MAX_STAGES, "FFT length %d needs too many stages", L);
    f.nstage = (int)r.size();
    for (int i = 0; i < f.nstage; ++i) f.radix[i] = r[i];
    return f;
}

const float2* fft_twiddles(int L) {
    static std::mutex mu;
    static std::map<std::pair<int, int>, float2*> cache;   // (device, L)
    int dev = 0;
    MMR_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> g(mu);
    auto it = cache.find({dev, L});
    if (it != cache.end()) return it->second;
    std::vector<float2> h(L);
    for (int m = 0; m < L; ++m) {
        // e^{-2 pi i m / L} in FP64, exact at the quarter points
        const double a = -2.0 * M_PI * (double)m / (double)L;
        h[m] = make_float2((float)std::cos(a), (float)std::sin(a));
        if (4 * m % L == 0) {
            const int q = (4 * m / L) & 3;
            const float c[4] = {1.f, 0.f, -1.f, 0.f}, s[4] = {0.f, -1.f, 0.f, 1.f};
            h[m] = make_float2(c[q], s[q]);
        }
    }
    float2* d = nullptr;
    MMR_CUDA(cudaMalloc(&d, L * sizeof(float2)));
    MMR_CUDA(cudaMemcpy(d, h.data(), L * sizeof(float2), cudaMemcpyHostToDevice));
    cache[{dev, L}] = d;
    return d;
}

template <int MODE, int SIGN, int LC>
__global__ void __launch_bounds__(256) fft_pass_kernel(const PassArgs a) {
    extern __shared__ float4 sm4[];
    float2* sm = reinterpret_cast<float2*>(sm4);
    pdl_wait();
    pdl_trigger();
    if (a.active && *a.active) return;
    const int L = LC ? LC : a.L, B = a.B;
    int lgB = 0;
    while ((1 << lgB) < B) ++lgB;
    const int ls = padded_len(L);

    // ---- tile decomposition: B consecutive lines (contiguous axis) or B adjacent lines of one
    //      outer slice (strided axis)
    const bool contiguous = a.inner == 1;
    const int bufw = fft_buf_words(L, B);
    float2* buf0 = sm;
    float2* buf1 = sm + bufw;
    long long l0 = 0, q0 = 0, o = 0;
    if (contiguous) {
        l0 = (long long)blockIdx.x * B;
    } else {
        const long long ntq = (a.inner + B - 1) / B;
        o = (long long)blockIdx.x / ntq;
        q0 = ((long long)blockIdx.x % ntq) * B;
    }
    auto line_valid = [&](int b) -> bool { return contiguous ? (l0 + b < a.outer) : (q0 + b < a.inner); };

    // first stage input: natural index n <- input position t = (n - in_start) mod L (zero padding beyond nin)
    auto line_in = [&](int b) -> float2 {
        return a.in_line ? a.in_line[(l0 + b) % a.lpc] : make_float2(1.f, 0.f);
    };
    auto line_out = [&](int b) -> float2 {
        return a.out_line ? a.out_line[q0 + b] : make_float2(1.f, 0.f);
    };
    auto ld = [&](int b, int n) -> float2 {
        int t = n - a.in_start;
        t += (t < 0) ? L : 0;
        if (t >= a.nin || !line_valid(b)) return make_float2(0.f, 0.f);
        float2 v;
        if (MODE == PASS_FWD_IMG) {
            const long long l = l0 + b;
            const float2 x = a.in[t + (long long)a.nin * (l % a.lpc)];
            v = a.maps ? cmul(x, a.maps[t + (long long)a.nin * l]) : x;
        } else if (contiguous) {
            v = a.in[t + (long long)a.nin * (l0 + b)];
        } else {
            v = a.in[(q0 + b) + a.inner * (t + (long long)a.nin * o)];
        }
        if (a.in_fac) v = cmul(v, a.in_fac[t]);
        if (a.in_line) v = cmul(v, line_in(b));
        return v;
    };
    // last stage output: natural index n -> output position t = (n - out_start) mod L (crop beyond nout)
    auto stf = [&](int b, int n, float2 v) {
        int t = n - a.out_start;
        t += (t < 0) ? L : 0;
        if (t >= a.nout || !line_valid(b)) return;
        v = cscale(v, a.scale);
        if (a.out_fac) v = cmul(v, a.out_fac[t]);
        if (a.out_line) v = cmul(v, line_out(b));
        if (contiguous) a.out[t + (long long)a.nout * (l0 + b)] = v;
        else a.out[(q0 + b) + a.inner * (t + (long long)a.nout * o)] = v;
    };
    if (contiguous) run_fft<LC, SIGN, false>(buf0, buf1, a.tw, a.f, B, lgB, ls, ld, stf);
    else run_fft<LC, SIGN, true>(buf0, buf1, a.tw, a.f, B, lgB, ls, ld, stf);
}

template <int MODE, int SIGN, int LC>
static void launch_mode(const PassArgs& a, cudaStream_t st) {
    const size_t smem = (size_t)2 * fft_buf_words(a.L, a.B) * sizeof(float2);
    auto kern = fft_pass_kernel<MODE, SIGN, LC>;
    static bool attr_done = false;   // one per instantiation
    if (!attr_done) {
        MMR_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
        attr_done = true;
    }
    const bool contiguous = a.inner == 1;
    const long long nblk = contiguous ? (a.outer + a.B - 1) / a.B : ((a.inner + a.B - 1) / a.B) * a.outer;
    MMR_REQUIRE(nblk < (1LL << 31), "FFT pass grid too large");
    if (nblk == 0) return;
    launch_dependent(kern, dim3((unsigned)nblk), dim3(256), smem, st, a);
}

template <int LC>
static void launch_len(int mode, const PassArgs& a, cudaStream_t st) {
    static_assert(LC == 0 || fft_has_cplan(LC), "no compile-time plan");
    if (a.sign < 0) {
        if (mode == PASS_PLAIN) launch_mode<PASS_PLAIN, -1, LC>(a, st);
        else launch_mode<PASS_FWD_IMG, -1, LC>(a, st);
    } else {
        if (mode == PASS_PLAIN) launch_mode<PASS_PLAIN, 1, LC>(a, st);
        else launch_mode<PASS_FWD_IMG, 1, LC>(a, st);
    }
}

void launch_fft_pass(int mode, const PassArgs& a, cudaStream_t st) {
    MMR_REQUIRE(!a.in_line || (a.inner == 1 && a.lpc >= 1), "per-line input factors need a contiguous pass");
    MMR_REQUIRE(!a.out_line || a.inner > 1, "per-line output factors need a strided pass");
    MMR_REQUIRE(a.nin <= a.L && a.nout <= a.L && a.nin > 0 && a.nout > 0, "bad FFT pass extents");
    MMR_REQUIRE(a.B >= 1 && (a.B & (a.B - 1)) == 0, "lines per block must be a power of two");
    switch (a.L) {
        case 512: launch_len<512>(mode, a, st); break;
        case 384: launch_len<384>(mode, a, st); break;
        case 256: launch_len<256>(mode, a, st); break;
        case 192: launch_len<192>(mode, a, st); break;
        case 128: launch_len<128>(mode, a, st); break;
        default: launch_len<0>(mode, a, st); break;
    }
}

}  // namespace mmr
