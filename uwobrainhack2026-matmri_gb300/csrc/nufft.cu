// @nufftOp on GB300: FP64 plan precompute (host) and the gridding kernels.
//
// Plan (operators/@nufftOp/nufftOp.m:138-274): oversampled size osN, the
// tabulated Kaiser-Bessel kernel with linear table interpolation, the
// deapodisation comp, per-sample tap weights and base cells.  The sparse
// interpolation matrix convMat (nufftOp.m:257) is never materialised: each
// sample keeps its base cell floor((k+0.5) osN) and its separable per-dim tap
// weights, exactly the factors whose products are convMat's entries.
//
// Gridding (nufftOp.m:359 convMat'*y and nufftOp.m:389 convMat*y):
//  * interp2d_binned  — forward interpolation; each CTA stages one grid tile
//    plus halo for a group of coils into shared memory with a TMA tensor
//    copy (cp.async.bulk.tensor.3d, mbarrier completion, bounded wait) and
//    evaluates the W x W taps of a sample with one lane per tap and a
//    warp-shuffle reduction;
//  * spread2d_binned  — adjoint spreading; samples are pre-sorted into the
//    tiles their footprint touches.  Tiles are adaptive (a quadtree): a
//    32 x 32 tile holding more samples than one work item allows — the dense
//    centre of a variable-density trajectory — is split into 16 x 16 and
//    8 x 8 sub-tiles.  Every output cell is owned by exactly one CTA, which
//    accumulates its (sub)tile in shared memory and flushes it with coalesced
//    plain stores: no global atomics, no memset of the grid, deterministic;
//  * gridnorm2d_binned — the two fused for the normal operator
//    C^H diag(w) C: interp from a staged tile + 2W halo (one thread per
//    sample and coil, separable weights), weight, spread into the owned tile
//    (one lane per tap); the samples never round-trip through HBM;
//  * interp_generic / spread_generic — any ndim / small grids.
#include <algorithm>
#include <cmath>
#include <cudaTypedefs.h>
#include <complex>
#include <functional>

#include "nufft.cuh"
#include "reduce.cuh"

namespace mmr {

__device__ int g_dev_error = 0;
// Poll limit of the gridding kernels' bounded TMA waits; a test lowers it to make a wait run out.
constexpr int kDefaultWaitPolls = 1 << 22;
__device__ int g_wait_polls = kDefaultWaitPolls;

// Device address of the error word, for kernels of other translation units that take it as an argument.
int* device_error_ptr() {
    int* p = nullptr;
    MMR_CUDA(cudaGetSymbolAddress((void**)&p, g_dev_error));
    return p;
}

void set_wait_polls(int polls) {
    const int v = polls > 0 ? polls : 0;
    MMR_CUDA(cudaMemcpyToSymbol(g_wait_polls, &v, sizeof(int)));
}

int device_error_word(cudaStream_t st) {
    int v = 0;
    MMR_CUDA(cudaMemcpyFromSymbolAsync(&v, g_dev_error, sizeof(int), 0, cudaMemcpyDeviceToHost, st));
    MMR_CUDA(cudaStreamSynchronize(st));
    if (v) {
        int z = 0;
        MMR_CUDA(cudaMemcpyToSymbol(g_dev_error, &z, sizeof(int)));
    }
    return v;
}

// ----------------------------------------------------------------- host plan --
static int max_prime_factor(int n) {
    int f = 1;
    for (int p = 2; p * p <= n; ++p)
        while (n % p == 0) { f = p; n /= p; }
    return n > 1 ? std::max(f, n) : f;
}

// I0 by its power series (positive terms); matches besseli(0,.) to ~1e-15 here.
static double bessel_i0(double z) {
    const double q = z * z / 4.0;
    double term = 1.0, acc = 1.0;
    for (int k = 1; k < 500; ++k) {
        term *= q / ((double)k * (double)k);
        acc += term;
        if (term <= 1e-17 * acc) break;
    }
    return acc;
}

static inline long long imod(long long a, long long m) {
    long long r = a % m;
    return r < 0 ? r + m : r;
}

void nufft_plan_build(NufftPlan& p, const mmr_nufft_desc& d) {
    MMR_REQUIRE(d.ndim >= 1 && d.ndim <= 3, "ndim must be 1..3 (got %d)", d.ndim);
    MMR_REQUIRE(d.nsamp >= 1, "need at least one sample");
    MMR_REQUIRE(d.kloc != nullptr, "kloc is NULL");
    p.nd = d.ndim;
    p.M = d.nsamp;
    p.os = d.os > 0 ? d.os : 1.5;                  // nufftOp.m:66
    p.W = d.kwidth > 0 ? d.kwidth : 6;             // nufftOp.m:65
    MMR_REQUIRE(p.W % 2 == 0 && p.W >= 2 && p.W <= 8, "kwidth must be even in 2..8 (got %d)", p.W);
    const double barg = p.W * (double)p.W / (p.os * p.os) * (p.os - 0.5) * (p.os - 0.5) - 0.8;
    MMR_REQUIRE(barg > 0, "kwidth/os combination gives a non-real Kaiser-Bessel beta");
    p.beta = M_PI * std::sqrt(barg);                                                 // 155
    p.Nkern = (int)(std::ceil(0.5 * (p.W + 1) * std::sqrt(0.37 / (p.os * p.os) / 1e-6)) * 2);   // 156
    p.Ntot = p.Gtot = 1;
    for (int k = 0; k < 3; ++k) { p.N[k] = 1; p.G[k] = 1; }
    for (int k = 0; k < p.nd; ++k) {
        MMR_REQUIRE(d.imN[k] >= 2 && d.imN[k] % 2 == 0 && d.imN[k] <= 32768,
                    "imN(%d) = %lld must be even in [2, 32768]", k + 1, (long long)d.imN[k]);
        p.N[k] = (int)d.imN[k];
        int g = (int)(std::ceil(p.N[k] * p.os / 2.0) * 2);                            // 146
        while (max_prime_factor(g) > 7) g += 2;                                       // 148-152
        MMR_REQUIRE(g >= p.N[k] && g >= 2 * p.W, "oversampled size %d too small", g);
        p.G[k] = g;
        p.Ntot *= p.N[k];
        p.Gtot *= g;
    }
    p.kloc.assign(d.kloc, d.kloc + p.M * p.nd);
    for (double v : p.kloc) MMR_REQUIRE(std::isfinite(v), "kloc holds NaN/Inf");

    // kernel table (157-165)
    const int Nk = p.Nkern;
    std::vector<double> kern(Nk + 1);
    double ksum = 0;
    for (int i = 0; i < Nk; ++i) {
        const double kx = -1.0 + 2.0 * i / (Nk - 1);
        kern[i] = bessel_i0(p.beta * std::sqrt(std::max(0.0, 1.0 - kx * kx)));
        ksum += kern[i];
    }
    kern[Nk] = 0.0;
    for (auto& v : kern) v = v / ksum * (double)(Nk - 1) / p.W;

    // deapodisation (171-181) and the fftShiftArray constant exp(+-i pi N/2)
    std::vector<std::complex<double>> fac64[3];
    for (int k = 0; k < p.nd; ++k) {
        const int n = p.N[k], g = p.G[k];
        std::vector<double> c(n);
        int imin = 0;
        for (int i = 0; i < n; ++i) {
            const double x0 = (i - n / 2) * M_PI * p.W / g;
            const double z = x0 * x0 - p.beta * p.beta;
            double v;
            if (z < 0) { const double y = std::sqrt(-z); v = y / std::sinh(y); }
            else if (z > 0) { const double x = std::sqrt(z); v = x / std::sin(x); }
            else v = 1.0;
            c[i] = v;
            if (std::fabs(v) < std::fabs(c[imin])) imin = i;
        }
        const double cm = c[imin], sc = std::sqrt((double)g / n);
        const double ph = M_PI * n / 2.0;
        std::vector<float2> ff(n), fa(n);
        fac64[k].resize(n);
        for (int i = 0; i < n; ++i) {
            const double v = c[i] / cm * sc;
            fac64[k][i] = {v * std::cos(ph), v * std::sin(ph)};
            ff[i] = make_float2((float)(v * std::cos(ph)), (float)(v * std::sin(ph)));
            fa[i] = make_float2((float)(v * std::cos(ph)), (float)(-v * std::sin(ph)));
        }
        p.d_fwd_fac[k].upload(ff);
        p.d_adj_fac[k].upload(fa);
        p.ff[k] = fft_factorize(g);
        p.tw[k] = fft_twiddles(g);
    }
    if (p.nd > 1) {
        // per-line products in FP64, rounded once: forward over axes 1.., adjoint over axes ..nd-2
        const long long nf = (long long)p.N[1] * p.N[2], na = (long long)p.N[0] * (p.nd > 2 ? p.N[1] : 1);
        std::vector<float2> fl((size_t)nf), al((size_t)na);
        for (long long l = 0; l < nf; ++l) {
            std::complex<double> f = fac64[1][l % p.N[1]];
            if (p.nd > 2) f *= fac64[2][l / p.N[1]];
            fl[(size_t)l] = make_float2((float)f.real(), (float)f.imag());
        }
        for (long long q = 0; q < na; ++q) {
            std::complex<double> f = std::conj(fac64[0][q % p.N[0]]);
            if (p.nd > 2) f *= std::conj(fac64[1][q / p.N[0]]);
            al[(size_t)q] = make_float2((float)f.real(), (float)f.imag());
        }
        p.d_fwd_line.upload(fl);
        p.d_adj_line.upload(al);
    }

    // per-sample base cells and tap weights (216-238)
    std::vector<int> base((size_t)p.nd * p.M);
    std::vector<float> wts((size_t)p.M * p.nd * p.W);
    for (long long s = 0; s < p.M; ++s) {
        for (int k = 0; k < p.nd; ++k) {
            const double ka = p.kloc[s + p.M * k] + 0.5;                   // 141
            const double xa = ka * p.G[k];                                 // 217
            const double fl = std::floor(xa);
            const double kia = fl - xa;                                    // 218
            base[(size_t)k * p.M + s] = (int)imod((long long)fl, p.G[k]);
            for (int t = 0; t < p.W; ++t) {
                const double off = -p.W / 2 + 1 + t;
                double ki = (kia + off) * (Nk - 1) / p.W + Nk / 2.0 + 0.5; // 220-221
                const double fi = std::floor(ki);
                const double frac = ki - fi;                               // 222
                long long idx = (long long)fi;                             // 1-based (223)
                idx = std::min<long long>(std::max<long long>(idx, 1), Nk);
                const double w = (1.0 - frac) * kern[idx - 1] + frac * kern[idx];   // 225
                wts[((size_t)s * p.nd + k) * p.W + t] = (float)w;
            }
        }
    }
    p.d_base.upload(base);
    p.d_w.upload(wts);
    nufft_set_dcf(p, d.dcf);
    if (p.nd == 2) nufft_build_bins(p, 32);
}

void nufft_set_dcf(NufftPlan& p, const double* dcf) {
    p.dcf_version++;
    if (!dcf) {
        p.has_dcf = false;
        p.dcf_h.clear();
        return;
    }
    p.dcf_h.assign(dcf, dcf + p.M);
    std::vector<float> f(p.M);
    for (long long s = 0; s < p.M; ++s) {
        MMR_REQUIRE(std::isfinite(dcf[s]), "dcf holds NaN/Inf");
        f[s] = (float)dcf[s];
    }
    p.d_dcf.upload(f);
    p.has_dcf = true;
}

// Work item encoding: {u0 | v0 << 16, e0, e1, tile side}.
static inline int4 item_of(int u0, int v0, int e0, int e1, int T) { return make_int4(u0 | (v0 << 16), e0, e1, T); }

void nufft_build_bins(NufftPlan& p, int Treq, int chunk) {
    p.use_bins = false;
    if (p.nd != 2) return;
    MMR_REQUIRE(chunk >= 8, "work-item chunk must be >= 8");
    MMR_REQUIRE(p.G[0] < 65536 && p.G[1] < 65536, "grid too large for the binned path");
    MMR_REQUIRE(p.G[0] % 2 == 0, "the binned path needs an even first grid extent");
    p.bins.chunk = chunk;
    int T = Treq;
    while (T >= 8 && (p.G[0] < 2 * (T + 2 * p.W) || p.G[1] < 2 * (T + 2 * p.W))) T /= 2;
    if (T < 8 || T < p.W) return;
    BinLists& b = p.bins;
    b.T = T;
    b.ntx = (int)cdiv(p.G[0], T);
    b.nty = (int)cdiv(p.G[1], T);
    const int ntile = b.ntx * b.nty;
    std::vector<int> base((size_t)2 * p.M);
    MMR_CUDA(cudaMemcpy(base.data(), p.d_base.p, base.size() * sizeof(int), cudaMemcpyDeviceToHost));
    const int off0 = -p.W / 2 + 1;
    auto sdist = [](long long a, int g) {   // signed representative of a mod g in [-g/2, g/2)
        long long r = imod(a, g);
        return (int)(r >= g / 2 ? r - g : r);
    };
    // ---- own lists (interpolation): each sample once, in the tile holding its base cell,
    //      split into items of <= chunk samples (no output conflicts)
    std::vector<int> cnt(ntile + 1, 0);
    for (long long s = 0; s < p.M; ++s) {
        const int c1 = base[s], c2 = base[p.M + s];
        cnt[(c2 / T) * b.ntx + c1 / T + 1]++;
    }
    for (int t = 0; t < ntile; ++t) cnt[t + 1] += cnt[t];
    std::vector<int> own_s(p.M), pos(cnt.begin(), cnt.end() - 1);
    std::vector<short2> own_lb(p.M);
    b.max_own = 0;
    for (int t = 0; t < ntile; ++t) b.max_own = std::max(b.max_own, cnt[t + 1] - cnt[t]);
    for (long long s = 0; s < p.M; ++s) {
        const int c1 = base[s], c2 = base[p.M + s];
        const int tx = c1 / T, ty = c2 / T, t = ty * b.ntx + tx;
        const int e = pos[t]++;
        own_s[e] = (int)s;
        own_lb[e] = make_short2((short)(c1 - tx * T), (short)(c2 - ty * T));
    }
    std::vector<int4> items;
    for (int t = 0; t < ntile; ++t) {
        const int u0 = (t % b.ntx) * T, v0 = (t / b.ntx) * T;
        for (int e0 = cnt[t]; e0 < cnt[t + 1]; e0 += chunk)
            items.push_back(item_of(u0, v0, e0, std::min(cnt[t + 1], e0 + chunk), T));
    }
    b.own_s.upload(own_s);
    b.own_lb.upload(own_lb);
    b.own_items.upload(items);
    b.n_own_items = (int)items.size();
    b.n_own = p.M;
    // ---- padded lists (spreading / fused normal op): every output tile owns its cells and
    //      lists every sample whose footprint touches it.  Tiles holding more than `chunk`
    //      samples (the dense centre of a variable-density trajectory) are split into
    //      quadrants down to 8 x 8 cells, so that work stays balanced without atomics.
    std::vector<std::vector<int>> tiles_s(ntile);
    for (long long s = 0; s < p.M; ++s) {
        const int c[2] = {base[s], base[p.M + s]};
        int tl[2][8], ntl[2] = {0, 0};
        for (int k = 0; k < 2; ++k) {
            for (int j = 0; j < p.W; ++j) {
                const int ti = (int)imod(c[k] + off0 + j, p.G[k]) / T;
                bool seen = false;
                for (int q = 0; q < ntl[k]; ++q) seen |= (tl[k][q] == ti);
                if (!seen) tl[k][ntl[k]++] = ti;
            }
        }
        for (int a = 0; a < ntl[0]; ++a)
            for (int bb = 0; bb < ntl[1]; ++bb) tiles_s[tl[1][bb] * b.ntx + tl[0][a]].push_back((int)s);
    }
    auto touches = [&](int s, int u0, int v0, int Tt) {
        const int c[2] = {base[s], base[p.M + s]}, o[2] = {u0, v0};
        for (int k = 0; k < 2; ++k) {
            bool hit = false;
            for (int j = 0; j < p.W && !hit; ++j) hit = imod((long long)c[k] + off0 + j - o[k], p.G[k]) < Tt;
            if (!hit) return false;
        }
        return true;
    };
    std::vector<float> wts((size_t)2 * p.W * p.M);
    MMR_CUDA(cudaMemcpy(wts.data(), p.d_w.p, wts.size() * sizeof(float), cudaMemcpyDeviceToHost));
    std::vector<int> ps;
    std::vector<short2> plb;
    std::vector<float> pw;
    std::vector<int2> heavy;   // {u0 | v0 << 16, side} of leaf tiles shared by several items
    items.clear();
    b.max_pad = 0;
    std::function<void(int, int, int, const std::vector<int>&)> split = [&](int u0, int v0, int Tt,
                                                                             const std::vector<int>& list) {
        if (u0 >= p.G[0] || v0 >= p.G[1]) return;
        if ((int)list.size() > chunk && Tt > 8) {
            const int h = Tt / 2;
            for (int dv = 0; dv < 2; ++dv)
                for (int du = 0; du < 2; ++du) {
                    std::vector<int> sub;
                    for (int s : list)
                        if (touches(s, u0 + du * h, v0 + dv * h, h)) sub.push_back(s);
                    split(u0 + du * h, v0 + dv * h, h, sub);
                }
            return;
        }
        const int e0 = (int)ps.size();
        for (int s : list) {
            ps.push_back(s);
            plb.push_back(make_short2((short)sdist((long long)base[s] - u0, p.G[0]),
                                      (short)sdist((long long)base[p.M + s] - v0, p.G[1])));
            pw.insert(pw.end(), wts.begin() + (size_t)s * 2 * p.W, wts.begin() + (size_t)(s + 1) * 2 * p.W);
        }
        b.max_pad = std::max(b.max_pad, (int)list.size());
        const int e1 = (int)ps.size();
        if (e1 - e0 <= chunk) {
            items.push_back(item_of(u0, v0, e0, e1, Tt));   // owned; empty tiles still write zeros
        } else {
            // an 8 x 8 leaf still denser than one item: zeroed first, then its chunks add
            heavy.push_back(make_int2(u0 | (v0 << 16), Tt));
            for (int c = e0; c < e1; c += chunk) items.push_back(item_of(u0, v0, c, std::min(e1, c + chunk), Tt | 256));
        }
    };
    for (int t = 0; t < ntile; ++t) split((t % b.ntx) * T, (t / b.ntx) * T, T, tiles_s[t]);
    // costliest items first (about 100 instructions per entry and coil, 10 per cell and coil), so
    // that the long ones start in the first wave of a launch instead of trailing in the last
    std::stable_sort(items.begin(), items.end(), [](const int4& x, const int4& y) {
        const long long tx = x.w & 255, ty = y.w & 255;
        return 100LL * (x.z - x.y) + 10 * tx * tx > 100LL * (y.z - y.y) + 10 * ty * ty;
    });
    b.heavy.upload(heavy);
    b.n_heavy = (int)heavy.size();
    b.pad_s.upload(ps);
    b.pad_lb.upload(plb);
    b.pad_w.upload(pw);
    b.n_pad = (long long)ps.size();
    b.pad_items.upload(items);
    b.n_pad_items = (int)items.size();
    p.use_bins = true;
    p.tmap_ptr = nullptr;   // invalidate descriptor caches (box depends on T)
}

// --------------------------------------------------------------- TMA helpers --
static PFN_cuTensorMapEncodeTiled_v12000 get_encode() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        cudaDriverEntryPointQueryResult q;
        void* f = nullptr;
        MMR_CUDA(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q));
        MMR_REQUIRE(q == cudaDriverEntryPointSuccess && f, "cuTensorMapEncodeTiled unavailable");
        fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
    }
    return fn;
}

// 3D map over a centered grid [G1, G2, nb] of complex64 viewed as floats.
static void encode_grid_map(CUtensorMap* m, const void* grid, int G1, int G2, long long nb, int box_cells, int cg) {
    MMR_REQUIRE(((uintptr_t)grid & 15) == 0, "grid buffer not 16-byte aligned");
    cuuint64_t dims[3] = {(cuuint64_t)2 * G1, (cuuint64_t)G2, (cuuint64_t)nb};
    cuuint64_t strides[2] = {(cuuint64_t)G1 * 8, (cuuint64_t)G1 * G2 * 8};
    cuuint32_t box[3] = {(cuuint32_t)(2 * box_cells), (cuuint32_t)box_cells, (cuuint32_t)cg};
    cuuint32_t es[3] = {1, 1, 1};
    MMR_REQUIRE((2 * box_cells * 4) % 16 == 0 && 2 * box_cells <= 256 && box_cells <= 256 && cg <= 256,
                "bad TMA box");
    CUresult r = get_encode()(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<void*>(grid), dims, strides, box,
                              es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                              CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    MMR_REQUIRE(r == CUDA_SUCCESS, "cuTensorMapEncodeTiled failed (%d)", (int)r);
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ bool mbar_poll(uint32_t a, uint32_t phase, int polls) {
    for (int it = 0; it < polls; ++it) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done)
            : "r"(a), "r"(phase)
            : "memory");
        if (done) return true;
    }
    return false;
}

// Bounded mbarrier wait for a TMA copy: returns false (and flags the device error word) when
// g_wait_polls polls run out.  Before it returns false it still waits (bounded, with the default
// limit) for the copy to land, so that the CTA never leaves with a copy into its shared memory in
// flight.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t phase) {
    const uint32_t a = smem_u32(bar);
    if (mbar_poll(a, phase, g_wait_polls)) return true;
    atomicExch(&g_dev_error, 1);
    mbar_poll(a, phase, kDefaultWaitPolls);
    return false;
}

// TMA only for regions fully inside the grid whose inner start (2*ox floats) is
// 16-byte aligned and whose row (2*R floats) is a multiple of 16 bytes.  Thread 0
// issues the copy; returns whether it did (the caller then waits on `bar`).
__device__ __forceinline__ bool region_issue(float2* reg, const CUtensorMap* tmap, bool use_tma, uint64_t* bar,
                                             int ox, int oy, int c0, int cg, int R, int G1, int G2) {
    const bool inside = use_tma && ox >= 0 && oy >= 0 && ox + R <= G1 && oy + R <= G2 && (ox & 1) == 0 &&
                        (R & 1) == 0;
    if (inside && threadIdx.x == 0) {
        const uint32_t bytes = (uint32_t)cg * R * R * 8;
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                     : "memory");
        asm volatile(
            "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, "
            "%4}], [%5];" ::"r"(smem_u32(reg)),
            "l"(tmap), "r"(2 * ox), "r"(oy), "r"(c0), "r"(smem_u32(bar))
            : "memory");
    }
    return inside;
}

// Wrapped plain loads of the region: one warp per (coil, row), lanes along the row.
__device__ __forceinline__ void region_plain(float2* reg, const float2* __restrict__ grid, int ox, int oy, int c0,
                                             int cg, int R, int G1, int G2, long long nb) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
    for (int cr = warp; cr < cg * R; cr += nwarp) {
        const int c = cr / R, ry = cr - c * R;
        int u2 = oy + ry;
        u2 += (u2 < 0) ? G2 : 0;
        u2 -= (u2 >= G2) ? G2 : 0;
        const bool cv = c0 + c < nb;
        const float2* src = grid + (long long)G1 * (u2 + (long long)G2 * (c0 + c));
        float2* dst = reg + (size_t)cr * R;
        for (int rx = lane; rx < R; rx += 32) {
            int u1 = ox + rx;
            u1 += (u1 < 0) ? G1 : 0;
            u1 -= (u1 >= G1) ? G1 : 0;
            dst[rx] = cv ? src[u1] : make_float2(0.f, 0.f);
        }
    }
    __syncthreads();
}

// Stage a [cg][R][R] complex region whose origin is (ox, oy) into smem.
// TMA when the region is inside the grid, wrapped plain loads otherwise.
__device__ __forceinline__ bool stage_region(float2* reg, const float2* __restrict__ grid, const CUtensorMap* tmap,
                                             bool use_tma, uint64_t* bar, int ox, int oy, int c0, int cg, int R,
                                             int G1, int G2, long long nb) {
    if (region_issue(reg, tmap, use_tma, bar, ox, oy, c0, cg, R, G1, G2)) return mbar_wait(bar, 0);
    region_plain(reg, grid, ox, oy, c0, cg, R, G1, G2, nb);
    return true;
}

// Dynamic smem layout for TMA kernels: [pad to 128 B][mbarrier, 128 B slot][region ...].
constexpr size_t kTmaSmemExtra = 256;
__device__ __forceinline__ float2* tma_layout(float4* sm, uint64_t** bar) {
    char* b = reinterpret_cast<char*>(sm);
    const uint32_t pad = (128u - (smem_u32(b) & 127u)) & 127u;
    *bar = reinterpret_cast<uint64_t*>(b + pad);
    return reinterpret_cast<float2*>(b + pad + 128);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar) {
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    __syncthreads();
}

template <int W>
struct TapMap {
    static constexpr int TAPS = W * W;
    static constexpr int LPP = TAPS <= 16 ? 16 : 32;          // lanes per (sample, coil) pair
    static constexpr int TPL = (TAPS + LPP - 1) / LPP;        // taps per lane
    static constexpr int PPW = 32 / LPP;                      // pairs per warp
};

template <int LPP>
__device__ __forceinline__ float2 group_sum(float2 v) {
#pragma unroll
    for (int o = LPP / 2; o >= 1; o >>= 1) {
        v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
        v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
    }
    return v;
}

// ------------------------------------------------------- binned 2D kernels ----
struct Bin2DArgs {
    const int4* items;       // {u0 | v0 << 16, e0, e1, tile side}
    const int* ent_s;
    const short2* ent_lb;
    const float* ent_w;      // padded lists: [entry][2][W] (the entry's sample's tap weights)
    const float* wts;        // [M][2][W]
    const float* wfac;       // per-sample weight or null
    long long wfac_bstride;  // 0 or M
    int G1, G2, T, lgT, ntx;
    long long M, nb;
    int cg;
    int use_tma;
    int chunk;               // max entries per phase batch (sval capacity)
    int n_items;             // work items in the list
    const int* active;
};

template <int W>
__global__ void __launch_bounds__(256) interp2d_binned(const float2* __restrict__ grid, float2* __restrict__ y,
                                                       const Bin2DArgs a, const __grid_constant__ CUtensorMap tmap) {
    using TM = TapMap<W>;
    extern __shared__ float4 sm4[];
    if (a.active && *a.active) return;
    const int R = a.T + W;
    uint64_t* bar;
    float2* reg = tma_layout(sm4, &bar);
    const int4 item = a.items[blockIdx.x];
    const int u0 = item.x & 0xffff, v0 = item.x >> 16;
    const int c0 = blockIdx.y * a.cg;
    const int e0 = item.y, e1 = item.z;
    if (e0 == e1) return;
    mbar_init(bar);
    if (!stage_region(reg, grid, &tmap, a.use_tma, bar, u0 - W / 2, v0 - W / 2, c0, a.cg, R, a.G1, a.G2, a.nb))
        return;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
    const int grp = lane / TM::LPP, gl = lane % TM::LPP;
    // warp per entry: the entry's taps are decoded once, then reused for every coil
    for (int e = e0 + warp; e < e1; e += nwarp) {
        const int s = a.ent_s[e];
        const short2 lb = a.ent_lb[e];
        const float* w = a.wts + (size_t)s * 2 * W;
        float wt[TM::TPL];
        int ro[TM::TPL];
#pragma unroll
        for (int i = 0; i < TM::TPL; ++i) {
            const int k = gl + i * TM::LPP;
            const int ta = k % W, tb = k / W;
            const bool ok = k < TM::TAPS;
            wt[i] = ok ? w[ta] * w[W + tb] : 0.f;
            ro[i] = ok ? (lb.y + tb + 1) * R + (lb.x + ta + 1) : 0;
        }
        for (int cb = 0; cb < a.cg; cb += TM::PPW) {
            const int c = cb + grp;
            const bool cv = c < a.cg;
            const float2* rc = reg + (size_t)(cv ? c : 0) * R * R;
            float2 v = make_float2(0.f, 0.f);
#pragma unroll
            for (int i = 0; i < TM::TPL; ++i) {
                const float2 g = rc[ro[i]];
                v.x += wt[i] * g.x;
                v.y += wt[i] * g.y;
            }
            v = group_sum<TM::LPP>(v);
            if (cv && gl == 0 && c0 + c < a.nb) {
                float f = 1.f;
                if (a.wfac) f = a.wfac[s + a.wfac_bstride * (c0 + c)];
                y[s + a.M * (c0 + c)] = make_float2(v.x * f, v.y * f);
            }
        }
    }
}

// Writes a CTA's accumulated tile: plain stores when the tile is owned by this
// CTA, vector reductions of the non-zero cells into a pre-zeroed region when
// several items share the tile.
// Two cells per thread-iteration (float4); T is a power of two, te1 is even.
// Owned (sub)tiles are written with plain float4 stores; a leaf tile shared by
// several items (pre-zeroed) receives vector reductions of its non-zero cells.
// Spreading accumulators in shared memory: per coil a real and an imaginary plane of
// T rows x (T + 4) floats (all real planes, then all imaginary planes), plane stride
// (T + 4) T + 16 floats.  Row stride = 4 (mod 32) words and adjacent coils' planes 16
// (mod 32) words apart put the 16 taps of a 4 x 4 footprint of two coils (one warp's
// atomics) on 32 distinct banks; a float2 tile with separate .x / .y atomics put four
// rows on the same banks.
__device__ __forceinline__ int acc_row(int T) { return T + 4; }
__device__ __forceinline__ int acc_plane(int T) { return (T + 4) * T + 16; }
inline size_t acc_plane_host(int T) { return (size_t)(T + 4) * T + 16; }

__device__ __forceinline__ void flush_tile(const float* acc, float2* __restrict__ out, bool shared, int T, int u0,
                                           int v0, int te1, int te2, int c0, const Bin2DArgs& a) {
    const int lgT = 31 - __clz(T);
    const int PS = acc_plane(T), RS = acc_row(T);
    const float* im = acc + (size_t)a.cg * PS;
    // two horizontally adjacent cells per iteration: T, te1 and the grid's first extent are
    // even (osN is, nufftOp.m:146-152), so a pair is valid as a whole, its accumulators are
    // float2-aligned and its grid cells float4-aligned
    const int lgh = 2 * lgT - 1;
    const int n = a.cg << lgh;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const int c = i >> lgh, r = (i & ((1 << lgh) - 1)) << 1, l2 = r >> lgT, l1 = r & (T - 1);
        if (l1 < te1 && l2 < te2 && c0 + c < a.nb) {
            float2* d = out + (u0 + l1) + (long long)a.G1 * ((v0 + l2) + (long long)a.G2 * (c0 + c));
            const int k = c * PS + l2 * RS + l1;
            const float2 re = *reinterpret_cast<const float2*>(acc + k);
            const float2 iv = *reinterpret_cast<const float2*>(im + k);
            if (!shared) {
                *reinterpret_cast<float4*>(d) = make_float4(re.x, iv.x, re.y, iv.y);
            } else {
                if (re.x != 0.f || iv.x != 0.f) atomicAdd(d, make_float2(re.x, iv.x));
                if (re.y != 0.f || iv.y != 0.f) atomicAdd(d + 1, make_float2(re.y, iv.y));
            }
        }
    }
}

// Zeroes the shared leaf tiles (block (k, c): tile k of plane c) before their items add into them.
__global__ void __launch_bounds__(256) zero_shared_tiles(float2* __restrict__ out, const int2* __restrict__ tiles,
                                                         int G1, int G2, const int* active) {
    pdl_wait();
    pdl_trigger();
    if (active && *active) return;
    const int2 t = tiles[blockIdx.x];
    const int u0 = t.x & 0xffff, v0 = t.x >> 16, T = t.y;
    float2* o = out + (long long)G1 * G2 * blockIdx.y;
    for (int i = threadIdx.x; i < T * T; i += blockDim.x) {
        const int l2 = i / T, l1 = i - l2 * T;
        if (u0 + l1 < G1 && v0 + l2 < G2) o[(u0 + l1) + (long long)G1 * (v0 + l2)] = make_float2(0.f, 0.f);
    }
}

static void zero_shared(NufftPlan& p, float2* out, long long nb, cudaStream_t st, const int* active) {
    const BinLists& b = p.bins;
    if (b.n_heavy == 0) return;
    launch_dependent(zero_shared_tiles, dim3((unsigned)b.n_heavy, (unsigned)nb), dim3(256), 0, st, out,
                     b.heavy.as<int2>(), p.G[0], p.G[1], active);
}

// Zeroes n floats (n a multiple of 4).
__device__ __forceinline__ void zero_acc(float* acc, int n) {
    float4* a4 = reinterpret_cast<float4*>(acc);
    for (int h = threadIdx.x; h < (n >> 2); h += blockDim.x) a4[h] = make_float4(0.f, 0.f, 0.f, 0.f);
}

template <int W>
__global__ void __launch_bounds__(256) spread2d_binned(const float2* __restrict__ y, float2* __restrict__ grid,
                                                       const Bin2DArgs a) {
    using TM = TapMap<W>;
    extern __shared__ float4 sm4[];
    if (a.active && *a.active) return;
    float* acc = reinterpret_cast<float*>(sm4);
    const int4 item = a.items[blockIdx.x];
    const int T = item.w & 255;                // this item's (sub)tile side
    const bool shared = (item.w >> 8) != 0;    // tile split across several items
    const int u0 = item.x & 0xffff, v0 = item.x >> 16;
    const int c0 = blockIdx.y * a.cg;
    const int te1 = min(T, a.G1 - u0), te2 = min(T, a.G2 - v0);
    const int PS = acc_plane(T), RS = acc_row(T);
    zero_acc(acc, 2 * a.cg * PS);
    __syncthreads();
    const int e0 = item.y, e1 = item.z;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
    const int grp = lane / TM::LPP, gl = lane % TM::LPP;
    constexpr int off0 = -W / 2 + 1;
    for (int e = e0 + warp; e < e1; e += nwarp) {
        const int s = a.ent_s[e];
        const short2 lb = a.ent_lb[e];
        const float* w = a.wts + (size_t)s * 2 * W;
        float wt[TM::TPL];
        int ao[TM::TPL];
#pragma unroll
        for (int i = 0; i < TM::TPL; ++i) {
            const int k = gl + i * TM::LPP;
            const int ta = k % W, tb = k / W;
            const int l1 = lb.x + off0 + ta, l2 = lb.y + off0 + tb;
            const bool ok = k < TM::TAPS && l1 >= 0 && l1 < te1 && l2 >= 0 && l2 < te2;
            wt[i] = ok ? w[ta] * w[W + tb] : 0.f;
            ao[i] = ok ? l2 * RS + l1 : -1;
        }
        for (int cb = 0; cb < a.cg; cb += TM::PPW) {
            const int c = cb + grp;
            if (c >= a.cg || c0 + c >= a.nb) continue;
            float2 v = y[s + a.M * (c0 + c)];
            if (a.wfac) {
                const float f = a.wfac[s + a.wfac_bstride * (c0 + c)];
                v.x *= f;
                v.y *= f;
            }
            float* re = acc + (size_t)c * PS;
            float* im = re + (size_t)a.cg * PS;
#pragma unroll
            for (int i = 0; i < TM::TPL; ++i) {
                if (ao[i] >= 0) {
                    atomicAdd(re + ao[i], wt[i] * v.x);
                    atomicAdd(im + ao[i], wt[i] * v.y);
                }
            }
        }
    }
    __syncthreads();
    flush_tile(acc, grid, shared, T, u0, v0, te1, te2, c0, a);
}

// Zeroes an owned (sub)tile of the coil group's output planes (an item no sample touches).
__device__ __forceinline__ void zero_tile(float2* __restrict__ out, int T, int u0, int v0, int te1, int te2, int c0,
                                          const Bin2DArgs& a) {
    const int lgT = 31 - __clz(T), lgh = 2 * lgT - 1;   // cell pairs, as in flush_tile
    const int n = a.cg << lgh;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const int c = i >> lgh, r = (i & ((1 << lgh) - 1)) << 1, l2 = r >> lgT, l1 = r & (T - 1);
        if (l1 < te1 && l2 < te2 && c0 + c < a.nb)
            *reinterpret_cast<float4*>(out + (u0 + l1) + (long long)a.G1 * ((v0 + l2) + (long long)a.G2 * (c0 + c))) =
                make_float4(0.f, 0.f, 0.f, 0.f);
    }
}

// Shared-memory float2 words of the input region / accumulator area per coil: the
// accumulators reuse the region once interpolation is done.
__host__ __device__ __forceinline__ int gn_area(int T, int W) {
    const int R = T + 2 * W, ps = (T + 4) * T + 16;   // acc_plane(T) floats, per real / imaginary plane
    return R * R > ps ? R * R : ps;
}

// Fused normal operator on the grid, out = C^H diag(wfac) C in per coil (nufftOp.m:354-394
// without the FFTs): one CTA per (work item, coil group).  The item's padded entries (at most
// `chunk`: items are built that way) are interpolated from the staged input region, weighted,
// and spread into the (sub)tile's accumulators, which alias the region.
template <int W>
__global__ void __launch_bounds__(256, 5) gridnorm2d_binned(const float2* __restrict__ gin, float2* __restrict__ gout,
                                                         const Bin2DArgs a, const __grid_constant__ CUtensorMap tmap) {
    using TM = TapMap<W>;
    extern __shared__ float4 sm4[];
    pdl_wait();
    pdl_trigger();
    if (a.active && *a.active) return;
    // all coil groups of an item launch together (blockIdx.x); items along y, then z past 65535
    const long long it = blockIdx.y + (long long)gridDim.y * blockIdx.z;
    if (it >= a.n_items) return;
    const int4 item = a.items[it];
    const int T = item.w & 255, R = T + 2 * W; // this item's (sub)tile and region sides
    const bool shared = (item.w >> 8) != 0;    // tile split across several items
    const int u0 = item.x & 0xffff, v0 = item.x >> 16;
    const int c0 = blockIdx.x * a.cg;
    const int te1 = min(T, a.G1 - u0), te2 = min(T, a.G2 - v0);
    const int e0 = item.y, ne = item.z - item.y;
    if (ne == 0) {
        zero_tile(gout, T, u0, v0, te1, te2, c0, a);
        return;
    }
    const int PS = acc_plane(T), RS = acc_row(T);
    uint64_t* bar;
    float2* reg = tma_layout(sm4, &bar);
    float* acc = reinterpret_cast<float*>(reg);
    // interpolated, weighted samples [entry][coil], then the entry lists: sample index,
    // base cell, the 2W tap weights, the per-sample weight of each (entry, coil)
    float2* sval = reg + (size_t)a.cg * gn_area(a.T, W);
    int* es = reinterpret_cast<int*>(sval + (size_t)a.chunk * a.cg);
    short2* elb = reinterpret_cast<short2*>(es + a.chunk);
    float* ew = reinterpret_cast<float*>(elb + a.chunk);
    float* ef = ew + (size_t)a.chunk * 2 * W;
    mbar_init(bar);
    // the region copy is issued first and waited for after the entry lists are loaded; the
    // tensor map's box is a full tile's region, so sub-tiles use plain loads
    const bool tma = region_issue(reg, &tmap, a.use_tma && T == a.T, bar, u0 - W, v0 - W, c0, a.cg, R, a.G1, a.G2);
    if (!tma) region_plain(reg, gin, u0 - W, v0 - W, c0, a.cg, R, a.G1, a.G2, a.nb);
    // the item's lists and inline tap weights are contiguous: independent, coalesced loads
    for (int i = threadIdx.x; i < ne; i += blockDim.x) {
        es[i] = a.ent_s[e0 + i];
        elb[i] = a.ent_lb[e0 + i];
    }
    for (int j = threadIdx.x; j < ne * 2 * W; j += blockDim.x) ew[j] = a.ent_w[(size_t)e0 * 2 * W + j];
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
    constexpr int off0 = -W / 2 + 1;
    int lgcg = 0;
    while ((1 << lgcg) < a.cg) ++lgcg;
    const int npair = ne << lgcg;
    // the weights are gathered by sample index while the region copy completes
    if (a.wfac) {
        for (int q = threadIdx.x; q < npair; q += blockDim.x) {
            const int i = q >> lgcg, c = q & (a.cg - 1);
            ef[q] = c0 + c < a.nb ? a.wfac[es[i] + a.wfac_bstride * (c0 + c)] : 0.f;
        }
    }
    if (tma && !mbar_wait(bar, 0)) return;
    __syncthreads();
    // phase 1 — interpolation, one thread per (entry, coil), separable weights:
    //   v = sum_b w2[b] sum_a w1[a] g[b][a]; independent loads, no shuffles, no atomics.
    //   The coil planes of the region lie a multiple of 32 banks apart, so with 4 or more coils
    //   consecutive threads take consecutive entries of one coil (with 2, consecutive coils of
    //   one entry measured faster).
    const bool coil_major = a.cg >= 4;
    for (int q = threadIdx.x; q < npair; q += blockDim.x) {
        const int c = coil_major ? q / ne : (q & (a.cg - 1));
        const int i = coil_major ? q - c * ne : (q >> lgcg);
        const int p = (i << lgcg) + c;
        const short2 lb = elb[i];
        const float* w1 = ew + i * 2 * W;
        const float* w2 = w1 + W;
        const float2* rc = reg + (size_t)c * R * R + (lb.y + off0 + W) * R + (lb.x + off0 + W);
        float2 v = make_float2(0.f, 0.f);
#pragma unroll
        for (int b = 0; b < W; ++b) {
            float2 row = make_float2(0.f, 0.f);
#pragma unroll
            for (int q = 0; q < W; ++q) {
                const float2 g = rc[b * R + q];
                row.x += w1[q] * g.x;
                row.y += w1[q] * g.y;
            }
            v.x += w2[b] * row.x;
            v.y += w2[b] * row.y;
        }
        const float f = a.wfac ? ef[p] : 1.f;
        sval[p] = make_float2(v.x * f, v.y * f);
    }
    __syncthreads();
    zero_acc(acc, 2 * a.cg * PS);   // the region is no longer read
    __syncthreads();
    // phase 2 — spreading, one lane per tap; the entry's taps are decoded once per warp
    const int grp = lane / TM::LPP, gl = lane % TM::LPP;
    for (int i = warp; i < ne; i += nwarp) {
        const short2 lb = elb[i];
        const float* w = ew + i * 2 * W;
        float wt[TM::TPL];
        int ao[TM::TPL];
#pragma unroll
        for (int t = 0; t < TM::TPL; ++t) {
            const int k = gl + t * TM::LPP;
            const int ta = k % W, tb = k / W;
            const int l1 = lb.x + off0 + ta, l2 = lb.y + off0 + tb;
            const bool ok = k < TM::TAPS && l1 >= 0 && l1 < te1 && l2 >= 0 && l2 < te2;
            wt[t] = ok ? w[ta] * w[W + tb] : 0.f;
            ao[t] = ok ? l2 * RS + l1 : -1;
        }
        const float2* sv = sval + (i << lgcg);
        for (int cb = 0; cb < a.cg; cb += TM::PPW) {
            const int c = cb + grp;
            if (c >= a.cg || c0 + c >= a.nb) continue;
            const float2 v = sv[c];
            float* re = acc + (size_t)c * PS;
            float* im = re + (size_t)a.cg * PS;
#pragma unroll
            for (int t = 0; t < TM::TPL; ++t) {
                if (ao[t] >= 0) {
                    atomicAdd(re + ao[t], wt[t] * v.x);
                    atomicAdd(im + ao[t], wt[t] * v.y);
                }
            }
        }
    }
    __syncthreads();
    flush_tile(acc, gout, shared, T, u0, v0, te1, te2, c0, a);
}

// ------------------------------------------------------------ generic kernels --
struct GenArgs {
    const int* base;     // [nd][M]
    const float* wts;    // [M][nd][W]
    const float* wfac;
    long long wfac_bstride;
    int nd, W;
    int G1, G2, G3;
    long long M, nb;
    const int* active;
};

__global__ void interp_generic(const float2* __restrict__ grid, float2* __restrict__ y, const GenArgs a) {
    if (a.active && *a.active) return;
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.M * a.nb) return;
    const long long s = i % a.M, bb = i / a.M;
    const int W = a.W, off0 = -W / 2 + 1;
    const float* w = a.wts + (size_t)s * a.nd * W;
    const int c1 = a.base[s];
    const int c2 = a.nd > 1 ? a.base[a.M + s] : 0;
    const int c3 = a.nd > 2 ? a.base[2 * a.M + s] : 0;
    const long long Gt = (long long)a.G1 * a.G2 * a.G3;
    const float2* g = grid + Gt * bb;
    float2 acc = make_float2(0.f, 0.f);
    const int n2 = a.nd > 1 ? W : 1, n3 = a.nd > 2 ? W : 1;
    for (int k3 = 0; k3 < n3; ++k3) {
        int u3 = 0;
        float w3 = 1.f;
        if (a.nd > 2) { u3 = c3 + off0 + k3; u3 += u3 < 0 ? a.G3 : 0; u3 -= u3 >= a.G3 ? a.G3 : 0; w3 = w[2 * W + k3]; }
        for (int k2 = 0; k2 < n2; ++k2) {
            int u2 = 0;
            float w2 = 1.f;
            if (a.nd > 1) { u2 = c2 + off0 + k2; u2 += u2 < 0 ? a.G2 : 0; u2 -= u2 >= a.G2 ? a.G2 : 0; w2 = w[W + k2]; }
            for (int k1 = 0; k1 < W; ++k1) {
                int u1 = c1 + off0 + k1;
                u1 += u1 < 0 ? a.G1 : 0;
                u1 -= u1 >= a.G1 ? a.G1 : 0;
                const float wt = w[k1] * w2 * w3;
                const float2 v = g[u1 + (long long)a.G1 * (u2 + (long long)a.G2 * u3)];
                acc.x += wt * v.x;
                acc.y += wt * v.y;
            }
        }
    }
    float f = 1.f;
    if (a.wfac) f = a.wfac[s + a.wfac_bstride * bb];
    y[i] = make_float2(acc.x * f, acc.y * f);
}

__global__ void spread_generic(const float2* __restrict__ y, float2* __restrict__ grid, const GenArgs a) {
    if (a.active && *a.active) return;
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.M * a.nb) return;
    const long long s = i % a.M, bb = i / a.M;
    const int W = a.W, off0 = -W / 2 + 1;
    const float* w = a.wts + (size_t)s * a.nd * W;
    float2 v = y[i];
    if (a.wfac) {
        const float f = a.wfac[s + a.wfac_bstride * bb];
        v.x *= f;
        v.y *= f;
    }
    const int c1 = a.base[s];
    const int c2 = a.nd > 1 ? a.base[a.M + s] : 0;
    const int c3 = a.nd > 2 ? a.base[2 * a.M + s] : 0;
    const long long Gt = (long long)a.G1 * a.G2 * a.G3;
    float2* g = grid + Gt * bb;
    const int n2 = a.nd > 1 ? W : 1, n3 = a.nd > 2 ? W : 1;
    for (int k3 = 0; k3 < n3; ++k3) {
        int u3 = 0;
        float w3 = 1.f;
        if (a.nd > 2) { u3 = c3 + off0 + k3; u3 += u3 < 0 ? a.G3 : 0; u3 -= u3 >= a.G3 ? a.G3 : 0; w3 = w[2 * W + k3]; }
        for (int k2 = 0; k2 < n2; ++k2) {
            int u2 = 0;
            float w2 = 1.f;
            if (a.nd > 1) { u2 = c2 + off0 + k2; u2 += u2 < 0 ? a.G2 : 0; u2 -= u2 >= a.G2 ? a.G2 : 0; w2 = w[W + k2]; }
            for (int k1 = 0; k1 < W; ++k1) {
                int u1 = c1 + off0 + k1;
                u1 += u1 < 0 ? a.G1 : 0;
                u1 -= u1 >= a.G1 ? a.G1 : 0;
                const float wt = w[k1] * w2 * w3;
                float2* d = g + u1 + (long long)a.G1 * (u2 + (long long)a.G2 * u3);
                atomicAdd(&d->x, wt * v.x);
                atomicAdd(&d->y, wt * v.y);
            }
        }
    }
}

// ---------------------------------------------------------------- dispatch ----
static int pick_cg(const NufftPlan& p, long long nb, size_t per_coil_bytes, size_t fixed) {
    const size_t lim = (size_t)std::min(device_smem_optin(), 200 * 1024);
    int cg = std::max(1, std::min(8, p.cg_pref));
    while (cg > 1 && fixed + per_coil_bytes * cg > lim) cg /= 2;
    while (cg > 1 && cg / 2 >= nb) cg /= 2;
    return cg;
}

static Bin2DArgs bin_args(const NufftPlan& p, bool own, const float* wfac, long long wfb, long long nb, int cg,
                          bool tma, const int* active) {
    Bin2DArgs a;
    const BinLists& b = p.bins;
    a.items = own ? b.own_items.as<int4>() : b.pad_items.as<int4>();
    a.ent_s = own ? b.own_s.as<int>() : b.pad_s.as<int>();
    a.ent_lb = own ? b.own_lb.as<short2>() : b.pad_lb.as<short2>();
    a.ent_w = own ? nullptr : b.pad_w.as<float>();
    a.wts = p.d_w.as<float>();
    a.wfac = wfac;
    a.wfac_bstride = wfb;
    a.G1 = p.G[0];
    a.G2 = p.G[1];
    a.T = b.T;
    a.lgT = 0;
    while ((1 << a.lgT) < b.T) ++a.lgT;
    a.ntx = b.ntx;
    a.M = p.M;
    a.nb = nb;
    a.cg = cg;
    a.use_tma = tma ? 1 : 0;
    a.chunk = b.chunk;
    a.n_items = own ? b.n_own_items : b.n_pad_items;
    a.active = active;
    return a;
}

template <class K>
static void set_smem(K kern, size_t smem) {
    MMR_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
}

#define MMR_W_DISPATCH(W, ...)                                \
    switch (W) {                                              \
        case 2: { constexpr int KW = 2; __VA_ARGS__; } break; \
        case 4: { constexpr int KW = 4; __VA_ARGS__; } break; \
        case 6: { constexpr int KW = 6; __VA_ARGS__; } break; \
        case 8: { constexpr int KW = 8; __VA_ARGS__; } break; \
        default: MMR_THROW(MMR_ERR_UNSUPPORTED, "kwidth %d", (W)); \
    }

static GenArgs gen_args(const NufftPlan& p, const float* wfac, long long wfb, long long nb, const int* active) {
    GenArgs g;
    g.base = p.d_base.as<int>();
    g.wts = p.d_w.as<float>();
    g.wfac = wfac;
    g.wfac_bstride = wfb;
    g.nd = p.nd;
    g.W = p.W;
    g.G1 = p.G[0];
    g.G2 = p.G[1];
    g.G3 = p.G[2];
    g.M = p.M;
    g.nb = nb;
    g.active = active;
    return g;
}

void nufft_interp(NufftPlan& p, const float2* grid, float2* y, long long nb, const float* wfac, long long wfb,
                  cudaStream_t st, const int* active) {
    if (!p.use_bins) {
        const long long n = p.M * nb;
        interp_generic<<<(unsigned)cdiv(n, 256), 256, 0, st>>>(grid, y, gen_args(p, wfac, wfb, nb, active));
        check_launch("interp_generic");
        return;
    }
    const int R = p.bins.T + p.W;
    const int cg = pick_cg(p, nb, (size_t)R * R * 8, kTmaSmemExtra);
    if (p.tmap_ptr != grid || p.tmap_nb != nb || p.tmap_cg != cg) {
        encode_grid_map(&p.tmap, grid, p.G[0], p.G[1], nb, R, cg);
        p.tmap_ptr = grid;
        p.tmap_nb = nb;
        p.tmap_cg = cg;
    }
    const size_t smem = kTmaSmemExtra + (size_t)cg * R * R * 8;
    Bin2DArgs a = bin_args(p, true, wfac, wfb, nb, cg, true, active);
    dim3 gridDim((unsigned)p.bins.n_own_items, (unsigned)cdiv(nb, cg));
    if (p.bins.n_own_items == 0) return;
    MMR_W_DISPATCH(p.W, {
        set_smem(interp2d_binned<KW>, smem);
        interp2d_binned<KW><<<gridDim, 256, smem, st>>>(grid, y, a, p.tmap);
    });
    check_launch("interp2d_binned");
}

void nufft_spread(NufftPlan& p, const float2* y, float2* grid, long long nb, const float* wfac, long long wfb,
                  cudaStream_t st, const int* active) {
    if (!p.use_bins) {
        MMR_CUDA(cudaMemsetAsync(grid, 0, (size_t)p.Gtot * nb * sizeof(float2), st));
        const long long n = p.M * nb;
        spread_generic<<<(unsigned)cdiv(n, 256), 256, 0, st>>>(y, grid, gen_args(p, wfac, wfb, nb, active));
        check_launch("spread_generic");
        return;
    }
    const int T = p.bins.T;
    const int cg = pick_cg(p, nb, acc_plane_host(T) * 8, 0);
    const size_t smem = (size_t)cg * acc_plane_host(T) * 8;
    Bin2DArgs a = bin_args(p, false, wfac, wfb, nb, cg, false, active);
    dim3 gridDim((unsigned)p.bins.n_pad_items, (unsigned)cdiv(nb, cg));
    zero_shared(p, grid, nb, st, active);
    MMR_W_DISPATCH(p.W, {
        set_smem(spread2d_binned<KW>, smem);
        spread2d_binned<KW><<<gridDim, 256, smem, st>>>(y, grid, a);
    });
    check_launch("spread2d_binned");
}

bool nufft_has_fused_normal(const NufftPlan& p) { return p.use_bins; }

static CUtensorMap g_norm_map;   // cache for the fused kernel's box

void nufft_grid_normal(NufftPlan& p, const float2* gin, float2* gout, long long nb, const float* wfac, long long wfb,
                       cudaStream_t st, const int* active) {
    MMR_REQUIRE(p.use_bins, "fused gridding needs the 2D binned path");
    const int T = p.bins.T, R = T + 2 * p.W;
    const size_t ent = (size_t)p.bins.chunk * (8 + 8 * p.W);    // staged entry lists (gridnorm2d_binned)
    // per coil: region / accumulators, interpolated samples, per-sample weights
    const size_t per_coil = ((size_t)gn_area(T, p.W) + p.bins.chunk) * 8 + (size_t)p.bins.chunk * 4;
    const int cg = pick_cg(p, nb, per_coil, kTmaSmemExtra + ent);
    static const void* cptr = nullptr;
    static long long cnb = 0;
    static int ccg = 0, cR = 0, cG1 = 0, cG2 = 0;
    if (cptr != gin || cnb != nb || ccg != cg || cR != R || cG1 != p.G[0] || cG2 != p.G[1]) {
        encode_grid_map(&g_norm_map, gin, p.G[0], p.G[1], nb, R, cg);
        cptr = gin;
        cnb = nb;
        ccg = cg;
        cR = R;
        cG1 = p.G[0];
        cG2 = p.G[1];
    }
    const size_t smem = kTmaSmemExtra + ent + (size_t)cg * per_coil;
    Bin2DArgs a = bin_args(p, false, wfac, wfb, nb, cg, true, active);
    const long long ny = std::min(p.bins.n_pad_items, 65535);
    dim3 gridDim((unsigned)cdiv(nb, cg), (unsigned)ny, (unsigned)cdiv(p.bins.n_pad_items, ny));
    zero_shared(p, gout, nb, st, active);
    MMR_W_DISPATCH(p.W, {
        set_smem(gridnorm2d_binned<KW>, smem);
        launch_dependent(gridnorm2d_binned<KW>, gridDim, dim3(256), smem, st, gin, gout, a, g_norm_map);
    });
}

// ------------------------------------------------------------- FFT pipelines --
static int pow2_floor(int v) {
    int r = 1;
    while (r * 2 <= v) r *= 2;
    return r;
}

static PassArgs base_pass(const NufftPlan& p, int axis, int sign) {
    PassArgs a;
    a.L = p.G[axis];
    a.f = p.ff[axis];
    a.tw = p.tw[axis];
    a.sign = sign;
    a.scale = (float)(1.0 / std::sqrt((double)p.G[axis]));
    a.B = pow2_floor(std::max(1, std::min(p.fft_lines, 4096 / a.L)));
    return a;
}

void nufft_img_to_grid(NufftPlan& p, const float2* x, const float2* maps, float2* grid, long long nb, cudaStream_t st,
                       const int* active) {
    // axis order 0, 1, 2: image extents shrink to grid extents one axis at a time
    long long ext[3] = {p.N[0], p.N[1], p.N[2]};
    float2* tmp = nullptr;
    if (p.nd > 1) {
        // intermediate buffers: after axis 0: [G1, N2, N3, nb]; after axis 1: [G1, G2, N3, nb]
        const size_t need = (size_t)p.G[0] * p.N[1] * p.N[2] * nb;
        const size_t need2 = p.nd > 2 ? (size_t)p.G[0] * p.G[1] * p.N[2] * nb : 0;
        p.s_tmp.ensure((need + need2) * sizeof(float2));
        tmp = p.s_tmp.as<float2>();
    }
    const float2* src = x;
    for (int ax = 0; ax < p.nd; ++ax) {
        PassArgs a = base_pass(p, ax, +1);
        long long inner = 1, outer = nb;
        for (int k = 0; k < ax; ++k) inner *= p.G[k];
        for (int k = ax + 1; k < 3; ++k) outer *= ext[k];
        a.inner = inner;
        a.outer = outer;
        a.nin = p.N[ax];
        a.in_start = p.G[ax] - p.N[ax] / 2;
        a.nout = p.G[ax];
        a.out_start = p.G[ax] / 2;
        // axis 0 applies its own factor per point and the others' per line; later axes none
        a.in_fac = ax == 0 ? p.d_fwd_fac[0].as<float2>() : nullptr;
        if (ax == 0 && p.nd > 1) {
            a.in_line = p.d_fwd_line.as<float2>();
            a.lpc = (long long)p.N[1] * p.N[2];
        }
        a.active = active;
        float2* dst;
        if (ax == p.nd - 1) dst = grid;
        else if (ax == 0) dst = tmp;
        else dst = tmp + (size_t)p.G[0] * p.N[1] * p.N[2] * nb;
        a.in = src;
        a.out = dst;
        int mode = PASS_PLAIN;
        if (ax == 0 && maps) {
            mode = PASS_FWD_IMG;
            a.maps = maps;
            a.lpc = (long long)p.N[1] * p.N[2];
        }
        prof_mark(ax == 0 ? 0 : 1, st);
        launch_fft_pass(mode, a, st);
        ext[ax] = p.G[ax];
        src = dst;
    }
}

size_t nufft_grid_to_img_scratch(const NufftPlan& p, long long nb) {
    if (p.nd < 2) return 0;
    const size_t need = (size_t)p.N[0] * p.G[1] * p.G[2] * nb;
    const size_t need2 = p.nd > 2 ? (size_t)p.N[0] * p.N[1] * p.G[2] * nb : 0;
    return need + need2;
}

// out (+)= sum_c conj(maps_c) .* img_c over nb per-coil images of n voxels (the rcvrOp adjoint,
// rcvrOp.m:144-157, after the per-coil nufftOp adjoint), summed in coil order: deterministic.
// With dacc: the DotEpilogue (out += tik .* dv, then dacc += v' out) in the same pass.
__global__ void __launch_bounds__(256) coil_combine_kernel(const float2* __restrict__ img,
                                                           const float2* __restrict__ maps, float2* __restrict__ out,
                                                           long long n, int nb, int accumulate, const int* active,
                                                           const float2* __restrict__ dv,
                                                           const float* __restrict__ tik, double* dacc) {
    pdl_wait();
    pdl_trigger();
    if (active && *active) return;
    double d[2] = {0, 0};
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        float2 s = make_float2(0.f, 0.f);
        // unrolled so the coils' loads issue together; the sum keeps the coil order
#pragma unroll 8
        for (int c = 0; c < nb; ++c) s = cadd(s, cmulc(img[i + n * c], maps[i + n * c]));
        if (accumulate) s = cadd(out[i], s);
        if (dacc) {
            const float2 v = dv[i];
            if (tik) s = make_float2(s.x + tik[i] * v.x, s.y + tik[i] * v.y);
            d[0] += (double)v.x * s.x + (double)v.y * s.y;     // re(conj(v) s)
            d[1] += (double)v.x * s.y - (double)v.y * s.x;     // im(conj(v) s)
        }
        out[i] = s;
    }
    if (dacc) {
        double* const dst[2] = {dacc, dacc + 1};
        block_accumulate<2>(d, dst);
    }
}

void nufft_grid_to_img(NufftPlan& p, const float2* grid, const float2* maps, float2* out, long long nb,
                       bool accumulate, cudaStream_t st, const int* active, float2* scratch,
                       const DotEpilogue* dot) {
    MMR_REQUIRE(!dot || maps, "the dot epilogue runs in the coil sum");
    long long ext[3] = {p.G[0], p.G[1], p.G[2]};
    float2* tmp = scratch;
    if (p.nd > 1 && !tmp) {
        p.s_tmp.ensure(nufft_grid_to_img_scratch(p, nb) * sizeof(float2));
        tmp = p.s_tmp.as<float2>();
    }
    // with maps, the last pass writes the per-coil images, then one kernel weights and sums them
    float2* per_coil = nullptr;
    if (maps) {
        p.s_coil.ensure((size_t)p.Ntot * nb * sizeof(float2));
        per_coil = p.s_coil.as<float2>();
    }
    const float2* src = grid;
    for (int ax = 0; ax < p.nd; ++ax) {
        PassArgs a = base_pass(p, ax, -1);
        long long inner = 1, outer = nb;
        for (int k = 0; k < ax; ++k) inner *= p.N[k];
        for (int k = ax + 1; k < 3; ++k) outer *= ext[k];
        a.inner = inner;
        a.outer = outer;
        a.nin = p.G[ax];
        a.in_start = p.G[ax] / 2;
        a.nout = p.N[ax];
        a.out_start = p.G[ax] - p.N[ax] / 2;
        // the last axis applies its own factor per point and the others' per line; earlier axes none
        const bool last = ax == p.nd - 1;
        a.out_fac = last ? p.d_adj_fac[ax].as<float2>() : nullptr;
        if (last && p.nd > 1) a.out_line = p.d_adj_line.as<float2>();
        a.active = active;
        float2* dst;
        if (last) dst = maps ? per_coil : out;
        else if (ax == 0) dst = tmp;
        else dst = tmp + (size_t)p.N[0] * p.G[1] * p.G[2] * nb;
        a.in = src;
        a.out = dst;
        prof_mark(last ? 4 : 3, st);
        launch_fft_pass(PASS_PLAIN, a, st);
        ext[ax] = p.N[ax];
        src = dst;
    }
    if (maps) {
        const long long n = p.Ntot;
        const unsigned blocks = (unsigned)std::min<long long>(cdiv(n, 256), (long long)device_sm_count() * 8);
        launch_dependent(coil_combine_kernel, dim3(blocks), dim3(256), 0, st, per_coil, maps, out, n, (int)nb,
                         accumulate ? 1 : 0, active, dot ? dot->v : nullptr, dot ? dot->tik : nullptr,
                         dot ? dot->acc : nullptr);
    }
}

void nufft_forward(NufftPlan& p, const float2* x, float2* y, long long nb, cudaStream_t st, const int* active) {
    p.s_grid.ensure((size_t)p.Gtot * nb * sizeof(float2));
    float2* grid = p.s_grid.as<float2>();
    nufft_img_to_grid(p, x, nullptr, grid, nb, st, active);
    nufft_interp(p, grid, y, nb, p.has_dcf ? p.d_dcf.as<float>() : nullptr, 0, st, active);
}

void nufft_adjoint(NufftPlan& p, const float2* y, float2* x, long long nb, cudaStream_t st, const int* active) {
    p.s_grid.ensure((size_t)p.Gtot * nb * sizeof(float2));
    float2* grid = p.s_grid.as<float2>();
    nufft_spread(p, y, grid, nb, p.has_dcf ? p.d_dcf.as<float>() : nullptr, 0, st, active);
    nufft_grid_to_img(p, grid, nullptr, x, nb, false, st, active);
}

// ------------------------------------------------------------------ Toeplitz --
__global__ void cmul_bcast_kernel(float2* __restrict__ x, const float2* __restrict__ t, long long n, long long nt) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) x[i] = cmul(x[i], t[i % nt]);
}

__global__ void cscale_kernel(float2* __restrict__ x, float s, long long n) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) x[i] = cscale(x[i], s);
}

// Centered (i)fft passes on a [2N]^d grid: ifftnc/fftnc with doShift = 1 (general/fftnc.m:32-42).
static void toep_passes(NufftPlan& p, const float2* in, float2* out, long long nb, int sign, int nin_mode,
                        cudaStream_t st, float2* tmp) {
    // nin_mode 0: input is the N-image (pad to 2N, centered) -> output full 2N grid
    // nin_mode 1: input is the full 2N grid -> output cropped N-image
    // nin_mode 2: full 2N grid -> full 2N grid
    long long ext[3];
    int L[3] = {1, 1, 1};
    for (int k = 0; k < 3; ++k) {
        L[k] = k < p.nd ? 2 * p.N[k] : 1;
        ext[k] = (nin_mode == 0) ? (k < p.nd ? p.N[k] : 1) : L[k];
    }
    const float2* src = in;
    for (int ax = 0; ax < p.nd; ++ax) {
        PassArgs a;
        a.L = L[ax];
        a.f = p.tff[ax];
        a.tw = p.ttw[ax];
        a.sign = sign;
        a.scale = (float)(1.0 / std::sqrt((double)L[ax]));
        a.B = pow2_floor(std::max(1, std::min(16, 2048 / a.L)));
        long long inner = 1, outer = nb;
        int outn = (nin_mode == 1) ? p.N[ax] : L[ax];
        for (int k = 0; k < ax; ++k) inner *= (nin_mode == 1 ? p.N[k] : L[k]);
        for (int k = ax + 1; k < 3; ++k) outer *= ext[k];
        a.inner = inner;
        a.outer = outer;
        if (nin_mode == 0) { a.nin = p.N[ax]; a.in_start = L[ax] - p.N[ax] / 2; }
        else { a.nin = L[ax]; a.in_start = L[ax] / 2; }
        a.nout = outn;
        a.out_start = (nin_mode == 1) ? L[ax] - p.N[ax] / 2 : L[ax] / 2;
        const bool last = ax == p.nd - 1;
        float2* dst = last ? out : tmp + (size_t)(ax & 1) * (size_t)(8LL * p.Ntot * nb);
        a.in = src;
        a.out = dst;
        launch_fft_pass(PASS_PLAIN, a, st);
        ext[ax] = outn;
        src = dst;
    }
}

void nufft_prep_toep(NufftPlan& p, double tos, int kw) {
    if (p.is_toep) return;
    if (tos <= 0) tos = 0.5 * (p.os - 1) + 1;                               // nufftOp.m:416
    if (kw <= 0) kw = p.W;
    mmr_nufft_desc d = {};
    d.ndim = p.nd;
    for (int k = 0; k < p.nd; ++k) d.imN[k] = 2 * p.N[k];
    d.nsamp = p.M;
    d.kloc = p.kloc.data();
    d.dcf = p.dcf_h.empty() ? nullptr : p.dcf_h.data();
    d.os = tos;
    d.kwidth = kw;
    NufftPlan S;
    nufft_plan_build(S, d);                                                 // nufftOp.m:421
    std::vector<float2> v(p.M);
    for (long long s = 0; s < p.M; ++s) v[s] = make_float2(p.dcf_h.empty() ? 1.f : (float)p.dcf_h[s], 0.f);
    DevBuf dv, dimg;
    dv.upload(v);
    long long n2 = 1;
    for (int k = 0; k < p.nd; ++k) {
        n2 *= 2 * p.N[k];
        p.tff[k] = fft_factorize(2 * p.N[k]);
        p.ttw[k] = fft_twiddles(2 * p.N[k]);
    }
    dimg.ensure(n2 * sizeof(float2));
    nufft_adjoint(S, dv.as<float2>(), dimg.as<float2>(), 1, 0, nullptr);   // S'*dcf (423/425)
    p.d_toep.ensure(n2 * sizeof(float2));
    DevBuf tmp;
    tmp.ensure((size_t)2 * 8 * p.Ntot * sizeof(float2));
    toep_passes(p, dimg.as<float2>(), p.d_toep.as<float2>(), 1, +1, 2, 0, tmp.as<float2>());  // ifftnc (427)
    cscale_kernel<<<(unsigned)cdiv(n2, 256), 256>>>(p.d_toep.as<float2>(), (float)(1 << p.nd), n2);
    check_launch("cscale");
    MMR_CUDA(cudaDeviceSynchronize());
    p.is_toep = true;
}

void nufft_toep_apply(NufftPlan& p, const float2* x, float2* y, long long nb, cudaStream_t st) {
    long long n2 = 1;
    for (int k = 0; k < p.nd; ++k) n2 *= 2 * p.N[k];
    p.s_grid.ensure((size_t)n2 * nb * sizeof(float2));
    p.s_grid2.ensure((size_t)2 * 8 * p.Ntot * nb * sizeof(float2));
    float2* g = p.s_grid.as<float2>();
    toep_passes(p, x, g, nb, +1, 0, st, p.s_grid2.as<float2>());           // ifftnc(padcrop(x, 2N))
    cmul_bcast_kernel<<<(unsigned)cdiv(n2 * nb, 256), 256, 0, st>>>(g, p.d_toep.as<float2>(), n2 * nb, n2);
    check_launch("toep multiply");
    toep_passes(p, g, y, nb, -1, 1, st, p.s_grid2.as<float2>());           // padcrop(fftnc(.), N)
}

}  // namespace mmr
