// bfista (iterativeSolvers/bfista.m), powermethod (iterativeSolvers/powermethod.m),
// softthresh (general/softthresh.m) and the undecimated db1 dwtND (operators/@dwtND)
// on the device.
//
// Haar filter bank (dwtND.m:108-116 with wfilters('db1') / sqrt(2) when
// undecimated): Lo_D = [1 1]/2, Hi_D = [-1 1]/2, Lo_R = [1 1]/2, Hi_R = [1 -1]/2.
// wavConv1D.m:22-43 (object domain, undecimated, shift 2^(j-1)):
//   decomposition   y[i] = f1 x[i] + f2 x[i + s]       (circshift(x, -(n-1)s))
//   reconstruction  y[i] = f1 x[i - s] + f2 x[i]
// Band order and the sequence of 1D filterings follow decompSep / reconSep
// (@dwtND/mtimes.m:74-122): bands = [low, high{1}{1..}, high{2}{1..}, ...].
// Vectors are complex64, every norm / inner product FP64.
#include <cmath>
#include <vector>

#include "sense.cuh"

namespace mmr {

struct DwtShape {
    int nd;
    long long n[3];
    long long tot;
    int J[3];
};

static int dwt_nbands(const DwtShape& s) {
    int jmax = 0;
    for (int d = 0; d < s.nd; ++d) jmax = std::max(jmax, s.J[d]);
    int nb = 1;
    for (int j = 1; j <= jmax; ++j) {
        int k = 0;
        for (int d = 0; d < s.nd; ++d) k += s.J[d] >= j;
        nb += (1 << k) - 1;
    }
    return nb;
}

// y = f1 * x[i] + f2 * x[i + s*dir] along dimension `dim` (periodic); accumulate: y +=.
__global__ void haar_conv_kernel(const float2* __restrict__ x, float2* __restrict__ y, long long n0, long long n1,
                                 long long n2, int dim, long long s, float f1, float f2, int recon, int accumulate) {
    const long long tot = n0 * n1 * n2;
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= tot) return;
    const long long i0 = i % n0, i1 = (i / n0) % n1, i2 = i / (n0 * n1);
    long long c[3] = {i0, i1, i2};
    const long long nn[3] = {n0, n1, n2};
    const long long stride[3] = {1, n0, n0 * n1};
    const long long L = nn[dim];
    long long shifted;
    if (!recon) shifted = (c[dim] + s) % L;                     // decomposition: x[i + s]
    else shifted = ((c[dim] - s) % L + L) % L;                  // reconstruction: x[i - s]
    const long long j = i + (shifted - c[dim]) * stride[dim];
    float2 v;
    if (!recon) v = make_float2(f1 * x[i].x + f2 * x[j].x, f1 * x[i].y + f2 * x[j].y);
    else v = make_float2(f1 * x[j].x + f2 * x[i].x, f1 * x[j].y + f2 * x[i].y);
    if (accumulate) v = cadd(y[i], v);
    y[i] = v;
}

struct DwtWork {
    DwtShape s;
    DevBuf tmp;   // scratch band
};

static void conv(const DwtShape& sh, const float2* x, float2* y, int dim, long long shift, const float* f, bool recon,
                 bool accumulate, cudaStream_t st) {
    const long long n0 = sh.n[0], n1 = sh.nd > 1 ? sh.n[1] : 1, n2 = sh.nd > 2 ? sh.n[2] : 1;
    haar_conv_kernel<<<(unsigned)cdiv(sh.tot, 256), 256, 0, st>>>(x, y, n0, n1, n2, dim, shift, f[0], f[1],
                                                                 recon ? 1 : 0, accumulate ? 1 : 0);
    check_launch("haar_conv");
}

static const float LO_D[2] = {0.5f, 0.5f}, HI_D[2] = {-0.5f, 0.5f}, LO_R[2] = {0.5f, 0.5f}, HI_R[2] = {0.5f, -0.5f};

// bands: nbands * tot complex values (band 0 = low).  decomp: x -> bands.
static void dwt_decomp(DwtWork& w, const float2* x, float2* bands, cudaStream_t st) {
    const DwtShape& sh = w.s;
    const long long T = sh.tot;
    w.tmp.ensure((size_t)T * sizeof(float2));
    float2* low = bands;
    MMR_CUDA(cudaMemcpyAsync(low, x, T * 8, cudaMemcpyDeviceToDevice, st));
    int jmax = 0;
    for (int d = 0; d < sh.nd; ++d) jmax = std::max(jmax, sh.J[d]);
    int bi = 1;   // first band index of this level's high set
    for (int j = 1; j <= jmax; ++j) {
        const long long shift = 1LL << (j - 1);
        int k = 0;
        for (int d = 0; d < sh.nd; ++d) k += sh.J[d] >= j;
        float2* hj = bands + (size_t)bi * T;     // high{j}{1..2^k-1}: hj + (m-1)*T
        int ds = 0;
        for (int d = 0; d < sh.nd; ++d) {
            if (sh.J[d] < j) continue;
            // high{2^ds} = conv(low, Hi)  (mtimes.m:86)
            conv(sh, low, hj + (size_t)((1 << ds) - 1) * T, d, shift, HI_D, false, false, st);
            for (int s = 1; s <= (1 << ds) - 1; ++s) {
                float2* hs = hj + (size_t)(s - 1) * T;
                conv(sh, hs, hj + (size_t)((1 << ds) + s - 1) * T, d, shift, HI_D, false, false, st);   // 88
                conv(sh, hs, w.tmp.as<float2>(), d, shift, LO_D, false, false, st);                   // 89
                MMR_CUDA(cudaMemcpyAsync(hs, w.tmp.p, T * 8, cudaMemcpyDeviceToDevice, st));
            }
            conv(sh, low, w.tmp.as<float2>(), d, shift, LO_D, false, false, st);                      // 92
            MMR_CUDA(cudaMemcpyAsync(low, w.tmp.p, T * 8, cudaMemcpyDeviceToDevice, st));
            ++ds;
        }
        bi += (1 << k) - 1;
    }
}

// recon: bands -> x (bands are consumed / overwritten).
static void dwt_recon(DwtWork& w, float2* bands, float2* x, cudaStream_t st) {
    const DwtShape& sh = w.s;
    const long long T = sh.tot;
    w.tmp.ensure((size_t)T * sizeof(float2));
    int jmax = 0;
    for (int d = 0; d < sh.nd; ++d) jmax = std::max(jmax, sh.J[d]);
    std::vector<int> first(jmax + 2, 1);
    for (int j = 1; j <= jmax; ++j) {
        int k = 0;
        for (int d = 0; d < sh.nd; ++d) k += sh.J[d] >= j;
        first[j + 1] = first[j] + (1 << k) - 1;
    }
    float2* low = bands;
    float2* tmp = w.tmp.as<float2>();
    for (int j = jmax; j >= 1; --j) {                                             // mtimes.m:57-62
        const long long shift = 1LL << (j - 1);
        int k = 0;
        for (int d = 0; d < sh.nd; ++d) k += sh.J[d] >= j;
        float2* hj = bands + (size_t)first[j] * T;
        int ds = k - 1;
        for (int d = sh.nd - 1; d >= 0; --d) {                                    // reconSep 98-122
            if (sh.J[d] < j) continue;
            conv(sh, low, tmp, d, shift, LO_R, true, false, st);                  // 109
            conv(sh, hj + (size_t)((1 << ds) - 1) * T, tmp, d, shift, HI_R, true, true, st);   // 112
            MMR_CUDA(cudaMemcpyAsync(low, tmp, T * 8, cudaMemcpyDeviceToDevice, st));
            for (int s = 1; s <= (1 << ds) - 1; ++s) {
                float2* hs = hj + (size_t)(s - 1) * T;
                conv(sh, hs, tmp, d, shift, LO_R, true, false, st);                                // 115
                conv(sh, hj + (size_t)((1 << ds) + s - 1) * T, tmp, d, shift, HI_R, true, true, st);
                MMR_CUDA(cudaMemcpyAsync(hs, tmp, T * 8, cudaMemcpyDeviceToDevice, st));
            }
            --ds;
        }
    }
    MMR_CUDA(cudaMemcpyAsync(x, low, T * 8, cudaMemcpyDeviceToDevice, st));
}

// ------------------------------------------------------------ vector kernels --
__device__ __forceinline__ double bwarp_sum(double v) {
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ void block_add(double v, double* dst) {
    __shared__ double red[32];
    v = bwarp_sum(v);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) red[warp] = v;
    __syncthreads();
    if (warp == 0) {
        double s = lane < (int)(blockDim.x >> 5) ? red[lane] : 0.0;
        s = bwarp_sum(s);
        if (lane == 0) atomicAdd(dst, s);
    }
    __syncthreads();
}

// z = a*x + b*y ; acc += |z|^2 (optional)
__global__ void axpby_kernel(float2* __restrict__ z, const float2* __restrict__ x, const float2* __restrict__ y,
                             double a, double b, long long n, double* acc) {
    double s = 0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float2 xi = x[i];
        const float2 yi = y ? y[i] : make_float2(0.f, 0.f);
        const float2 v = make_float2((float)(a * xi.x + b * yi.x), (float)(a * xi.y + b * yi.y));
        z[i] = v;
        s += (double)v.x * v.x + (double)v.y * v.y;
    }
    if (acc) block_add(s, acc);
}

// acc[0] += |x|^2, acc[1..2] += x^H y (re, im)
__global__ void dots_kernel(const float2* __restrict__ x, const float2* __restrict__ y, long long n, double* acc) {
    double s0 = 0, s1 = 0, s2 = 0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float2 a = x[i];
        s0 += (double)a.x * a.x + (double)a.y * a.y;
        if (y) {
            const float2 b = y[i];
            s1 += (double)a.x * b.x + (double)a.y * b.y;
            s2 += (double)a.x * b.y - (double)a.y * b.x;
        }
    }
    block_add(s0, acc);
    if (y) {
        block_add(s1, acc + 1);
        block_add(s2, acc + 2);
    }
}

// acc += lam * |w| (the l1 cost, before thresholding), then w = softthresh(w, thr)
//   softthresh.m:4 -- sign(w) .* max(abs(w) - thr, 0), sign(w) = w / |w|.
__global__ void softthresh_kernel(float2* __restrict__ w, long long n, float lam, float thr, double* acc) {
    double s = 0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float2 v = w[i];
        const float a = hypotf(v.x, v.y);
        s += (double)fabsf(lam) * a;
        const float m = fmaxf(a - thr, 0.f);
        w[i] = a > 0.f ? make_float2(v.x / a * m, v.y / a * m) : make_float2(0.f, 0.f);
    }
    block_add(s, acc);
}

__global__ void cmul_mask_kernel(float2* __restrict__ x, const float2* __restrict__ m, long long n) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) x[i] = cmul(x[i], m[i]);
}

static unsigned vgrid(long long n) {
    return (unsigned)std::max<long long>(1, std::min<long long>(cdiv(n, 256), 2LL * device_sm_count()));
}

struct Scal {
    DevBuf d;
    double* p(int i = 0) { return d.as<double>() + i; }
    void zero(cudaStream_t st, int n) { MMR_CUDA(cudaMemsetAsync(d.p, 0, n * sizeof(double), st)); }
    void read(double* h, int n, cudaStream_t st) {
        MMR_CUDA(cudaMemcpyAsync(h, d.p, n * sizeof(double), cudaMemcpyDeviceToHost, st));
        MMR_CUDA(cudaStreamSynchronize(st));
    }
};

// powermethod.m:31-65 with doAtA = 1 on the normal operator A'A.
static void power_method(SenseOp& a, const float2* x0, int nitmax, double thresh, double* eig_re, double* eig_im,
                         cudaStream_t st) {
    const long long n = a.Nimg;
    DevBuf x, xp, ax;
    x.ensure(n * 8);
    xp.ensure(n * 8);
    ax.ensure(n * 8);
    Scal s;
    s.d.ensure(8 * sizeof(double));
    MMR_CUDA(cudaMemcpyAsync(x.p, x0, n * 8, cudaMemcpyDefault, st));
    MMR_CUDA(cudaMemcpyAsync(xp.p, x0, n * 8, cudaMemcpyDefault, st));
    double h[3];
    for (int nit = 0; nit < nitmax;) {
        sense_normal(a, x.as<float2>(), ax.as<float2>(), st, nullptr);        // 40
        s.zero(st, 3);
        dots_kernel<<<vgrid(n), 256, 0, st>>>(ax.as<float2>(), nullptr, n, s.p());
        check_launch("dots");
        s.read(h, 1, st);
        const double nrm = std::sqrt(h[0]);
        axpby_kernel<<<vgrid(n), 256, 0, st>>>(x.as<float2>(), ax.as<float2>(), nullptr, 1.0 / nrm, 0.0, n, nullptr);  // 44
        check_launch("axpby");
        s.zero(st, 3);
        axpby_kernel<<<vgrid(n), 256, 0, st>>>(ax.as<float2>(), x.as<float2>(), xp.as<float2>(), 1.0, -1.0, n, s.p());
        check_launch("axpby");
        s.read(h, 1, st);
        const double xdiff = std::sqrt(h[0]);                                  // 47
        MMR_CUDA(cudaMemcpyAsync(xp.p, x.p, n * 8, cudaMemcpyDeviceToDevice, st));
        ++nit;
        if (xdiff < thresh) break;                                             // 51-56
    }
    sense_normal(a, x.as<float2>(), ax.as<float2>(), st, nullptr);            // 61
    s.zero(st, 3);
    dots_kernel<<<vgrid(n), 256, 0, st>>>(x.as<float2>(), ax.as<float2>(), n, s.p());
    check_launch("dots");
    s.read(h, 3, st);
    *eig_re = h[1] / h[0];                                                     // 65
    *eig_im = h[2] / h[0];
}

}  // namespace mmr

using namespace mmr;

extern "C" int mmr_powermethod(mmr_sense* A, const void* x0, int32_t nit_max, double xdiff_thresh, double* re,
                               double* im, void* stream) {
    return guarded([&] {
        MMR_REQUIRE(A && x0 && re && im, "NULL argument");
        SenseOp& a = A->a;
        sense_set_weights(a, nullptr, false);
        power_method(a, (const float2*)x0, nit_max > 0 ? nit_max : 50, xdiff_thresh > 0 ? xdiff_thresh : 1e-3, re,
                     im, as_stream(stream));
    });
}

extern "C" int mmr_dwt_haar(int32_t ndim, const int64_t imN[3], const int32_t levels[3], int adjoint, const void* in,
                            void* out, void* stream) {
    return guarded([&] {
        MMR_REQUIRE(imN && levels && in && out && ndim >= 1 && ndim <= 3, "bad argument");
        DwtWork w;
        w.s.nd = ndim;
        w.s.tot = 1;
        for (int d = 0; d < 3; ++d) {
            w.s.n[d] = d < ndim ? imN[d] : 1;
            w.s.J[d] = d < ndim ? (imN[d] == 1 ? 0 : levels[d]) : 0;    // dwtND.m:55
            MMR_REQUIRE(w.s.J[d] >= 0 && w.s.J[d] <= 16, "levels must be 0..16");
            w.s.tot *= w.s.n[d];
        }
        const int nb = dwt_nbands(w.s);
        cudaStream_t st = as_stream(stream);
        const size_t bimg = (size_t)w.s.tot * 8, bband = bimg * nb;
        Staged si, so;
        const float2* din = (const float2*)stage_in(si, in, adjoint ? bband : bimg, st);
        float2* dout = (float2*)stage_out(so, out, adjoint ? bimg : bband);
        if (!adjoint) {
            dwt_decomp(w, din, dout, st);
        } else {
            DevBuf copy;
            copy.ensure(bband);
            MMR_CUDA(cudaMemcpyAsync(copy.p, din, bband, cudaMemcpyDeviceToDevice, st));
            dwt_recon(w, copy.as<float2>(), dout, st);
        }
        finish_out(so, adjoint ? bimg : bband, st);
        if (!so.host) MMR_CUDA(cudaStreamSynchronize(st));
    });
}

extern "C" int mmr_bfista_solve(mmr_sense* A, const void* b, const int32_t* levels, const float* lam, int32_t nbands,
                                const void* x0, const mmr_bfista_opts* opts, void* x_out, mmr_bfista_hist* hist,
                                void* stream) {
    return guarded([&] {
        MMR_REQUIRE(A && b && levels && lam && opts && x_out, "NULL argument");
        SenseOp& a = A->a;
        cudaStream_t st = as_stream(stream);
        sense_set_weights(a, nullptr, false);
        const long long n = a.Nimg, nd = a.M * a.C;
        DwtWork w;
        const int ndim = a.nufft ? a.nufft->nd : 2;
        w.s.nd = ndim;
        w.s.tot = 1;
        for (int d = 0; d < 3; ++d) {
            long long ext = 1;
            if (a.nufft) ext = d < ndim ? a.nufft->N[d] : 1;
            w.s.n[d] = ext;
            w.s.J[d] = (d < ndim && ext > 1) ? levels[d] : 0;
            w.s.tot *= ext;
        }
        if (!a.nufft) {   // sampHighOrder: treat the voxels as a 1D signal unless levels say otherwise
            w.s.nd = 1;
            w.s.n[0] = n;
            w.s.tot = n;
            w.s.J[0] = levels[0];
        }
        MMR_REQUIRE(w.s.tot == n, "wavelet shape does not match the image");
        const int nb = dwt_nbands(w.s);
        MMR_REQUIRE(nbands == nb, "lam has %d bands, the transform has %d", nbands, nb);
        const int nit_max = opts->nit_max > 0 ? opts->nit_max : 200;            // bfista.m:22-25
        const double res_thresh = opts->res_thresh;
        const int n_restart = opts->n_restart > 0 ? opts->n_restart : nit_max + 1;
        Staged sb;
        const float2* bin = (const float2*)stage_in(sb, b, (size_t)nd * 8, st);
        DevBuf x, y, xp, g, resid, bands, mask;
        for (DevBuf* bb : {&x, &y, &xp, &g}) bb->ensure(n * 8);
        resid.ensure((size_t)nd * 8);
        bands.ensure((size_t)nb * n * 8);
        if (x0) MMR_CUDA(cudaMemcpyAsync(xp.p, x0, n * 8, cudaMemcpyDefault, st));
        else sense_adjoint(a, bin, xp.as<float2>(), st, nullptr);               // x0 = A'b (73-75)
        if (opts->x_mask) {
            mask.ensure(n * 8);
            MMR_CUDA(cudaMemcpyAsync(mask.p, opts->x_mask, n * 8, cudaMemcpyDefault, st));
        }
        double max_eig = opts->max_eig;
        if (!(max_eig > 0)) {                                                   // 81-89
            double re, im;
            power_method(a, xp.as<float2>(), 50, 1e-3, &re, &im, st);
            max_eig = std::hypot(re, im);
        }
        const double step = 0.9 / (2.0 * std::fabs(max_eig));                  // 90
        MMR_CUDA(cudaMemcpyAsync(y.p, xp.p, n * 8, cudaMemcpyDeviceToDevice, st));   // y = x0
        Scal s;
        s.d.ensure(8 * sizeof(double));
        std::vector<double> rs, rx, t0, t1;
        double t_prev = 1.0;
        int nit = 1, nit_restart = 1;
        std::vector<float> lamv(lam, lam + nb);
        while (true) {                                                           // 127-233
            // residual_y = A*y - b ; grad = 2*A'*residual_y (129-131)
            sense_forward(a, y.as<float2>(), resid.as<float2>(), st, nullptr);
            s.zero(st, 4);
            axpby_kernel<<<vgrid(nd), 256, 0, st>>>(resid.as<float2>(), resid.as<float2>(), bin, 1.0, -1.0, nd, s.p(0));
            check_launch("axpby");
            sense_adjoint(a, resid.as<float2>(), g.as<float2>(), st, nullptr);
            // g = y - step*grad = y - 2*step*A'r (134)
            axpby_kernel<<<vgrid(n), 256, 0, st>>>(g.as<float2>(), y.as<float2>(), g.as<float2>(), 1.0, -2.0 * step, n,
                                                  nullptr);
            check_launch("axpby");
            // x = R'(softthresh(R g, lam*step)) (146-150), RxAll = sum |lam * R g|
            dwt_decomp(w, g.as<float2>(), bands.as<float2>(), st);
            for (int k = 0; k < nb; ++k) {
                softthresh_kernel<<<vgrid(n), 256, 0, st>>>(bands.as<float2>() + (size_t)k * n, n, lamv[k],
                                                           (float)(lamv[k] * step), s.p(1));
                check_launch("softthresh");
            }
            dwt_recon(w, bands.as<float2>(), x.as<float2>(), st);
            if (opts->x_mask) {                                                  // 153-155
                cmul_mask_kernel<<<(unsigned)cdiv(n, 256), 256, 0, st>>>(x.as<float2>(), mask.as<float2>(), n);
                check_launch("mask");
            }
            // xdiff = x - x_prev (195); |xdiff|^2 and |x|^2 for testAll(:,2)
            axpby_kernel<<<vgrid(n), 256, 0, st>>>(g.as<float2>(), x.as<float2>(), xp.as<float2>(), 1.0, -1.0, n, s.p(2));
            check_launch("axpby");
            dots_kernel<<<vgrid(n), 256, 0, st>>>(x.as<float2>(), nullptr, n, s.p(3));
            check_launch("dots");
            double h[4];
            s.read(h, 4, st);
            rs.push_back(h[0]);
            rx.push_back(h[1]);
            const double t = 0.5 * (1.0 + std::sqrt(1.0 + 4.0 * t_prev * t_prev));   // 196
            // y = x + (t_prev - 1)/t * xdiff (197)
            axpby_kernel<<<vgrid(n), 256, 0, st>>>(y.as<float2>(), x.as<float2>(), g.as<float2>(), 1.0, (t_prev - 1.0) / t,
                                                  n, nullptr);
            check_launch("axpby");
            t_prev = t;
            MMR_CUDA(cudaMemcpyAsync(xp.p, x.p, n * 8, cudaMemcpyDeviceToDevice, st));   // x_prev = x (201)
            bool finished = nit >= nit_max;                                      // 204-207
            double testVal = NAN;
            if (nit > 1) {                                                       // 208-222
                const int i1 = std::max(1, nit - 3);
                double acc = 0;
                int cnt = 0;
                for (int q = i1; q <= nit - 1; ++q) {
                    acc += std::fabs((rs[q] + rx[q]) - (rs[q - 1] + rx[q - 1])) / (rs[nit - 1] + rx[nit - 1]);
                    ++cnt;
                }
                testVal = acc / cnt;
                t0.push_back(testVal);
                t1.push_back(h[2] / h[3]);
            } else {
                t0.push_back(NAN);
                t1.push_back(NAN);
            }
            if (nit > 1 && testVal < res_thresh) finished = true;               // 223-226
            ++nit;
            ++nit_restart;
            if (nit_restart >= n_restart) {                                      // 229-232
                nit_restart = 1;
                t_prev = 1.0;
            }
            if (finished) break;
        }
        Staged sx;
        float2* xo = (float2*)stage_out(sx, x_out, n * 8);
        MMR_CUDA(cudaMemcpyAsync(xo, x.p, n * 8, cudaMemcpyDeviceToDevice, st));
        finish_out(sx, n * 8, st);
        MMR_CUDA(cudaStreamSynchronize(st));
        if (hist) {
            const int m = (int)rs.size();
            hist->n = m;
            hist->max_eig = max_eig;
            for (int i = 0; i < m && i < hist->capacity; ++i) {
                if (hist->res_sq) hist->res_sq[i] = rs[i];
                if (hist->rx) hist->rx[i] = rx[i];
                if (hist->test) {
                    hist->test[i] = t0[i];
                    hist->test[i + hist->capacity] = t1[i];
                }
            }
        }
    });
}
