// @sampHighOrder approach 1 (interpolated) on GB300.
//
// prepForInterp (sampHighOrder.m:700-889) factors the encoding less its
// in-plane linear terms as exp(i b) ~ svdSpace * svdTime.' (rank L, truncated
// SVD) and moves the linear terms into a 2D nufftOp trajectory with a phase
// shift phsShft (createNufftForInterp, sampHighOrder.m:624-698).  The plan is
// formed on the host; this file applies it (useInterpWorker, 314-359):
//   forward  y[m] = phsShft[m] sum_l svdTime[m,l] (N (svdSpace_l .* x))[m]
//   adjoint  x    = sum_l conj(svdSpace_l) .* N'(conj(svdTime_l .* phsShft) .* y)
// Per batch column the L terms run in chunks of at most 16 through the same
// kernels as the coil-weighted SENSE path: the term weights svdSpace_l play
// the part of coil maps (multiplied in the first FFT pass, conjugated and
// summed in the last), and the oversampled grids of a chunk stay in L2.  The
// product wt = phsShft .* svdTime is formed once in FP64 and stored as complex64.
#include <algorithm>
#include <cmath>
#include <vector>

#include "sho_interp.cuh"

namespace mmr {

struct ShoInterp {
    NufftPlan traj;
    long long V = 0, M = 0;
    int L = 0;
    int chunk = 0;
    DevBuf d_space;   // complex64 [V, L]
    DevBuf d_wt;      // complex64 [M, L]
    DevBuf s_grid;    // complex64 [Gtot, chunk]
    DevBuf s_samp;    // complex64 [M, chunk]
};

long long sho_interp_nvox(const ShoInterp& s) { return s.V; }
long long sho_interp_nsamp(const ShoInterp& s) { return s.M; }

// y[m] (+)= sum_{l<n} wt[m, l] t[m, l]
__global__ void interp_combine_kernel(const float2* __restrict__ t, const float2* __restrict__ wt,
                                      float2* __restrict__ y, long long M, int n, int accumulate, const int* active) {
    if (active && *active) return;
    const long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= M) return;
    float2 acc = accumulate ? y[m] : make_float2(0.f, 0.f);
    for (int l = 0; l < n; ++l) acc = cadd(acc, cmul(wt[m + M * l], t[m + M * l]));
    y[m] = acc;
}

// u[m, l] = conj(wt[m, l]) y[m]
__global__ void interp_expand_kernel(const float2* __restrict__ y, const float2* __restrict__ wt,
                                     float2* __restrict__ u, long long M, int n, const int* active) {
    if (active && *active) return;
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= M * n) return;
    u[i] = cmulc(y[i % M], wt[i]);
}

std::shared_ptr<ShoInterp> sho_interp_build(const mmr_sho_interp_desc& d) {
    MMR_REQUIRE(d.ndim == 2, "the interpolated approach is built for 2D images");
    MMR_REQUIRE(d.imN[0] >= 2 && d.imN[1] >= 2, "bad image size");
    MMR_REQUIRE(d.nsamp >= 1 && d.nterms >= 1, "nsamp and nterms must be >= 1");
    MMR_REQUIRE(d.kloc && d.svd_space && d.svd_time && d.phs_shift, "missing interpolation factor");
    auto s = std::make_shared<ShoInterp>();
    s->V = d.imN[0] * d.imN[1];
    s->M = d.nsamp;
    s->L = d.nterms;
    mmr_nufft_desc nd{};
    nd.ndim = 2;
    nd.imN[0] = d.imN[0];
    nd.imN[1] = d.imN[1];
    nd.imN[2] = 1;
    nd.nsamp = d.nsamp;
    nd.kloc = d.kloc;
    nd.dcf = nullptr;
    nd.os = d.os;
    nd.kwidth = d.kwidth;
    nufft_plan_build(s->traj, nd);                                       // sampHighOrder.m:695
    const long long V = s->V, M = s->M, L = s->L;
    std::vector<float2> space((size_t)(V * L)), wt((size_t)(M * L));
    for (long long i = 0; i < V * L; ++i) {
        const double re = d.svd_space[2 * i], im = d.svd_space[2 * i + 1];
        MMR_REQUIRE(std::isfinite(re) && std::isfinite(im), "non-finite svdSpace");
        space[i] = make_float2((float)re, (float)im);
    }
    for (long long l = 0; l < L; ++l)
        for (long long m = 0; m < M; ++m) {
            const long long i = m + M * l;
            const double tr = d.svd_time[2 * i], ti = d.svd_time[2 * i + 1];
            const double pr = d.phs_shift[2 * m], pi = d.phs_shift[2 * m + 1];
            MMR_REQUIRE(std::isfinite(tr) && std::isfinite(ti) && std::isfinite(pr) && std::isfinite(pi),
                        "non-finite svdTime / phsShft");
            wt[i] = make_float2((float)(pr * tr - pi * ti), (float)(pr * ti + pi * tr));   // 351-352
        }
    s->d_space.upload(space);
    s->d_wt.upload(wt);
    // balanced chunks of at most 16 terms
    const int npass = (int)cdiv(L, 16);
    s->chunk = (int)cdiv(L, npass);
    s->s_grid.ensure((size_t)s->traj.Gtot * s->chunk * sizeof(float2));
    s->s_samp.ensure((size_t)M * s->chunk * sizeof(float2));
    return s;
}

void sho_interp_forward(ShoInterp& s, const float2* x, float2* y, long long nb, cudaStream_t st, const int* active) {
    NufftPlan& p = s.traj;
    float2* grid = s.s_grid.as<float2>();
    float2* samp = s.s_samp.as<float2>();
    const float2* space = s.d_space.as<float2>();
    const float2* wt = s.d_wt.as<float2>();
    for (long long b = 0; b < nb; ++b) {
        for (int l0 = 0; l0 < s.L; l0 += s.chunk) {
            const int n = std::min(s.chunk, s.L - l0);
            nufft_img_to_grid(p, x + s.V * b, space + s.V * l0, grid, n, st, active);     // 344-345
            nufft_interp(p, grid, samp, n, nullptr, 0, st, active);
            interp_combine_kernel<<<(unsigned)cdiv(s.M, 256), 256, 0, st>>>(samp, wt + s.M * l0, y + s.M * b, s.M,
                                                                           n, l0 > 0, active);   // 351-353
            check_launch("sho_interp_combine");
        }
    }
}

void sho_interp_adjoint(ShoInterp& s, const float2* y, float2* x, long long nb, cudaStream_t st, const int* active) {
    NufftPlan& p = s.traj;
    float2* grid = s.s_grid.as<float2>();
    float2* samp = s.s_samp.as<float2>();
    const float2* space = s.d_space.as<float2>();
    const float2* wt = s.d_wt.as<float2>();
    for (long long b = 0; b < nb; ++b) {
        for (int l0 = 0; l0 < s.L; l0 += s.chunk) {
            const int n = std::min(s.chunk, s.L - l0);
            interp_expand_kernel<<<(unsigned)cdiv(s.M * n, 256), 256, 0, st>>>(y + s.M * b, wt + s.M * l0, samp,
                                                                             s.M, n, active);   // 326-327
            check_launch("sho_interp_expand");
            nufft_spread(p, samp, grid, n, nullptr, 0, st, active);                     // 334
            nufft_grid_to_img(p, grid, space + s.V * l0, x + s.V * b, n, l0 > 0, st, active);   // 335-336
        }
    }
}

}  // namespace mmr
