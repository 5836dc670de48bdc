// @rcvrOp kernels, the mrSampFunc composition A = S*R (forward, adjoint and the
// fused normal operator), and the C ABI of nufftOp / rcvrOp / mrSampFunc.
//
// rcvrOp.m:148-152: forward y = x .* maps, adjoint sum(y .* conj(maps), nDim+1).
// mrSampFunc.m:83-159: notransp x -> R*x -> S*x; transp W.*x -> S'*x -> R'*x.
// For a 2D nufftOp sampling operator the coil weighting is fused into the FFT
// passes (maps multiply in the first forward pass, conj(maps) and the coil
// sum in the last adjoint pass), coils are processed in chunks whose
// oversampled grids stay resident in L2, and the normal operator
// A^H diag(w) A never writes the k-space samples.
#include <algorithm>
#include <cmath>

#include "sense.cuh"

namespace mmr {

// ------------------------------------------------------------------ rcvrOp ----
__global__ void rcvr_fwd_kernel(const float2* __restrict__ x, const float2* __restrict__ maps, float2* __restrict__ y,
                                long long n, long long C, const int* active) {
    if (active && *active) return;
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n * C) return;
    y[i] = cmul(x[i % n], maps[i]);
}

__global__ void rcvr_adj_kernel(const float2* __restrict__ y, const float2* __restrict__ maps, float2* __restrict__ x,
                                long long n, long long C, const int* active) {
    if (active && *active) return;
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float2 acc = make_float2(0.f, 0.f);
    for (long long c = 0; c < C; ++c) acc = cadd(acc, cmulc(y[i + n * c], maps[i + n * c]));
    x[i] = acc;
}

void rcvr_forward(const RcvrPlan& r, const float2* x, float2* y, cudaStream_t st, const int* active) {
    const long long n = r.Ntot * r.C;
    rcvr_fwd_kernel<<<(unsigned)cdiv(n, 256), 256, 0, st>>>(x, r.d_maps.as<float2>(), y, r.Ntot, r.C, active);
    check_launch("rcvr_fwd");
}

void rcvr_adjoint(const RcvrPlan& r, const float2* y, float2* x, cudaStream_t st, const int* active) {
    rcvr_adj_kernel<<<(unsigned)cdiv(r.Ntot, 256), 256, 0, st>>>(y, r.d_maps.as<float2>(), x, r.Ntot, r.C, active);
    check_launch("rcvr_adj");
}

// ---------------------------------------------------------------- helpers ----
__global__ void weight_kernel(const float2* __restrict__ y, const float* __restrict__ w, float2* __restrict__ out,
                              long long M, long long nb, long long bstride, const int* active) {
    if (active && *active) return;
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= M * nb) return;
    const long long s = i % M, c = i / M;
    out[i] = cscale(y[i], w[s + bstride * c]);
}

__global__ void axpy_real_kernel(float2* __restrict__ y, const float2* __restrict__ x, float a, long long n,
                                 const int* active) {
    pdl_wait();
    pdl_trigger();
    if (active && *active) return;
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    y[i] = make_float2(y[i].x + a * x[i].x, y[i].y + a * x[i].y);
}

int sense_chunk(const SenseOp& a) {
    if (!a.rcvr) return 1;
    int cc = a.coil_chunk > 0 ? a.coil_chunk : 8;
    cc = (int)std::min<long long>(cc, a.C);
    return std::max(1, std::min(cc, 32));
}

void sense_set_weights(SenseOp& a, const float* cgW, bool cgW_per_coil) {
    const bool dcf = a.nufft && a.nufft->has_dcf;
    const long long key = a.nufft ? a.nufft->dcf_version : 0;
    if (!cgW && a.wkey == key) return;
    a.wkey = cgW ? -2 : key;
    const bool any = dcf || a.has_optW || cgW;
    if (!any) {
        a.d_wadj.release();
        a.d_wnorm.release();
        a.wnorm_h.clear();
        a.w_bstride = 0;
        ++a.wversion;
        return;
    }
    const bool per_coil = (a.has_optW && a.optW_per_coil) || (cgW && cgW_per_coil);
    const long long nc = per_coil ? a.C : 1;
    std::vector<float> wa((size_t)a.M * nc), wn((size_t)a.M * nc);
    const std::vector<float>& ow = a.optW_h;
    for (long long c = 0; c < nc; ++c)
        for (long long s = 0; s < a.M; ++s) {
            const double d = dcf ? a.nufft->dcf_h[s] : 1.0;
            double w = 1.0;
            if (a.has_optW) w *= ow[s + (a.optW_per_coil ? a.M * c : 0)];
            if (cgW) w *= cgW[s + (cgW_per_coil ? a.M * c : 0)];
            wa[s + a.M * c] = (float)(d * w);
            wn[s + a.M * c] = (float)(d * d * w);
        }
    a.d_wadj.upload(wa);
    a.d_wnorm.upload(wn);
    a.wnorm_h = wn;
    a.w_bstride = per_coil ? a.M : 0;
    ++a.wversion;
}

// The stencil form needs one weight per sample (shared by all coils).
static bool use_stencil(const SenseOp& a) {
    const NufftPlan& p = *a.nufft;
    if (!nufft_stencil_supported(p) || a.w_bstride != 0) return false;
    if (p.normal_mode == 1) return false;
    if (p.normal_mode == 2) return true;
    return p.W <= 4 && p.use_bins;     // auto: (2W-1)^2 floats per cell stays modest
}

static const float* wptr(const DevBuf& b, long long off) {
    return b.p ? b.as<float>() + off : nullptr;
}

// --------------------------------------------------------------- operators ----
void sense_forward(SenseOp& a, const float2* x, float2* y, cudaStream_t st, const int* active) {
    if (a.sho) {
        if (a.rcvr) {
            a.s_img.ensure((size_t)a.Nimg * a.C * sizeof(float2));
            rcvr_forward(*a.rcvr, x, a.s_img.as<float2>(), st, active);
            sho_forward(*a.sho, a.s_img.as<float2>(), y, a.C, st, active);
        } else {
            sho_forward(*a.sho, x, y, 1, st, active);
        }
        return;
    }
    NufftPlan& p = *a.nufft;
    const float* dcf = p.has_dcf ? p.d_dcf.as<float>() : nullptr;
    if (!a.rcvr) {
        p.s_grid.ensure((size_t)p.Gtot * sizeof(float2));
        nufft_img_to_grid(p, x, nullptr, p.s_grid.as<float2>(), 1, st, active);
        nufft_interp(p, p.s_grid.as<float2>(), y, 1, dcf, 0, st, active);
        return;
    }
    const int cc = sense_chunk(a);
    a.s_grid.ensure((size_t)p.Gtot * cc * sizeof(float2));
    const float2* maps = a.rcvr->d_maps.as<float2>();
    for (long long c0 = 0; c0 < a.C; c0 += cc) {
        const long long n = std::min<long long>(cc, a.C - c0);
        nufft_img_to_grid(p, x, maps + c0 * a.Nimg, a.s_grid.as<float2>(), n, st, active);
        nufft_interp(p, a.s_grid.as<float2>(), y + c0 * a.M, n, dcf, 0, st, active);
    }
}

void sense_adjoint(SenseOp& a, const float2* y, float2* x, cudaStream_t st, const int* active) {
    if (a.sho) {
        const float2* yy = y;
        const long long nb = a.rcvr ? a.C : 1;
        if (a.d_wadj.p) {
            a.s_samp.ensure((size_t)a.M * nb * sizeof(float2));
            weight_kernel<<<(unsigned)cdiv(a.M * nb, 256), 256, 0, st>>>(y, a.d_wadj.as<float>(), a.s_samp.as<float2>(),
                                                                       a.M, nb, a.w_bstride, active);
            check_launch("weight");
            yy = a.s_samp.as<float2>();
        }
        if (a.rcvr) {
            a.s_img.ensure((size_t)a.Nimg * a.C * sizeof(float2));
            sho_adjoint(*a.sho, yy, a.s_img.as<float2>(), a.C, st, active);
            rcvr_adjoint(*a.rcvr, a.s_img.as<float2>(), x, st, active);
        } else {
            sho_adjoint(*a.sho, yy, x, 1, st, active);
        }
        return;
    }
    NufftPlan& p = *a.nufft;
    if (!a.rcvr) {
        p.s_grid.ensure((size_t)p.Gtot * sizeof(float2));
        nufft_spread(p, y, p.s_grid.as<float2>(), 1, wptr(a.d_wadj, 0), 0, st, active);
        nufft_grid_to_img(p, p.s_grid.as<float2>(), nullptr, x, 1, false, st, active);
        return;
    }
    const int cc = sense_chunk(a);
    a.s_grid.ensure((size_t)p.Gtot * cc * sizeof(float2));
    const float2* maps = a.rcvr->d_maps.as<float2>();
    for (long long c0 = 0; c0 < a.C; c0 += cc) {
        const long long n = std::min<long long>(cc, a.C - c0);
        nufft_spread(p, y + c0 * a.M, a.s_grid.as<float2>(), n, wptr(a.d_wadj, a.w_bstride * c0), a.w_bstride, st,
                     active);
        nufft_grid_to_img(p, a.s_grid.as<float2>(), maps + c0 * a.Nimg, x, n, c0 > 0, st, active);
    }
}

static void normal_impl(SenseOp& a, const float2* x, float2* y, cudaStream_t st, const int* active,
                        const DotEpilogue* dot) {
    if (a.sho) {
        const long long nb = a.rcvr ? a.C : 1;
        a.s_samp.ensure((size_t)a.M * nb * sizeof(float2));
        float2* smp = a.s_samp.as<float2>();
        const float2* xin = x;
        if (a.rcvr) {
            a.s_img.ensure((size_t)a.Nimg * a.C * sizeof(float2));
            rcvr_forward(*a.rcvr, x, a.s_img.as<float2>(), st, active);
            xin = a.s_img.as<float2>();
        }
        prof_mark(2, st);
        sho_forward(*a.sho, xin, smp, nb, st, active);
        if (a.d_wnorm.p) {
            weight_kernel<<<(unsigned)cdiv(a.M * nb, 256), 256, 0, st>>>(smp, a.d_wnorm.as<float>(), smp, a.M, nb,
                                                                       a.w_bstride, active);
            check_launch("weight");
        }
        prof_mark(2, st);
        if (a.rcvr) {
            sho_adjoint(*a.sho, smp, a.s_img.as<float2>(), a.C, st, active);
            prof_mark(4, st);
            rcvr_adjoint(*a.rcvr, a.s_img.as<float2>(), y, st, active);
        } else {
            sho_adjoint(*a.sho, smp, y, 1, st, active);
        }
    } else {
        NufftPlan& p = *a.nufft;
        const int cc = sense_chunk(a);
        a.s_grid.ensure((size_t)p.Gtot * cc * sizeof(float2));
        a.s_grid2.ensure((size_t)p.Gtot * cc * sizeof(float2));
        const bool stencil = use_stencil(a);
        const bool fused = !stencil && nufft_has_fused_normal(p);
        if (stencil) nufft_build_stencil(p, a.wnorm_h.empty() ? nullptr : a.wnorm_h.data(), (long long)(intptr_t)&a * 64 + a.wversion);
        if (!fused && !stencil) a.s_samp.ensure((size_t)a.M * cc * sizeof(float2));
        const float2* maps = a.rcvr ? a.rcvr->d_maps.as<float2>() : nullptr;
        for (long long c0 = 0; c0 < a.C; c0 += cc) {
            const long long n = std::min<long long>(cc, a.C - c0);
            const float* w = wptr(a.d_wnorm, a.w_bstride * c0);
            nufft_img_to_grid(p, x, maps ? maps + c0 * a.Nimg : nullptr, a.s_grid.as<float2>(), n, st, active);
            prof_mark(2, st);
            if (stencil) {
                nufft_grid_normal_stencil(p, a.s_grid.as<float2>(), a.s_grid2.as<float2>(), n, st, active);
            } else if (fused) {
                nufft_grid_normal(p, a.s_grid.as<float2>(), a.s_grid2.as<float2>(), n, w, a.w_bstride, st, active);
            } else {
                nufft_interp(p, a.s_grid.as<float2>(), a.s_samp.as<float2>(), n, w, a.w_bstride, st, active);
                nufft_spread(p, a.s_samp.as<float2>(), a.s_grid2.as<float2>(), n, nullptr, 0, st, active);
            }
            const bool last = c0 + cc >= a.C;
            nufft_grid_to_img(p, a.s_grid2.as<float2>(), maps ? maps + c0 * a.Nimg : nullptr, y, n, c0 > 0, st,
                              active, nullptr, last ? dot : nullptr);
        }
    }
    prof_mark(-1, st);
    if (a.tikreg != 0) {
        launch_dependent(axpy_real_kernel, dim3((unsigned)cdiv(a.Nimg, 256)), dim3(256), 0, st, y, x,
                         (float)(a.tikreg * a.tikreg), a.Nimg, active);
    }
}

void sense_normal(SenseOp& a, const float2* x, float2* y, cudaStream_t st, const int* active) {
    normal_impl(a, x, y, st, active, nullptr);
}

bool sense_normal_dot(SenseOp& a, const float2* x, float2* y, const float* tik, double* dot, cudaStream_t st,
                      const int* active) {
    // the coil sum of the nufftOp path is the last kernel unless a Tikhonov term follows it
    if (a.sho || !a.nufft || !a.rcvr || a.tikreg != 0) return false;
    DotEpilogue e;
    e.v = x;
    e.tik = tik;
    e.acc = dot;
    normal_impl(a, x, y, st, active, &e);
    return true;
}

}  // namespace mmr

using namespace mmr;

// ===================================================================== C ABI ==
extern "C" int mmr_nufft_create(const mmr_nufft_desc* desc, mmr_nufft** out) {
    return guarded([&] {
        MMR_REQUIRE(desc && out, "NULL argument");
        *out = nullptr;
        auto* h = new mmr_nufft();
        try {
            nufft_plan_build(h->p, *desc);
        } catch (...) {
            delete h;
            throw;
        }
        *out = h;
    });
}

extern "C" int mmr_nufft_set_dcf(mmr_nufft* plan, const double* dcf) {
    return guarded([&] {
        MMR_REQUIRE(plan, "NULL plan");
        nufft_set_dcf(plan->p, dcf);
    });
}

extern "C" int mmr_nufft_info(const mmr_nufft* plan, int64_t osN[3], double* beta, int64_t* nkern) {
    return guarded([&] {
        MMR_REQUIRE(plan, "NULL plan");
        for (int k = 0; k < 3; ++k)
            if (osN) osN[k] = k < plan->p.nd ? plan->p.G[k] : 1;
        if (beta) *beta = plan->p.beta;
        if (nkern) *nkern = plan->p.Nkern;
    });
}

extern "C" int mmr_nufft_apply(mmr_nufft* plan, int adjoint, const void* in, void* out, int64_t nbatch, void* stream) {
    return guarded([&] {
        MMR_REQUIRE(plan && in && out, "NULL argument");
        MMR_REQUIRE(nbatch >= 1, "nbatch must be >= 1");
        NufftPlan& p = plan->p;
        cudaStream_t st = as_stream(stream);
        size_t bin, bout;
        if (p.is_toep) bin = bout = (size_t)p.Ntot * nbatch * 8;
        else if (adjoint) { bin = (size_t)p.M * nbatch * 8; bout = (size_t)p.Ntot * nbatch * 8; }
        else { bin = (size_t)p.Ntot * nbatch * 8; bout = (size_t)p.M * nbatch * 8; }
        const float2* din = (const float2*)stage_in(p.st_in, in, bin, st);
        float2* dout = (float2*)stage_out(p.st_out, out, bout);
        if (p.is_toep) nufft_toep_apply(p, din, dout, nbatch, st);
        else if (adjoint) nufft_adjoint(p, din, dout, nbatch, st);
        else nufft_forward(p, din, dout, nbatch, st);
        finish_out(p.st_out, bout, st);
        if (p.st_out.host && device_error_word(st)) MMR_THROW(MMR_ERR_TIMEOUT, "a bounded device wait ran out");
    });
}

extern "C" int mmr_check_device_error(void* stream) {
    return guarded([&] {
        if (device_error_word(as_stream(stream))) MMR_THROW(MMR_ERR_TIMEOUT, "a bounded device wait ran out");
    });
}

extern "C" int mmr_debug_set_wait_polls(int32_t polls) {
    return guarded([&] {
        MMR_REQUIRE(polls >= 0, "polls must be >= 0");
        set_wait_polls(polls);
    });
}

extern "C" int mmr_nufft_prep_toep(mmr_nufft* plan, double tos, int32_t kwidth) {
    return guarded([&] {
        MMR_REQUIRE(plan, "NULL plan");
        nufft_prep_toep(plan->p, tos, kwidth);
    });
}

extern "C" int mmr_nufft_destroy(mmr_nufft* plan) {
    return guarded([&] { delete plan; });
}

extern "C" int mmr_rcvr_create(int32_t ndim, const int64_t imN[3], int64_t ncoil, const void* maps, mmr_rcvr** out) {
    return guarded([&] {
        MMR_REQUIRE(out && maps && imN, "NULL argument");
        MMR_REQUIRE(ndim >= 1 && ndim <= 3 && ncoil >= 1, "bad rcvr shape");
        auto* h = new mmr_rcvr();
        RcvrPlan& r = h->r;
        r.nd = ndim;
        r.Ntot = 1;
        for (int k = 0; k < ndim; ++k) {
            r.N[k] = (int)imN[k];
            r.Ntot *= imN[k];
        }
        r.C = ncoil;
        const size_t bytes = (size_t)r.Ntot * r.C * 8;
        try {
            r.d_maps.ensure(bytes);
            MMR_CUDA(cudaMemcpy(r.d_maps.p, maps, bytes, cudaMemcpyDefault));
        } catch (...) {
            delete h;
            throw;
        }
        *out = h;
    });
}

extern "C" int mmr_rcvr_apply(mmr_rcvr* h, int adjoint, const void* in, void* out, void* stream) {
    return guarded([&] {
        MMR_REQUIRE(h && in && out, "NULL argument");
        RcvrPlan& r = h->r;
        cudaStream_t st = as_stream(stream);
        const size_t bi = (size_t)r.Ntot * 8 * (adjoint ? r.C : 1), bo = (size_t)r.Ntot * 8 * (adjoint ? 1 : r.C);
        const float2* din = (const float2*)stage_in(r.st_in, in, bi, st);
        float2* dout = (float2*)stage_out(r.st_out, out, bo);
        if (adjoint) rcvr_adjoint(r, din, dout, st, nullptr);
        else rcvr_forward(r, din, dout, st, nullptr);
        finish_out(r.st_out, bo, st);
    });
}

extern "C" int mmr_rcvr_destroy(mmr_rcvr* h) {
    return guarded([&] { delete h; });
}

extern "C" int mmr_sense_create(const mmr_sense_desc* d, mmr_sense** out) {
    return guarded([&] {
        MMR_REQUIRE(d && out, "NULL argument");
        MMR_REQUIRE((d->nufft != nullptr) != (d->sho != nullptr), "exactly one of nufft / sho must be given");
        auto* h = new mmr_sense();
        SenseOp& a = h->a;
        try {
            a.nufft = d->nufft ? &d->nufft->p : nullptr;
            a.sho = d->sho ? reinterpret_cast<ShoPlan*>(d->sho) : nullptr;
            a.rcvr = d->rcvr ? &d->rcvr->r : nullptr;
            a.Nimg = a.nufft ? a.nufft->Ntot : sho_nvox(*a.sho);
            a.M = a.nufft ? a.nufft->M : sho_nsamp(*a.sho);
            a.C = a.rcvr ? a.rcvr->C : 1;
            if (a.rcvr) MMR_REQUIRE(a.rcvr->Ntot == a.Nimg, "rcvrOp maps size does not match the image size");
            MMR_REQUIRE(!(a.nufft && a.nufft->is_toep), "a Toeplitz nufftOp cannot be used inside mrSampFunc");
            a.tikreg = d->tikreg;
            if (d->W) {
                const long long n = a.M * (d->w_per_coil ? a.C : 1);
                a.optW_h.assign(d->W, d->W + n);
                a.d_optW.upload(a.optW_h);
                a.has_optW = true;
                a.optW_per_coil = d->w_per_coil != 0;
            }
            MMR_CUDA(cudaStreamCreateWithFlags(&a.stream, cudaStreamNonBlocking));
            sense_set_weights(a, nullptr, false);
        } catch (...) {
            delete h;
            throw;
        }
        *out = h;
    });
}

extern "C" int mmr_sense_apply(mmr_sense* h, int transp, const void* in, void* out, void* stream) {
    return guarded([&] {
        MMR_REQUIRE(h && in && out, "NULL argument");
        SenseOp& a = h->a;
        cudaStream_t st = as_stream(stream);
        sense_set_weights(a, nullptr, false);
        const size_t bimg = (size_t)a.Nimg * 8, bdat = (size_t)a.M * a.C * 8;
        const float2* din = (const float2*)stage_in(a.st_in, in, transp ? bdat : bimg, st);
        float2* dout = (float2*)stage_out(a.st_out, out, transp ? bimg : bdat);
        if (transp) sense_adjoint(a, din, dout, st, nullptr);
        else sense_forward(a, din, dout, st, nullptr);
        finish_out(a.st_out, transp ? bimg : bdat, st);
    });
}

extern "C" int mmr_sense_normal(mmr_sense* h, const void* in, void* out, void* stream) {
    return guarded([&] {
        MMR_REQUIRE(h && in && out, "NULL argument");
        SenseOp& a = h->a;
        cudaStream_t st = as_stream(stream);
        sense_set_weights(a, nullptr, false);
        const size_t bimg = (size_t)a.Nimg * 8;
        const float2* din = (const float2*)stage_in(a.st_in, in, bimg, st);
        float2* dout = (float2*)stage_out(a.st_out, out, bimg);
        sense_normal(a, din, dout, st, nullptr);
        finish_out(a.st_out, bimg, st);
    });
}

extern "C" int mmr_sense_set_tuning(mmr_sense* h, const mmr_tuning* t) {
    return guarded([&] {
        MMR_REQUIRE(h && t, "NULL argument");
        SenseOp& a = h->a;
        MMR_REQUIRE(t->coil_chunk >= 0 && t->coil_chunk <= 32, "coil_chunk must be 0..32");
        MMR_REQUIRE(t->coil_group == 0 || t->coil_group == 1 || t->coil_group == 2 || t->coil_group == 4 ||
                        t->coil_group == 8, "coil_group must be 1, 2, 4 or 8");
        MMR_REQUIRE(t->item == 0 || t->item >= 8, "item must be >= 8");
        MMR_REQUIRE(t->normal_mode >= 0 && t->normal_mode <= 2, "normal_mode must be 0, 1 or 2");
        MMR_REQUIRE(t->fft_lines == 0 || (t->fft_lines >= 1 && t->fft_lines <= 16 && (t->fft_lines & (t->fft_lines - 1)) == 0),
                    "fft_lines must be a power of two in 1..16");
        if (t->coil_chunk > 0) a.coil_chunk = t->coil_chunk;
        if (a.nufft) {
            NufftPlan& p = *a.nufft;
            if (t->coil_group > 0) p.cg_pref = t->coil_group;
            if (t->fft_lines > 0) p.fft_lines = t->fft_lines;
            if (t->normal_mode > 0) p.normal_mode = t->normal_mode;
            const int tile = t->tile > 0 ? t->tile : p.bins.T;
            const int item = t->item > 0 ? t->item : p.bins.chunk;
            if (p.nd == 2 && (tile != p.bins.T || item != p.bins.chunk)) {
                MMR_REQUIRE(tile == 8 || tile == 16 || tile == 32 || tile == 64, "tile must be 8, 16, 32 or 64");
                nufft_build_bins(p, tile, item);
            }
            a.tile = p.use_bins ? p.bins.T : 0;
        }
        cg_release(a);   // graphs captured with the old tuning are stale
    });
}

extern "C" int mmr_sense_get_tuning(const mmr_sense* h, mmr_tuning* t) {
    return guarded([&] {
        MMR_REQUIRE(h && t, "NULL argument");
        const SenseOp& a = h->a;
        t->coil_chunk = sense_chunk(a);
        t->tile = a.nufft && a.nufft->use_bins ? a.nufft->bins.T : 0;
        t->coil_group = a.nufft ? a.nufft->cg_pref : 0;
        t->item = a.nufft && a.nufft->use_bins ? a.nufft->bins.chunk : 0;
        t->fft_lines = a.nufft ? a.nufft->fft_lines : 0;
        t->normal_mode = a.nufft ? (use_stencil(a) ? 2 : 1) : 0;
    });
}

extern "C" int mmr_sense_destroy(mmr_sense* h) {
    return guarded([&] {
        if (!h) return;
        cg_release(h->a);
        if (h->a.stream) cudaStreamDestroy(h->a.stream);
        delete h;
    });
}

extern "C" int mmr_sense_profile_normal(mmr_sense* h, const void* in, void* out, int32_t reps, double* stage_ms,
                                        int32_t* launches, void* stream) {
    return guarded([&] {
        MMR_REQUIRE(h && in && out && stage_ms && launches && reps >= 1, "bad argument");
        SenseOp& a = h->a;
        cudaStream_t st = as_stream(stream);
        sense_set_weights(a, nullptr, false);
        const size_t bimg = (size_t)a.Nimg * 8;
        const float2* din = (const float2*)stage_in(a.st_in, in, bimg, st);
        float2* dout = (float2*)stage_out(a.st_out, out, bimg);
        sense_normal(a, din, dout, st, nullptr);   // sizes scratch outside the measurement
        MMR_CUDA(cudaStreamSynchronize(st));
        prof_begin();
        try {
            for (int r = 0; r < reps; ++r) sense_normal(a, din, dout, st, nullptr);
        } catch (...) {
            double d[5];
            int c[5];
            prof_end(d, c, 5);
            throw;
        }
        double ms[5];
        int cnt[5];
        prof_end(ms, cnt, 5);
        for (int i = 0; i < 5; ++i) {
            stage_ms[i] = ms[i];
            launches[i] = cnt[i];
        }
        finish_out(a.st_out, bimg, st);
    });
}
