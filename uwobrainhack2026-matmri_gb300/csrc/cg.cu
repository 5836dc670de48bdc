// cgne (iterativeSolvers/cgne.m) as a device-resident solver.
//
// Vectors (x, p, res, Ap) are complex64; every inner product, alph, beta and
// the stopping tests are FP64.  One iteration is captured as a CUDA graph:
//   Ap = A'(W.*A(p)) [+ gam R'R p]          (cgne.m:214-227)
//   alph = res_sq_old / (p' Ap)             (228)
//   x = xold + alph p                       (229)
//   res = b - A'(W.*A(x)) ... (explicit, mod(nit, expResN) == 0, beta = 0)  (230-246)
//   res = res - alph Ap       (otherwise)   (248)
//   histories, stopping rules               (252-326)
//   p = res + beta p                        (328)
// The last block of each reduction kernel runs the scalar epilogue, so the
// host never synchronises inside the loop; a device flag stops all later
// kernels once a rule fires, and the host polls it between graph batches only
// when a data-dependent rule is enabled.
#include <algorithm>
#include <cmath>
#include <random>

#include "reduce.cuh"
#include "sense.cuh"

namespace mmr {

struct CgState {
    double res_sq_old;
    double pAp_re, pAp_im;
    double acc_res, acc_xn, acc_xd, acc_mse;
    double beta;
    double stop_thresh;
    // options
    double resThresh, resChangeThresh, xChangeThresh, resIncThresh;
    int has_resThresh, has_resChange, has_xChange, has_stop;
    int stopOnResInc, stopOnXdifInc, nseExtraIt;
    int findxnorm, findxdiff, has_gt;
    int cap;
    // progress
    int nit, nitmax, finished, status;
    int resIncs, xdifIncs, lastXdifInc;
    unsigned int counter;
};

struct CgWorkspace {
    long long n = 0;
    DevBuf x, p, res, Ap, b, tmp, tik, gt, state, hist, noise, nimg;
    Staged sb, sxo;
    // graph cache
    cudaGraphExec_t g_norm = nullptr, g_expl = nullptr, g_run = nullptr;
    int k_norm = 0, k_expl = 0, k_run = 0;   // kernel nodes per graph
    const void* key[8] = {nullptr};
    long long keyv[4] = {0};
    ~CgWorkspace() {
        if (g_norm) cudaGraphExecDestroy(g_norm);
        if (g_expl) cudaGraphExecDestroy(g_expl);
        if (g_run) cudaGraphExecDestroy(g_run);
    }
};

void cg_release(SenseOp& a) {
    delete static_cast<CgWorkspace*>(a.solver_ws);
    a.solver_ws = nullptr;
    lpcg_release(a);
}

// True in exactly one thread (thread 0 of the last block to arrive).
__device__ __forceinline__ bool last_block(CgState* st) { return last_block_of(&st->counter); }

// The state is read with independent L2 loads (st.global.cg / ld.global.cg,
// written by other blocks' atomics) into a register copy, updated, and
// written back; one thread of the last block runs this.
static_assert(sizeof(CgState) % 8 == 0, "CgState must be a whole number of 8-byte words");
__device__ __forceinline__ void state_load(CgState& s, const CgState* st) {
    const unsigned long long* src = reinterpret_cast<const unsigned long long*>(st);
    unsigned long long* dst = reinterpret_cast<unsigned long long*>(&s);
#pragma unroll
    for (int i = 0; i < (int)(sizeof(CgState) / 8); ++i) dst[i] = __ldcg(src + i);
}
__device__ __forceinline__ void state_store(CgState* st, const CgState& s) {
    unsigned long long* dst = reinterpret_cast<unsigned long long*>(st);
    const unsigned long long* src = reinterpret_cast<const unsigned long long*>(&s);
#pragma unroll
    for (int i = 0; i < (int)(sizeof(CgState) / 8); ++i) __stcg(dst + i, src[i]);
}

// Scalar epilogue of one iteration (cgne.m:252-335).
__device__ void cg_finalize(CgState* st, double* hist, bool expl) {
    CgState ls;
    state_load(ls, st);
    CgState* vs = &ls;
    const int nit = vs->nit;
    const int cap = vs->cap;
    double* hr = hist;
    double* hm = hist + cap;
    double* hxn = hist + 2 * cap;
    double* hxd = hist + 3 * cap;
    const double rsn = vs->acc_res;
    const int k = nit + 1;
    if (k < cap) {
        hr[k] = rsn;
        if (vs->findxnorm) hxn[k] = vs->acc_xn;
        if (vs->findxdiff) hxd[k] = vs->acc_xd;
        if (vs->has_gt) hm[k] = vs->acc_mse;
    }
    int finished = 0, status = vs->status;
    const double xd = vs->findxdiff ? vs->acc_xd : 0.0;
    if (vs->has_xChange && xd < vs->xChangeThresh) { finished = 1; status = 10; }
    if (vs->has_resThresh && rsn < vs->resThresh) { finished = 1; status = 1; }
    if (vs->has_resChange && fabs((rsn - hr[nit]) / hr[nit]) < vs->resChangeThresh) { finished = 1; status = 2; }
    int nitmax = vs->nitmax;
    if (vs->has_stop && rsn < vs->stop_thresh) {
        nitmax = nit + vs->nseExtraIt;
        vs->stop_thresh = 0.0;
        status = 3;
    }
    if (vs->stopOnResInc > 0 && rsn / hr[nit] > vs->resIncThresh) {
        vs->resIncs = vs->resIncs + 1;
        if (vs->resIncs >= vs->stopOnResInc) { finished = 1; status = 4; }
    }
    const double xdprev = vs->findxdiff ? hxd[nit] : 0.0;
    if (vs->stopOnXdifInc > 0 && xd > xdprev) {
        if (!vs->lastXdifInc) {
            vs->xdifIncs = vs->xdifIncs + 1;
            vs->lastXdifInc = 1;
            if (vs->xdifIncs >= vs->stopOnXdifInc) { finished = 1; status = 5; }
        }
    } else {
        vs->lastXdifInc = 0;
    }
    vs->beta = expl ? 0.0 : rsn / vs->res_sq_old;
    vs->res_sq_old = rsn;
    const int nn = nit + 1;
    if (nn >= nitmax) { finished = 1; status = 0; }
    vs->nit = nn;
    vs->nitmax = nitmax;
    vs->status = status;
    vs->pAp_re = vs->pAp_im = 0.0;
    vs->acc_res = vs->acc_xn = vs->acc_xd = vs->acc_mse = 0.0;
    vs->counter = 0;
    if (finished) vs->finished = 1;
    state_store(st, ls);
    __threadfence();
}

// res = b - Ax - tik.*x0 ; p = res ; histories at index 0 (cgne.m:164-207)
__global__ void cg_init_kernel(const float2* __restrict__ b, const float2* __restrict__ ax,
                               const float2* __restrict__ x, const float* __restrict__ tik,
                               const float2* __restrict__ gt, float2* __restrict__ res, float2* __restrict__ p,
                               long long n, CgState* st, double* hist) {
    double v[4] = {0, 0, 0, 0};
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float2 xi = x[i];
        float2 r = csub(b[i], ax[i]);
        if (tik) r = make_float2(r.x - tik[i] * xi.x, r.y - tik[i] * xi.y);
        res[i] = r;
        p[i] = r;
        v[0] += (double)r.x * r.x + (double)r.y * r.y;
        v[1] += (double)xi.x * xi.x + (double)xi.y * xi.y;
        if (gt) {
            const double dx = (double)gt[i].x - xi.x, dy = (double)gt[i].y - xi.y;
            v[2] += dx * dx + dy * dy;
        }
    }
    double* const dst[4] = {&st->acc_res, &st->acc_xn, &st->acc_mse, nullptr};
    block_accumulate<4>(v, dst);
    if (last_block(st)) {
        volatile CgState* vs = st;
        const int cap = vs->cap;
        const double r0 = vs->acc_res;
        hist[0] = r0;
        const double xn = vs->findxnorm ? vs->acc_xn : 0.0;
        hist[2 * cap] = xn;
        hist[3 * cap] = vs->findxdiff ? xn : 0.0;
        hist[cap] = vs->has_gt ? vs->acc_mse : 0.0;
        vs->res_sq_old = r0;
        vs->pAp_re = vs->pAp_im = 0.0;
        vs->acc_res = vs->acc_xn = vs->acc_xd = vs->acc_mse = 0.0;
        vs->counter = 0;
    }
}

// Ap += tik.*p ; pAp = p' * Ap
__global__ void cg_pap_kernel(const float2* __restrict__ p, float2* __restrict__ Ap, const float* __restrict__ tik,
                              long long n, CgState* st) {
    pdl_wait();
    pdl_trigger();
    if (st->finished) return;
    double v[2] = {0, 0};
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float2 pi = p[i];
        float2 a = Ap[i];
        if (tik) {
            a = make_float2(a.x + tik[i] * pi.x, a.y + tik[i] * pi.y);
            Ap[i] = a;
        }
        v[0] += (double)pi.x * a.x + (double)pi.y * a.y;    // re(conj(p) a)
        v[1] += (double)pi.x * a.y - (double)pi.y * a.x;    // im(conj(p) a)
    }
    double* const dst[2] = {&st->pAp_re, &st->pAp_im};
    block_accumulate<2>(v, dst);
}

// mode 0: x += alph p, res -= alph Ap, all accumulators, finalize.
// mode 1: x += alph p only (explicit-residual iteration); finalize happens later.
template <int MODE>
__global__ void cg_update_kernel(float2* __restrict__ x, const float2* __restrict__ p, const float2* __restrict__ Ap,
                                 float2* __restrict__ res, const float2* __restrict__ gt, long long n, CgState* st,
                                 double* hist) {
    pdl_wait();
    pdl_trigger();
    if (st->finished) return;
    const double rso = st->res_sq_old, ar = st->pAp_re, ai = st->pAp_im;
    const double den = ar * ar + ai * ai;
    const double alr = rso * ar / den, ali = -rso * ai / den;     // res_sq_old / (p' Ap)
    // The vector updates run as FP32 FMAs with alpha rounded once (the vectors are complex64); the
    // norms take FP32 squares of each element (positive terms: no cancellation) summed in FP64.
    // |x|^2 and |x - xold|^2 only when a history or a stopping rule needs them (cgne.m:101-108).
    const float fr = (float)alr, fi = (float)ali;
    const bool fxn = st->findxnorm, fxd = st->findxdiff;
    double v[4] = {0, 0, 0, 0};
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float2 pi = p[i];
        const float2 xo = x[i];
        const float2 xn = make_float2(fmaf(fr, pi.x, fmaf(-fi, pi.y, xo.x)), fmaf(fr, pi.y, fmaf(fi, pi.x, xo.y)));
        x[i] = xn;
        if (fxn) v[1] += (double)fmaf(xn.x, xn.x, xn.y * xn.y);
        if (fxd) {
            const float dx = xn.x - xo.x, dy = xn.y - xo.y;
            v[2] += (double)fmaf(dx, dx, dy * dy);
        }
        if (gt) {
            const double ex = (double)gt[i].x - xn.x, ey = (double)gt[i].y - xn.y;
            v[3] += ex * ex + ey * ey;
        }
        if (MODE == 0) {
            const float2 a = Ap[i], r = res[i];
            const float2 rn = make_float2(fmaf(-fr, a.x, fmaf(fi, a.y, r.x)), fmaf(-fr, a.y, fmaf(-fi, a.x, r.y)));
            res[i] = rn;
            v[0] += (double)fmaf(rn.x, rn.x, rn.y * rn.y);
        }
    }
    double* const dst[4] = {MODE == 0 ? &st->acc_res : nullptr, &st->acc_xn, &st->acc_xd, &st->acc_mse};
    block_accumulate<4>(v, dst);
    if (MODE == 0) {
        if (last_block(st)) cg_finalize(st, hist, false);
    } else {
        // keep the block counter consistent: mode 1 does not finalize
    }
}

// Explicit residual: res = b - Ax - tik.*x ; finalize with beta = 0.
__global__ void cg_res_explicit_kernel(const float2* __restrict__ b, const float2* __restrict__ ax,
                                       const float2* __restrict__ x, const float* __restrict__ tik,
                                       float2* __restrict__ res, long long n, CgState* st, double* hist) {
    pdl_wait();
    pdl_trigger();
    if (st->finished) return;
    double v[1] = {0};
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        float2 r = csub(b[i], ax[i]);
        if (tik) r = make_float2(r.x - tik[i] * x[i].x, r.y - tik[i] * x[i].y);
        res[i] = r;
        v[0] += (double)r.x * r.x + (double)r.y * r.y;
    }
    double* const dst[1] = {&st->acc_res};
    block_accumulate<1>(v, dst);
    if (last_block(st)) cg_finalize(st, hist, true);
}

__global__ void cg_p_kernel(float2* __restrict__ p, const float2* __restrict__ res, long long n, const CgState* st) {
    // runs after the finalize of the same iteration: skip only if finished *before* it
    pdl_wait();
    pdl_trigger();
    const float beta = (float)st->beta;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float2 r = res[i], pi = p[i];
        p[i] = make_float2(fmaf(beta, pi.x, r.x), fmaf(beta, pi.y, r.y));
    }
}

__global__ void norm2_kernel(const float2* __restrict__ v, long long n, double* out) {
    double s[1] = {0};
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        s[0] += (double)v[i].x * v[i].x + (double)v[i].y * v[i].y;
    double* const dst[1] = {out};
    block_accumulate<1>(s, dst);
}

static unsigned red_grid(long long n) {
    const long long b = cdiv(n, 256);
    return (unsigned)std::max<long long>(1, std::min<long long>(b, (long long)device_sm_count()));
}

static bool isset(double v) { return !std::isnan(v); }

// The kernels of one iteration (explicit residual or not) of the solve in `w`, issued on `st`.
static void iter_body(SenseOp& a, CgWorkspace& w, bool expl, bool has_tik, bool has_gt, cudaStream_t st) {
    CgState* sp = w.state.as<CgState>();
    double* hist = w.hist.as<double>();
    const long long n = w.n;
    const int* active = &sp->finished;
    const unsigned g = red_grid(n);
    float2* x = w.x.as<float2>();
    float2* p = w.p.as<float2>();
    float2* res = w.res.as<float2>();
    float2* Ap = w.Ap.as<float2>();
    const float* tik = has_tik ? w.tik.as<float>() : nullptr;
    const float2* gt = has_gt ? w.gt.as<float2>() : nullptr;
    // Ap = A'A p; Ap += tik.*p and pAp in the coil sum when the operator allows, else cg_pap.
    // The vector kernels are launched the ordinary way: with programmatic dependent launch a
    // CG iteration measured 14 us slower; their pdl_trigger() still lets the next iteration's
    // first (dependent-launched) kernel start early.
    if (!sense_normal_dot(a, p, Ap, tik, &sp->pAp_re, st, active)) {
        sense_normal(a, p, Ap, st, active);
        cg_pap_kernel<<<g, 256, 0, st>>>(p, Ap, tik, n, sp);
    }
    if (expl) {
        cg_update_kernel<1><<<g, 256, 0, st>>>(x, p, Ap, res, gt, n, sp, hist);
        sense_normal(a, x, w.tmp.as<float2>(), st, active);
        cg_res_explicit_kernel<<<g, 256, 0, st>>>(w.b.as<float2>(), w.tmp.as<float2>(), x, tik, res, n, sp, hist);
    } else {
        cg_update_kernel<0><<<g, 256, 0, st>>>(x, p, Ap, res, gt, n, sp, hist);
    }
    cg_p_kernel<<<g, 256, 0, st>>>(p, res, n, sp);
}

static cudaGraphExec_t instantiate_counted(cudaGraph_t gr, int& kernels);

// Captures `body` (issued on `st`) as a graph; the capture is closed on every error path.
template <class F>
static cudaGraphExec_t capture(cudaStream_t st, F&& body, int& kernels) {
    MMR_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed));
    set_capturing(true);
    try {
        body();
    } catch (...) {
        set_capturing(false);
        cudaGraph_t gr = nullptr;
        cudaStreamEndCapture(st, &gr);
        if (gr) cudaGraphDestroy(gr);
        throw;
    }
    set_capturing(false);
    cudaGraph_t gr = nullptr;
    MMR_CUDA(cudaStreamEndCapture(st, &gr));
    return instantiate_counted(gr, kernels);
}

// Captures one iteration (explicit or not) on the operator's stream.
static cudaGraphExec_t capture_iter(SenseOp& a, CgWorkspace& w, bool expl, bool has_tik, bool has_gt,
                                    int& kernels) {
    return capture(a.stream, [&] { iter_body(a, w, expl, has_tik, has_gt, a.stream); }, kernels);
}

// Plain iterations per run graph: consecutive iterations captured back to back in one graph,
// so the kernels at iteration boundaries overlap like those inside an iteration.
constexpr int kRunIters = 8;
static cudaGraphExec_t capture_run(SenseOp& a, CgWorkspace& w, bool has_tik, bool has_gt, int& kernels) {
    return capture(a.stream, [&] {
        for (int i = 0; i < kRunIters; ++i) iter_body(a, w, false, has_tik, has_gt, a.stream);
    }, kernels);
}

// Instantiates `gr` (destroyed here) and counts its kernel nodes.
static cudaGraphExec_t instantiate_counted(cudaGraph_t gr, int& kernels) {
    size_t nn = 0;
    MMR_CUDA(cudaGraphGetNodes(gr, nullptr, &nn));
    std::vector<cudaGraphNode_t> nodes(nn);
    MMR_CUDA(cudaGraphGetNodes(gr, nodes.data(), &nn));
    kernels = 0;
    for (auto nd : nodes) {
        cudaGraphNodeType t;
        MMR_CUDA(cudaGraphNodeGetType(nd, &t));
        if (t == cudaGraphNodeTypeKernel) ++kernels;
    }
    cudaGraphExec_t ex = nullptr;
    cudaError_t e = cudaGraphInstantiate(&ex, gr, 0);
    cudaGraphDestroy(gr);
    MMR_CUDA(e);
    return ex;
}

// What one solve needs between its set-up and its read-back.
struct CgRun {
    int nitmax0 = 0, extra = 0, cap = 0, expResN = 1, limit = 0;
    bool has_tik = false, has_gt = false, has_stop = false, dynamic = false;
    double stop_thresh_out = NAN;
    cudaEvent_t ev = nullptr;
};

// Set-up of one solve on the operator's stream (ordered after `ust`): inputs, b = A'(W.*y),
// x0, the options in the device state, the initial residual (cgne.m:135-207).
static CgRun cg_begin(SenseOp& a, const void* b_user, const void* x0_user, const float* W, const mmr_cgne_opts& o,
                      bool hist_out, cudaStream_t ust) {
    CgRun run;
    if (!a.solver_ws) a.solver_ws = new CgWorkspace();
    CgWorkspace& w = *static_cast<CgWorkspace*>(a.solver_ws);
    const long long n = a.Nimg;
    const long long nd = a.M * a.C;
    w.n = n;
    for (DevBuf* bb : {&w.x, &w.p, &w.res, &w.Ap, &w.b, &w.tmp}) bb->ensure(n * sizeof(float2));
    const int nitmax0 = o.nit_max > 0 ? o.nit_max : 1000;
    const int extra = std::max(0, o.nse_extra_it);
    const int cap = nitmax0 + extra + 1;
    w.state.ensure(sizeof(CgState));
    w.hist.ensure((size_t)4 * cap * sizeof(double));
    cudaStream_t st = a.stream;
    // order the internal stream after the caller's stream
    cudaEvent_t ev;
    MMR_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    run.ev = ev;
    MMR_CUDA(cudaEventRecord(ev, ust));
    MMR_CUDA(cudaStreamWaitEvent(st, ev, 0));

    sense_set_weights(a, W, W && o.w_per_coil);
    // inputs
    const float2* b_in = (const float2*)stage_in(w.sb, b_user, (size_t)nd * 8, st);
    const bool has_tik = o.tik_diag != nullptr;
    const bool has_gt = o.gtruth != nullptr;
    if (has_tik) {
        w.tik.ensure(n * sizeof(float));
        MMR_CUDA(cudaMemcpyAsync(w.tik.p, o.tik_diag, n * sizeof(float), cudaMemcpyDefault, st));
    }
    if (has_gt) {
        w.gt.ensure(n * sizeof(float2));
        MMR_CUDA(cudaMemcpyAsync(w.gt.p, o.gtruth, n * sizeof(float2), cudaMemcpyDefault, st));
    }
    // b = A'(W.*bin)  (cgne.m:136-140)
    sense_adjoint(a, b_in, w.b.as<float2>(), st, nullptr);
    if (x0_user) MMR_CUDA(cudaMemcpyAsync(w.x.p, x0_user, n * 8, cudaMemcpyDefault, st));
    else MMR_CUDA(cudaMemcpyAsync(w.x.p, w.b.p, n * 8, cudaMemcpyDeviceToDevice, st));   // x0 = b (143-145)

    CgState h = {};
    h.resThresh = o.res_thresh;
    h.has_resThresh = isset(o.res_thresh);
    h.resChangeThresh = o.res_change_thresh;
    h.has_resChange = isset(o.res_change_thresh);
    h.xChangeThresh = o.x_change_thresh;
    h.has_xChange = isset(o.x_change_thresh);
    h.resIncThresh = o.res_inc_thresh;
    h.stopOnResInc = o.stop_on_res_inc;
    h.stopOnXdifInc = o.stop_on_xdif_inc;
    h.nseExtraIt = o.nse_extra_it;
    // cgne.m:101-108: |x|^2 when histories are returned (nargout > 3) or xChangeThresh is set; |dx|^2
    // also for stopOnXdifInc
    const bool want_hist = hist_out && o.want_history;
    h.findxnorm = want_hist || h.has_xChange;
    h.findxdiff = want_hist || h.has_xChange || h.stopOnXdifInc > 0;
    h.has_gt = has_gt;
    h.cap = cap;
    h.nitmax = nitmax0;
    h.stop_thresh = 0;
    h.has_stop = 0;
    // discrepancy-principle threshold (148-162)
    if (isset(o.noise_var) && o.noise_var > 0) {
        w.noise.ensure((size_t)nd * 8);
        if (o.noise) {
            MMR_CUDA(cudaMemcpyAsync(w.noise.p, o.noise, (size_t)nd * 8, cudaMemcpyDefault, st));
        } else {
            std::mt19937_64 gen(o.noise_seed);
            std::normal_distribution<double> nrm(0.0, 1.0);
            std::vector<float2> nz(nd);
            const double s = std::sqrt(o.noise_var / 2.0);
            for (auto& z : nz) z = make_float2((float)(s * nrm(gen)), (float)(s * nrm(gen)));
            MMR_CUDA(cudaMemcpyAsync(w.noise.p, nz.data(), (size_t)nd * 8, cudaMemcpyHostToDevice, st));
            MMR_CUDA(cudaStreamSynchronize(st));
        }
        w.nimg.ensure(n * 8 + 64);
        sense_adjoint(a, w.noise.as<float2>(), w.nimg.as<float2>(), st, nullptr);
        double* acc = reinterpret_cast<double*>(w.nimg.as<char>() + n * 8);
        MMR_CUDA(cudaMemsetAsync(acc, 0, sizeof(double), st));
        norm2_kernel<<<red_grid(n), 256, 0, st>>>(w.nimg.as<float2>(), n, acc);
        check_launch("norm2");
        double nn = 0;
        MMR_CUDA(cudaMemcpyAsync(&nn, acc, sizeof(double), cudaMemcpyDeviceToHost, st));
        MMR_CUDA(cudaStreamSynchronize(st));
        h.stop_thresh = o.nse_thresh_fact * nn;
        h.has_stop = 1;
    }
    const double stop_thresh_out = h.has_stop ? h.stop_thresh : NAN;
    MMR_CUDA(cudaMemcpyAsync(w.state.p, &h, sizeof(CgState), cudaMemcpyHostToDevice, st));
    MMR_CUDA(cudaMemsetAsync(w.hist.p, 0, (size_t)4 * cap * sizeof(double), st));
    CgState* sp = w.state.as<CgState>();
    // initial residual (164-181)
    sense_normal(a, w.x.as<float2>(), w.tmp.as<float2>(), st, nullptr);
    cg_init_kernel<<<red_grid(n), 256, 0, st>>>(w.b.as<float2>(), w.tmp.as<float2>(), w.x.as<float2>(),
                                               has_tik ? w.tik.as<float>() : nullptr,
                                               has_gt ? w.gt.as<float2>() : nullptr, w.res.as<float2>(),
                                               w.p.as<float2>(), n, sp, w.hist.as<double>());
    check_launch("cg_init");
    run.nitmax0 = nitmax0;
    run.extra = extra;
    run.cap = cap;
    run.expResN = std::max(1, o.exp_res_n);
    run.has_tik = has_tik;
    run.has_gt = has_gt;
    run.has_stop = h.has_stop;
    run.stop_thresh_out = stop_thresh_out;
    run.dynamic = h.has_resThresh || h.has_resChange || h.has_xChange || h.has_stop || h.stopOnResInc > 0 ||
                  h.stopOnXdifInc > 0;
    run.limit = nitmax0 + (h.has_stop ? extra : 0);
    return run;
}

// Read-back of one solve: x, histories, status (cgne.m:336-340); releases the run's event.
static void cg_end(SenseOp& a, CgRun& run, void* x_user, mmr_cgne_hist* hist, cudaStream_t ust) {
    CgWorkspace& w = *static_cast<CgWorkspace*>(a.solver_ws);
    cudaStream_t st = a.stream;
    CgState* sp = w.state.as<CgState>();
    const long long n = w.n;
    const int cap = run.cap;
    cudaEvent_t ev = run.ev;
    CgState fs;
    MMR_CUDA(cudaMemcpyAsync(&fs, sp, sizeof(CgState), cudaMemcpyDeviceToHost, st));
    float2* xo = (float2*)stage_out(w.sxo, x_user, n * 8);
    MMR_CUDA(cudaMemcpyAsync(xo, w.x.p, n * 8, cudaMemcpyDeviceToDevice, st));
    finish_out(w.sxo, n * 8, st);
    MMR_CUDA(cudaStreamSynchronize(st));
    if (hist) {
        hist->nit = fs.nit;
        hist->n = fs.nit + 1;
        hist->status = fs.status;
        // cgne.m:305 sets stopThresh = 0 once the discrepancy rule has fired
        hist->stop_thresh = run.has_stop ? fs.stop_thresh : run.stop_thresh_out;
        const int m = std::min(hist->capacity, fs.nit + 1);
        std::vector<double> hh((size_t)4 * cap);
        MMR_CUDA(cudaMemcpy(hh.data(), w.hist.p, hh.size() * sizeof(double), cudaMemcpyDeviceToHost));
        for (int i = 0; i < m; ++i) {
            if (hist->res_sq) hist->res_sq[i] = hh[i];
            if (hist->mse) hist->mse[i] = hh[cap + i];
            if (hist->xnorm) hist->xnorm[i] = hh[2 * cap + i];
            if (hist->xdiff) hist->xdiff[i] = hh[3 * cap + i];
        }
    }
    MMR_CUDA(cudaEventRecord(ev, st));
    MMR_CUDA(cudaStreamWaitEvent(ust, ev, 0));
    cudaEventDestroy(ev);
    run.ev = nullptr;
    if (device_error_word(st)) MMR_THROW(MMR_ERR_TIMEOUT, "a bounded device wait ran out during cgne");
}

static void cg_solve(SenseOp& a, const void* b_user, const void* x0_user, const float* W, const mmr_cgne_opts& o,
                     void* x_user, mmr_cgne_hist* hist, cudaStream_t ust) {
    CgRun run = cg_begin(a, b_user, x0_user, W, o, hist != nullptr, ust);
    CgWorkspace& w = *static_cast<CgWorkspace*>(a.solver_ws);
    cudaStream_t st = a.stream;
    CgState* sp = w.state.as<CgState>();
    // graphs (re-captured when buffers or options that change kernel arguments differ)
    const void* key[8] = {a.d_wnorm.p, a.s_grid.p, a.s_grid2.p, w.x.p, w.hist.p, (const void*)(intptr_t)run.has_tik,
                          (const void*)(intptr_t)run.has_gt, a.nufft ? a.nufft->s_tmp.p : nullptr};
    const long long keyv[4] = {a.w_bstride, sense_chunk(a), a.nufft && a.nufft->use_bins ? a.nufft->bins.T : 0,
                               run.cap};
    bool same = w.g_norm != nullptr;
    for (int i = 0; i < 8 && same; ++i) same = key[i] == w.key[i];
    for (int i = 0; i < 4 && same; ++i) same = keyv[i] == w.keyv[i];
    if (!same) {
        if (w.g_norm) cudaGraphExecDestroy(w.g_norm);
        if (w.g_expl) cudaGraphExecDestroy(w.g_expl);
        if (w.g_run) cudaGraphExecDestroy(w.g_run);
        w.g_norm = w.g_expl = w.g_run = nullptr;
        // the eager initial residual has sized every scratch buffer before capture
        w.g_norm = capture_iter(a, w, false, run.has_tik, run.has_gt, w.k_norm);
        w.g_expl = capture_iter(a, w, true, run.has_tik, run.has_gt, w.k_expl);
        w.g_run = capture_run(a, w, run.has_tik, run.has_gt, w.k_run);
        for (int i = 0; i < 8; ++i) w.key[i] = key[i];
        for (int i = 0; i < 4; ++i) w.keyv[i] = keyv[i];
    }
    // with a data-dependent stopping rule the host reads the finished flag every kRunIters
    // iterations (one run graph); iterations after the rule fired skip their work on the device
    const int poll = run.dynamic ? kRunIters : run.limit;
    int it = 0;
    while (it < run.limit) {
        const int end = std::min(run.limit, it + poll);
        while (it < end) {
            // kRunIters plain iterations in one launch when none of them needs the explicit residual
            bool plain_run = it + kRunIters <= end;
            for (int j = it; j < it + kRunIters && plain_run; ++j) plain_run = j % run.expResN != 0;
            if (plain_run) {
                MMR_CUDA(cudaGraphLaunch(w.g_run, st));
                add_launches(w.k_run);
                it += kRunIters;
                continue;
            }
            const bool ex = it % run.expResN == 0;
            MMR_CUDA(cudaGraphLaunch(ex ? w.g_expl : w.g_norm, st));
            add_launches(ex ? w.k_expl : w.k_norm);
            ++it;
        }
        int fin = 0;
        MMR_CUDA(cudaMemcpyAsync(&fin, &sp->finished, sizeof(int), cudaMemcpyDeviceToHost, st));
        MMR_CUDA(cudaStreamSynchronize(st));
        if (fin) break;
    }
    cg_end(a, run, x_user, hist, ust);
}

// Many independent solves (slices of different sizes, coil counts and trajectories) advanced
// together: one CUDA graph holds one iteration of every solve as parallel branches (fork/join
// on the operators' own streams), so each graph launch moves the whole batch one iteration.
static void cg_solve_batch(SenseOp* const* ops, int nops, const void* const* b_user, void* const* x_user,
                           const mmr_cgne_opts& o, mmr_cgne_hist* hists, cudaStream_t ust) {
    std::vector<CgRun> runs;
    runs.reserve(nops);
    for (int i = 0; i < nops; ++i)
        for (int j = 0; j < i; ++j) MMR_REQUIRE(ops[i] != ops[j], "operators of a batch must be distinct");
    cudaStream_t origin = nullptr;
    std::vector<cudaEvent_t> evs;
    cudaGraphExec_t g[2] = {nullptr, nullptr};
    auto cleanup = [&] {
        for (auto e : evs) cudaEventDestroy(e);
        for (auto& gg : g)
            if (gg) cudaGraphExecDestroy(gg);
        if (origin) cudaStreamDestroy(origin);
        for (int i = 0; i < (int)runs.size(); ++i)
            if (runs[i].ev) cudaEventDestroy(runs[i].ev);
    };
    try {
        for (int i = 0; i < nops; ++i) runs.push_back(cg_begin(*ops[i], b_user[i], nullptr, nullptr, o, hists != nullptr, ust));
        MMR_CUDA(cudaStreamCreateWithFlags(&origin, cudaStreamNonBlocking));
        evs.resize(nops + 1);
        for (auto& e : evs) MMR_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        // the origin stream starts after every set-up
        for (int i = 0; i < nops; ++i) {
            MMR_CUDA(cudaEventRecord(evs[i], ops[i]->stream));
            MMR_CUDA(cudaStreamWaitEvent(origin, evs[i], 0));
        }
        int kern[2] = {0, 0};
        for (int v = 0; v < 2; ++v) {
            g[v] = capture(origin, [&] {
                MMR_CUDA(cudaEventRecord(evs[nops], origin));
                for (int i = 0; i < nops; ++i) {
                    SenseOp& a = *ops[i];
                    MMR_CUDA(cudaStreamWaitEvent(a.stream, evs[nops], 0));
                    iter_body(a, *static_cast<CgWorkspace*>(a.solver_ws), v == 1, runs[i].has_tik, runs[i].has_gt,
                              a.stream);
                    MMR_CUDA(cudaEventRecord(evs[i], a.stream));
                    MMR_CUDA(cudaStreamWaitEvent(origin, evs[i], 0));
                }
            }, kern[v]);
        }
        int limit = 0;
        bool dynamic = false;
        for (auto& r : runs) {
            limit = std::max(limit, r.limit);
            dynamic = dynamic || r.dynamic;
        }
        const int expResN = runs.empty() ? 1 : runs[0].expResN;
        const int poll = dynamic ? 4 : limit;
        std::vector<int> fin(nops);
        int it = 0;
        while (it < limit) {
            const int end = std::min(limit, it + poll);
            for (; it < end; ++it) {
                const int v = it % expResN == 0 ? 1 : 0;
                MMR_CUDA(cudaGraphLaunch(g[v], origin));
                add_launches(kern[v]);
            }
            bool all = true;
            for (int i = 0; i < nops; ++i) {
                CgState* sp = static_cast<CgWorkspace*>(ops[i]->solver_ws)->state.as<CgState>();
                MMR_CUDA(cudaMemcpyAsync(&fin[i], &sp->finished, sizeof(int), cudaMemcpyDeviceToHost, origin));
            }
            MMR_CUDA(cudaStreamSynchronize(origin));
            for (int i = 0; i < nops; ++i) all = all && fin[i];
            if (all) break;
        }
        // each operator's stream continues after the last batch graph
        MMR_CUDA(cudaEventRecord(evs[nops], origin));
        for (int i = 0; i < nops; ++i) {
            MMR_CUDA(cudaStreamWaitEvent(ops[i]->stream, evs[nops], 0));
            cg_end(*ops[i], runs[i], x_user[i], hists ? hists + i : nullptr, ust);
        }
    } catch (...) {
        cleanup();
        throw;
    }
    cleanup();
}

}  // namespace mmr

using namespace mmr;

extern "C" int mmr_cgne_default_opts(mmr_cgne_opts* o) {
    return guarded([&] {
        MMR_REQUIRE(o, "NULL opts");
        memset(o, 0, sizeof(*o));
        o->nit_max = 1000;
        o->res_thresh = 1e-10;
        o->res_change_thresh = NAN;
        o->x_change_thresh = 1e-10;
        o->exp_res_n = 100;
        o->nse_thresh_fact = 1.0;
        o->nse_extra_it = 4;
        o->stop_on_res_inc = 0;
        o->res_inc_thresh = 1.0;
        o->stop_on_xdif_inc = 0;
        o->noise_var = NAN;
        o->want_history = 1;
    });
}

extern "C" int mmr_cgne_solve(mmr_sense* A, const void* b, const void* x0, const float* W, const mmr_cgne_opts* opts,
                              void* x_out, mmr_cgne_hist* hist, void* stream) {
    return guarded([&] {
        MMR_REQUIRE(A && b && x_out, "NULL argument");
        mmr_cgne_opts o;
        if (opts) o = *opts;
        else mmr_cgne_default_opts(&o);
        cg_solve(A->a, b, x0, W, o, x_out, hist, as_stream(stream));
    });
}

extern "C" int mmr_cgne_solve_batch(mmr_sense* const* A, int32_t n, const void* const* b, void* const* x_out,
                                    const mmr_cgne_opts* opts, mmr_cgne_hist* hists, void* stream) {
    return guarded([&] {
        MMR_REQUIRE(A && b && x_out && n > 0, "NULL argument or empty batch");
        std::vector<SenseOp*> ops(n);
        for (int i = 0; i < n; ++i) {
            MMR_REQUIRE(A[i] && b[i] && x_out[i], "NULL operator, data or output in slot %d", i);
            ops[i] = &A[i]->a;
        }
        mmr_cgne_opts o;
        if (opts) o = *opts;
        else mmr_cgne_default_opts(&o);
        cg_solve_batch(ops.data(), n, b, x_out, o, hists, as_stream(stream));
    });
}
