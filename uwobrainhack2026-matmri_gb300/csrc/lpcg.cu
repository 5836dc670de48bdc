// Learned-preconditioned CG-SENSE: flexible CG on
//     H x = b,   H = A'WA + T   (T: optional Tikhonov diagonal, cgne.m:171-179)
//     b = A'W y                (cgne.m:136-140)
// with the preconditioner z = net(r) (cnn.cuh) or z = r (plain CG):
//     q = H p;  alpha = (p'r)/(p'q);  x += alpha p;  r -= alpha q
//     z = net(r);  p = z - sum_j (q_j'z)/(p_j'q_j) p_j
// over the m most recent directions p_j (FCG(m); a ring of (p_j, q_j) in
// HBM).  alpha is the exact line minimiser of the H-norm error along p, so
// every step lowers it whatever the network returns; the sum makes p
// H-conjugate to the last m directions, which keeps the method close to PCG
// when the preconditioner is not exactly the same operator from one
// application to the next (BF16 activations round differently for every
// residual).  r is updated with exact H products, so it tracks the true
// residual b - Hx up to rounding.  The network's first application (to
// r0 = b when x0 = 0) is the warm start.
//
// Fallback: when |r|^2 has not fallen over `stall_window` iterations (while
// still above the complex64 precision floor), or a direction has no
// curvature (a zero or non-finite network output), the same iteration
// switches the solve to plain CG on the device: z = r from then on and the
// directions restart from r at the current x.  No host round trip is needed,
// so the host only polls when a residual tolerance can end the solve early.
// At exit the true residual |b - Hx| / |b| is computed once more and
// returned (the exit check).
//
// Vectors are complex64; inner products, alpha, beta and the stopping tests
// are FP64.  One iteration (learned or plain) is a captured CUDA graph.
#include <algorithm>
#include <cmath>
#include <cstddef>

#include "cnn.cuh"
#include "reduce.cuh"
#include "sense.cuh"

namespace mmr {

constexpr int LP_MAXM = 8;          // directions kept for the conjugation
constexpr double LP_FLOOR = 1e-12;  // |r|^2 / |r0|^2 below which a stall is not acted on

struct LpState {
    // per-iteration accumulators (zeroed together: keep them first)
    double pq_re, pq_im, pr_re, pr_im, rr, mse;
    double qz[2 * LP_MAXM];          // q_j' z (re, im) per ring slot
    double pqh[2 * LP_MAXM];         // p_j' q_j per ring slot
    double beta[2 * LP_MAXM];        // -(q_j' z) / (p_j' q_j)
    double rr0, tol2;
    int nit, nitmax, finished, status, stalled, window, plain, cap;
    int m, slot, nstored, restart;   // ring size, slot of the current direction, valid slots, restart pending
    int fell_at, pad;                // iteration of the switch to plain CG (-1: none)
    unsigned int counter, counter2;
};
constexpr size_t LP_ACC_BYTES = offsetof(LpState, pqh);

struct LpWorkspace {
    long long n = 0;
    DevBuf x, p, q, r, z, b, tmp, tik, gt, state, hist, nrm, ring_p, ring_q;
    Staged sy, sxo;
    cudaGraphExec_t g_learn = nullptr, g_plain = nullptr;
    int k_learn = 0, k_plain = 0;
    static constexpr int NKEY = 13;
    const void* key[NKEY] = {nullptr};
    long long keyv[4] = {0};
    ~LpWorkspace() {
        if (g_learn) cudaGraphExecDestroy(g_learn);
        if (g_plain) cudaGraphExecDestroy(g_plain);
    }
};

void lpcg_release(SenseOp& a) {
    delete static_cast<LpWorkspace*>(a.lpcg_ws);
    a.lpcg_ws = nullptr;
}

__device__ __forceinline__ double2 cdiv_d(double ar, double ai, double br, double bi) {
    const double d = br * br + bi * bi;
    return make_double2((ar * br + ai * bi) / d, (ai * br - ar * bi) / d);
}

// r = b - Hx - tik.*x (Hx may be NULL: x = 0); |r|^2, |x - gt|^2; rr0 and history[0]
// (exit_check = 1: only leaves |b - Hx - tik.*x|^2 in rr)
__global__ void lp_init_kernel(const float2* __restrict__ b, const float2* __restrict__ hx,
                               const float2* __restrict__ x, const float* __restrict__ tik,
                               const float2* __restrict__ gt, float2* __restrict__ r, long long n, LpState* st,
                               double* hist, int exit_check) {
    double v[2] = {0, 0};
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float2 xi = x[i];
        float2 ri = b[i];
        if (hx) ri = make_float2(ri.x - hx[i].x, ri.y - hx[i].y);
        if (tik) ri = make_float2(ri.x - tik[i] * xi.x, ri.y - tik[i] * xi.y);
        r[i] = ri;
        v[0] += (double)ri.x * ri.x + (double)ri.y * ri.y;
        if (gt) {
            const double dx = (double)gt[i].x - xi.x, dy = (double)gt[i].y - xi.y;
            v[1] += dx * dx + dy * dy;
        }
    }
    double* const dst[2] = {&st->rr, &st->mse};
    block_accumulate<2>(v, dst);
    if (last_block_of(&st->counter)) {
        if (!exit_check) {
            const double rr = __ldcg(&st->rr), mse = __ldcg(&st->mse);
            st->rr0 = rr;
            hist[0] = rr;
            hist[st->cap] = mse;
        }
        st->counter = 0;
        __threadfence();
    }
}

// q += tik.*p ; p'q.  Only when the normal operator cannot accumulate p'q in its last kernel
// (sense_normal_dot): p'r comes from lp_p, the ring copies from lp_update and lp_p.
__global__ void lp_pq_kernel(const float2* __restrict__ p, float2* __restrict__ q, const float* __restrict__ tik,
                             long long n, LpState* st) {
    if (st->finished) return;
    double v[2] = {0, 0};
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float2 pi = p[i];
        float2 qi = q[i];
        if (tik) {
            qi = make_float2(qi.x + tik[i] * pi.x, qi.y + tik[i] * pi.y);
            q[i] = qi;
        }
        v[0] += (double)pi.x * qi.x + (double)pi.y * qi.y;
        v[1] += (double)pi.x * qi.y - (double)pi.y * qi.x;
    }
    double* const dst[2] = {&st->pq_re, &st->pq_im};
    block_accumulate<2>(v, dst);
}

// x += alpha p ; r -= alpha q ; q into the ring slot of this iteration ; |r|^2 ; |x - gt|^2 ;
// history, stopping and stall tests
__global__ void lp_update_kernel(float2* __restrict__ x, const float2* __restrict__ p, const float2* __restrict__ q,
                                 float2* __restrict__ r, float2* __restrict__ ring_q, const float2* __restrict__ gt,
                                 long long n, LpState* st, double* hist) {
    if (st->finished) return;
    float2* __restrict__ rq = ring_q + (long long)st->slot * n;
    // a direction without curvature (p = 0, or a non-finite network output) takes no step;
    // the finalize below then reports a stall so that the host falls back to plain CG
    const double pqr = st->pq_re, pqi = st->pq_im;
    const bool bad = !(pqr * pqr + pqi * pqi > 0.0) || !isfinite(pqr + pqi + st->pr_re + st->pr_im);
    const double2 al = bad ? make_double2(0.0, 0.0) : cdiv_d(st->pr_re, st->pr_im, pqr, pqi);
    // FP32 FMAs with alpha rounded once (complex64 vectors); |r|^2 from FP32 squares summed in FP64
    const float ar = (float)al.x, ai = (float)al.y;
    double v[2] = {0, 0};
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float2 xo = x[i], ro = r[i];
        float2 xn = xo, rn = ro;
        const float2 qi = q[i];
        rq[i] = qi;
        if (!bad) {
            const float2 pi = p[i];
            xn = make_float2(fmaf(ar, pi.x, fmaf(-ai, pi.y, xo.x)), fmaf(ar, pi.y, fmaf(ai, pi.x, xo.y)));
            rn = make_float2(fmaf(-ar, qi.x, fmaf(ai, qi.y, ro.x)), fmaf(-ar, qi.y, fmaf(-ai, qi.x, ro.y)));
            x[i] = xn;
            r[i] = rn;
        }
        v[0] += (double)fmaf(rn.x, rn.x, rn.y * rn.y);
        if (gt) {
            const double dx = (double)gt[i].x - xn.x, dy = (double)gt[i].y - xn.y;
            v[1] += dx * dx + dy * dy;
        }
    }
    double* const dst[2] = {&st->rr, &st->mse};
    block_accumulate<2>(v, dst);
    if (last_block_of(&st->counter)) {
        LpState s;
        state_copy_in(s, st);
        const int k = s.nit + 1;
        const double rr = s.rr;
        const int cap = s.cap;
        s.pqh[2 * s.slot] = bad ? 0.0 : pqr;
        s.pqh[2 * s.slot + 1] = bad ? 0.0 : pqi;
        if (k < cap) {
            hist[k] = rr;
            hist[cap + k] = s.mse;
        }
        // a stall counts only above the precision floor of complex64 vectors (|r| ~ 1e-6 |r0|),
        // where any residual stops falling
        if (s.window > 0 && !s.plain && k >= s.window && k - s.window < cap && rr >= __ldcg(hist + k - s.window) &&
            rr > LP_FLOOR * s.rr0)
            s.stalled = 1;
        if (bad && !s.plain) s.stalled = 1;
        if (s.stalled && !s.plain) {   // fall back to plain CG from this x
            s.plain = 1;
            s.restart = 1;
            s.fell_at = k;
        }
        int fin = 0;
        if (s.tol2 > 0 && rr <= s.tol2 * s.rr0) {
            fin = 1;
            s.status = 1;
        }
        if (k >= s.nitmax) fin = 1;
        s.nit = k;
        if (fin) s.finished = 1;
        s.counter = 0;
        state_copy_out(st, s);
    }
}

// q_j'z for every valid ring slot j (the current direction included); the last block forms
// beta_j = -(q_j'z)/(p_j'q_j), advances the ring and zeroes the accumulators.  After the
// switch to plain CG z is r; on the switch itself the directions restart (all beta_j = 0).
__global__ void lp_qz_kernel(const float2* __restrict__ ring_q, const float2* __restrict__ zn,
                             const float2* __restrict__ r, long long n, LpState* st) {
    if (st->finished) return;
    const float2* __restrict__ z = st->plain ? r : zn;
    const int m = st->m;
    const int nv = min(st->nstored + 1, m);
    double v[2 * LP_MAXM];
#pragma unroll
    for (int j = 0; j < 2 * LP_MAXM; ++j) v[j] = 0.0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float2 zi = z[i];
#pragma unroll
        for (int j = 0; j < LP_MAXM; ++j) {
            if (j < nv) {
                const float2 qi = ring_q[(long long)j * n + i];
                v[2 * j] += (double)qi.x * zi.x + (double)qi.y * zi.y;
                v[2 * j + 1] += (double)qi.x * zi.y - (double)qi.y * zi.x;
            }
        }
    }
    double* dst[2 * LP_MAXM];
#pragma unroll
    for (int j = 0; j < 2 * LP_MAXM; ++j) dst[j] = j < 2 * nv ? &st->qz[j] : nullptr;
    block_accumulate<2 * LP_MAXM>(v, dst);
    if (last_block_of(&st->counter2)) {
        LpState s;
        state_copy_in(s, st);
        const bool restart = s.restart;
#pragma unroll
        for (int j = 0; j < LP_MAXM; ++j) {
            double2 bt = make_double2(0.0, 0.0);
            const double pr = s.pqh[2 * j], pi = s.pqh[2 * j + 1];
            if (!restart && j < nv && pr * pr + pi * pi > 0.0) bt = cdiv_d(-s.qz[2 * j], -s.qz[2 * j + 1], pr, pi);
            if (!isfinite(bt.x + bt.y)) bt = make_double2(0.0, 0.0);
            s.beta[2 * j] = bt.x;
            s.beta[2 * j + 1] = bt.y;
        }
        // valid ring entries are always slots [0, nstored): a restart begins again at slot 0
        s.nstored = restart ? 0 : nv;
        s.restart = 0;
        s.slot = restart ? 0 : (s.slot + 1) % m;
        s.pq_re = s.pq_im = s.pr_re = s.pr_im = s.rr = s.mse = 0.0;
#pragma unroll
        for (int j = 0; j < 2 * LP_MAXM; ++j) s.qz[j] = 0.0;
        s.counter2 = 0;
        state_copy_out(st, s);
    }
}

// p = z + sum_j beta_j p_j over the valid ring slots (z = r after the switch to plain CG); p into
// the ring slot of the next iteration; p'r for the next step length
__global__ void lp_p_kernel(float2* __restrict__ p, const float2* __restrict__ zn, const float2* __restrict__ r,
                            float2* __restrict__ ring_p, long long n, LpState* st) {
    if (st->finished) return;
    const float2* __restrict__ z = st->plain ? r : zn;
    const int nv = st->nstored;
    float2* __restrict__ rp = ring_p + (long long)st->slot * n;
    double d[2] = {0, 0};
    // the combination in FP32 FMAs with the FP64 betas rounded once (p is complex64)
    float br[LP_MAXM], bi[LP_MAXM];
#pragma unroll
    for (int j = 0; j < LP_MAXM; ++j) {
        br[j] = (float)st->beta[2 * j];
        bi[j] = (float)st->beta[2 * j + 1];
    }
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float2 zi = z[i];
        float ax = zi.x, ay = zi.y;
#pragma unroll
        for (int j = 0; j < LP_MAXM; ++j) {
            if (j < nv) {
                const float2 pj = ring_p[(long long)j * n + i];
                ax = fmaf(br[j], pj.x, fmaf(-bi[j], pj.y, ax));
                ay = fmaf(br[j], pj.y, fmaf(bi[j], pj.x, ay));
            }
        }
        const float2 pn = make_float2(ax, ay);
        const float2 ri = r[i];
        p[i] = pn;
        rp[i] = pn;
        d[0] += (double)pn.x * ri.x + (double)pn.y * ri.y;
        d[1] += (double)pn.x * ri.y - (double)pn.y * ri.x;
    }
    double* const dst[2] = {&st->pr_re, &st->pr_im};
    block_accumulate<2>(d, dst);
}

// |v|^2 into *out (zeroed by the caller)
__global__ void lp_norm2_kernel(const float2* __restrict__ v, long long n, double* out) {
    double s[1] = {0};
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        s[0] += (double)v[i].x * v[i].x + (double)v[i].y * v[i].y;
    double* const dst[1] = {out};
    block_accumulate<1>(s, dst);
}

static unsigned lp_grid(long long n) {
    return (unsigned)std::max<long long>(1, std::min<long long>(cdiv(n, 256), 2LL * device_sm_count()));
}

struct LpCall {
    SenseOp* a;
    CnnNet* net;
    int nx, ny, flags;
    bool has_tik, has_gt;
};

static void lp_iter(const LpCall& c, LpWorkspace& w, bool learned, cudaStream_t st) {
    LpState* sp = w.state.as<LpState>();
    const long long n = w.n;
    const unsigned g = lp_grid(n);
    float2* p = w.p.as<float2>();
    float2* q = w.q.as<float2>();
    float2* r = w.r.as<float2>();
    float2* z = learned ? w.z.as<float2>() : r;
    const float* tik = c.has_tik ? w.tik.as<float>() : nullptr;
    float2* ring_p = w.ring_p.as<float2>();
    float2* ring_q = w.ring_q.as<float2>();
    // q = H p with p'q accumulated in the normal operator's coil sum when it is the last kernel
    if (!sense_normal_dot(*c.a, p, q, tik, &sp->pq_re, st, &sp->finished)) {
        sense_normal(*c.a, p, q, st, &sp->finished);
        lp_pq_kernel<<<g, 256, 0, st>>>(p, q, tik, n, sp);
        check_launch("lp_pq");
    }
    lp_update_kernel<<<g, 256, 0, st>>>(w.x.as<float2>(), p, q, r, ring_q, c.has_gt ? w.gt.as<float2>() : nullptr,
                                        n, sp, w.hist.as<double>());
    check_launch("lp_update");
    if (learned) cnn_forward(*c.net, r, z, c.nx, c.ny, 1, &sp->rr, c.flags, st);
    lp_qz_kernel<<<g, 256, 0, st>>>(ring_q, z, r, n, sp);
    check_launch("lp_qz");
    lp_p_kernel<<<g, 256, 0, st>>>(p, z, r, ring_p, n, sp);
    check_launch("lp_p");
}

static cudaGraphExec_t lp_capture(const LpCall& c, LpWorkspace& w, bool learned, int& kernels) {
    cudaStream_t st = c.a->stream;
    MMR_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed));
    set_capturing(true);
    try {
        lp_iter(c, w, learned, st);
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

// Sets x, r, p (and rr) from scratch: r = b - Hx - tik.*x, z = M(r), p = z.
static void lp_start(const LpCall& c, LpWorkspace& w, bool learned, bool have_x, cudaStream_t st) {
    LpState* sp = w.state.as<LpState>();
    const long long n = w.n;
    const unsigned g = lp_grid(n);
    MMR_CUDA(cudaMemsetAsync(w.state.p, 0, LP_ACC_BYTES, st));
    const float2* hx = nullptr;
    if (have_x) {
        sense_normal(*c.a, w.x.as<float2>(), w.tmp.as<float2>(), st, nullptr);
        hx = w.tmp.as<float2>();
    }
    lp_init_kernel<<<g, 256, 0, st>>>(w.b.as<float2>(), hx, w.x.as<float2>(), c.has_tik ? w.tik.as<float>() : nullptr,
                                      c.has_gt ? w.gt.as<float2>() : nullptr, w.r.as<float2>(), n, sp,
                                      w.hist.as<double>(), 0);
    check_launch("lp_init");
    if (learned) cnn_forward(*c.net, w.r.as<float2>(), w.z.as<float2>(), c.nx, c.ny, 1, &sp->rr, c.flags, st);
    MMR_CUDA(cudaMemsetAsync(w.state.p, 0, LP_ACC_BYTES, st));
    // p = z (r for plain CG; no stored directions yet), its ring slot 0 and p'r
    lp_p_kernel<<<g, 256, 0, st>>>(w.p.as<float2>(), learned ? w.z.as<float2>() : w.r.as<float2>(), w.r.as<float2>(),
                                   w.ring_p.as<float2>(), n, sp);
    check_launch("lp_p");
}

static void lp_solve(SenseOp& a, const void* y_user, CnnNet* net, const void* x0_user, const mmr_lpcg_opts& o,
                     void* x_user, mmr_lpcg_hist* hist, cudaStream_t ust) {
    MMR_REQUIRE(a.nufft || a.sho, "operator without a sampling operator");
    if (!a.lpcg_ws) a.lpcg_ws = new LpWorkspace();
    LpWorkspace& w = *static_cast<LpWorkspace*>(a.lpcg_ws);
    const long long n = a.Nimg;
    const long long nd = a.M * a.C;
    int nx = 0, ny = 1;
    if (net) {
        MMR_REQUIRE(a.nufft && a.nufft->nd == 2, "the learned preconditioner needs a 2D image");
        nx = a.nufft->N[0];
        ny = a.nufft->N[1];
    }
    w.n = n;
    for (DevBuf* bb : {&w.x, &w.p, &w.q, &w.r, &w.z, &w.b, &w.tmp}) bb->ensure(n * sizeof(float2));
    const int nitmax = o.nit_max > 0 ? o.nit_max : 100;
    const int cap = nitmax + 1;
    const int m = net ? std::min(std::max(o.fcg_m, 1), LP_MAXM) : 1;
    // sized for the largest ring once, so that captured graphs never see these buffers move
    w.ring_p.ensure((size_t)LP_MAXM * n * sizeof(float2));
    w.ring_q.ensure((size_t)LP_MAXM * n * sizeof(float2));
    w.state.ensure(sizeof(LpState));
    w.hist.ensure((size_t)2 * cap * sizeof(double));
    w.nrm.ensure(2 * sizeof(double));
    cudaStream_t st = a.stream;
    cudaEvent_t ev;
    MMR_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    MMR_CUDA(cudaEventRecord(ev, ust));
    MMR_CUDA(cudaStreamWaitEvent(st, ev, 0));

    sense_set_weights(a, nullptr, false);
    const float2* y_in = (const float2*)stage_in(w.sy, y_user, (size_t)nd * 8, st);
    LpCall c{&a, net, nx, ny, o.flags, o.tik_diag != nullptr || o.lam != 0.0, o.gtruth != nullptr};
    if (c.has_tik) {
        w.tik.ensure(n * sizeof(float));
        std::vector<float> t(n, (float)o.lam);
        if (o.tik_diag) {
            std::vector<float> td(n);
            MMR_CUDA(cudaMemcpy(td.data(), o.tik_diag, n * sizeof(float), cudaMemcpyDefault));
            for (long long i = 0; i < n; ++i) t[i] += td[i];
        }
        MMR_CUDA(cudaMemcpyAsync(w.tik.p, t.data(), n * sizeof(float), cudaMemcpyHostToDevice, st));
        MMR_CUDA(cudaStreamSynchronize(st));
    }
    if (c.has_gt) {
        w.gt.ensure(n * sizeof(float2));
        MMR_CUDA(cudaMemcpyAsync(w.gt.p, o.gtruth, n * sizeof(float2), cudaMemcpyDefault, st));
    }
    sense_adjoint(a, y_in, w.b.as<float2>(), st, nullptr);
    if (x0_user) MMR_CUDA(cudaMemcpyAsync(w.x.p, x0_user, n * 8, cudaMemcpyDefault, st));
    else MMR_CUDA(cudaMemsetAsync(w.x.p, 0, n * 8, st));
    if (net) cnn_pack(*net, st);

    LpState h = {};
    h.tol2 = o.tol > 0 ? o.tol * o.tol : 0.0;
    h.nitmax = nitmax;
    h.window = o.stall_window;
    h.cap = cap;
    h.plain = net ? 0 : 1;
    h.m = m;
    h.fell_at = -1;
    MMR_CUDA(cudaMemcpyAsync(w.state.p, &h, sizeof(LpState), cudaMemcpyHostToDevice, st));
    MMR_CUDA(cudaMemsetAsync(w.hist.p, 0, (size_t)2 * cap * sizeof(double), st));
    lp_start(c, w, net != nullptr, x0_user != nullptr, st);

    // every buffer the captured kernels touch that can move between calls
    const void* key[LpWorkspace::NKEY] = {a.d_wnorm.p, a.s_grid.p, a.s_grid2.p, w.x.p, w.hist.p, net,
                                          net ? net->act.p : nullptr, w.ring_p.p, w.ring_q.p,
                                          net ? net->wmma.p : nullptr, net ? net->sumsq.p : nullptr,
                                          net ? net->fold.p : nullptr,
                                          a.nufft ? a.nufft->s_tmp.p : nullptr};
    const long long keyv[4] = {a.w_bstride, sense_chunk(a), (n << 2) | ((long long)c.has_tik << 1) | (long long)c.has_gt,
                               ((long long)o.flags << 32) | (long long)(a.nufft && a.nufft->use_bins ? a.nufft->bins.T : 0)};
    bool same = w.g_plain != nullptr;
    for (int i = 0; i < LpWorkspace::NKEY && same; ++i) same = key[i] == w.key[i];
    for (int i = 0; i < 4 && same; ++i) same = keyv[i] == w.keyv[i];
    if (!same) {
        if (w.g_learn) cudaGraphExecDestroy(w.g_learn);
        if (w.g_plain) cudaGraphExecDestroy(w.g_plain);
        w.g_learn = w.g_plain = nullptr;
        w.g_plain = lp_capture(c, w, false, w.k_plain);
        if (net) w.g_learn = lp_capture(c, w, true, w.k_learn);
        for (int i = 0; i < LpWorkspace::NKEY; ++i) w.key[i] = key[i];
        for (int i = 0; i < 4; ++i) w.keyv[i] = keyv[i];
    }
    // The fallback to plain CG happens on the device (the learned graph reads z = r once the
    // solve has switched), so the host only has to watch for a tolerance that ends it early.
    cudaGraphExec_t gx = net ? w.g_learn : w.g_plain;
    const int kx = net ? w.k_learn : w.k_plain;
    const int poll = h.tol2 > 0 ? (o.poll > 0 ? o.poll : 8) : nitmax;
    int it = 0;
    LpState* sp = w.state.as<LpState>();
    while (it < nitmax) {
        const int end = std::min(nitmax, it + poll);
        for (; it < end; ++it) {
            MMR_CUDA(cudaGraphLaunch(gx, st));
            add_launches(kx);
        }
        if (end >= nitmax) break;
        int fin = 0;
        MMR_CUDA(cudaMemcpyAsync(&fin, &sp->finished, sizeof(int), cudaMemcpyDeviceToHost, st));
        MMR_CUDA(cudaStreamSynchronize(st));
        if (fin) break;
    }
    // exit check: true residual |b - Hx - tik.*x| / |b|
    sense_normal(a, w.x.as<float2>(), w.tmp.as<float2>(), st, nullptr);
    MMR_CUDA(cudaMemsetAsync(w.state.p, 0, LP_ACC_BYTES, st));
    lp_init_kernel<<<lp_grid(n), 256, 0, st>>>(w.b.as<float2>(), w.tmp.as<float2>(), w.x.as<float2>(),
                                               c.has_tik ? w.tik.as<float>() : nullptr, nullptr, w.q.as<float2>(), n,
                                               sp, w.hist.as<double>(), 1);
    check_launch("lp_init");
    MMR_CUDA(cudaMemsetAsync(w.nrm.p, 0, 2 * sizeof(double), st));
    lp_norm2_kernel<<<lp_grid(n), 256, 0, st>>>(w.b.as<float2>(), n, w.nrm.as<double>());
    check_launch("lp_norm2");
    LpState fs;
    double bn = 0;
    MMR_CUDA(cudaMemcpyAsync(&fs, sp, sizeof(LpState), cudaMemcpyDeviceToHost, st));
    MMR_CUDA(cudaMemcpyAsync(&bn, w.nrm.p, sizeof(double), cudaMemcpyDeviceToHost, st));
    float2* xo = (float2*)stage_out(w.sxo, x_user, n * 8);
    MMR_CUDA(cudaMemcpyAsync(xo, w.x.p, n * 8, cudaMemcpyDeviceToDevice, st));
    finish_out(w.sxo, n * 8, st);
    MMR_CUDA(cudaStreamSynchronize(st));
    if (hist) {
        hist->nit = fs.nit;
        hist->n = std::min(cap, fs.nit + 1);
        hist->status = fs.status;
        hist->fell_back_at = fs.fell_at;
        hist->true_res_rel = bn > 0 ? std::sqrt(fs.rr / bn) : 0.0;
        std::vector<double> hh((size_t)2 * cap);
        MMR_CUDA(cudaMemcpy(hh.data(), w.hist.p, hh.size() * sizeof(double), cudaMemcpyDeviceToHost));
        const int m = std::min(hist->capacity, hist->n);
        for (int i = 0; i < m; ++i) {
            if (hist->res_sq) hist->res_sq[i] = hh[i];
            if (hist->err_sq) hist->err_sq[i] = hh[cap + i];
        }
    }
    MMR_CUDA(cudaEventRecord(ev, st));
    MMR_CUDA(cudaStreamWaitEvent(ust, ev, 0));
    cudaEventDestroy(ev);
}

}  // namespace mmr

using namespace mmr;

extern "C" int mmr_lpcg_default_opts(mmr_lpcg_opts* o) {
    return guarded([&] {
        MMR_REQUIRE(o, "NULL opts");
        memset(o, 0, sizeof(*o));
        o->nit_max = 100;
        o->tol = 0.0;
        o->stall_window = 10;
        o->flags = 2;   // tensor-core network forward
        o->poll = 8;
        o->fcg_m = 4;
    });
}

extern "C" int mmr_lpcg_solve(mmr_sense* A, const void* y, mmr_cnn* net, const void* x0, const mmr_lpcg_opts* opts,
                              void* x_out, mmr_lpcg_hist* hist, void* stream) {
    return guarded([&] {
        MMR_REQUIRE(A && y && x_out, "NULL argument");
        mmr_lpcg_opts o;
        if (opts) o = *opts;
        else mmr_lpcg_default_opts(&o);
        lp_solve(A->a, y, net ? &net->n : nullptr, x0, o, x_out, hist, as_stream(stream));
    });
}
