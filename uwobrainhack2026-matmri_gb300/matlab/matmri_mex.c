/*
 * matmri_mex.c — MATLAB gateway to libmatmri_gb300 (the C ABI in
 * include/matmri_gb300.h).  Build (MATLAB R2018a or newer, interleaved complex,
 * Parallel Computing Toolbox for gpuArray data):
 *
 *   mex -R2018a matmri_mex.c -I../../include -L../matmri_gb300 -lmatmri_gb300 -lmwgpu
 *
 * Called as  varargout = matmri_mex(command, args...)  by the classdef wrappers
 * in this folder (@nufftOp, @rcvrOp, @sampHighOrder, cgne.m, bfista.m).
 * Handles travel as uint64 scalars.
 *
 * Numeric data:
 *   - host arrays (double or single, real or complex) are converted to
 *     interleaved complex single and the result is returned in the class of
 *     the input (nufftOp.m:288-299, 404-406 preserve the input class);
 *   - gpuArray data (nufftOp.m:335-347 accepts gpuArray input) must be complex
 *     single (the classdef wrappers convert on the GPU); its device pointer is
 *     handed to the library directly and the result is a complex single
 *     gpuArray, with no host copy.
 * Any non-zero status raises matmri:gb300:<code> with the library's message;
 * combinations the device path does not implement raise matmri:gb300:unsupported.
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include "gpu/mxGPUArray.h"
#include "matrix.h"
#include "mex.h"
#include "matmri_gb300.h"

static void check(int rc) {
    if (rc != MMR_OK) {
        char msg[1024];
        char id[64];
        mmr_last_error(msg, sizeof(msg));
        snprintf(id, sizeof(id), "matmri:gb300:e%d", rc);
        mexErrMsgIdAndTxt(id, "%s", msg);
    }
}

static void* get_handle(const mxArray* a) {
    if (!mxIsUint64(a) || mxGetNumberOfElements(a) != 1) mexErrMsgIdAndTxt("matmri:gb300:arg", "bad handle");
    return (void*)(uintptr_t)(*(uint64_t*)mxGetData(a));
}

static mxArray* put_handle(void* h) {
    mxArray* a = mxCreateNumericMatrix(1, 1, mxUINT64_CLASS, mxREAL);
    *(uint64_t*)mxGetData(a) = (uint64_t)(uintptr_t)h;
    return a;
}

/* Copy of a real array as double (caller frees). */
static double* as_double(const mxArray* a) {
    size_t n = mxGetNumberOfElements(a);
    double* d = (double*)mxMalloc(n * sizeof(double) + 1);
    if (mxIsDouble(a) && !mxIsComplex(a)) {
        memcpy(d, mxGetDoubles(a), n * sizeof(double));
    } else if (mxIsSingle(a) && !mxIsComplex(a)) {
        const float* f = mxGetSingles(a);
        for (size_t i = 0; i < n; ++i) d[i] = f[i];
    } else if (mxIsLogical(a)) {
        const mxLogical* l = mxGetLogicals(a);
        for (size_t i = 0; i < n; ++i) d[i] = l[i] ? 1.0 : 0.0;
    } else {
        mexErrMsgIdAndTxt("matmri:gb300:arg", "expected a real numeric array");
    }
    return d;
}

/* Copy of a real array as float (caller frees). */
static float* as_float(const mxArray* a) {
    size_t n = mxGetNumberOfElements(a);
    double* d = as_double(a);
    float* f = (float*)mxMalloc(n * sizeof(float) + 4);
    for (size_t i = 0; i < n; ++i) f[i] = (float)d[i];
    mxFree(d);
    return f;
}

/* Interleaved complex single copy of any host numeric array (caller frees). */
static float* as_c64(const mxArray* a) {
    size_t n = mxGetNumberOfElements(a);
    float* f = (float*)mxMalloc(2 * n * sizeof(float) + 8);
    if (mxIsComplex(a)) {
        if (mxIsDouble(a)) {
            const mxComplexDouble* c = mxGetComplexDoubles(a);
            for (size_t i = 0; i < n; ++i) { f[2 * i] = (float)c[i].real; f[2 * i + 1] = (float)c[i].imag; }
        } else {
            memcpy(f, mxGetComplexSingles(a), 2 * n * sizeof(float));
        }
    } else if (mxIsDouble(a)) {
        const double* d = mxGetDoubles(a);
        for (size_t i = 0; i < n; ++i) { f[2 * i] = (float)d[i]; f[2 * i + 1] = 0.f; }
    } else if (mxIsSingle(a)) {
        const float* s = mxGetSingles(a);
        for (size_t i = 0; i < n; ++i) { f[2 * i] = s[i]; f[2 * i + 1] = 0.f; }
    } else {
        mexErrMsgIdAndTxt("matmri:gb300:arg", "expected a numeric array");
    }
    return f;
}

/* Complex result array of the given dims in the class of `like`, filled from complex64. */
static mxArray* from_c64(const float* f, mwSize nd, const mwSize* dims, const mxArray* like) {
    mxArray* o;
    size_t n = 1;
    for (mwSize k = 0; k < nd; ++k) n *= dims[k];
    if (like && mxIsDouble(like)) {
        o = mxCreateNumericArray(nd, dims, mxDOUBLE_CLASS, mxCOMPLEX);
        mxComplexDouble* c = mxGetComplexDoubles(o);
        for (size_t i = 0; i < n; ++i) { c[i].real = f[2 * i]; c[i].imag = f[2 * i + 1]; }
    } else {
        o = mxCreateNumericArray(nd, dims, mxSINGLE_CLASS, mxCOMPLEX);
        memcpy(mxGetComplexSingles(o), f, 2 * n * sizeof(float));
    }
    return o;
}

static double scalar_or(const mxArray* a, double dflt) {
    return (a && !mxIsEmpty(a)) ? mxGetScalar(a) : dflt;
}

static size_t read_dims(const mxArray* a, mwSize* dims, mwSize* nd) {
    double* od = as_double(a);
    size_t n = 1;
    *nd = (mwSize)mxGetNumberOfElements(a);
    if (*nd > 8) mexErrMsgIdAndTxt("matmri:gb300:arg", "at most 8 dimensions");
    for (mwSize k = 0; k < *nd; ++k) { dims[k] = (mwSize)od[k]; n *= dims[k]; }
    mxFree(od);
    return n;
}

/* ---- data that may live on the host or on the GPU ------------------------ */
typedef struct {
    const mxGPUArray* g;     /* gpuArray input, or NULL */
    float* host;             /* host copy, or NULL */
} in_buf;

static int gpu_ready = 0;
static void gpu_init(void) {
    if (!gpu_ready) {
        if (mxInitGPU() != MX_GPU_SUCCESS) mexErrMsgIdAndTxt("matmri:gb300:gpu", "mxInitGPU failed");
        gpu_ready = 1;
    }
}

static const void* in_data(const mxArray* a, in_buf* b) {
    b->g = NULL;
    b->host = NULL;
    if (mxIsGPUArray(a)) {
        gpu_init();
        b->g = mxGPUCreateFromMxArray(a);
        if (mxGPUGetClassID(b->g) != mxSINGLE_CLASS || mxGPUGetComplexity(b->g) != mxCOMPLEX)
            mexErrMsgIdAndTxt("matmri:gb300:arg", "gpuArray data must be complex single");
        return mxGPUGetDataReadOnly(b->g);
    }
    b->host = as_c64(a);
    return b->host;
}
static void in_free(in_buf* b) {
    if (b->g) mxGPUDestroyGPUArray(b->g);
    if (b->host) mxFree(b->host);
}

typedef struct {
    mxGPUArray* g;
    float* host;
} out_buf;

/* Output of dims: on the GPU when `like` is a gpuArray, else on the host. */
static void* out_data(const mxArray* like, mwSize nd, const mwSize* dims, size_t n, out_buf* o) {
    o->g = NULL;
    o->host = NULL;
    if (like && mxIsGPUArray(like)) {
        gpu_init();
        o->g = mxGPUCreateGPUArray(nd, dims, mxSINGLE_CLASS, mxCOMPLEX, MX_GPU_DO_NOT_INITIALIZE);
        return mxGPUGetData(o->g);
    }
    o->host = (float*)mxMalloc(2 * n * sizeof(float) + 8);
    return o->host;
}
/* The MATLAB array of an output (frees the buffer); NULL when the call failed. */
static mxArray* out_take(out_buf* o, int rc, mwSize nd, const mwSize* dims, const mxArray* like) {
    mxArray* r = NULL;
    if (o->g) {
        if (rc == MMR_OK) r = mxGPUCreateMxArrayOnGPU(o->g);
        mxGPUDestroyGPUArray(o->g);
    } else {
        if (rc == MMR_OK) r = from_c64(o->host, nd, dims, like);
        mxFree(o->host);
    }
    return r;
}

/* mrSampFunc(., ., S, R, opt) with the options the device path implements (opt.W, opt.tikReg). */
static mmr_sense* make_sense(const mxArray* hn, const mxArray* hs, const mxArray* hr, const mxArray* Wsense,
                             double tikreg, int w_per_coil, float** wkeep) {
    mmr_sense_desc sd;
    memset(&sd, 0, sizeof(sd));
    sd.nufft = (mmr_nufft*)get_handle(hn);
    sd.sho = (mmr_sho*)get_handle(hs);
    sd.rcvr = (mmr_rcvr*)get_handle(hr);
    *wkeep = NULL;
    if (Wsense && !mxIsEmpty(Wsense)) {
        *wkeep = as_float(Wsense);
        sd.W = *wkeep;
        sd.w_per_coil = w_per_coil;
    }
    sd.tikreg = tikreg;
    mmr_sense* A = NULL;
    check(mmr_sense_create(&sd, &A));
    return A;
}

static void cgne_opts_from(const mxArray* opt, mmr_cgne_opts* o) {
    if (!opt || !mxIsStruct(opt)) return;
    mxArray* f;
#define OPTD(name, field) if ((f = mxGetField(opt, 0, name))) o->field = mxIsEmpty(f) ? NAN : mxGetScalar(f);
#define OPTI(name, field) if ((f = mxGetField(opt, 0, name)) && !mxIsEmpty(f)) o->field = (int32_t)mxGetScalar(f);
    OPTD("resThresh", res_thresh) OPTD("resChangeThresh", res_change_thresh)
    OPTD("xChangeThresh", x_change_thresh) OPTI("expResN", exp_res_n)
    OPTD("nseThreshFact", nse_thresh_fact) OPTI("nseExtraIt", nse_extra_it)
    OPTI("stopOnResInc", stop_on_res_inc) OPTD("resIncThresh", res_inc_thresh)
    OPTI("stopOnXdifInc", stop_on_xdif_inc) OPTD("noiseVar", noise_var)
#undef OPTD
#undef OPTI
}

void mexFunction(int nlhs, mxArray* plhs[], int nrhs, const mxArray* prhs[]) {
    char cmd[64];
    if (nrhs < 1 || mxGetString(prhs[0], cmd, sizeof(cmd)))
        mexErrMsgIdAndTxt("matmri:gb300:arg", "first argument must be a command string");

    /* ------------------------------------------------------------------ @nufftOp */
    if (!strcmp(cmd, "nufft_create")) {            /* (imN, kloc, dcf, os, kwidth) */
        mmr_nufft_desc d;
        memset(&d, 0, sizeof(d));
        double* imN = as_double(prhs[1]);
        d.ndim = (int32_t)mxGetNumberOfElements(prhs[1]);
        for (int k = 0; k < d.ndim && k < 3; ++k) d.imN[k] = (int64_t)imN[k];
        d.nsamp = (int64_t)mxGetM(prhs[2]);
        double* kloc = as_double(prhs[2]);
        d.kloc = kloc;
        double* dcf = (nrhs > 3 && !mxIsEmpty(prhs[3])) ? as_double(prhs[3]) : NULL;
        d.dcf = dcf;
        d.os = scalar_or(nrhs > 4 ? prhs[4] : NULL, 1.5);
        d.kwidth = (int32_t)scalar_or(nrhs > 5 ? prhs[5] : NULL, 6);
        mmr_nufft* h = NULL;
        int rc = mmr_nufft_create(&d, &h);
        mxFree(imN); mxFree(kloc); if (dcf) mxFree(dcf);
        check(rc);
        plhs[0] = put_handle(h);
        return;
    }
    if (!strcmp(cmd, "nufft_set_dcf")) {           /* (h, dcf or []) */
        double* dcf = mxIsEmpty(prhs[2]) ? NULL : as_double(prhs[2]);
        int rc = mmr_nufft_set_dcf((mmr_nufft*)get_handle(prhs[1]), dcf);
        if (dcf) mxFree(dcf);
        check(rc);
        return;
    }
    if (!strcmp(cmd, "nufft_apply")) {             /* (h, adjoint, x, outDims, nbatch) */
        mwSize dims[8], nd;
        size_t nout = read_dims(prhs[4], dims, &nd);
        in_buf ib;
        out_buf ob;
        const void* in = in_data(prhs[3], &ib);
        void* out = out_data(prhs[3], nd, dims, nout, &ob);
        int rc = mmr_nufft_apply((mmr_nufft*)get_handle(prhs[1]), (int)mxGetScalar(prhs[2]), in, out,
                                 (int64_t)mxGetScalar(prhs[5]), NULL);
        in_free(&ib);
        plhs[0] = out_take(&ob, rc, nd, dims, prhs[3]);
        check(rc);
        return;
    }
    if (!strcmp(cmd, "nufft_prep_toep")) {         /* (h, tos, kwidth) */
        check(mmr_nufft_prep_toep((mmr_nufft*)get_handle(prhs[1]), scalar_or(prhs[2], -1),
                                  (int32_t)scalar_or(prhs[3], -1)));
        return;
    }
    if (!strcmp(cmd, "nufft_destroy")) { check(mmr_nufft_destroy((mmr_nufft*)get_handle(prhs[1]))); return; }

    /* ------------------------------------------------------------------- @rcvrOp */
    if (!strcmp(cmd, "rcvr_create")) {             /* (maps) with the coil dimension last */
        const mxArray* m = prhs[1];
        mwSize nd = mxGetNumberOfDimensions(m);
        const mwSize* dm = mxGetDimensions(m);
        int64_t imN[3] = {1, 1, 1};
        for (mwSize k = 0; k + 1 < nd && k < 3; ++k) imN[k] = (int64_t)dm[k];
        float* maps = as_c64(m);
        mmr_rcvr* h = NULL;
        int rc = mmr_rcvr_create((int32_t)(nd - 1), imN, (int64_t)dm[nd - 1], maps, &h);
        mxFree(maps);
        check(rc);
        plhs[0] = put_handle(h);
        return;
    }
    if (!strcmp(cmd, "rcvr_apply")) {              /* (h, adjoint, x, outDims) */
        mwSize dims[8], nd;
        size_t nout = read_dims(prhs[4], dims, &nd);
        in_buf ib;
        out_buf ob;
        const void* in = in_data(prhs[3], &ib);
        void* out = out_data(prhs[3], nd, dims, nout, &ob);
        int rc = mmr_rcvr_apply((mmr_rcvr*)get_handle(prhs[1]), (int)mxGetScalar(prhs[2]), in, out, NULL);
        in_free(&ib);
        plhs[0] = out_take(&ob, rc, nd, dims, prhs[3]);
        check(rc);
        return;
    }
    if (!strcmp(cmd, "rcvr_destroy")) { check(mmr_rcvr_destroy((mmr_rcvr*)get_handle(prhs[1]))); return; }

    /* ------------------------------------------------------------ @sampHighOrder */
    if (!strcmp(cmd, "sho_create")) {              /* (b0, t, spha, conc, gx, gy, gz, mask) */
        mmr_sho_desc d;
        memset(&d, 0, sizeof(d));
        const mwSize* dm = mxGetDimensions(prhs[5]);
        mwSize nd = mxGetNumberOfDimensions(prhs[5]);
        d.ndim = (dm[nd - 1] == 1 && nd == 2) ? 1 : (int32_t)nd;
        for (int k = 0; k < d.ndim && k < 3; ++k) d.imN[k] = (int64_t)dm[k];
        d.nsamp = (int64_t)mxGetNumberOfElements(prhs[2]);
        d.nspha = (int32_t)mxGetM(prhs[3]);
        d.nconc = mxIsEmpty(prhs[4]) ? 0 : (int32_t)mxGetM(prhs[4]);
        double *b0 = mxIsEmpty(prhs[1]) ? NULL : as_double(prhs[1]), *t = as_double(prhs[2]),
               *sp = as_double(prhs[3]), *cc = d.nconc ? as_double(prhs[4]) : NULL, *gx = as_double(prhs[5]),
               *gy = as_double(prhs[6]), *gz = as_double(prhs[7]),
               *mk = (nrhs > 8 && !mxIsEmpty(prhs[8])) ? as_double(prhs[8]) : NULL;
        d.b0 = b0; d.t = t; d.spha = sp; d.conc = cc; d.gx = gx; d.gy = gy; d.gz = gz; d.mask = mk;
        mmr_sho* h = NULL;
        int rc = mmr_sho_create(&d, &h);
        if (b0) mxFree(b0);
        if (cc) mxFree(cc);
        if (mk) mxFree(mk);
        mxFree(t); mxFree(sp); mxFree(gx); mxFree(gy); mxFree(gz);
        check(rc);
        plhs[0] = put_handle(h);
        return;
    }
    if (!strcmp(cmd, "sho_apply")) {               /* (h, adjoint, x, outDims, nbatch) */
        mwSize dims[8], nd;
        size_t nout = read_dims(prhs[4], dims, &nd);
        in_buf ib;
        out_buf ob;
        const void* in = in_data(prhs[3], &ib);
        void* out = out_data(prhs[3], nd, dims, nout, &ob);
        int rc = mmr_sho_apply((mmr_sho*)get_handle(prhs[1]), (int)mxGetScalar(prhs[2]), in, out,
                               (int64_t)mxGetScalar(prhs[5]), NULL);
        in_free(&ib);
        plhs[0] = out_take(&ob, rc, nd, dims, prhs[3]);
        check(rc);
        return;
    }
    if (!strcmp(cmd, "sho_kbase")) {               /* (h, V, M) -> double [V x M] (sampHighOrder kbase) */
        const mwSize V = (mwSize)mxGetScalar(prhs[2]), M = (mwSize)mxGetScalar(prhs[3]);
        mxArray* o = mxCreateDoubleMatrix(V, M, mxREAL);
        int rc = mmr_sho_kbase((const mmr_sho*)get_handle(prhs[1]), mxGetDoubles(o));
        if (rc != MMR_OK) mxDestroyArray(o);
        check(rc);
        plhs[0] = o;
        return;
    }
    if (!strcmp(cmd, "sho_phidiv_create")) {       /* (h, ksphaDiv [nspha x M], kconcDiv [nconc x M]) */
        const int32_t ns = mxIsEmpty(prhs[2]) ? 0 : (int32_t)mxGetM(prhs[2]);
        const int32_t nc = mxIsEmpty(prhs[3]) ? 0 : (int32_t)mxGetM(prhs[3]);
        double* ks = ns ? as_double(prhs[2]) : NULL;
        double* kc = nc ? as_double(prhs[3]) : NULL;
        mmr_sho* h = NULL;
        int rc = mmr_sho_phidiv_create((mmr_sho*)get_handle(prhs[1]), ns, nc, ks, kc, &h);
        if (ks) mxFree(ks);
        if (kc) mxFree(kc);
        check(rc);
        plhs[0] = put_handle(h);
        return;
    }
    if (!strcmp(cmd, "sho_set_tensor")) {          /* (h, mode) */
        check(mmr_sho_set_tensor((mmr_sho*)get_handle(prhs[1]), (int)mxGetScalar(prhs[2])));
        return;
    }
    if (!strcmp(cmd, "sho_destroy")) { check(mmr_sho_destroy((mmr_sho*)get_handle(prhs[1]))); return; }

    /* ----------------------------------------------------------------------- cgne */
    if (!strcmp(cmd, "cgne")) {
        /* (hn, hs, hr, b, x0 or [], NitMax, opt, W or [], imDims, tikDiag or [], senseW or [], tikReg,
         *  senseWperCoil) -> [x, resSqAll, mseAll, xnormAll, xdiffAll, stopThresh, status]   (cgne.m:1)
         * tikDiag: sum_k gam_k |R_k|^2 for elementwise R (cgne.m:171-179); senseW / tikReg: the
         * mrSampFunc options opt.W and opt.tikReg (mrSampFunc.m:126-128, 91-95). */
        float* wsense = NULL;
        mmr_sense* A = make_sense(prhs[1], prhs[2], prhs[3], nrhs > 11 ? prhs[11] : NULL,
                                  scalar_or(nrhs > 12 ? prhs[12] : NULL, 0.0),
                                  (int)scalar_or(nrhs > 13 ? prhs[13] : NULL, 0.0), &wsense);
        mmr_cgne_opts o;
        mmr_cgne_default_opts(&o);
        o.nit_max = (int32_t)scalar_or(prhs[6], 1000);
        o.want_history = 1;
        cgne_opts_from(prhs[7], &o);
        float* tik = NULL;
        if (nrhs > 10 && !mxIsEmpty(prhs[10])) {
            tik = as_float(prhs[10]);
            o.tik_diag = tik;
        }
        in_buf bb, xb;
        const void* b = in_data(prhs[4], &bb);
        const void* x0 = NULL;
        xb.g = NULL;
        xb.host = NULL;
        if (!mxIsEmpty(prhs[5])) x0 = in_data(prhs[5], &xb);
        float* W = NULL;
        if (!mxIsEmpty(prhs[8])) {
            W = as_float(prhs[8]);
            o.w_per_coil = mxGetNumberOfElements(prhs[8]) > (size_t)mxGetM(prhs[4]);
        }
        mwSize dims[8], nd;
        size_t nimg = read_dims(prhs[9], dims, &nd);
        const int32_t cap = o.nit_max + o.nse_extra_it + 1;
        double* hh = (double*)mxCalloc(4 * (size_t)cap, sizeof(double));
        mmr_cgne_hist hist = {hh, hh + cap, hh + 2 * cap, hh + 3 * cap, cap, 0, 0, 0, 0};
        out_buf ob;
        void* x = out_data(prhs[4], nd, dims, nimg, &ob);
        int rc = mmr_cgne_solve(A, b, x0, W, &o, x, &hist, NULL);
        mmr_sense_destroy(A);
        in_free(&bb);
        in_free(&xb);
        if (W) mxFree(W);
        if (tik) mxFree(tik);
        if (wsense) mxFree(wsense);
        plhs[0] = out_take(&ob, rc, nd, dims, prhs[4]);
        if (rc == MMR_OK) {
            for (int k = 0; k < 4 && k + 1 < nlhs; ++k) {   /* resSqAll, mseAll, xnormAll, xdiffAll */
                mxArray* v = mxCreateDoubleMatrix((mwSize)hist.n, 1, mxREAL);
                memcpy(mxGetDoubles(v), hh + (size_t)k * cap, (size_t)hist.n * sizeof(double));
                plhs[k + 1] = v;
            }
            if (nlhs > 5) plhs[5] = isnan(hist.stop_thresh) ? mxCreateDoubleMatrix(0, 0, mxREAL)
                                                            : mxCreateDoubleScalar(hist.stop_thresh);
            if (nlhs > 6) plhs[6] = mxCreateDoubleScalar(hist.status);
        }
        mxFree(hh);
        check(rc);
        return;
    }
    if (!strcmp(cmd, "cgne_batch")) {
        /* ({hn}, {hs}, {hr}, {b}, NitMax, opt, {imDims}) -> [{x}, statuses, iterations]: independent cgne
         * solves (a loop of cgne calls over slices) advanced together on the device */
        const mwSize n = mxGetNumberOfElements(prhs[4]);
        mmr_sense** A = (mmr_sense**)mxCalloc(n, sizeof(mmr_sense*));
        const void** b = (const void**)mxCalloc(n, sizeof(void*));
        void** x = (void**)mxCalloc(n, sizeof(void*));
        in_buf* ib = (in_buf*)mxCalloc(n, sizeof(in_buf));
        out_buf* ob = (out_buf*)mxCalloc(n, sizeof(out_buf));
        mwSize (*dims)[8] = (mwSize(*)[8])mxCalloc(n, sizeof(mwSize[8]));
        mwSize* nds = (mwSize*)mxCalloc(n, sizeof(mwSize));
        mmr_cgne_hist* hs = (mmr_cgne_hist*)mxCalloc(n, sizeof(mmr_cgne_hist));
        float* wk = NULL;
        for (mwSize i = 0; i < n; ++i) {
            A[i] = make_sense(mxGetCell(prhs[1], i), mxGetCell(prhs[2], i), mxGetCell(prhs[3], i), NULL, 0.0, 0, &wk);
            b[i] = in_data(mxGetCell(prhs[4], i), &ib[i]);
            size_t nimg = read_dims(mxGetCell(prhs[7], i), dims[i], &nds[i]);
            x[i] = out_data(mxGetCell(prhs[4], i), nds[i], dims[i], nimg, &ob[i]);
        }
        mmr_cgne_opts o;
        mmr_cgne_default_opts(&o);
        o.nit_max = (int32_t)scalar_or(prhs[5], 1000);
        cgne_opts_from(prhs[6], &o);
        int rc = mmr_cgne_solve_batch(A, (int32_t)n, b, x, &o, hs, NULL);
        mxArray* cx = mxCreateCellMatrix(n, 1);
        mxArray* st = mxCreateDoubleMatrix(n, 1, mxREAL);
        mxArray* it = mxCreateDoubleMatrix(n, 1, mxREAL);
        for (mwSize i = 0; i < n; ++i) {
            mmr_sense_destroy(A[i]);
            in_free(&ib[i]);
            mxArray* xi = out_take(&ob[i], rc, nds[i], dims[i], mxGetCell(prhs[4], i));
            if (xi) mxSetCell(cx, i, xi);
            mxGetDoubles(st)[i] = hs[i].status;
            mxGetDoubles(it)[i] = hs[i].nit;
        }
        mxFree(A); mxFree(b); mxFree(x); mxFree(ib); mxFree(ob); mxFree(dims); mxFree(nds); mxFree(hs);
        check(rc);
        plhs[0] = cx;
        if (nlhs > 1) plhs[1] = st;
        if (nlhs > 2) plhs[2] = it;
        return;
    }

    /* ------------------------------------------------------------------ bfista */
    if (!strcmp(cmd, "bfista")) {
        /* (hn, hs, hr, b, levels, lam, x0 or [], NitMax, opt, imDims) -> [x, resSqAll, RxAll, testAll]
         * with R = dwtND(levels, imSize, false, 'db1') (bfista.m:1, @dwtND undecimated Haar) */
        float* wk = NULL;
        mmr_sense* A = make_sense(prhs[1], prhs[2], prhs[3], NULL, 0.0, 0, &wk);
        double* lv = as_double(prhs[5]);
        int32_t levels[3] = {0, 0, 0};
        for (size_t k = 0; k < mxGetNumberOfElements(prhs[5]) && k < 3; ++k) levels[k] = (int32_t)lv[k];
        mxFree(lv);
        float* lam = as_float(prhs[6]);
        mmr_bfista_opts o;
        memset(&o, 0, sizeof(o));
        o.nit_max = (int32_t)scalar_or(prhs[8], 200);
        o.res_thresh = 1e-5;
        o.n_restart = o.nit_max + 1;
        if (mxIsStruct(prhs[9])) {
            mxArray* f;
            if ((f = mxGetField(prhs[9], 0, "resThresh")) && !mxIsEmpty(f)) o.res_thresh = mxGetScalar(f);
            if ((f = mxGetField(prhs[9], 0, "maxEig")) && !mxIsEmpty(f)) o.max_eig = mxGetScalar(f);
            if ((f = mxGetField(prhs[9], 0, "nRestart")) && !mxIsEmpty(f)) o.n_restart = (int32_t)mxGetScalar(f);
            if ((f = mxGetField(prhs[9], 0, "xMask")) && !mxIsEmpty(f))
                mexErrMsgIdAndTxt("matmri:gb300:unsupported", "opt.xMask: pass it through the C ABI");
        }
        in_buf bb, xb;
        const void* b = in_data(prhs[4], &bb);
        const void* x0 = NULL;
        xb.g = NULL;
        xb.host = NULL;
        if (!mxIsEmpty(prhs[7])) x0 = in_data(prhs[7], &xb);
        mwSize dims[8], nd;
        size_t nimg = read_dims(prhs[10], dims, &nd);
        const int32_t cap = o.nit_max;
        double* hh = (double*)mxCalloc(4 * (size_t)cap + 4, sizeof(double));
        mmr_bfista_hist hist;
        memset(&hist, 0, sizeof(hist));
        hist.res_sq = hh;
        hist.rx = hh + cap;
        hist.test = hh + 2 * cap;
        hist.capacity = cap;
        out_buf ob;
        void* x = out_data(prhs[4], nd, dims, nimg, &ob);
        int rc = mmr_bfista_solve(A, b, levels, lam, (int32_t)mxGetNumberOfElements(prhs[6]), x0, &o, x, &hist, NULL);
        mmr_sense_destroy(A);
        in_free(&bb);
        in_free(&xb);
        mxFree(lam);
        plhs[0] = out_take(&ob, rc, nd, dims, prhs[4]);
        if (rc == MMR_OK) {
            if (nlhs > 1) {
                plhs[1] = mxCreateDoubleMatrix((mwSize)hist.n, 1, mxREAL);
                memcpy(mxGetDoubles(plhs[1]), hist.res_sq, (size_t)hist.n * sizeof(double));
            }
            if (nlhs > 2) {
                plhs[2] = mxCreateDoubleMatrix((mwSize)hist.n, 1, mxREAL);
                memcpy(mxGetDoubles(plhs[2]), hist.rx, (size_t)hist.n * sizeof(double));
            }
            if (nlhs > 3) {
                plhs[3] = mxCreateDoubleMatrix((mwSize)hist.n, 2, mxREAL);
                for (int32_t i = 0; i < hist.n; ++i) {
                    mxGetDoubles(plhs[3])[i] = hist.test[i];
                    mxGetDoubles(plhs[3])[i + hist.n] = hist.test[i + cap];
                }
            }
        }
        mxFree(hh);
        check(rc);
        return;
    }

    /* ------------------------------------------------ learned-preconditioned CG */
    if (!strcmp(cmd, "lpcg")) {
        /* (hn, hs, hr, y, channels, theta or [], x0 or [], opt, imDims) -> [x, resSq, errSq, info]
         * (no counterpart in the reference): flexible CG on (A'A + lam) x = A'y with the network
         * z = net(r) of `channels` (2, 32, ..., 2) and FP32 parameters theta; theta = [] runs plain CG. */
        float* wk = NULL;
        mmr_sense* A = make_sense(prhs[1], prhs[2], prhs[3], NULL, 0.0, 0, &wk);
        mmr_cnn* net = NULL;
        if (!mxIsEmpty(prhs[6])) {
            double* ch = as_double(prhs[5]);
            const int32_t nl = (int32_t)mxGetNumberOfElements(prhs[5]) - 1;
            int32_t chi[16];
            for (int32_t k = 0; k <= nl && k < 16; ++k) chi[k] = (int32_t)ch[k];
            mxFree(ch);
            check(mmr_cnn_create(nl, chi, &net));
            float* th = as_float(prhs[6]);
            int rc0 = mmr_cnn_set_params(net, th);
            mxFree(th);
            if (rc0 != MMR_OK) mmr_cnn_destroy(net);
            check(rc0);
        }
        mmr_lpcg_opts o;
        mmr_lpcg_default_opts(&o);
        if (mxIsStruct(prhs[8])) {
            mxArray* f;
            if ((f = mxGetField(prhs[8], 0, "NitMax")) && !mxIsEmpty(f)) o.nit_max = (int32_t)mxGetScalar(f);
            if ((f = mxGetField(prhs[8], 0, "tol")) && !mxIsEmpty(f)) o.tol = mxGetScalar(f);
            if ((f = mxGetField(prhs[8], 0, "lam")) && !mxIsEmpty(f)) o.lam = mxGetScalar(f);
            if ((f = mxGetField(prhs[8], 0, "stallWindow")) && !mxIsEmpty(f)) o.stall_window = (int32_t)mxGetScalar(f);
            if ((f = mxGetField(prhs[8], 0, "flags")) && !mxIsEmpty(f)) o.flags = (int32_t)mxGetScalar(f);
            if ((f = mxGetField(prhs[8], 0, "fcgM")) && !mxIsEmpty(f)) o.fcg_m = (int32_t)mxGetScalar(f);
        }
        in_buf yb, xb;
        const void* y = in_data(prhs[4], &yb);
        const void* x0 = NULL;
        xb.g = NULL;
        xb.host = NULL;
        if (!mxIsEmpty(prhs[7])) x0 = in_data(prhs[7], &xb);
        mwSize dims[8], nd;
        size_t nimg = read_dims(prhs[9], dims, &nd);
        const int32_t cap = o.nit_max + 1;
        double* hh = (double*)mxCalloc(2 * (size_t)cap, sizeof(double));
        mmr_lpcg_hist hist;
        memset(&hist, 0, sizeof(hist));
        hist.res_sq = hh;
        hist.err_sq = hh + cap;
        hist.capacity = cap;
        out_buf ob;
        void* x = out_data(prhs[4], nd, dims, nimg, &ob);
        int rc = mmr_lpcg_solve(A, y, net, x0, &o, x, &hist, NULL);
        mmr_sense_destroy(A);
        if (net) mmr_cnn_destroy(net);
        in_free(&yb);
        in_free(&xb);
        plhs[0] = out_take(&ob, rc, nd, dims, prhs[4]);
        if (rc == MMR_OK) {
            if (nlhs > 1) {
                plhs[1] = mxCreateDoubleMatrix((mwSize)hist.n, 1, mxREAL);
                memcpy(mxGetDoubles(plhs[1]), hist.res_sq, (size_t)hist.n * sizeof(double));
            }
            if (nlhs > 2) {
                plhs[2] = mxCreateDoubleMatrix((mwSize)hist.n, 1, mxREAL);
                memcpy(mxGetDoubles(plhs[2]), hist.err_sq, (size_t)hist.n * sizeof(double));
            }
            if (nlhs > 3) {
                const char* names[4] = {"nit", "status", "fellBackAt", "trueResRel"};
                plhs[3] = mxCreateStructMatrix(1, 1, 4, names);
                mxSetField(plhs[3], 0, "nit", mxCreateDoubleScalar(hist.nit));
                mxSetField(plhs[3], 0, "status", mxCreateDoubleScalar(hist.status));
                mxSetField(plhs[3], 0, "fellBackAt", mxCreateDoubleScalar(hist.fell_back_at));
                mxSetField(plhs[3], 0, "trueResRel", mxCreateDoubleScalar(hist.true_res_rel));
            }
        }
        mxFree(hh);
        check(rc);
        return;
    }

    /* --------------------------------------------------- mrSampFuncMat (dense) */
    if (!strcmp(cmd, "dense_normal")) {
        /* (hs, hr or 0, vox (1-based voxel indices of imMask)) -> AtA, complex single gpuArray
         * [nvox x nvox] (operators/mrSampFuncMat.m:22-47) */
        gpu_init();
        const mwSize nv = (mwSize)mxGetNumberOfElements(prhs[3]);
        double* vd = as_double(prhs[3]);
        int64_t* vox = (int64_t*)mxMalloc(nv * sizeof(int64_t) + 8);
        for (mwSize i = 0; i < nv; ++i) vox[i] = (int64_t)vd[i] - 1;
        mxFree(vd);
        const mwSize dims[2] = {nv, nv};
        mxGPUArray* g = mxGPUCreateGPUArray(2, dims, mxSINGLE_CLASS, mxCOMPLEX, MX_GPU_DO_NOT_INITIALIZE);
        int rc = mmr_dense_normal((mmr_sho*)get_handle(prhs[1]), (mmr_rcvr*)get_handle(prhs[2]), vox, (int64_t)nv,
                                  mxGPUGetData(g), NULL);
        mxFree(vox);
        if (rc == MMR_OK) plhs[0] = mxGPUCreateMxArrayOnGPU(g);
        mxGPUDestroyGPUArray(g);
        check(rc);
        return;
    }
    if (!strcmp(cmd, "dense_solve")) {
        /* (AtA gpuArray, lam2, b) -> [x gpuArray, method]: (AtA + lam2 I) \ b (demo_denseMat.m:98-106) */
        gpu_init();
        if (!mxIsGPUArray(prhs[1])) mexErrMsgIdAndTxt("matmri:gb300:arg", "AtA must be the gpuArray of dense_normal");
        const mxGPUArray* a = mxGPUCreateFromMxArray(prhs[1]);
        const mwSize n = mxGPUGetDimensions(a)[0];
        const mwSize dims[2] = {n, 1};
        const mxGPUArray* bg = NULL;
        if (mxIsGPUArray(prhs[3])) {
            bg = mxGPUCreateFromMxArray(prhs[3]);
            if (mxGPUGetClassID(bg) != mxSINGLE_CLASS || mxGPUGetComplexity(bg) != mxCOMPLEX)
                mexErrMsgIdAndTxt("matmri:gb300:arg", "gpuArray data must be complex single");
        } else {   /* host right-hand side: one copy to the device */
            float* bh = as_c64(prhs[3]);
            mxArray* tmp = mxCreateNumericArray(2, dims, mxSINGLE_CLASS, mxCOMPLEX);
            memcpy(mxGetComplexSingles(tmp), bh, 2 * n * sizeof(float));
            mxFree(bh);
            bg = mxGPUCopyFromMxArray(tmp);
            mxDestroyArray(tmp);
        }
        mxGPUArray* xg = mxGPUCreateGPUArray(2, dims, mxSINGLE_CLASS, mxCOMPLEX, MX_GPU_DO_NOT_INITIALIZE);
        int32_t method = 0;
        int rc = mmr_dense_solve(mxGPUGetDataReadOnly(a), (int64_t)n, mxGetScalar(prhs[2]), mxGPUGetDataReadOnly(bg),
                                 mxGPUGetData(xg), &method, NULL);
        mxGPUDestroyGPUArray(bg);
        mxGPUDestroyGPUArray(a);
        if (rc == MMR_OK) plhs[0] = mxGPUCreateMxArrayOnGPU(xg);
        mxGPUDestroyGPUArray(xg);
        check(rc);
        if (nlhs > 1) plhs[1] = mxCreateDoubleScalar(method);
        return;
    }
    /* --------------------------------------------------------------- library */
    if (!strcmp(cmd, "check_device_error")) {
        /* () raises matmri:gb300:e4 if a bounded device wait ran out during a call given gpuArray
           data (calls given host arrays report it themselves); clears the flag */
        check(mmr_check_device_error(NULL));
        return;
    }
    mexErrMsgIdAndTxt("matmri:gb300:arg", "unknown command %s", cmd);
}
