/*
 * matmri_mex.c — MATLAB gateway to libmatmri_gb300 (the C ABI in
 * include/matmri_gb300.h).  Build (MATLAB R2018a or newer, interleaved complex):
 *
 *   mex -R2018a matmri_mex.c -I../../include -L../matmri_gb300 -lmatmri_gb300
 *
 * Called as  varargout = matmri_mex(command, args...)  by the classdef wrappers
 * in this folder (@nufftOp, @rcvrOp, @sampHighOrder, cgne.m).  Handles travel
 * as uint64 scalars.  Numeric arrays: double or single host arrays are
 * converted to interleaved complex single; the result is returned in the
 * class of the input (nufftOp.m:288-299, 404-406 preserve the input class).
 * Any non-zero status raises matmri:gb300:<code> with the library's message.
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

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
    } else {
        mexErrMsgIdAndTxt("matmri:gb300:arg", "expected a real numeric array");
    }
    return d;
}

/* Interleaved complex single copy of any numeric array (caller frees). */
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

void mexFunction(int nlhs, mxArray* plhs[], int nrhs, const mxArray* prhs[]) {
    char cmd[64];
    if (nrhs < 1 || mxGetString(prhs[0], cmd, sizeof(cmd)))
        mexErrMsgIdAndTxt("matmri:gb300:arg", "first argument must be a command string");

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
    if (!strcmp(cmd, "nufft_apply")) {             /* (h, adjoint, x, outDims) */
        mmr_nufft* h = (mmr_nufft*)get_handle(prhs[1]);
        const int adjoint = (int)mxGetScalar(prhs[2]);
        const mxArray* x = prhs[3];
        double* od = as_double(prhs[4]);
        mwSize nd = (mwSize)mxGetNumberOfElements(prhs[4]);
        mwSize dims[8];
        size_t nout = 1;
        for (mwSize k = 0; k < nd && k < 8; ++k) { dims[k] = (mwSize)od[k]; nout *= dims[k]; }
        const int64_t nbatch = (int64_t)mxGetScalar(prhs[5]);
        float* in = as_c64(x);
        float* out = (float*)mxMalloc(2 * nout * sizeof(float) + 8);
        int rc = mmr_nufft_apply(h, adjoint, in, out, nbatch, NULL);
        mxFree(in);
        if (rc == MMR_OK) plhs[0] = from_c64(out, nd, dims, x);
        mxFree(out); mxFree(od);
        check(rc);
        return;
    }
    if (!strcmp(cmd, "nufft_prep_toep")) {         /* (h, tos, kwidth) */
        check(mmr_nufft_prep_toep((mmr_nufft*)get_handle(prhs[1]), scalar_or(prhs[2], -1),
                                  (int32_t)scalar_or(prhs[3], -1)));
        return;
    }
    if (!strcmp(cmd, "nufft_destroy")) { check(mmr_nufft_destroy((mmr_nufft*)get_handle(prhs[1]))); return; }

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
        mmr_rcvr* h = (mmr_rcvr*)get_handle(prhs[1]);
        double* od = as_double(prhs[4]);
        mwSize nd = (mwSize)mxGetNumberOfElements(prhs[4]);
        mwSize dims[8];
        size_t nout = 1;
        for (mwSize k = 0; k < nd && k < 8; ++k) { dims[k] = (mwSize)od[k]; nout *= dims[k]; }
        float* in = as_c64(prhs[3]);
        float* out = (float*)mxMalloc(2 * nout * sizeof(float) + 8);
        int rc = mmr_rcvr_apply(h, (int)mxGetScalar(prhs[2]), in, out, NULL);
        mxFree(in);
        if (rc == MMR_OK) plhs[0] = from_c64(out, nd, dims, prhs[3]);
        mxFree(out); mxFree(od);
        check(rc);
        return;
    }
    if (!strcmp(cmd, "rcvr_destroy")) { check(mmr_rcvr_destroy((mmr_rcvr*)get_handle(prhs[1]))); return; }

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
        mxFree(t);
        mxFree(sp);
        mxFree(gx);
        mxFree(gy);
        mxFree(gz);
        check(rc);
        plhs[0] = put_handle(h);
        return;
    }
    if (!strcmp(cmd, "sho_apply")) {               /* (h, adjoint, x, outDims, nbatch) */
        mmr_sho* h = (mmr_sho*)get_handle(prhs[1]);
        double* od = as_double(prhs[4]);
        mwSize nd = (mwSize)mxGetNumberOfElements(prhs[4]);
        mwSize dims[8];
        size_t nout = 1;
        for (mwSize k = 0; k < nd && k < 8; ++k) { dims[k] = (mwSize)od[k]; nout *= dims[k]; }
        float* in = as_c64(prhs[3]);
        float* out = (float*)mxMalloc(2 * nout * sizeof(float) + 8);
        int rc = mmr_sho_apply(h, (int)mxGetScalar(prhs[2]), in, out, (int64_t)mxGetScalar(prhs[5]), NULL);
        mxFree(in);
        if (rc == MMR_OK) plhs[0] = from_c64(out, nd, dims, prhs[3]);
        mxFree(out); mxFree(od);
        check(rc);
        return;
    }
    if (!strcmp(cmd, "sho_destroy")) { check(mmr_sho_destroy((mmr_sho*)get_handle(prhs[1]))); return; }

    if (!strcmp(cmd, "cgne")) {
        /* (nufftHandle or 0, shoHandle or 0, rcvrHandle or 0, b, x0 or [], NitMax, opt struct, W or [],
         *  imDims) -> [x, resSqAll, mseAll, xnormAll, xdiffAll, stopThresh, status]   (cgne.m:1) */
        mmr_sense_desc sd;
        memset(&sd, 0, sizeof(sd));
        sd.nufft = (mmr_nufft*)get_handle(prhs[1]);
        sd.sho = (mmr_sho*)get_handle(prhs[2]);
        sd.rcvr = (mmr_rcvr*)get_handle(prhs[3]);
        mmr_sense* A = NULL;
        check(mmr_sense_create(&sd, &A));
        mmr_cgne_opts o;
        mmr_cgne_default_opts(&o);
        o.nit_max = (int32_t)scalar_or(prhs[6], 1000);
        o.want_history = 1;
        const mxArray* opt = prhs[7];
        if (mxIsStruct(opt)) {
            mxArray* f;
#define OPTD(name, field) if ((f = mxGetField(opt, 0, name))) o.field = mxIsEmpty(f) ? NAN : mxGetScalar(f);
#define OPTI(name, field) if ((f = mxGetField(opt, 0, name)) && !mxIsEmpty(f)) o.field = (int32_t)mxGetScalar(f);
            OPTD("resThresh", res_thresh) OPTD("resChangeThresh", res_change_thresh)
            OPTD("xChangeThresh", x_change_thresh) OPTI("expResN", exp_res_n)
            OPTD("nseThreshFact", nse_thresh_fact) OPTI("nseExtraIt", nse_extra_it)
            OPTI("stopOnResInc", stop_on_res_inc) OPTD("resIncThresh", res_inc_thresh)
            OPTI("stopOnXdifInc", stop_on_xdif_inc) OPTD("noiseVar", noise_var)
#undef OPTD
#undef OPTI
        }
        float* b = as_c64(prhs[4]);
        float* x0 = mxIsEmpty(prhs[5]) ? NULL : as_c64(prhs[5]);
        float* W = NULL;
        if (!mxIsEmpty(prhs[8])) {
            double* wd = as_double(prhs[8]);
            size_t n = mxGetNumberOfElements(prhs[8]);
            W = (float*)mxMalloc(n * sizeof(float) + 4);
            for (size_t i = 0; i < n; ++i) W[i] = (float)wd[i];
            mxFree(wd);
            o.w_per_coil = n > (size_t)mxGetM(prhs[4]);
        }
        double* idim = as_double(prhs[9]);
        mwSize nd = (mwSize)mxGetNumberOfElements(prhs[9]);
        mwSize dims[4];
        size_t nimg = 1;
        for (mwSize k = 0; k < nd && k < 4; ++k) { dims[k] = (mwSize)idim[k]; nimg *= dims[k]; }
        const int32_t cap = o.nit_max + o.nse_extra_it + 1;
        double* hh = (double*)mxCalloc(4 * (size_t)cap, sizeof(double));
        mmr_cgne_hist hist = {hh, hh + cap, hh + 2 * cap, hh + 3 * cap, cap, 0, 0, 0, 0};
        float* x = (float*)mxMalloc(2 * nimg * sizeof(float) + 8);
        int rc = mmr_cgne_solve(A, b, x0, W, &o, x, &hist, NULL);
        mmr_sense_destroy(A);
        mxFree(b); if (x0) mxFree(x0); if (W) mxFree(W); mxFree(idim);
        if (rc == MMR_OK) {
            plhs[0] = from_c64(x, nd, dims, prhs[4]);
            for (int k = 0; k < 4 && k + 1 < nlhs; ++k) {
                static const int order[4] = {0, 1, 2, 3};   /* resSqAll, mseAll, xnormAll, xdiffAll */
                mxArray* v = mxCreateDoubleMatrix((mwSize)hist.n, 1, mxREAL);
                memcpy(mxGetDoubles(v), hh + (size_t)order[k] * cap, (size_t)hist.n * sizeof(double));
                plhs[k + 1] = v;
            }
            if (nlhs > 5) plhs[5] = isnan(hist.stop_thresh) ? mxCreateDoubleMatrix(0, 0, mxREAL)
                                                            : mxCreateDoubleScalar(hist.stop_thresh);
            if (nlhs > 6) plhs[6] = mxCreateDoubleScalar(hist.status);
        }
        mxFree(x); mxFree(hh);
        check(rc);
        return;
    }
    mexErrMsgIdAndTxt("matmri:gb300:arg", "unknown command %s", cmd);
}
