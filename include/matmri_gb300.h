/*
 * matmri_gb300.h — C ABI of the GB300 (sm_103a) MatMRI reconstruction hot path.
 *
 * Plain C: opaque handles, pointers and sizes; no C++ or torch types.
 * Every entry point returns an int status (MMR_OK == 0); the message of the
 * last failure on the calling thread is available from mmr_last_error().
 *
 * Data conventions (the MATLAB R2018a interleaved-complex API):
 *   - complex data is interleaved complex64 (float re, float im);
 *   - arrays are column-major with MATLAB index order: an image is
 *     [imN(1), imN(2), ..., extra], samples are [M, extra];
 *   - array pointers may be device pointers (gpuArray data) or host
 *     pointers; host pointers are staged through device memory and the call
 *     returns after the result is back on the host (nufftOp.m:335-347,396-398
 *     accept host or gpuArray input the same way);
 *   - trajectories, density compensation, coil maps and encoding phases are
 *     given as host arrays at construction (the constructors of the
 *     reference take MATLAB host arrays).
 *   - `stream` is a cudaStream_t (NULL = the legacy default stream).
 * Threading: a handle is used by one thread at a time; distinct handles are
 * independent.
 */
#ifndef MATMRI_GB300_H
#define MATMRI_GB300_H

#include <stdint.h>
#include <stddef.h>

#if defined(__GNUC__)
#define MMR_API __attribute__((visibility("default")))
#else
#define MMR_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define MMR_OK              0
#define MMR_ERR_BADARG      1   /* invalid argument / shape                      */
#define MMR_ERR_NOMEM       2   /* device or host allocation failed              */
#define MMR_ERR_CUDA        3   /* CUDA runtime error                            */
#define MMR_ERR_TIMEOUT     4   /* a bounded device wait ran out                 */
#define MMR_ERR_NONFINITE   5   /* NaN/Inf in an input where it is not allowed   */
#define MMR_ERR_UNSUPPORTED 6   /* option combination not implemented            */

#define MMR_ABI_VERSION 1

typedef struct mmr_nufft mmr_nufft;   /* @nufftOp plan                 */
typedef struct mmr_rcvr  mmr_rcvr;    /* @rcvrOp (precomputed maps)    */
typedef struct mmr_sho   mmr_sho;     /* @sampHighOrder plan           */
typedef struct mmr_sense mmr_sense;   /* mrSampFunc(., ., S, R, opt)   */

/* ---- library ------------------------------------------------------------ */
MMR_API int  mmr_abi_version(void);
/* Copies the last error message of this thread (NUL-terminated). */
MMR_API int  mmr_last_error(char* buf, size_t len);
/* Device properties used by the autotuner (SM count, smem per block). */
MMR_API int  mmr_device_info(int* sm_count, int* smem_optin_bytes, int* cc_major, int* cc_minor);
/* Kernels this library has launched in the process (eager launches plus the
 * kernel nodes of every replayed CUDA graph). */
MMR_API int  mmr_kernel_launches(uint64_t* count);
/* Reports a bounded device wait that ran out since the last check, for callers that pass
 * device pointers (entry points given host buffers check it themselves before returning):
 * synchronises `stream`, returns MMR_ERR_TIMEOUT and clears the flag if it was set, else
 * MMR_OK.  No reference counterpart (MATLAB has no asynchronous device calls). */
MMR_API int  mmr_check_device_error(void* stream);
/* Test hook: poll limit of the gridding kernels' bounded TMA waits (default 4194304; 0 makes
 * every wait run out, after which the kernel still lets its copy land and returns). */
MMR_API int  mmr_debug_set_wait_polls(int32_t polls);

/* ---- @nufftOp ------------------------------------------------------------
 * Replaces nufftOp(imN, kloc, dcf, useGPU, os, kwidth)
 *   (operators/@nufftOp/nufftOp.m:89-136; doPrep 138-274).
 * kloc: host double [M x ndim] column-major, in [-0.5, 0.5) (values outside
 *       wrap, as nufftOp.m:20-22 documents).  dcf: host double [M] or NULL.
 * os <= 0 selects the reference default 1.5; kwidth <= 0 selects 6
 *   (nufftOp.m:65-66). kwidth must be even, 2..8.                       */
typedef struct mmr_nufft_desc {
    int32_t       ndim;        /* 1, 2 or 3                                    */
    int64_t       imN[3];
    int64_t       nsamp;       /* M                                            */
    const double* kloc;
    const double* dcf;
    double        os;
    int32_t       kwidth;
} mmr_nufft_desc;

MMR_API int mmr_nufft_create(const mmr_nufft_desc* desc, mmr_nufft** out);
/* Nop.dcf = dcf (demos/demo_regridding.m:35); dcf == NULL clears it. */
MMR_API int mmr_nufft_set_dcf(mmr_nufft* plan, const double* dcf);
/* osN, beta, Nkern of the plan (nufftOp.m:146-156). */
MMR_API int mmr_nufft_info(const mmr_nufft* plan, int64_t osN[3], double* beta, int64_t* nkern);
/* N*x (adjoint = 0: x [imN, nbatch] -> y [M, nbatch]) and N'*y (adjoint = 1)
 * (nufftOp.m:284-408 incl. the extra-dim batching of 302-331).          */
MMR_API int mmr_nufft_apply(mmr_nufft* plan, int adjoint, const void* in, void* out,
                    int64_t nbatch, void* stream);
/* prepToep: switches the plan to Toeplitz mode where apply() computes
 * N'*(N*x) on a 2N grid (nufftOp.m:410-432, 348-352).  tos <= 0 selects
 * 0.5*(os-1)+1, kwidth <= 0 the plan's kwidth.                         */
MMR_API int mmr_nufft_prep_toep(mmr_nufft* plan, double tos, int32_t kwidth);
MMR_API int mmr_nufft_destroy(mmr_nufft* plan);
/* N'*y without allocating device memory (no counterpart in the reference; an
 * addition of this library).  For callers that must not allocate while they
 * apply the operator: a MEX function or plug-in that its host application
 * holds to a fixed device-memory budget, or a real-time loop that cannot
 * afford a cudaMalloc/cudaFree (their implicit synchronisation, or a failure)
 * in the middle of a scan.  Same kernels and result as
 * mmr_nufft_apply(plan, 1, ...).  y [M, nbatch] and x [imN, nbatch] must be
 * device pointers.  The grid scratch comes from one 8 MiB array in the
 * library's device image (held on every GPU that loads the library until
 * exit): nbatch * (prod(osN) + osN-pass intermediate) must fit in 1 Mi
 * complex values, otherwise MMR_ERR_BADARG.  The first call on a device looks
 * up the array's device address; make that first call before any stream
 * capture.  All calls share the array: calls that overlap on the GPU race, so
 * issue them on one stream.  Not available for a Toeplitz plan.            */
MMR_API int mmr_nufft_adjoint_noalloc(mmr_nufft* plan, const void* y, void* x, int64_t nbatch,
                                      void* stream);

/* ---- @rcvrOp ---------------------------------------------------------------
 * Replaces rcvrOp(maps, 0) (operators/@rcvrOp/rcvrOp.m:47-94, isCalDat = 0).
 * maps: host complex64 [imN, C].                                         */
MMR_API int mmr_rcvr_create(int32_t ndim, const int64_t imN[3], int64_t ncoil,
                    const void* maps, mmr_rcvr** out);
/* R*x (x [imN] -> [imN, C]) and R'*y (sum(y.*conj(maps), nDim+1))
 * (rcvrOp.m:104-159).                                                    */
MMR_API int mmr_rcvr_apply(mmr_rcvr* r, int adjoint, const void* in, void* out, void* stream);
MMR_API int mmr_rcvr_destroy(mmr_rcvr* r);

/* ---- @sampHighOrder --------------------------------------------------------
 * Replaces sampHighOrder(b0, sampTimes, phs_spha, phs_conc, phs_grid, imMask)
 *   (operators/@sampHighOrder/sampHighOrder.m:129-291, prepForDirect 496-588).
 * Host doubles: b0 [V] rad/s (NULL = 0), t [M] s, spha [nspha x M],
 * conc [nconc x M] (NULL when nconc = 0), grid x/y/z [V], mask [V] or NULL.
 * nspha <= 36, nconc <= 4.                                                 */
typedef struct mmr_sho_desc {
    int32_t       ndim;        /* image dims (1..3)                           */
    int64_t       imN[3];
    int64_t       nsamp;       /* M = numel(sampTimes)                        */
    int32_t       nspha;
    int32_t       nconc;
    const double* b0;
    const double* t;
    const double* spha;
    const double* conc;
    const double* gx;
    const double* gy;
    const double* gz;
    const double* mask;
} mmr_sho_desc;

MMR_API int mmr_sho_create(const mmr_sho_desc* desc, mmr_sho** out);
/* S*x (x [V, nbatch] -> y [M, nbatch]) and S'*y (useDirectWorker,
 * sampHighOrder.m:361-391; the segmented approaches 2/3 compute the same
 * sums, sampHighOrder.m:393-457).                                         */
MMR_API int mmr_sho_apply(mmr_sho* s, int adjoint, const void* in, void* out,
                  int64_t nbatch, void* stream);
/* Selects the contraction of the direct encoding: on = 1 (default) the
 * tcgen05 tensor-core kernel (TMA-staged phase tiles, TMEM accumulators;
 * operands split into FP16 hi + scaled lo parts, FP32 accumulation), on = 2
 * the mma.sync tensor-core kernel (same splits), on = 0 the SIMT FP32
 * kernels.  All read the FP32-turns phase table; without room for the table
 * the SIMT kernels evaluate the phase per element in FP64.                */
MMR_API int mmr_sho_set_tensor(mmr_sho* s, int on);
MMR_API int mmr_sho_destroy(mmr_sho* s);
/* The public property S.kbase of a direct plan (prepForDirect,
 * sampHighOrder.m:496-588; read by operators/mrSampFuncMat.m:35): host FP64
 * [V x M] column-major, kbase[v + V m] = sum_k basis_k(r_v) coef_k(m) +
 * b0(v) t(m).  A setPhiDiv handle gives its base's kbase; not available for
 * the interpolated approach.                                              */
MMR_API int mmr_sho_kbase(const mmr_sho* s, double* kbase);
/* Replaces S2 = S.setPhiDiv(ksphaDiv, kconcDiv) (sampHighOrder.m:590-622):
 * a new handle whose forward is (1i * exp(1i*kbase) .* phiDiv).' * x / sqrt(V)
 * with phiDiv from prepForDirect on the derivative coefficients (no B0 term;
 * sampHighOrder.m:376-380) and whose adjoint is the base's (369-372).
 * kspha_div [nspha x M], kconc_div [nconc x M] host doubles, nspha / nconc at
 * most the base plan's.  The new handle refers to `base`, which must outlive
 * it.  Not available for the interpolated approach.                       */
MMR_API int mmr_sho_phidiv_create(mmr_sho* base, int32_t nspha, int32_t nconc, const double* kspha_div,
                                  const double* kconc_div, mmr_sho** out);

/* Replaces sampHighOrder(..., approach = 1, opt): the SVD + NUFFT
 * interpolated encoding (useInterpWorker, sampHighOrder.m:314-359).  The
 * caller passes the factors that prepForInterp forms (sampHighOrder.m:700-889,
 * createNufftForInterp 624-698): kloc [M x 2] of the trajectory nufftOp,
 * svd_space [V x L], svd_time [M x L] and phs_shift [M], all host doubles,
 * the last three interleaved complex.  os / kwidth of the trajectory nufftOp
 * (<= 0: the nufftOp defaults 1.5 / 6).  2D images only.  The handle works
 * with mmr_sho_apply and mmr_sense_create like the direct encoding.        */
typedef struct mmr_sho_interp_desc {
    int32_t       ndim;        /* 2                                           */
    int64_t       imN[3];
    int64_t       nsamp;       /* M                                           */
    int32_t       nterms;      /* L (number of singular triplets kept)        */
    const double* kloc;
    const double* svd_space;
    const double* svd_time;
    const double* phs_shift;
    double        os;
    int32_t       kwidth;
} mmr_sho_interp_desc;
MMR_API int mmr_sho_interp_create(const mmr_sho_interp_desc* desc, mmr_sho** out);

/* ---- mrSampFuncMat (dense normal matrix) -------------------------------------
 * Replaces [AtA, ~] = mrSampFuncMat(y, Crcvr, b0, sampTimes, phs_spha, phs_conc,
 *   phs_grid, imMask) (operators/mrSampFuncMat.m:22-47) for the matrix part:
 *   AtA = sum_c conj(r_c) r_c.' .* (S'*S),  S = exp(1i*kbase(vox,:)).'/sqrt(nvox)
 * over the nvox voxels listed in vox (host, 0-based, column-major order; the
 * imMask voxels).  S must be a direct sampHighOrder plan (mmr_sho_create),
 * R an rcvrOp over the same image or NULL (single coil of ones).  AtA: device
 * complex64 [nvox x nvox] column-major, written.  Aty = R'*(S'*y) on the mask
 * comes from mmr_sense_apply.                                              */
MMR_API int mmr_dense_normal(mmr_sho* S, mmr_rcvr* R, const int64_t* vox, int64_t nvox, void* AtA, void* stream);
/* x = (AtA + lam2*I) \ b (demos/demo_denseMat.m:98-106) on device complex64
 * buffers; AtA is not modified.  Cholesky, or LU with partial pivoting when
 * the shifted matrix is not numerically positive definite; *method (may be
 * NULL) receives 1 or 2 accordingly.  Synchronises the stream.             */
MMR_API int mmr_dense_solve(const void* AtA, int64_t n, double lam2, const void* b, void* x, int32_t* method,
                            void* stream);

/* ---- mrSampFunc --------------------------------------------------------------
 * Replaces opFunc = @(x,transp) mrSampFunc(x, transp, S, R, opt)
 *   (operators/mrSampFunc.m:1-160) for S a nufftOp or sampHighOrder and R an
 * rcvrOp (or none).  Exactly one of nufft / sho is non-NULL.
 * W: host float [M] or [M x C] data weights (opt.W, mrSampFunc.m:126-128),
 *    or NULL.  tikreg: opt.tikReg scalar (0 = none).                       */
typedef struct mmr_sense_desc {
    mmr_nufft*   nufft;
    mmr_sho*     sho;
    mmr_rcvr*    rcvr;
    const float* W;
    int32_t      w_per_coil;
    double       tikreg;
} mmr_sense_desc;

MMR_API int mmr_sense_create(const mmr_sense_desc* desc, mmr_sense** out);
/* transp = 0: image [imN] -> data [M, C];  transp = 1: data -> image.     */
MMR_API int mmr_sense_apply(mmr_sense* a, int transp, const void* in, void* out, void* stream);
/* A'*(A*x) with the fused gridding (used by cgne.m:215-218).             */
MMR_API int mmr_sense_normal(mmr_sense* a, const void* in, void* out, void* stream);
/* Runs the normal operator `reps` times with a CUDA event before every kernel
 * and returns, per stage, the summed time (ms) and the number of launches:
 * stage 0 first image->grid FFT pass (deapod + coil maps), 1 remaining
 * image->grid passes, 2 gridding (fused interp/spread, or sampHighOrder
 * encode), 3 grid->image passes before the last, 4 last pass per coil (crop,
 * deapod) and the conj-maps coil sum.  stage_ms / launches hold 5 entries. */
MMR_API int mmr_sense_profile_normal(mmr_sense* a, const void* in, void* out, int32_t reps,
                                     double* stage_ms, int32_t* launches, void* stream);
/* Tuning knobs chosen by the autotuner (0 = keep / automatic):
 *   coil_chunk  coils per pipeline pass (1..32; a pass's grids stay in L2 when they fit)
 *   tile        gridding tile side (8, 16, 32, 64)
 *   coil_group  coils per CTA in the gridding kernels (1, 2, 4, 8)
 *   item        max samples per gridding work item (>= 8)
 *   fft_lines   transform lines per CTA in the FFT passes (1..16, power of two)
 *   normal_mode gridding step of the normal operator: 1 fused interpolate /
 *               weight / spread, 2 precomputed C^H diag(w) C stencil       */
typedef struct mmr_tuning {
    int32_t coil_chunk;
    int32_t tile;
    int32_t coil_group;
    int32_t item;
    int32_t fft_lines;
    int32_t normal_mode;
} mmr_tuning;
MMR_API int mmr_sense_set_tuning(mmr_sense* a, const mmr_tuning* t);
MMR_API int mmr_sense_get_tuning(const mmr_sense* a, mmr_tuning* t);
MMR_API int mmr_sense_destroy(mmr_sense* a);

/* ---- cgne -------------------------------------------------------------------
 * Replaces [x,resSqAll,mseAll,xnormAll,xdiffAll,stopThresh,status] =
 *   cgne(A, b, x0, NitMax, opt, gam, R, W)  (iterativeSolvers/cgne.m:1-341).
 * Options mirror cgne.m:21-89; a NaN double means MATLAB's [] (rule off).
 * The whole iteration runs on the device (FP64 scalars and reductions,
 * complex64 vectors) and is captured as a CUDA graph.                      */
typedef struct mmr_cgne_opts {
    int32_t       nit_max;           /* NitMax (<= 0 selects 1000)            */
    double        res_thresh;        /* default 1e-10                         */
    double        res_change_thresh; /* default []                            */
    double        x_change_thresh;   /* default 1e-10                         */
    int32_t       exp_res_n;         /* default 100                           */
    double        nse_thresh_fact;   /* default 1.0                           */
    int32_t       nse_extra_it;      /* default 4                             */
    int32_t       stop_on_res_inc;   /* default 0                             */
    double        res_inc_thresh;    /* default 1.0                           */
    int32_t       stop_on_xdif_inc;  /* default 0                             */
    double        noise_var;         /* default []                            */
    const void*   noise;             /* optional noise draw [M x C] (complex64) for the
                                        discrepancy rule; NULL = internal seeded draw */
    uint64_t      noise_seed;
    const void*   gtruth;            /* optional [imN] complex64 (opt.gtruth) */
    const float*  tik_diag;          /* optional [imN] real: sum_k gam_k |R_k|^2 for
                                        elementwise-mask R (cgne.m:171-179)  */
    int32_t       w_per_coil;        /* W passed to mmr_cgne_solve is [M x C] */
    int32_t       want_history;      /* 1: fill the history arrays            */
} mmr_cgne_opts;

/* Fills opts with cgne.m's defaults. */
MMR_API int mmr_cgne_default_opts(mmr_cgne_opts* opts);

/* History outputs (host doubles, capacity nit_max + nse_extra_it + 1 each;
 * res_sq, mse, xnorm, xdiff are complex in the reference and are returned
 * as their real parts). */
typedef struct mmr_cgne_hist {
    double* res_sq;
    double* mse;
    double* xnorm;
    double* xdiff;
    int32_t capacity;
    int32_t n;            /* out: nit + 1 entries written                    */
    double  stop_thresh;  /* out: NaN when no noise rule                     */
    int32_t status;       /* out: cgne.m status code                         */
    int32_t nit;          /* out                                              */
} mmr_cgne_hist;

/* b: data [M, C]; x0: image or NULL (x0 = A'*b, cgne.m:143-145);
 * W: cgne's data weights [M] / [M x C] host float, or NULL. */
MMR_API int mmr_cgne_solve(mmr_sense* A, const void* b, const void* x0, const float* W,
                   const mmr_cgne_opts* opts, void* x_out, mmr_cgne_hist* hist,
                   void* stream);

/* n independent cgne solves (e.g. slices with different matrix sizes, coil
 * counts and trajectories: one mmr_sense each, all distinct) run together:
 * one CUDA graph holds one iteration of every solve as parallel branches, so
 * each graph launch advances the whole batch (a loop over cgne calls in the
 * reference).  Same options for all (x0 = A'b, no W); stopping rules act per
 * solve; hists may be NULL or an array of n.                               */
MMR_API int mmr_cgne_solve_batch(mmr_sense* const* A, int32_t n, const void* const* b, void* const* x_out,
                                 const mmr_cgne_opts* opts, mmr_cgne_hist* hists, void* stream);

/* ---- powermethod / bfista --------------------------------------------------
 * powermethod(A, x0, NitMax, doAtA=1, xdiffThresh)  (iterativeSolvers/powermethod.m:1-67) */
MMR_API int mmr_powermethod(mmr_sense* A, const void* x0, int32_t nit_max, double xdiff_thresh,
                    double* max_eig_re, double* max_eig_im, void* stream);

/* W*x and W'*w for W = dwtND(levels, imN, false, 'db1') (operators/@dwtND/
 * mtimes.m:1-122, wavConv1D.m:1-44): adjoint = 0 maps x [imN] to the bands
 * [nbands][imN] in waveletObj order (low, high{1}{1..}, high{2}{1..}, ...);
 * adjoint = 1 maps bands back to an image.                                  */
MMR_API int mmr_dwt_haar(int32_t ndim, const int64_t imN[3], const int32_t levels[3], int adjoint,
                         const void* in, void* out, void* stream);

/* bfista(A, b, dwtND(J, imSize, false, 'db1'), lam, x0, NitMax, opt)
 *   (iterativeSolvers/bfista.m:1-246; operators/@dwtND, undecimated Haar).
 * levels[ndim]: J per dim; lam: per-band thresholds (nbands = 1 + sum over
 * levels of (2^dims_decomposed - 1), band order low, high{1}{1..}, ...).
 * max_eig <= 0: run powermethod (bfista.m:81-89).                          */
typedef struct mmr_bfista_opts {
    int32_t       nit_max;     /* default 200                                  */
    double        res_thresh;  /* default 1e-5                                 */
    double        max_eig;     /* opt.maxEig (<= 0 = [])                       */
    int32_t       n_restart;   /* default NitMax + 1                           */
    const void*   x_mask;      /* optional [imN] complex64                     */
} mmr_bfista_opts;

typedef struct mmr_bfista_hist {
    double* res_sq;     /* capacity nit_max                                    */
    double* rx;
    double* test;       /* [nit_max x 2] column-major                          */
    int32_t capacity;
    int32_t n;          /* out: iterations run                                 */
    double  max_eig;    /* out                                                 */
} mmr_bfista_hist;

MMR_API int mmr_bfista_solve(mmr_sense* A, const void* b, const int32_t* levels,
                     const float* lam, int32_t nbands, const void* x0,
                     const mmr_bfista_opts* opts, void* x_out, mmr_bfista_hist* hist,
                     void* stream);

/* ---- learned preconditioner ---------------------------------------------------
 * No counterpart in the reference (an addition of this library): a small
 * convolutional network used as preconditioner and warm start of CG-SENSE.
 * A bias-free 3x3 CNN on complex images (2 real channels), hidden width 32,
 * ReLU between layers, global skip:
 *   s = sqrt(mean|r|^2);  a0 = r/s;  a_{l+1} = relu(conv(a_l, W_l));
 *   z = s * (conv(a_{L-1}, W_{L-1}) + skip * a0)
 * channels[] = {2, 32, ..., 32, 2} (nlayers + 1 entries).  Parameters: FP32,
 * W_l in [co][ci][ky][kx] order, layer by layer, then skip.  Images are
 * complex64 [nx, ny, batch], column-major (x fastest).                      */
typedef struct mmr_cnn mmr_cnn;

#define MMR_CNN_FP32_ACT 1   /* keep activations in FP32 (default BF16)       */
#define MMR_CNN_TENSOR   2   /* forward on the tensor-core path (mma.sync, FP16
                                activations, FP32 accumulation)               */
#define MMR_CNN_LOSS_COS 4   /* loss_grad: 1 - |<z,e>|^2/(|z|^2 |e|^2) instead of
                                the relative L2 (invariant to a complex scale)  */
#define MMR_CNN_LINEAR   8   /* identity activations: the network is a fixed
                                linear operator (forward and loss_grad)       */
#define MMR_CNN_FOLDED   16  /* with MMR_CNN_LINEAR: apply the network as its
                                folded (2L+1)^2 filter (2x2 real per tap) on the
                                zero-extended image, composed in FP64 from the
                                weights; FP32 arithmetic                      */

MMR_API int mmr_cnn_create(int32_t nlayers, const int32_t* channels, mmr_cnn** out);
MMR_API int mmr_cnn_num_params(const mmr_cnn* net, int64_t* n);
/* theta: host or device FP32 [n]; set_params also resets the optimiser state. */
MMR_API int mmr_cnn_set_params(mmr_cnn* net, const float* theta);
MMR_API int mmr_cnn_get_params(const mmr_cnn* net, float* theta);
/* z = net(r) */
MMR_API int mmr_cnn_forward(mmr_cnn* net, const void* r, void* z, int64_t nx, int64_t ny, int64_t batch,
                            int32_t flags, void* stream);
/* Loss L = mean_b |m.*(net(r_b) - e_b)|^2 / |m.*e_b|^2 (m: the interior
 * mask without `margin` pixels on each side; MMR_CNN_LOSS_COS selects
 * mean_b 1 - |<m z_b, m e_b>|^2 / (|m z_b|^2 |m e_b|^2)) and dL/dtheta, kept
 * on the device for mmr_cnn_adam_step and copied to `grad` (host, or NULL). */
MMR_API int mmr_cnn_loss_grad(mmr_cnn* net, const void* r, const void* e, int64_t nx, int64_t ny, int64_t batch,
                              int32_t margin, int32_t flags, double* loss, float* grad, void* stream);
/* One Adam step (beta1 0.9, beta2 0.999, eps 1e-8) with the last gradient. */
MMR_API int mmr_cnn_adam_step(mmr_cnn* net, float lr, void* stream);
MMR_API int mmr_cnn_destroy(mmr_cnn* net);

/* Learned-preconditioned CG-SENSE (no counterpart in the reference): flexible
 * CG on (A'WA + T) x = A'W y, the system cgne solves (cgne.m:136-227), with
 * z = net(r) as preconditioner (net == NULL: plain CG).  alpha = p'r / p'Hp is
 * the exact line search along p; beta = -(Hp)'z / p'Hp.  When |r|^2 has not
 * fallen over stall_window iterations the solver restarts plain CG from the
 * current x (the fallback); the true residual is recomputed at exit.        */
typedef struct mmr_lpcg_opts {
    int32_t       nit_max;       /* iterations (default 100)                      */
    double        tol;           /* stop when |r| <= tol |r0| (0: run nit_max)    */
    const float*  tik_diag;      /* optional [imN] real diagonal T (host/device)  */
    double        lam;           /* scalar added to T (Tikhonov gam with R = 1)   */
    const void*   gtruth;        /* optional [imN] complex64 for the error history */
    int32_t       stall_window;  /* fallback window (default 10; 0 = never)       */
    int32_t       flags;         /* MMR_CNN_* network flags (default TENSOR)      */
    int32_t       poll;          /* with tol > 0: the host checks for the stop every
                                    poll iterations (8); the fallback needs no host */
    int32_t       fcg_m;         /* directions the new one is made H-conjugate to
                                    (1..8, default 4; plain CG uses 1)          */
} mmr_lpcg_opts;

typedef struct mmr_lpcg_hist {
    double*  res_sq;        /* |r_k|^2, capacity nit_max + 1                   */
    double*  err_sq;        /* |x_k - gtruth|^2 (when gtruth is given)         */
    int32_t  capacity;
    int32_t  n;             /* out: entries written                            */
    int32_t  nit;           /* out: iterations run                             */
    int32_t  status;        /* out: 0 nit_max reached, 1 tol reached           */
    int32_t  fell_back_at;  /* out: iteration where plain CG took over, or -1  */
    double   true_res_rel;  /* out: |b - Hx| / |b| at exit                     */
} mmr_lpcg_hist;

MMR_API int mmr_lpcg_default_opts(mmr_lpcg_opts* opts);
/* y: data [M, C] (b = A'W y is formed inside); x0: image or NULL (zeros). */
MMR_API int mmr_lpcg_solve(mmr_sense* A, const void* y, mmr_cnn* net, const void* x0,
                           const mmr_lpcg_opts* opts, void* x_out, mmr_lpcg_hist* hist, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* MATMRI_GB300_H */
