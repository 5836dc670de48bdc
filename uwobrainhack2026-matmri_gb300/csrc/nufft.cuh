// @nufftOp plan and gridding kernels (Kaiser-Bessel interpolation / spreading).
#pragma once

#include <cuda.h>

#include "fft.cuh"

namespace mmr {

// Binned sample lists for one tile size (2D fast path).
//
// Work is split into items of about `chunk` entries so that the dense centre
// of a variable-density trajectory is spread over many CTAs: interpolation
// items are chunks of a tile's own samples; spreading items are quadtree
// (sub)tiles of 32, 16 or 8 cells that each own their output cells.
struct BinLists {
    int T = 0;                 // full tile side (grid cells)
    int chunk = 0;             // target entries per work item
    int ntx = 0, nty = 0;
    DevBuf own_s, own_lb;            // interp: each sample once (tile containing its base cell)
    DevBuf pad_s, pad_lb;            // spread/normal: every (sub)tile its footprint touches
    DevBuf pad_w;                    // float [n_pad][2][W]: each padded entry's tap weights
    DevBuf own_items, pad_items;     // int4 {u0 | v0 << 16, e0, e1, tile side | shared << 8}
    DevBuf heavy;                    // int2 {u0 | v0 << 16, side}: leaf tiles split across items
    int n_own_items = 0, n_pad_items = 0, n_heavy = 0;
    long long n_own = 0, n_pad = 0;
    int max_own = 0, max_pad = 0;
};

struct NufftPlan {
    int nd = 0;
    int N[3] = {1, 1, 1};
    int G[3] = {1, 1, 1};
    long long M = 0;
    int W = 0;
    double os = 0, beta = 0;
    int Nkern = 0;
    long long Ntot = 1, Gtot = 1;
    std::vector<double> kloc;     // host copy [M x nd] (Toeplitz re-plans from it)
    std::vector<double> dcf_h;    // host copy (empty = no dcf)
    DevBuf d_base;                // int  [nd][M]: floor((k+0.5) G) mod G
    DevBuf d_w;                   // float [M][nd][W] tap weights
    DevBuf d_dcf;                 // float [M]
    bool has_dcf = false;
    int dcf_version = 0;
    DevBuf d_fwd_fac[3], d_adj_fac[3];   // float2 [N_d]: deapod * exp(+-i pi N_d / 2)
    // the other axes' factors folded into one per transform line (nd > 1): the first
    // image->grid pass multiplies line (j, k) by fwd_1[j] fwd_2[k], the last grid->image pass
    // line (i, j) by adj_0[i] adj_1[j]; the passes in between apply none
    DevBuf d_fwd_line, d_adj_line;
    FftFactors ff[3];
    const float2* tw[3] = {nullptr, nullptr, nullptr};
    BinLists bins;                // valid when use_bins
    bool use_bins = false;
    int cg_pref = 4;              // coils per CTA in the gridding kernels (autotuned)
    // Gridding normal operator C^H diag(w) C as a (2W-1)^2 stencil per grid cell
    // (float [(2W-1)^2][G1*G2]), built from the per-sample weights w.
    DevBuf d_stencil;
    long long stencil_key = -1;   // identifies the weights it was built from
    int normal_mode = 0;          // 0 auto, 1 fused interp/spread, 2 stencil (autotuned)
    int fft_lines = 8;            // lines per CTA in the FFT passes (autotuned, power of two)
    // scratch
    DevBuf s_tmp, s_grid, s_grid2;
    DevBuf s_coil;                // per-coil images before the coil sum
    Staged st_in, st_out;
    // TMA descriptor cache for the interp kernel (keyed by grid buffer / batch)
    CUtensorMap tmap;
    const void* tmap_ptr = nullptr;
    long long tmap_nb = 0;
    int tmap_cg = 0;
    // Toeplitz mode
    bool is_toep = false;
    DevBuf d_toep;                // complex64 [2N...] transfer function (centered)
    FftFactors tff[3];
    const float2* ttw[3] = {nullptr, nullptr, nullptr};
};

void nufft_plan_build(NufftPlan& p, const mmr_nufft_desc& d);
void nufft_set_dcf(NufftPlan& p, const double* dcf);
void nufft_build_bins(NufftPlan& p, int T, int chunk = 64);

// Operations on device buffers (all on `st`).  `active` (nullable) makes every
// kernel a no-op while *active != 0 (device-resident solver termination).
// x: [N..., nb]   grid: [G..., nb] centered   y: [M, nb]
void nufft_forward(NufftPlan& p, const float2* x, float2* y, long long nb, cudaStream_t st,
                   const int* active = nullptr);
void nufft_adjoint(NufftPlan& p, const float2* y, float2* x, long long nb, cudaStream_t st,
                   const int* active = nullptr);
void nufft_toep_apply(NufftPlan& p, const float2* x, float2* y, long long nb, cudaStream_t st);
void nufft_prep_toep(NufftPlan& p, double tos, int kw);

// Building blocks used by the SENSE pipeline.
// Image-domain -> centered oversampled grid for `nb` lines-sets.  When maps != null
// the input is one image shared by the nb coils and multiplied by maps[.., c].
void nufft_img_to_grid(NufftPlan& p, const float2* x, const float2* maps, float2* grid,
                       long long nb, cudaStream_t st, const int* active);
// Centered grid -> image (crop + deapod).  When maps != null, conj(maps) weighted sum
// over the nb coils into out (accumulate: out += ...).
// `scratch` (optional) replaces the plan's intermediate buffer; it must hold
// nufft_grid_to_img_scratch(p, nb) complex values.
// An epilogue of the coil sum for a solver: out += tik .* v (tik nullable), then
// acc[0] += re(v' out), acc[1] += im(v' out) (FP64).
struct DotEpilogue {
    const float2* v = nullptr;
    const float* tik = nullptr;
    double* acc = nullptr;
};
void nufft_grid_to_img(NufftPlan& p, const float2* grid, const float2* maps, float2* out,
                       long long nb, bool accumulate, cudaStream_t st, const int* active,
                       float2* scratch = nullptr, const DotEpilogue* dot = nullptr);
size_t nufft_grid_to_img_scratch(const NufftPlan& p, long long nb);
// Gridding: interpolation (grid -> samples, times wfac) and spreading (samples*wfac -> grid).
// wfac: per-sample real weight [M] or per-sample-per-batch [M x nb] (wfac_bstride = M), or null.
void nufft_interp(NufftPlan& p, const float2* grid, float2* y, long long nb, const float* wfac,
                  long long wfac_bstride, cudaStream_t st, const int* active);
void nufft_spread(NufftPlan& p, const float2* y, float2* grid, long long nb, const float* wfac,
                  long long wfac_bstride, cudaStream_t st, const int* active);
// Fused C^H diag(wfac) C on the grid (interp -> weight -> spread), 2D binned path.
void nufft_grid_normal(NufftPlan& p, const float2* gin, float2* gout, long long nb, const float* wfac,
                       long long wfac_bstride, cudaStream_t st, const int* active);
bool nufft_has_fused_normal(const NufftPlan& p);
// Stencil form of the gridding normal operator.  `w` (host, M entries, or null
// for all ones) are the per-sample weights; `key` identifies them so that the
// stencil is rebuilt only when they change.  2D only.
bool nufft_stencil_supported(const NufftPlan& p);
void nufft_build_stencil(NufftPlan& p, const float* w, long long key);
void nufft_grid_normal_stencil(NufftPlan& p, const float2* gin, float2* gout, long long nb, cudaStream_t st,
                               const int* active);

// Device error word set by bounded waits that ran out (0 = none).
int device_error_word(cudaStream_t st);
// Sets the poll limit of the gridding kernels' bounded TMA waits (test hook; 0 makes every wait run out).
void set_wait_polls(int polls);
int* device_error_ptr();

}  // namespace mmr
