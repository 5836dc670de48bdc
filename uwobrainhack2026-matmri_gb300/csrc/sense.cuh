// @rcvrOp, @sampHighOrder handle types and the mrSampFunc composition.
#pragma once

#include <cuda_fp16.h>

#include "nufft.cuh"

namespace mmr {

struct RcvrPlan {
    int nd = 0;
    int N[3] = {1, 1, 1};
    long long Ntot = 0, C = 0;
    DevBuf d_maps;   // complex64 [Ntot, C]
    Staged st_in, st_out;
};

struct ShoPlan;   // sho.cuh

// Forward / adjoint of sampHighOrder on device buffers (nb = batch columns).
void sho_forward(ShoPlan& s, const float2* x, float2* y, long long nb, cudaStream_t st, const int* active);
void sho_adjoint(ShoPlan& s, const float2* y, float2* x, long long nb, cudaStream_t st, const int* active);
long long sho_nvox(const ShoPlan& s);
long long sho_nsamp(const ShoPlan& s);
// E [M, nvox] complex64, E[m + M j] = exp(i kbase[vox[j], m]) (vox: device indices).
void sho_encoding_matrix(ShoPlan& s, const long long* vox, long long nvox, float2* E, cudaStream_t st);
// The Gram operands [4][rows][kpad] FP16 (cos hi, cos lo, sin hi, sin lo; rows >= nvox, kpad >= M,
// zero-padded) of the mask voxels' encoding rows.
void sho_gram_operands(ShoPlan& s, const long long* vox, long long nvox, long long rows, long long kpad, __half* op,
                       cudaStream_t st);
// (1 / n) E^H E for the Gram operands above on the tcgen05 tensor cores, written to AtA [n x n]
// column-major (both triangles); false when the device has no tcgen05.
bool gram_umma(const __half* op, long long n, long long rows, long long kpad, float2* AtA, cudaStream_t st);
bool gram_umma_supported();

void rcvr_forward(const RcvrPlan& r, const float2* x, float2* y, cudaStream_t st, const int* active);
void rcvr_adjoint(const RcvrPlan& r, const float2* y, float2* x, cudaStream_t st, const int* active);

// mrSampFunc(x, transp, S, R, opt) on device buffers.
struct SenseOp {
    NufftPlan* nufft = nullptr;
    ShoPlan* sho = nullptr;
    RcvrPlan* rcvr = nullptr;
    long long Nimg = 0;     // voxels
    long long M = 0;        // samples per coil
    long long C = 1;        // coils (1 without R)
    double tikreg = 0;
    // opt.W (data weights, applied before the adjoint): [M] or [M x C]
    DevBuf d_optW;
    bool has_optW = false;
    bool optW_per_coil = false;
    int coil_chunk = 0;     // 0 = auto
    int tile = 32;
    // per-call weight buffers: dcf*W (adjoint) and dcf^2*W (normal)
    DevBuf d_wadj, d_wnorm;
    long long w_bstride = 0;
    long long wkey = -2;    // cache key of d_wadj/d_wnorm when no cgne W is applied
    std::vector<float> wnorm_h;   // host copy of d_wnorm (empty: no weights)
    long long wversion = 0;       // bumped whenever d_wadj / d_wnorm change
    std::vector<float> optW_h;
    // scratch
    DevBuf s_grid, s_grid2, s_samp, s_img;
    Staged st_in, st_out;
    cudaStream_t stream = nullptr;       // internal non-blocking stream (graphs)
    void* solver_ws = nullptr;           // cg workspace (cg.cu)
    void* lpcg_ws = nullptr;             // learned-PCG workspace (lpcg.cu)
};

int sense_chunk(const SenseOp& a);
// Rebuilds d_wadj / d_wnorm from dcf, opt.W and an optional cgne W (host floats).
void sense_set_weights(SenseOp& a, const float* cgW, bool cgW_per_coil);
void sense_forward(SenseOp& a, const float2* x, float2* y, cudaStream_t st, const int* active);
// adjoint applies d_wadj (dcf * opt.W * cgW)
void sense_adjoint(SenseOp& a, const float2* y, float2* x, cudaStream_t st, const int* active);
// normal op A^H diag(d_wnorm) A (+ tikreg^2) x.  With dot: y += tik .* x (tik nullable) and
// dot = (re, im)(x' y) accumulated into dot[0..1] in the last kernel; returns false (and does
// neither) when this operator's last kernel cannot carry it, so the caller does it separately.
void sense_normal(SenseOp& a, const float2* x, float2* y, cudaStream_t st, const int* active);
bool sense_normal_dot(SenseOp& a, const float2* x, float2* y, const float* tik, double* dot, cudaStream_t st,
                      const int* active);

// Frees the solver workspaces and their CUDA graphs (cg and learned PCG).
void cg_release(SenseOp& a);
void lpcg_release(SenseOp& a);

}  // namespace mmr

struct mmr_nufft { mmr::NufftPlan p; };
struct mmr_rcvr { mmr::RcvrPlan r; };
struct mmr_sense { mmr::SenseOp a; };
