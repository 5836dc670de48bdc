// Tensor-core path of the sampHighOrder encoding (sho_tc.cu).
#pragma once

#include "common.h"

namespace mmr {

constexpr long long SHO_TC_MAX_COILS = 4096;

// Device scratch of one plan, allocated once at its full size when the plan is
// built, so that graphs captured with these buffers stay valid.
struct ShoTcScratch {
    DevBuf bhi, blo;       // B operand hi / lo' [32][Kpad] halves (Kpad = 2 roundup(max(V, M), 8)), zero padded
    DevBuf partial;        // split-K partial sums
    DevBuf cmax;           // per-coil max |re|, |im|
    long long kpad = 0;
    int nsplit[2] = {1, 1};   // forward, adjoint
};

void sho_tc_alloc(ShoTcScratch& s, long long V, long long M);

// tcgen05 path (sho_umma.cu): the blocked radians copy of the phase table and the device scratch of
// one plan.
struct ShoUmma {
    bool ok = false;
    DevBuf tblk;            // the phase table as radians in 128 x 128 blocks [V / 128][M / 128][128][128]
    long long mblk = 0;     // blocks along M
    DevBuf b;               // B operand per stage (largest coil group), FP16 hi / lo, swizzled
    DevBuf partial;         // split-K partial sums [nsplit][rows][2 coils]
    DevBuf cmax;            // per-column max |re|, |im|
    long long lpad = 0;     // inputs padded to whole phase blocks (128)
    int nsplit[2] = {1, 1};   // forward, adjoint
    int* err = nullptr;       // device error word
};
// Builds the blocked phase table and scratch; false when the blocked copy does not fit in half of
// the free device memory or the device is not an sm_10x part.
bool sho_umma_prepare(ShoUmma& u, const float* turn, long long V, long long M);
void sho_umma_forward(ShoUmma& u, long long V, long long M, const float2* x, float2* y, long long nb, cudaStream_t st,
                      const int* active);
void sho_umma_adjoint(ShoUmma& u, long long V, long long M, const float2* y, float2* x, long long nb, cudaStream_t st,
                      const int* active);
void sho_tc_forward(ShoTcScratch& s, const float* turn, long long V, long long M, const float2* x, float2* y,
                    long long nb, cudaStream_t st, const int* active);
void sho_tc_adjoint(ShoTcScratch& s, const float* turn, long long V, long long M, const float2* y, float2* x,
                    long long nb, cudaStream_t st, const int* active);

}  // namespace mmr
