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
void sho_tc_forward(ShoTcScratch& s, const float* turn, long long V, long long M, const float2* x, float2* y,
                    long long nb, cudaStream_t st, const int* active);
void sho_tc_adjoint(ShoTcScratch& s, const float* turn, long long V, long long M, const float2* y, float2* x,
                    long long nb, cudaStream_t st, const int* active);

}  // namespace mmr
