// @sampHighOrder approach 1: SVD + NUFFT interpolated encoding (sho_interp.cu).
#pragma once

#include <memory>

#include "nufft.cuh"

namespace mmr {

struct ShoInterp;

std::shared_ptr<ShoInterp> sho_interp_build(const mmr_sho_interp_desc& d);
long long sho_interp_nvox(const ShoInterp& s);
long long sho_interp_nsamp(const ShoInterp& s);
// x [V, nb] -> y [M, nb] and back (useInterpWorker, sampHighOrder.m:314-359).
void sho_interp_forward(ShoInterp& s, const float2* x, float2* y, long long nb, cudaStream_t st, const int* active);
void sho_interp_adjoint(ShoInterp& s, const float2* y, float2* x, long long nb, cudaStream_t st, const int* active);

}  // namespace mmr
