// Learned preconditioner network: a bias-free 3x3 CNN on complex images
// (2 real channels), hidden width 32, ReLU (or identity: CNN_LINEAR) between
// layers, global skip.
//
//   s  = sqrt(mean |r|^2);  a0 = r / s  (complex = channels 0, 1)
//   a_{l+1} = relu(conv3x3(a_l, W_l))      l < L-1
//   z  = s * (conv3x3(a_{L-1}, W_{L-1}) + skip * a0)
//
// Activations are NHWC (channel fastest) over an image whose first index x
// is the fastest (the column-major MATLAB layout): a complex image is then
// exactly the 2-channel activation.  Weights are FP32 (theta layout
// [co][ci][ky][kx] per layer, then skip).  Hidden activations: BF16 in the
// SIMT path (training) unless the caller asks for FP32; FP16 in the
// tensor-core inference path (CNN_TENSOR).
#pragma once

#include <cuda_bf16.h>

#include "common.h"

namespace mmr {

constexpr int CNN_HIDDEN = 32;

struct CnnNet {
    int L = 0;                       // conv layers
    std::vector<int> ch;             // L + 1 channel counts
    long long nparam = 0;
    std::vector<long long> woff;     // offset of each layer in theta
    DevBuf theta, grad, adam_m, adam_v;
    DevBuf wpk, wpkT;                // packed forward / data-gradient weights (per layer, at woff)
    DevBuf wmma;                     // tensor-core weights (fp16), hidden layers
    DevBuf fold;                     // linear network folded into one filter: float4 [(2R+1)^2] (2x2 per tap)
    int fold_radius = 0;
    long long version = 0, packed_version = -1, folded_version = -1;
    long long adam_t = 0;
    // scratch
    DevBuf act, gbuf, gv, z, sumsq, lossacc, partial, dskip;
    size_t act_elems = 0;
    Staged st_in, st_out, st_tgt;
};

enum CnnFlags { CNN_FP32_ACT = 1, CNN_TENSOR = 2, CNN_LOSS_COS = 4, CNN_LINEAR = 8, CNN_FOLDED = 16 };

// z = net(r) for `batch` complex images of nx x ny on device memory.  `sumsq`
// (device, per image sum |r|^2) may be supplied by the caller (e.g. from a
// solver's residual norm); otherwise it is computed.  Scratch is sized on
// the first call of a shape, so make one eager call before stream capture.
void cnn_forward(CnnNet& n, const float2* r, float2* z, int nx, int ny, int batch, const double* sumsq, int flags,
                 cudaStream_t st);
// Re-packs the forward / data-gradient / tensor-core weights after a change.
void cnn_pack(CnnNet& n, cudaStream_t st);

}  // namespace mmr

struct mmr_cnn { mmr::CnnNet n; };
