// mmr_nufft_adjoint_noalloc: the nufftOp adjoint without any device allocation.
//
// Some callers cannot allocate device memory when they apply the operator: a
// MATLAB MEX function or plug-in that its host application hands a fixed
// device budget, or a real-time pipeline that must not risk an allocation
// failure or the implicit synchronisation of cudaMalloc/cudaFree in the
// middle of a scan.  This entry point runs the same kernels as
// mmr_nufft_apply(adjoint = 1) — spreading onto the oversampled grid, then
// the FFT passes with crop and deapodisation — but takes its grid scratch
// from a fixed-size array in device global memory that is part of the
// library image, instead of from buffers the plan allocates.
//
// The array is a file-scope __device__ variable, so every GPU that loads the
// library holds it (kNoallocScratchBytes) until the process exits.  All calls
// share it and it keeps the previous call's contents; every cell a call
// reads is written by that call first, so nothing has to start at zero.
// Calls whose GPU work overlaps (several host threads, or several streams)
// race on the array: serialise them on one stream.
#include <mutex>

#include "sense.cuh"

namespace mmr {

// 8 MiB: 1 Mi complex64 values.
constexpr size_t kNoallocScratchElems = (size_t)1 << 20;
constexpr size_t kNoallocScratchBytes = kNoallocScratchElems * sizeof(float2);

static __device__ __align__(256) float2 g_noalloc_scratch[kNoallocScratchElems];

// The host-side name of g_noalloc_scratch is only a stand-in: the kernels need
// its device address, looked up once per device (with that device current) by
// the first call on that device, which should therefore come before any
// stream capture.
static float2* noalloc_scratch_address() {
    static std::mutex mu;
    static float2* addr[64] = {nullptr};
    int dev = 0;
    MMR_CUDA(cudaGetDevice(&dev));
    MMR_REQUIRE(dev >= 0 && dev < 64, "device index out of range");
    std::lock_guard<std::mutex> g(mu);
    if (!addr[dev]) {
        float2* ptr = nullptr;
        MMR_CUDA(cudaGetSymbolAddress((void**)&ptr, g_noalloc_scratch));
        MMR_REQUIRE(ptr != nullptr, "scratch symbol has no device address");
        addr[dev] = ptr;
    }
    return addr[dev];
}

}  // namespace mmr

using namespace mmr;

extern "C" int mmr_nufft_adjoint_noalloc(mmr_nufft* plan, const void* y, void* x, int64_t nbatch, void* stream) {
    return guarded([&] {
        MMR_REQUIRE(plan && y && x, "NULL argument");
        MMR_REQUIRE(nbatch >= 1, "nbatch must be >= 1");
        NufftPlan& p = plan->p;
        MMR_REQUIRE(!p.is_toep, "the allocation-free adjoint is not available for a Toeplitz plan");
        MMR_REQUIRE(is_device_ptr(y) && is_device_ptr(x),
                    "the allocation-free adjoint takes device pointers only (host staging would allocate)");
        // scratch per batch column (the grid and the FFT intermediate both grow linearly with nbatch);
        // nbatch is bounded by the array before anything is multiplied by it
        const size_t grid_col = (size_t)p.Gtot;
        const size_t tmp_col = nufft_grid_to_img_scratch(p, 1);
        const size_t per_col = grid_col + tmp_col;
        if (per_col == 0 || (uint64_t)nbatch > kNoallocScratchElems / per_col)
            MMR_THROW(MMR_ERR_BADARG,
                      "the allocation-free adjoint needs %zu complex values of scratch per batch column (grid %zu + "
                      "FFT %zu) and its fixed array holds %zu (%zu MiB): %lld columns do not fit; use fewer batch "
                      "columns per call or mmr_nufft_apply",
                      per_col, grid_col, tmp_col, kNoallocScratchElems, kNoallocScratchBytes >> 20, (long long)nbatch);
        const size_t grid = grid_col * (size_t)nbatch;
        float2* scratch = noalloc_scratch_address();
        cudaStream_t st = as_stream(stream);
        const float2* dy = static_cast<const float2*>(y);
        float2* dx = static_cast<float2*>(x);
        nufft_spread(p, dy, scratch, nbatch, p.has_dcf ? p.d_dcf.as<float>() : nullptr, 0, st, nullptr);
        nufft_grid_to_img(p, scratch, nullptr, dx, nbatch, false, st, nullptr, scratch + grid);
    });
}
