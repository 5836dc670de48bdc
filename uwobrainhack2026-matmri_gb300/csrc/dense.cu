// Dense normal matrix of the high-order encoding and its direct solve.
//
// mrSampFuncMat (operators/mrSampFuncMat.m:22-47) forms, over the voxels of
// imMask (Vm of them),
//   S   = exp(1i * kbase(mask, :)).' / sqrt(Vm)                [M x Vm]
//   AtA = sum_c conj(r_c) r_c.' .* (S' * S)                    [Vm x Vm]
// with r_c the coil-c sensitivities on the mask.  Here the Gram S'S runs on the
// repository's own tcgen05 kernel (gram_umma.cu): the encoding rows are written
// once as FP16 hi / lo parts of cos and sin (sincospi of the plan's FP32 turns,
// sho.cu) and contracted with FP32 accumulation in TMEM.  On a device without
// tcgen05 the Gram is one complex GEMM in cuBLAS with the FP32 BF16x9 emulation
// instead.  The coil weighting runs as a tiled in-place epilogue.  The direct solve
// of the demo (demos/demo_denseMat.m:98-106: lam2 added to the diagonal, then
// AtA \ Aty) factors a copy with cuSOLVER: Cholesky, and LU when the shifted
// matrix is not numerically positive definite (MATLAB's backslash makes the
// same choice for Hermitian input).
#include <cublas_v2.h>
#include <cusolverDn.h>

#include <vector>

#include "sense.cuh"

namespace mmr {

#define MMR_CUBLAS(x)                                                                  \
    do {                                                                               \
        cublasStatus_t st_ = (x);                                                      \
        MMR_REQUIRE(st_ == CUBLAS_STATUS_SUCCESS, "cuBLAS error %d in %s", (int)st_, #x); \
    } while (0)
#define MMR_CUSOLVER(x)                                                                  \
    do {                                                                                 \
        cusolverStatus_t st_ = (x);                                                      \
        MMR_REQUIRE(st_ == CUSOLVER_STATUS_SUCCESS, "cuSOLVER error %d in %s", (int)st_, #x); \
    } while (0)

static cublasHandle_t blas_handle() {
    static cublasHandle_t h = nullptr;
    if (!h) {
        MMR_CUBLAS(cublasCreate(&h));
        MMR_CUBLAS(cublasSetMathMode(h, CUBLAS_FP32_EMULATED_BF16X9_MATH));
    }
    return h;
}

static cusolverDnHandle_t solver_handle() {
    static cusolverDnHandle_t h = nullptr;
    if (!h) MMR_CUSOLVER(cusolverDnCreate(&h));
    return h;
}

// AtA[v + n w] *= sum_c conj(maps[vox[v], c]) maps[vox[w], c]     (mrSampFuncMat.m:40-45)
constexpr int DT = 32;
constexpr int DC = 16;   // coils staged per pass
__global__ void __launch_bounds__(DT * 8) coil_hadamard_kernel(float2* __restrict__ A, long long n,
                                                              const float2* __restrict__ maps, long long V, int C,
                                                              const long long* __restrict__ vox) {
    __shared__ float2 rv[DC][DT], rw[DC][DT];
    const long long v0 = (long long)blockIdx.x * DT, w0 = (long long)blockIdx.y * DT;
    const int tx = threadIdx.x & (DT - 1), ty = threadIdx.x / DT;   // 32 x 8 threads, 4 rows each
    float2 q[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) q[r] = make_float2(0.f, 0.f);
    for (int c0 = 0; c0 < C; c0 += DC) {
        const int nc = min(DC, C - c0);
        __syncthreads();
        for (int i = threadIdx.x; i < DC * DT; i += blockDim.x) {
            const int c = i / DT, k = i % DT;
            float2 a = make_float2(0.f, 0.f), b = make_float2(0.f, 0.f);
            if (c < nc && v0 + k < n) a = maps[vox[v0 + k] + V * (c0 + c)];
            if (c < nc && w0 + k < n) b = maps[vox[w0 + k] + V * (c0 + c)];
            rv[c][k] = a;
            rw[c][k] = b;
        }
        __syncthreads();
        for (int c = 0; c < nc; ++c) {
            const float2 av = rv[c][tx];
#pragma unroll
            for (int r = 0; r < 4; ++r) q[r] = cadd(q[r], cmulc(rw[c][ty * 4 + r], av));   // conj(r_v) r_w
        }
    }
    const long long v = v0 + tx;
    if (v >= n) return;
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        const long long w = w0 + ty * 4 + r;
        if (w < n) A[v + n * w] = cmul(A[v + n * w], q[r]);
    }
}

__global__ void add_diag_kernel(float2* __restrict__ A, long long n, float lam) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) A[i + n * i].x += lam;
}

void dense_normal(ShoPlan& S, const RcvrPlan* R, const long long* vox_h, long long nvox, float2* AtA,
                  cudaStream_t st) {
    const long long V = sho_nvox(S), M = sho_nsamp(S);
    MMR_REQUIRE(nvox >= 1 && nvox <= V, "bad voxel count");
    for (long long j = 0; j < nvox; ++j) MMR_REQUIRE(vox_h[j] >= 0 && vox_h[j] < V, "voxel index out of range");
    MMR_REQUIRE(!R || R->Ntot == V, "rcvrOp and sampHighOrder image sizes differ");
    DevBuf d_vox, d_E;
    std::vector<long long> vh(vox_h, vox_h + nvox);
    d_vox.upload(vh);
    // S'S with S = E / sqrt(nvox): (1/nvox) E^H E     (mrSampFuncMat.m:37-38)
    if (gram_umma_supported()) {
        const long long rows = cdiv(nvox, 128) * 128, kpad = cdiv(M, 128) * 128;
        d_E.ensure((size_t)4 * rows * kpad * sizeof(__half));
        sho_gram_operands(S, d_vox.as<long long>(), nvox, rows, kpad, d_E.as<__half>(), st);
        MMR_REQUIRE(gram_umma(d_E.as<__half>(), nvox, rows, kpad, AtA, st), "tcgen05 Gram unavailable");
    } else {
        d_E.ensure((size_t)M * nvox * sizeof(float2));
        float2* E = d_E.as<float2>();
        sho_encoding_matrix(S, d_vox.as<long long>(), nvox, E, st);
        cublasHandle_t h = blas_handle();
        MMR_CUBLAS(cublasSetStream(h, st));
        const cuComplex alpha = make_cuComplex((float)(1.0 / (double)nvox), 0.f), beta = make_cuComplex(0.f, 0.f);
        MMR_CUBLAS(cublasCgemm(h, CUBLAS_OP_C, CUBLAS_OP_N, (int)nvox, (int)nvox, (int)M, &alpha,
                               reinterpret_cast<const cuComplex*>(E), (int)M, reinterpret_cast<const cuComplex*>(E),
                               (int)M, &beta, reinterpret_cast<cuComplex*>(AtA), (int)nvox));
    }
    if (R) {
        dim3 grid((unsigned)cdiv(nvox, DT), (unsigned)cdiv(nvox, DT));
        coil_hadamard_kernel<<<grid, DT * 8, 0, st>>>(AtA, nvox, R->d_maps.as<float2>(), V, (int)R->C,
                                                      d_vox.as<long long>());
        check_launch("coil_hadamard");
    }
    MMR_CUDA(cudaStreamSynchronize(st));   // the scratch buffers are freed on return
}

int dense_solve(const float2* AtA, long long n, double lam2, const float2* b, float2* x, cudaStream_t st) {
    cusolverDnHandle_t h = solver_handle();
    MMR_CUSOLVER(cusolverDnSetStream(h, st));
    DevBuf d_A, d_info, d_work, d_piv;
    const size_t bytes = (size_t)n * n * sizeof(float2);
    d_A.ensure(bytes);
    d_info.ensure(sizeof(int));
    cuComplex* A = d_A.as<cuComplex>();
    auto load = [&] {
        MMR_CUDA(cudaMemcpyAsync(A, AtA, bytes, cudaMemcpyDeviceToDevice, st));
        if (lam2 != 0) {
            add_diag_kernel<<<(unsigned)cdiv(n, 256), 256, 0, st>>>(reinterpret_cast<float2*>(A), n, (float)lam2);
            check_launch("add_diag");
        }
        MMR_CUDA(cudaMemcpyAsync(x, b, (size_t)n * sizeof(float2), cudaMemcpyDeviceToDevice, st));
    };
    load();
    int lwork = 0, info = 0;
    MMR_CUSOLVER(cusolverDnCpotrf_bufferSize(h, CUBLAS_FILL_MODE_LOWER, (int)n, A, (int)n, &lwork));
    d_work.ensure((size_t)std::max(lwork, 1) * sizeof(cuComplex));
    MMR_CUSOLVER(cusolverDnCpotrf(h, CUBLAS_FILL_MODE_LOWER, (int)n, A, (int)n, d_work.as<cuComplex>(), lwork,
                                  d_info.as<int>()));
    MMR_CUDA(cudaMemcpyAsync(&info, d_info.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    MMR_CUDA(cudaStreamSynchronize(st));
    MMR_REQUIRE(info >= 0, "potrf argument %d invalid", -info);
    if (info == 0) {
        MMR_CUSOLVER(cusolverDnCpotrs(h, CUBLAS_FILL_MODE_LOWER, (int)n, 1, A, (int)n,
                                      reinterpret_cast<cuComplex*>(x), (int)n, d_info.as<int>()));
        MMR_CUDA(cudaStreamSynchronize(st));
        return 1;   // Cholesky
    }
    load();       // not positive definite: LU with partial pivoting
    MMR_CUSOLVER(cusolverDnCgetrf_bufferSize(h, (int)n, (int)n, A, (int)n, &lwork));
    d_work.ensure((size_t)std::max(lwork, 1) * sizeof(cuComplex));
    d_piv.ensure((size_t)n * sizeof(int));
    MMR_CUSOLVER(cusolverDnCgetrf(h, (int)n, (int)n, A, (int)n, d_work.as<cuComplex>(), d_piv.as<int>(),
                                  d_info.as<int>()));
    MMR_CUDA(cudaMemcpyAsync(&info, d_info.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    MMR_CUDA(cudaStreamSynchronize(st));
    MMR_REQUIRE(info == 0, "the dense normal matrix is singular (getrf info %d)", info);
    MMR_CUSOLVER(cusolverDnCgetrs(h, CUBLAS_OP_N, (int)n, 1, A, (int)n, d_piv.as<int>(),
                                  reinterpret_cast<cuComplex*>(x), (int)n, d_info.as<int>()));
    MMR_CUDA(cudaStreamSynchronize(st));
    return 2;       // LU
}

}  // namespace mmr

using namespace mmr;

extern "C" int mmr_dense_normal(mmr_sho* S, mmr_rcvr* R, const int64_t* vox, int64_t nvox, void* AtA, void* stream) {
    return guarded([&] {
        MMR_REQUIRE(S && vox && AtA, "NULL argument");
        MMR_REQUIRE(is_device_ptr(AtA), "AtA must be device memory");
        static_assert(sizeof(long long) == sizeof(int64_t), "int64");
        dense_normal(*reinterpret_cast<ShoPlan*>(S), R ? &R->r : nullptr, reinterpret_cast<const long long*>(vox),
                     nvox, static_cast<float2*>(AtA), as_stream(stream));
    });
}

extern "C" int mmr_dense_solve(const void* AtA, int64_t n, double lam2, const void* b, void* x, int32_t* method,
                               void* stream) {
    return guarded([&] {
        MMR_REQUIRE(AtA && b && x && n >= 1, "bad argument");
        MMR_REQUIRE(is_device_ptr(AtA) && is_device_ptr(b) && is_device_ptr(x), "device pointers required");
        const int m = dense_solve(static_cast<const float2*>(AtA), n, lam2, static_cast<const float2*>(b),
                                  static_cast<float2*>(x), as_stream(stream));
        if (method) *method = m;
    });
}
