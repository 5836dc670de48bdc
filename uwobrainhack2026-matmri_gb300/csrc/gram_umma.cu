// The dense Gram (1 / n) E^H E of mrSampFuncMat (operators/mrSampFuncMat.m:37-38) on the
// 5th-generation tensor cores, without a library GEMM.
//
// E[m, v] = exp(i kbase[v, m]) over the n mask voxels and M samples.  With c = cos, s = sin of
// the phase:
//   Re G[v, w] = sum_m c_v c_w + s_v s_w        Im G[v, w] = sum_m c_v s_w - s_v c_w
// Each of c, s is split in fixed point into an FP16 high part hi = round(2^11 x) (an integer, exact)
// and a residual lo = 2^11 x - hi (|lo| <= 1/2), prepared once per voxel and sample
// (sho_gram_operands, sho.cu) as four K-major FP16 matrices [rows][kpad].  The products hi*hi,
// hi*lo, lo*hi (lo*lo is below FP32 resolution) accumulate in FP32 in TMEM: Re in one accumulator,
// the two Im terms in two more (subtracted in the epilogue), 12 tcgen05.mma (kind::f16, M 128,
// N 64, K 16) per 16 samples.
//
// FP32 accumulation in the tensor cores loses accuracy over long sums, so TMEM accumulates 128
// samples at a time: the MMA thread alternates between two accumulation sets and the epilogue warps
// add each finished set into FP32 register totals while the other fills.
//
// One CTA per 128 x 64 output tile (v rows, w columns) on or above the diagonal 128-blocks (tiles
// visited in super-blocks, so that the CTAs resident at a time share operand rows in L2).  Warp
// roles:
//   TMA warp    one thread loads, per stage of 32 samples, the four parts of the tile's 128 row
//               voxels (A) and 64 column voxels (B) with cp.async.bulk.tensor (64-byte swizzle)
//               into a 4-deep ring, 48 KB per stage;
//   MMA warp    one thread: per stage one bounded wait and one tcgen05 fence, 24 MMAs (M 128,
//               N 64), one commit that frees the slot; per 4 stages it waits for a free
//               accumulation set and commits the finished one to the epilogue; it owns the TMEM
//               allocation (512 columns: two sets of Re, c_v s_w and s_v c_w, 64 columns each);
//   8 epilogue warps: two per 32-lane TMEM quarter, each 32 of the 64 columns; per set they add
//               Re and the two Im terms into registers; at the end they scale by 2^-22 / n and
//               write G[v, w] and, above the diagonal blocks, the mirrored conj(G) at [w, v].
// Every wait is bounded; a wait that runs out sets the device error word and all roles drain and
// return.
#include <algorithm>
#include <cmath>
#include <vector>

#include <cuda.h>
#include <cudaTypedefs.h>

#include "sense.cuh"
#include "umma.cuh"

namespace mmr {

namespace gram {

constexpr int TV = 128;                     // tile rows (v, TMEM lanes)
constexpr int TW = 64;                      // tile columns (w, MMA N)
constexpr int GK = 32;                      // samples per stage (64-byte rows)
constexpr int CH = 4;                       // stages per accumulation set (128 samples)
constexpr int NSTG = 4;                     // stage ring depth
constexpr int SUBA = TV * GK * 2;           // 8 KB: one part of the A side of a stage
constexpr int SUBB = TW * GK * 2;           // 4 KB: one part of the B side
constexpr int STAGE = 4 * SUBA + 4 * SUBB;  // A parts 0..3, then B parts 0..3
constexpr int SET_COLS = 256;               // TMEM columns per accumulation set (192 used)
constexpr int SUPER = 12;                   // super-block side, in 128-row blocks
constexpr int NEPI = 8;                     // epilogue warps
constexpr int NTHREADS = (2 + NEPI) * 32;   // TMA, MMA, epilogue warps
// barriers: full[NSTG] empty[NSTG] setfull[2] setempty[2] done, then the TMEM address slot
constexpr int NBARS = 2 * NSTG + 5;
constexpr int BAR_OFF = NSTG * STAGE;
constexpr int SMEM_BYTES = BAR_OFF + NBARS * 8 + 16 + 1024;
static_assert(SMEM_BYTES <= 232448, "shared memory");

}  // namespace gram

__global__ void __launch_bounds__(gram::NTHREADS, 1)
    gram_umma_kernel(const __grid_constant__ CUtensorMap map, const int2* __restrict__ tiles, long long n,
                     long long rows, int nst, float scale, float2* __restrict__ A, int* err) {
    using namespace gram;
    using namespace umma;
    extern __shared__ uint8_t smem_raw[];
    uint8_t* sm = smem_raw + ((1024u - (su32(smem_raw) & 1023u)) & 1023u);
    const uint32_t s0 = su32(sm);
    const uint32_t bars = s0 + BAR_OFF;
    auto full = [&](int i) { return bars + 8u * i; };
    auto empty = [&](int i) { return bars + 8u * (NSTG + i); };
    auto setfull = [&](int i) { return bars + 8u * (2 * NSTG + i); };
    auto setempty = [&](int i) { return bars + 8u * (2 * NSTG + 2 + i); };
    const uint32_t done = bars + 8u * (2 * NSTG + 4);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(sm + BAR_OFF + NBARS * 8);
    __shared__ volatile int abort_flag;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int2 tile = tiles[blockIdx.x];
    const int bi = tile.x, bj = tile.y;     // row block of 128 (v), column block of 64 (w)
    const int nsets = nst / CH;
    if (tid == 0) {
        abort_flag = 0;
        for (int i = 0; i < NSTG; ++i) {
            bar_init(full(i), 1);
            bar_init(empty(i), 1);
        }
        for (int i = 0; i < 2; ++i) {
            bar_init(setfull(i), 1);
            bar_init(setempty(i), NEPI);   // one arrival per epilogue warp
        }
        bar_init(done, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(tslot)), "r"(512));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = *tslot;

    if (warp == 0) {
        // ------------------------------------------------------------------ TMA --
        if (lane == 0) {
            int s = 0;
            for (; s < nst && !abort_flag; ++s) {
                const int slot = s % NSTG;
                if (s >= NSTG && !bar_wait(empty(slot), (uint32_t)(((s / NSTG) + 1) & 1), &abort_flag, err)) break;
                bar_expect(full(slot), (uint32_t)STAGE);
                const uint32_t dst = s0 + slot * STAGE;
                // boxes of 64 rows: A parts in two halves, B parts whole
#pragma unroll
                for (int q = 0; q < 12; ++q) {
                    const int part = q < 8 ? (q >> 1) : q - 8;
                    const long long r0 = q < 8 ? (long long)bi * TV + (q & 1) * 64 : (long long)bj * TW;
                    const uint32_t d = q < 8 ? dst + part * SUBA + (q & 1) * (SUBA / 2) : dst + 4 * SUBA + part * SUBB;
                    asm volatile(
                        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, "
                        "{%2, %3}], [%4];" ::"r"(d),
                        "l"(&map), "r"(s * GK), "r"((int)(part * rows + r0)), "r"(full(slot))
                        : "memory");
                }
            }
            if (abort_flag) {   // the loads in flight land before the CTA exits
                for (int k = std::max(0, s - NSTG); k < s; ++k)
                    bar_wait(full(k % NSTG), (uint32_t)((k / NSTG) & 1), &abort_flag, err, true);
            }
        }
        __syncwarp();
    } else if (warp == 1) {
        // ------------------------------------------------------------------ MMA --
        if (lane == 0) {
            constexpr uint32_t ID = idesc(TV, TW);
            const uint64_t d0 = sdesc_sw64(s0);
            const uint32_t dlo = (uint32_t)d0, dhi = (uint32_t)(d0 >> 32);
            bool ok = true;
            for (int c = 0; c < nsets && ok; ++c) {
                const int set = c & 1;
                if (c >= 2 && !bar_wait(setempty(set), (uint32_t)(((c >> 1) + 1) & 1), &abort_flag, err)) {
                    ok = false;
                    break;
                }
                const uint32_t dre = tmem + set * SET_COLS, di1 = dre + 64, di2 = dre + 128;
                for (int ss = 0; ss < CH; ++ss) {
                    const int s = c * CH + ss, slot = s % NSTG;
                    if (!bar_wait(full(slot), (uint32_t)((s / NSTG) & 1), &abort_flag, err)) {
                        ok = false;
                        break;
                    }
                    fence_after();
                    const uint32_t base = dlo + (uint32_t)(slot * (STAGE >> 4));
#pragma unroll
                    for (int h = 0; h < GK / 16; ++h) {
                        // parts: 0 cos hi, 1 cos lo, 2 sin hi, 3 sin lo; A (rows v), B (columns w)
                        const uint32_t k = (uint32_t)h * (32 >> 4);
                        auto a = [&](int q) { return base + (uint32_t)(q * (SUBA >> 4)) + k; };
                        auto b = [&](int q) { return base + (uint32_t)((4 * SUBA + q * SUBB) >> 4) + k; };
                        const uint32_t first = (ss == 0 && h == 0) ? 0u : 1u;
                        mma2(dre, a(0), dhi, b(0), dhi, ID, first);      // c_v c_w
                        mma2(dre, a(0), dhi, b(1), dhi, ID, 1u);
                        mma2(dre, a(1), dhi, b(0), dhi, ID, 1u);
                        mma2(dre, a(2), dhi, b(2), dhi, ID, 1u);         // s_v s_w
                        mma2(dre, a(2), dhi, b(3), dhi, ID, 1u);
                        mma2(dre, a(3), dhi, b(2), dhi, ID, 1u);
                        mma2(di1, a(0), dhi, b(2), dhi, ID, first);      // c_v s_w
                        mma2(di1, a(0), dhi, b(3), dhi, ID, 1u);
                        mma2(di1, a(1), dhi, b(2), dhi, ID, 1u);
                        mma2(di2, a(2), dhi, b(0), dhi, ID, first);      // s_v c_w
                        mma2(di2, a(2), dhi, b(1), dhi, ID, 1u);
                        mma2(di2, a(3), dhi, b(0), dhi, ID, 1u);
                    }
                    commit(empty(slot));
                }
                if (ok) commit(setfull(set));
            }
            // every MMA this thread issued completes before TMEM is freed
            commit(done);
            bar_wait(done, 0u, &abort_flag, err, true);
        }
        __syncwarp();
    } else {
        // ------------------------------------------------------------- epilogue --
        const int quarter = warp & 3;               // TMEM lanes 32 quarter .. 32 quarter + 31
        const int half = (warp - 2) >> 2;           // columns 32 half .. 32 half + 31
        const uint32_t tq = tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(half * 32);
        float re[32], i1[32], i2[32];
#pragma unroll
        for (int k = 0; k < 32; ++k) re[k] = i1[k] = i2[k] = 0.f;
        bool ok = true;
        for (int c = 0; c < nsets; ++c) {
            const int set = c & 1;
            int got = 1;
            if (lane == 0) got = bar_wait(setfull(set), (uint32_t)((c >> 1) & 1), &abort_flag, err);
            __syncwarp();
            if (!__shfl_sync(0xffffffffu, got, 0)) {
                ok = false;
                break;
            }
            fence_after();
            const uint32_t ts = tq + set * SET_COLS;
#pragma unroll
            for (int cb = 0; cb < 32; cb += 16) {
                float a[16], b[16], d[16];
                tmem_ld16x2(ts + cb, ts + 64 + cb, a, b);
                tmem_ld16(ts + 128 + cb, d);
#pragma unroll
                for (int k = 0; k < 16; ++k) {
                    re[cb + k] += a[k];
                    i1[cb + k] += b[k];
                    i2[cb + k] += d[k];
                }
            }
            fence_before();
            __syncwarp();
            if (lane == 0) bar_arrive(setempty(set));
        }
        if (ok && !abort_flag) {
            const long long v = (long long)bi * TV + quarter * 32 + lane;
            const long long w0 = (long long)bj * TW + half * 32;
            const bool mirror = (long long)bj * TW >= (long long)(bi + 1) * TV;   // tile above the diagonal block
            if (v < n) {
#pragma unroll
                for (int k = 0; k < 32; ++k) {
                    const long long w = w0 + k;
                    if (w < n) {
                        const float2 g = make_float2(re[k] * scale, (i1[k] - i2[k]) * scale);
                        A[v + n * w] = g;                                 // column w: rows v coalesced
                        if (mirror) A[w + n * v] = make_float2(g.x, -g.y);   // mirrored: row v's run of w
                    }
                }
            }
        }
    }
    fence_before();
    __syncthreads();
    if (warp == 1) {
        fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512));
    }
}

static PFN_cuTensorMapEncodeTiled_v12000 gram_encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        cudaDriverEntryPointQueryResult q;
        void* f = nullptr;
        MMR_CUDA(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q));
        MMR_REQUIRE(q == cudaDriverEntryPointSuccess && f, "cuTensorMapEncodeTiled unavailable");
        fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
    }
    return fn;
}

bool gram_umma_supported() {
    int major = 0, dev = 0;
    MMR_CUDA(cudaGetDevice(&dev));
    MMR_CUDA(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev));
    return major == 10;
}

bool gram_umma(const __half* op, long long n, long long rows, long long kpad, float2* AtA, cudaStream_t st) {
    using namespace gram;
    if (!gram_umma_supported()) return false;
    MMR_REQUIRE(rows % TV == 0 && rows >= n && kpad % (GK * CH) == 0 && kpad / GK <= (1LL << 30),
                "Gram operands: rows a multiple of 128, samples of 128");
    MMR_REQUIRE(4 * rows <= (1LL << 31) && kpad <= (1LL << 31), "Gram operands too large for the tensor map");
    CUtensorMap map;
    const cuuint64_t dims[2] = {(cuuint64_t)kpad, (cuuint64_t)(4 * rows)};
    const cuuint64_t strides[1] = {(cuuint64_t)kpad * 2};
    const cuuint32_t box[2] = {(cuuint32_t)GK, (cuuint32_t)TW};
    const cuuint32_t estr[2] = {1, 1};
    const CUresult r = gram_encode_fn()(&map, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, const_cast<__half*>(op), dims,
                                        strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B,
                                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    MMR_REQUIRE(r == CUDA_SUCCESS, "cuTensorMapEncodeTiled (Gram operands) failed (%d)", (int)r);
    // the 128 x 64 tiles on or above the diagonal 128-blocks, in super-blocks of SUPER x SUPER
    // 128-blocks
    const int nb = (int)cdiv(n, TV), nw = (int)cdiv(n, TW);
    std::vector<int2> tl;
    tl.reserve((size_t)nb * (nb + 1));
    for (int I = 0; I < nb; I += SUPER)
        for (int J = I; J < nb; J += SUPER)
            for (int i = I; i < std::min(I + SUPER, nb); ++i)
                for (int j = 2 * std::max(J, i); j < std::min(2 * (J + SUPER), nw); ++j) tl.push_back(make_int2(i, j));
    DevBuf d_tiles;
    d_tiles.upload(tl);
    static bool attr = false;
    if (!attr) {
        MMR_CUDA(cudaFuncSetAttribute(gram_umma_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES));
        attr = true;
    }
    // 2^-11 per operand, 1 / n for S = E / sqrt(n)
    const float scale = (float)(1.0 / ((double)n * 4194304.0));
    gram_umma_kernel<<<(unsigned)tl.size(), NTHREADS, SMEM_BYTES, st>>>(map, d_tiles.as<int2>(), n, rows,
                                                                        (int)(kpad / GK), scale, AtA,
                                                                        device_error_ptr());
    check_launch("gram_umma");
    MMR_CUDA(cudaStreamSynchronize(st));   // the tile list is freed on return
    return true;
}

}  // namespace mmr
