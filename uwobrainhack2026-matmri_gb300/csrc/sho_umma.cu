// sampHighOrder encoding on the 5th-generation tensor cores (tcgen05.mma, TMEM
// accumulators, TMA-fed phase tiles).
//
// Forward  y[m, c] = sum_v exp(+i 2 pi t[v, m]) x[v, c] / sqrt(V)   (sampHighOrder.m:376, 387)
// adjoint  x[v, c] = sum_m exp(-i 2 pi t[v, m]) y[m, c] / sqrt(V)   (sampHighOrder.m:371, 387)
// with t the plan's FP32 phase table in turns ([V][M], reduced to [-1/2, 1/2)).
//
// As real GEMMs, per output row r (sample for the forward, voxel for the
// adjoint) and input i:  D[r, n] = sum_i cos(2 pi t) Bc[n, i] + sin(2 pi t) Bs[n, i]
// with N0 = 2 cg columns (cg coils: real parts, then imaginary parts):
//   forward  Bc = [ x_r ; x_i ]   Bs = [ -x_i ; x_r ]
//   adjoint  Bc = [ y_r ; y_i ]   Bs = [  y_i ; -y_r ]
// Precision: cos and sin are split in fixed point, hi = round(2^11 v) (an
// integer, exact in FP16) and lo = 2^11 (2^11 v - hi); the column-normalised
// coil data in floating point, hi = FP16(b), lo = FP16(2^11 (b - hi)).  TMEM
// accumulators take hi*hi (main) and hi*lo, lo*hi (two corrections) in FP32,
// combined as main + (corr1 + corr2) / 2^11 (about 22-bit operands).  Every
// accumulation in TMEM covers 64 inputs; the epilogue adds the accumulation
// sets in FP32 registers and the split-K partials are summed in FP64 in a
// fixed order by a second kernel.
//
// One persistent CTA per SM walks (row tile, K split) work items; warp roles
// (16 producer warps for up to 16 coils per pass, 8 for 32):
//   producers   per stage (32 inputs x 128 rows) read the phase tile from
//               shared memory, evaluate sincos on the SFU, split to FP16 hi/lo
//               and store the A operand in the no-swizzle K-major UMMA layout
//               (a 2-deep ring);
//   TMA warp    cp.async.bulk.tensor of the phase tiles into an 8-deep ring
//               (6 for 32-coil groups), each tile prefetched into L2 twelve
//               stages ahead;
//   B loader    one bulk copy per stage of the pre-split coil data into a
//               4-deep ring that the MMA thread releases;
//   MMA warp    one thread issues tcgen05.mma (kind::f16, M 128, K 16),
//               commits stage completion to the operand ring's mbarriers and
//               chunk completion to its own, and after seeing a chunk complete
//               hands its accumulation set to the epilogue; the warp owns the
//               TMEM allocation (all 512 columns);
//   4 epilogue warps: every two stages (64 inputs) the MMA warp moves on to the
//               next accumulation set of a TMEM ring, and the epilogue warps
//               (each its 32-lane quarter) read the finished set with
//               tcgen05.ld and add it to FP32 register totals, which they store
//               as the item's partial sums at its end.
// Generic stores into an A slot that MMAs read through the async proxy follow
// a fence.proxy.async after the slot's release; without it, adjoint rows came
// out wrong on a GB300.
// The B operand stacks hi and lo rows, so per 16 inputs and per cos / sin part
// two MMAs cover the three products: A_hi x [B_hi; B_lo] (N = 2 N0: main and
// the first correction) and A_lo x B_hi (N = N0: the second correction).  A
// set is [main | corr1 | corr2 | unused], 4 N0 columns, so that every MMA's
// accumulator starts at a column aligned to its own width and no two MMAs of a
// set write overlapping columns from different start columns.
// Every mbarrier wait is bounded; a wait that runs out sets the device error
// word and makes all roles stop, drain what they issued, free TMEM and return.
#include <algorithm>
#include <cmath>

#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_fp16.h>

#include "nufft.cuh"
#include "sho_tc.cuh"

namespace mmr {

namespace umma {

constexpr int BM = 128;                      // output rows per work item (TMEM lanes)
constexpr int KS = 32;                       // inputs per pipeline stage
constexpr int SA = 2;                        // A operand ring depth
constexpr int SB = 4;                        // B operand ring depth
constexpr int PS = 2;                        // stages per TMEM accumulation set (64 inputs)
constexpr int PF = 12;                       // L2 prefetch distance of the phase tiles, in stages
constexpr int TURN_BYTES = BM * KS * 4;      // 16 KB
constexpr int A_SUB_BYTES = BM * KS * 2;     // 8 KB per sub-tile (cos hi, cos lo, sin hi, sin lo)
constexpr int A_BYTES = 4 * A_SUB_BYTES;
constexpr int TMEM_COLS = 512;
constexpr int MAX_SETS = 16;
constexpr float LO_SCALE = 2048.f;
constexpr float ROUND_MAGIC = 12582912.f;    // 1.5 * 2^23: x + m - m rounds |x| < 2^22 to an integer
constexpr uint32_t WAIT_POLLS = 1u << 22;

// warps 0 .. NPW-1 producers, NPW the TMA warp (phase tiles), NPW+1 the MMA warp, NPW+2 the B loader,
// NPW+3 .. NPW+6 the epilogue
__host__ __device__ constexpr int nprod_warps(int N0) { return N0 <= 32 ? 16 : 8; }
__host__ __device__ constexpr int nthreads(int N0) { return (nprod_warps(N0) + 7) * 32; }
// phase-tile ring depth: as many 16 KB tiles in flight as shared memory leaves (HBM latency x
// bandwidth per SM is about 90 KB)
__host__ __device__ constexpr int n_turn_stages(int N0) { return N0 <= 32 ? 8 : 6; }
// B operand of one stage: a cos and a sin sub-tile, each [KS / 8][2 N0 rows: hi then lo][8] halves
__host__ __device__ constexpr int b_sub_bytes(int N0) { return 2 * N0 * KS * 2; }
__host__ __device__ constexpr int b_bytes(int N0) { return 2 * b_sub_bytes(N0); }
// TMEM accumulation sets: SET_W(N0) columns each, main at 0, corr1 at N0, corr2 at 2 N0
__host__ __device__ constexpr int set_w(int N0) { return 4 * N0; }
__host__ __device__ constexpr int nsets(int N0) {
    return TMEM_COLS / set_w(N0) < MAX_SETS ? TMEM_COLS / set_w(N0) : MAX_SETS;
}

// offsets in the 1024-aligned dynamic shared memory: phase tiles, A stages, B stages, barriers
__host__ __device__ constexpr int off_a(int N0) { return n_turn_stages(N0) * TURN_BYTES; }
__host__ __device__ constexpr int off_b(int N0) { return off_a(N0) + SA * A_BYTES; }
__host__ __device__ constexpr int bar_off(int N0) { return off_b(N0) + SB * b_bytes(N0); }
// barriers: tfull[ST] tempty[ST] afull[SA] aempty[SA] bfull[SB] bempty[SB] setfull[MAX_SETS]
// setempty[MAX_SETS] drain chunk[2], then the TMEM address slot
constexpr int MAX_ST = 8;
__host__ __device__ constexpr int nbars() { return 2 * MAX_ST + 2 * SA + 2 * SB + 2 * MAX_SETS + 3; }
__host__ __device__ constexpr int smem_bytes(int N0) { return bar_off(N0) + nbars() * 8 + 16 + 1024; }

__device__ __forceinline__ uint32_t su32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void bar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void bar_arrive(uint32_t bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void bar_expect(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
// Bounded wait for the completion of the phase with the given parity; on timeout
// flags `err` and the CTA's abort word and returns false.  A wait that is not a
// drain also gives up early once another role has aborted.
__device__ __forceinline__ bool bar_wait(uint32_t bar, uint32_t parity, volatile int* abort_flag, int* err,
                                         bool drain = false) {
    for (uint32_t it = 0; it < WAIT_POLLS; ++it) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done)
            : "r"(bar), "r"(parity)
            : "memory");
        if (done) return true;
        if (!drain && (it & 1023u) == 1023u && *abort_flag) return false;
    }
    *abort_flag = 1;
    atomicExch(err, 1);
    return false;
}

// Shared-memory matrix descriptor: no swizzle, K-major; lbo = byte distance of
// the core matrices adjacent along K, sbo = of those adjacent along M / N.
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | ((uint64_t)1 << 46);
}
// Instruction descriptor, kind::f16: D F32 (bits 4-5 = 1), A and B F16, both K-major,
// N >> 3 at bit 17, M >> 4 at bit 24.
__host__ __device__ constexpr uint32_t idesc(int M, int N) {
    return (1u << 4) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma(uint32_t d, uint64_t a, uint64_t b, uint32_t id, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d),
        "l"(a), "l"(b), "r"(id), "r"(acc));
}
__device__ __forceinline__ void commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
                 : "memory");
}
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }

// 16 consecutive TMEM columns at one or two addresses, this warp's 32 lanes (one row per thread).
// The loads and their wait are one asm statement: tcgen05.ld fills its destination registers
// asynchronously, so no use of them may be scheduled before tcgen05.wait::ld.
__device__ __forceinline__ void tmem_ld16x2(uint32_t ta, uint32_t tb, float (&a)[16], float (&b)[16]) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%32];\n\t"
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, "
        "[%33];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(ta), "r"(tb)
        : "memory");
#pragma unroll
    for (int j = 0; j < 16; ++j) {
        a[j] = __uint_as_float(r[j]);
        b[j] = __uint_as_float(r[16 + j]);
    }
}
__device__ __forceinline__ void tmem_ld16(uint32_t ta, float (&a)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(ta)
        : "memory");
#pragma unroll
    for (int j = 0; j < 16; ++j) a[j] = __uint_as_float(r[j]);
}

__device__ __forceinline__ uint32_t h2bits(__half2 h) { return *reinterpret_cast<uint32_t*>(&h); }

// Work item w -> row tile and the stage range of its K split (balanced integer split).
__device__ __forceinline__ void item_range(long long w, int nsplit, long long Q, long long& rt, long long& sp,
                                           long long& qa, long long& qb) {
    rt = w / nsplit;
    sp = w - rt * nsplit;
    qa = sp * Q / nsplit;
    qb = (sp + 1) * Q / nsplit;
}

}  // namespace umma

// partial[sp][row][N0] for every work item.  `turn_map` tiles the [V][M] phase table: forward
// box {128 samples, 32 voxels} (no swizzle), adjoint box {32 samples, 128 voxels} (128-byte
// swizzle).  bglob: the B operand in per-stage blocks laid out as in shared memory.
template <bool ADJ, int N0>
__global__ void __launch_bounds__(umma::nthreads(N0), 1)
    sho_umma_kernel(const __grid_constant__ CUtensorMap turn_map, const __half* __restrict__ bglob,
                    float* __restrict__ partial, long long R, long long Q, int nsplit, long long nitems, int* err,
                    const int* active) {
    using namespace umma;
    constexpr int NS = nsets(N0);
    constexpr int SW = set_w(N0);
    constexpr int NPW = nprod_warps(N0), NPROD = NPW * 32;
    constexpr int WARP_TMA = NPW, WARP_MMA = NPW + 1, WARP_B = NPW + 2;
    constexpr int ST = n_turn_stages(N0);
    constexpr int OFF_A = off_a(N0), OFF_B = off_b(N0);
    constexpr int CPT = (BM * KS / 8) / NPROD;     // 8-input chunks per producer thread and stage
    if (active && *active) return;
    extern __shared__ uint8_t smem_raw[];
    uint8_t* sm = smem_raw + ((1024u - (su32(smem_raw) & 1023u)) & 1023u);
    const uint32_t s0 = su32(sm);
    const uint32_t bars = s0 + bar_off(N0);
    auto tfull = [&](int i) { return bars + 8u * i; };
    auto tempty = [&](int i) { return bars + 8u * (MAX_ST + i); };
    auto afull = [&](int i) { return bars + 8u * (2 * MAX_ST + i); };
    auto aempty = [&](int i) { return bars + 8u * (2 * MAX_ST + SA + i); };
    auto bfull = [&](int i) { return bars + 8u * (2 * MAX_ST + 2 * SA + i); };
    auto bempty = [&](int i) { return bars + 8u * (2 * MAX_ST + 2 * SA + SB + i); };
    constexpr int SET0 = 2 * MAX_ST + 2 * SA + 2 * SB;
    auto setfull = [&](int i) { return bars + 8u * (SET0 + i); };
    auto setempty = [&](int i) { return bars + 8u * (SET0 + MAX_SETS + i); };
    const uint32_t drain = bars + 8u * (SET0 + 2 * MAX_SETS);
    auto chunkbar = [&](int i) { return bars + 8u * (SET0 + 2 * MAX_SETS + 1 + i); };
    uint32_t* tslot = reinterpret_cast<uint32_t*>(sm + bar_off(N0) + nbars() * 8);
    __shared__ volatile int abort_flag;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (tid == 0) {
        abort_flag = 0;
        for (int i = 0; i < ST; ++i) {
            bar_init(tfull(i), 1);
            bar_init(tempty(i), NPROD);
        }
        for (int i = 0; i < SA; ++i) {
            bar_init(afull(i), NPROD);
            bar_init(aempty(i), 1);
        }
        for (int i = 0; i < SB; ++i) {
            bar_init(bfull(i), 1);
            bar_init(bempty(i), 1);
        }
        for (int i = 0; i < NS; ++i) {
            bar_init(setfull(i), 1);
            bar_init(setempty(i), 128);
        }
        bar_init(drain, 1);
        bar_init(chunkbar(0), 1);
        bar_init(chunkbar(1), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == WARP_MMA) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(tslot)),
                     "r"(TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = *tslot;

    if (warp < NPW) {
        // ------------------------------------------------------------ producers --
        // A = cos / sin of the phase, each split into a high part hi = round(2^11 v) (an integer of at
        // most 2048, exact in FP16) and a low part lo = 2^11 (2^11 v - hi) (|lo| <= 1024): the MMAs
        // then give 2^11 main and 2^22 corr, which the reduce kernel scales back
        const int r = tid & (BM - 1);
        const int kq = tid >> 7;          // chunks kq + j NPROD / 128 of each stage (8 inputs each)
        long long g = 0;
        for (long long w = blockIdx.x; w < nitems && !abort_flag; w += gridDim.x) {
            long long rt, sp, qa, qb;
            item_range(w, nsplit, Q, rt, sp, qa, qb);
            for (long long q = qa; q < qb; ++q, ++g) {
                const int ts = (int)(g % ST), as = (int)(g % SA);
                if (!bar_wait(tfull(ts), (uint32_t)((g / ST) & 1), &abort_flag, err)) break;
                if (g >= SA && !bar_wait(aempty(as), (uint32_t)(((g / SA) + 1) & 1), &abort_flag, err)) break;
                // the MMAs of this slot's previous use read it through the async proxy: order them
                // before this thread's generic stores to it
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                const float* tile = reinterpret_cast<const float*>(sm + ts * TURN_BYTES);
                float t[CPT][8];
#pragma unroll
                for (int j = 0; j < CPT; ++j) {
                    const int kc = kq + j * (NPROD / BM);
                    if (ADJ) {
                        // [128 voxels][32 samples], 128-byte swizzle: 16-byte chunk c of row r at c ^ (r & 7)
                        const float4 lo4 = *reinterpret_cast<const float4*>(
                            reinterpret_cast<const uint8_t*>(tile) + r * 128 + (((2 * kc) ^ (r & 7)) << 4));
                        const float4 hi4 = *reinterpret_cast<const float4*>(
                            reinterpret_cast<const uint8_t*>(tile) + r * 128 + (((2 * kc + 1) ^ (r & 7)) << 4));
                        t[j][0] = lo4.x; t[j][1] = lo4.y; t[j][2] = lo4.z; t[j][3] = lo4.w;
                        t[j][4] = hi4.x; t[j][5] = hi4.y; t[j][6] = hi4.z; t[j][7] = hi4.w;
                    } else {
                        // [32 voxels][128 samples]
#pragma unroll
                        for (int e = 0; e < 8; ++e) t[j][e] = tile[(kc * 8 + e) * BM + r];
                    }
                }
                bar_arrive(tempty(ts));
                uint8_t* a = sm + OFF_A + as * A_BYTES;
#pragma unroll
                for (int j = 0; j < CPT; ++j) {
                    const int kc = kq + j * (NPROD / BM);
                    uint32_t chi[4], clo[4], shi[4], slo[4];
#pragma unroll
                    for (int e = 0; e < 4; ++e) {
                        float chv[2], shv[2], clv[2], slv[2];
#pragma unroll
                        for (int u = 0; u < 2; ++u) {
                            float sv, cv;
                            __sincosf(6.28318530717958647692f * t[j][2 * e + u], &sv, &cv);
                            const float cs = __fmul_rn(cv, LO_SCALE), ss = __fmul_rn(sv, LO_SCALE);
                            chv[u] = __fsub_rn(__fadd_rn(cs, ROUND_MAGIC), ROUND_MAGIC);
                            shv[u] = __fsub_rn(__fadd_rn(ss, ROUND_MAGIC), ROUND_MAGIC);
                            clv[u] = __fmul_rn(__fsub_rn(cs, chv[u]), LO_SCALE);
                            slv[u] = __fmul_rn(__fsub_rn(ss, shv[u]), LO_SCALE);
                        }
                        chi[e] = h2bits(__floats2half2_rn(chv[0], chv[1]));
                        shi[e] = h2bits(__floats2half2_rn(shv[0], shv[1]));
                        clo[e] = h2bits(__floats2half2_rn(clv[0], clv[1]));
                        slo[e] = h2bits(__floats2half2_rn(slv[0], slv[1]));
                    }
                    const int off = kc * (BM * 16) + r * 16;   // core matrices: 8 rows x 16 B, rows 16 B apart
                    *reinterpret_cast<uint4*>(a + 0 * A_SUB_BYTES + off) = make_uint4(chi[0], chi[1], chi[2], chi[3]);
                    *reinterpret_cast<uint4*>(a + 1 * A_SUB_BYTES + off) = make_uint4(clo[0], clo[1], clo[2], clo[3]);
                    *reinterpret_cast<uint4*>(a + 2 * A_SUB_BYTES + off) = make_uint4(shi[0], shi[1], shi[2], shi[3]);
                    *reinterpret_cast<uint4*>(a + 3 * A_SUB_BYTES + off) = make_uint4(slo[0], slo[1], slo[2], slo[3]);
                }
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                bar_arrive(afull(as));
            }
        }
    } else if (warp == WARP_B) {
        // -------------------------------------------------------------- B loader --
        // the stage's B operand (coil data, FP16 hi / lo, both parts) by one bulk copy into a ring
        // that the MMA thread releases stage by stage
        long long g = 0;
        if (lane == 0) {
            for (long long w = blockIdx.x; w < nitems && !abort_flag; w += gridDim.x) {
                long long rt, sp, qa, qb;
                item_range(w, nsplit, Q, rt, sp, qa, qb);
                bool ok = true;
                for (long long q = qa; q < qb; ++q, ++g) {
                    const int bs = (int)(g % SB);
                    if (g >= SB && !bar_wait(bempty(bs), (uint32_t)(((g / SB) + 1) & 1), &abort_flag, err)) {
                        ok = false;
                        break;
                    }
                    bar_expect(bfull(bs), (uint32_t)b_bytes(N0));
                    asm volatile(
                        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                            s0 + OFF_B + bs * b_bytes(N0)),
                        "l"(bglob + (size_t)q * (b_bytes(N0) / 2)), "r"((uint32_t)b_bytes(N0)), "r"(bfull(bs))
                        : "memory");
                }
                if (!ok) break;
            }
            if (abort_flag) {   // the copies in flight land before the CTA exits
                for (long long k = std::max<long long>(0, g - SB); k < g; ++k)
                    bar_wait(bfull((int)(k % SB)), (uint32_t)((k / SB) & 1), &abort_flag, err, true);
            }
        }
        __syncwarp();
    } else if (warp == WARP_TMA) {
        // ------------------------------------------------------------------ TMA --
        // Each phase tile is also prefetched into L2 PF stages before its load, so that the
        // ring's loads see L2 rather than HBM latency.
        long long g = 0;
        if (lane == 0) {
            long long w2 = blockIdx.x, rt2 = 0, sp2 = 0, qa2 = 0, qb2 = 0, q2 = 0;
            bool la = w2 < nitems;
            if (la) {
                item_range(w2, nsplit, Q, rt2, sp2, qa2, qb2);
                q2 = qa2;
            }
            auto prefetch_next = [&]() {
                if (!la) return;
                const int px = ADJ ? (int)(q2 * KS) : (int)(rt2 * BM);
                const int py = ADJ ? (int)(rt2 * BM) : (int)(q2 * KS);
                asm volatile("cp.async.bulk.prefetch.tensor.2d.L2.global.tile [%0, {%1, %2}];" ::"l"(&turn_map),
                             "r"(px), "r"(py)
                             : "memory");
                if (++q2 >= qb2) {
                    w2 += gridDim.x;
                    la = w2 < nitems;
                    if (la) {
                        item_range(w2, nsplit, Q, rt2, sp2, qa2, qb2);
                        q2 = qa2;
                    }
                }
            };
            for (int k = 0; k < PF; ++k) prefetch_next();
            for (long long w = blockIdx.x; w < nitems && !abort_flag; w += gridDim.x) {
                long long rt, sp, qa, qb;
                item_range(w, nsplit, Q, rt, sp, qa, qb);
                bool ok = true;
                for (long long q = qa; q < qb; ++q, ++g) {
                    const int ts = (int)(g % ST);
                    if (g >= ST && !bar_wait(tempty(ts), (uint32_t)(((g / ST) + 1) & 1), &abort_flag, err)) {
                        ok = false;
                        break;
                    }
                    bar_expect(tfull(ts), (uint32_t)TURN_BYTES);
                    const int cx = ADJ ? (int)(q * KS) : (int)(rt * BM);    // samples (inner dimension)
                    const int cy = ADJ ? (int)(rt * BM) : (int)(q * KS);    // voxels
                    asm volatile(
                        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, "
                        "{%2, %3}], [%4];" ::"r"(s0 + ts * TURN_BYTES),
                        "l"(&turn_map), "r"(cx), "r"(cy), "r"(tfull(ts))
                        : "memory");
                    prefetch_next();
                }
                if (!ok) break;
            }
            if (abort_flag) {   // let the phase tiles in flight land
                for (long long k = std::max<long long>(0, g - ST); k < g; ++k)
                    bar_wait(tfull((int)(k % ST)), (uint32_t)((k / ST) & 1), &abort_flag, err, true);
            }
        }
        __syncwarp();
    } else if (warp == WARP_MMA) {
        // ------------------------------------------------------------------ MMA --
        if (lane == 0) {
            constexpr uint32_t ID2 = idesc(BM, 2 * N0), ID1 = idesc(BM, N0);
            constexpr uint32_t LBO_A = BM * 16, LBO_B = 2 * N0 * 16;   // K-direction core-matrix strides
            long long g = 0, c = 0;
            bool ok = true;
            // A set goes to the epilogue only after this thread has seen its MMAs complete: each
            // chunk's MMAs are committed to chunkbar[c & 1], and once the next chunk's MMAs are
            // queued this thread waits for that barrier and then arrives on setfull.  (Epilogue
            // warps waiting directly on a tcgen05.commit arrival read incomplete accumulators.)
            long long pend = -1;
            int pend_set = 0;
            auto release_pending = [&]() {
                if (pend < 0) return true;
                if (!bar_wait(chunkbar((int)(pend & 1)), (uint32_t)((pend >> 1) & 1), &abort_flag, err)) return false;
                fence_before();
                bar_arrive(setfull(pend_set));
                pend = -1;
                return true;
            };
            for (long long w = blockIdx.x; w < nitems && ok && !abort_flag; w += gridDim.x) {
                long long rt, sp, qa, qb;
                item_range(w, nsplit, Q, rt, sp, qa, qb);
                for (long long q0 = qa; q0 < qb && ok; q0 += PS, ++c) {
                    const int set = (int)(c % NS);
                    if (c >= NS && !bar_wait(setempty(set), (uint32_t)(((c / NS) + 1) & 1), &abort_flag, err)) {
                        ok = false;
                        break;
                    }
                    fence_after();
                    const uint32_t dset = tmem + (uint32_t)(set * SW);
                    const long long q1 = std::min<long long>(q0 + PS, qb);
                    for (long long q = q0; q < q1; ++q, ++g) {
                        const int as = (int)(g % SA), bs = (int)(g % SB);
                        if (!bar_wait(bfull(bs), (uint32_t)((g / SB) & 1), &abort_flag, err) ||
                            !bar_wait(afull(as), (uint32_t)((g / SA) & 1), &abort_flag, err)) {
                            ok = false;
                            break;
                        }
                        fence_after();
                        const uint32_t a0 = s0 + OFF_A + as * A_BYTES;
                        const uint32_t b0 = s0 + OFF_B + bs * b_bytes(N0);
#pragma unroll
                        for (int j = 0; j < KS / 16; ++j) {
                            const uint32_t ao = j * 2 * LBO_A, bo = j * 2 * LBO_B;
                            const uint64_t ach = sdesc(a0 + 0 * A_SUB_BYTES + ao, LBO_A, 128);
                            const uint64_t acl = sdesc(a0 + 1 * A_SUB_BYTES + ao, LBO_A, 128);
                            const uint64_t ash = sdesc(a0 + 2 * A_SUB_BYTES + ao, LBO_A, 128);
                            const uint64_t asl = sdesc(a0 + 3 * A_SUB_BYTES + ao, LBO_A, 128);
                            const uint64_t bc = sdesc(b0 + bo, LBO_B, 128);
                            const uint64_t bs = sdesc(b0 + b_sub_bytes(N0) + bo, LBO_B, 128);
                            const uint32_t acc = (q == q0 && j == 0) ? 0u : 1u;
                            mma(dset, ach, bc, ID2, acc);            // [main | corr1] += cos_hi x [Bc_hi; Bc_lo]
                            mma(dset + 2 * N0, acl, bc, ID1, acc);   // corr2 += cos_lo x Bc_hi
                            mma(dset, ash, bs, ID2, 1u);
                            mma(dset + 2 * N0, asl, bs, ID1, 1u);
                        }
                        commit(aempty(as));
                        commit(bempty(bs));
                    }
                    if (!ok) break;
                    commit(chunkbar((int)(c & 1)));
                    if (!release_pending()) {
                        ok = false;
                        break;
                    }
                    pend = c;
                    pend_set = set;
                }
            }
            if (ok) release_pending();
            // every MMA this thread issued completes before TMEM is freed
            commit(drain);
            bar_wait(drain, 0u, &abort_flag, err, true);
        }
        __syncwarp();
    } else {
        // ------------------------------------------------------------- epilogue --
        const int quarter = warp & 3;                 // TMEM lanes 32 quarter .. 32 quarter + 31
        const int row = quarter * 32 + lane;
        const uint32_t tq = tmem + ((uint32_t)(quarter * 32) << 16);
        long long c = 0;
        bool ok = true;
        for (long long w = blockIdx.x; w < nitems && ok && !abort_flag; w += gridDim.x) {
            long long rt, sp, qa, qb;
            item_range(w, nsplit, Q, rt, sp, qa, qb);
            float tot[N0];
#pragma unroll
            for (int k = 0; k < N0; ++k) tot[k] = 0.f;
            for (long long q0 = qa; q0 < qb; q0 += PS, ++c) {
                const int set = (int)(c % NS);
                // every lane waits (acquire), then the warp reconverges before the warp-collective
                // tcgen05.ld; a wait that ran out on any lane stops the whole warp
                const bool got = bar_wait(setfull(set), (uint32_t)((c / NS) & 1), &abort_flag, err);
                if (!__all_sync(0xffffffffu, got)) {
                    ok = false;
                    break;
                }
                fence_after();
                const uint32_t ts = tq + (uint32_t)(set * SW);
#pragma unroll
                for (int cb = 0; cb < N0; cb += 16) {
                    float mv[16], cv[16];
                    tmem_ld16x2(ts + N0 + cb, ts + 2 * N0 + cb, mv, cv);     // corr1, corr2
#pragma unroll
                    for (int k = 0; k < 16; ++k) cv[k] += mv[k];
                    tmem_ld16(ts + cb, mv);                                  // main
#pragma unroll
                    for (int k = 0; k < 16; ++k) tot[cb + k] += mv[k] + cv[k] * (1.f / LO_SCALE);
                }
                fence_before();
                bar_arrive(setempty(set));
            }
            if (!ok) break;
            const long long grow = rt * BM + row;
            if (grow < R) {
                float* dst = partial + ((size_t)sp * R + grow) * N0;
#pragma unroll
                for (int k = 0; k < N0; k += 4)
                    *reinterpret_cast<float4*>(dst + k) = make_float4(tot[k], tot[k + 1], tot[k + 2], tot[k + 3]);
            }
        }
    }
    fence_before();
    __syncthreads();
    if (warp == WARP_MMA) {
        fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS));
    }
}

// Per-column max |re|, |im| of in[L, nb] as float bits (cmax zeroed by the caller).
__global__ void sho_umma_colmax_kernel(const float2* __restrict__ in, long long L, int nb,
                                       unsigned* __restrict__ cmax, const int* active) {
    if (active && *active) return;
    const int c = blockIdx.y;
    float m = 0.f;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < L; i += (long long)gridDim.x * blockDim.x) {
        const float2 v = in[i + L * c];
        m = fmaxf(m, fmaxf(fabsf(v.x), fabsf(v.y)));
    }
    for (int o = 16; o; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(cmax + c, __float_as_uint(m));
}

// B operand of coils c0 .. c0 + N0/2 - 1 in per-stage blocks: [sub][k / 8][row][k % 8] halves, sub =
// cos part, sin part; rows 0 .. N0 - 1 the FP16 high parts of the N0 output columns (real parts of the
// coils, then imaginary parts), rows N0 .. 2 N0 - 1 the low parts scaled by 2^11; inputs >= L and coils
// >= nb are zero.
template <bool ADJ, int N0>
__global__ void sho_umma_prep_kernel(const float2* __restrict__ in, long long L, long long Lpad, int nb, int c0,
                                     const unsigned* __restrict__ cmax, __half* __restrict__ b, const int* active) {
    using namespace umma;
    if (active && *active) return;
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int cl = blockIdx.y;
    if (i >= Lpad) return;
    const int c = c0 + cl;
    float re = 0.f, im = 0.f;
    if (c < nb && i < L) {
        const float mx = __uint_as_float(cmax[c]);
        const float inv = mx > 0.f ? 1.f / mx : 0.f;
        const float2 v = in[i + L * c];
        re = v.x * inv;
        im = v.y * inv;
    }
    const float bc0 = re, bc1 = im;                 // cos part: columns cl (real output), N0/2 + cl (imaginary)
    const float bs0 = ADJ ? im : -im, bs1 = ADJ ? -re : re;
    const long long q = i / KS;
    const int k = (int)(i - q * KS);
    __half* blk = b + q * (b_bytes(N0) / 2);
    auto put = [&](int sub, int n, float v) {
        const __half h = __float2half_rn(v);
        const __half l = __float2half_rn((v - __half2float(h)) * LO_SCALE);
        __half* p = blk + (long long)sub * (2 * N0 * KS) + (long long)(k >> 3) * (2 * N0 * 8) + (k & 7);
        p[n * 8] = h;
        p[(N0 + n) * 8] = l;
    };
    put(0, cl, bc0);
    put(0, N0 / 2 + cl, bc1);
    put(1, cl, bs0);
    put(1, N0 / 2 + cl, bs1);
}

// out[row + R c] = scale * max|in_c| * (sum_sp partial[sp][row][cl] + i partial[sp][row][N0/2 + cl]),
// summed over the splits in a fixed order (FP64).
template <int N0>
__global__ void sho_umma_reduce_kernel(const float* __restrict__ partial, int nsplit, long long R, int nb, int c0,
                                       const unsigned* __restrict__ cmax, float scale, float2* __restrict__ out,
                                       const int* active) {
    if (active && *active) return;
    const long long row = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int cl = blockIdx.y;
    const int c = c0 + cl;
    if (row >= R || c >= nb) return;
    double re = 0, im = 0;
    for (int s = 0; s < nsplit; ++s) {
        const float* p = partial + ((size_t)s * R + row) * N0;
        re += p[cl];
        im += p[N0 / 2 + cl];
    }
    const float f = scale * __uint_as_float(cmax[c]);
    out[row + R * c] = make_float2((float)re * f, (float)im * f);
}

// ------------------------------------------------------------------------ host --
static PFN_cuTensorMapEncodeTiled_v12000 umma_encode_fn() {
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

// K split per row tile: the persistent CTAs get equal numbers of equal items, items as long as
// the balance allows.
static int umma_nsplit(long long rtiles, long long Q, int nsm) {
    int best = 1;
    double best_cost = 1e300;
    for (int ns = 1; ns <= std::min<long long>(Q, 128); ++ns) {
        const long long items = rtiles * ns;
        const long long per_cta = cdiv(items, std::min<long long>(items, nsm));
        const double cost = (double)per_cta * ((double)cdiv(Q, ns) + 2.0);
        if (cost < best_cost - 1e-9) {
            best_cost = cost;
            best = ns;
        }
    }
    return best;
}

bool sho_umma_prepare(ShoUmma& u, const float* turn, long long V, long long M) {
    using namespace umma;
    u.ok = false;
    // TMA: the table's row pitch (M floats) must be a multiple of 16 bytes, tile coordinates fit int
    if (M % 4 != 0 || V > (1LL << 30) || M > (1LL << 30)) return false;
    int major = 0, dev = 0;
    MMR_CUDA(cudaGetDevice(&dev));
    MMR_CUDA(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev));
    if (major != 10) return false;
    const cuuint64_t dims[2] = {(cuuint64_t)M, (cuuint64_t)V};
    const cuuint64_t strides[1] = {(cuuint64_t)M * 4};
    const cuuint32_t estr[2] = {1, 1};
    const cuuint32_t box_f[2] = {(cuuint32_t)BM, (cuuint32_t)KS};
    const cuuint32_t box_a[2] = {(cuuint32_t)KS, (cuuint32_t)BM};
    CUresult r = umma_encode_fn()(&u.map_fwd, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float*>(turn), dims,
                                  strides, box_f, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    MMR_REQUIRE(r == CUDA_SUCCESS, "cuTensorMapEncodeTiled (phase table, forward) failed (%d)", (int)r);
    r = umma_encode_fn()(&u.map_adj, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float*>(turn), dims, strides,
                         box_a, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                         CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    MMR_REQUIRE(r == CUDA_SUCCESS, "cuTensorMapEncodeTiled (phase table, adjoint) failed (%d)", (int)r);
    const int nsm = device_sm_count();
    u.lpad = cdiv(std::max(V, M), KS) * KS;
    u.b.ensure((size_t)(u.lpad / KS) * b_bytes(64));
    for (int d = 0; d < 2; ++d) {
        const long long R = d ? V : M, L = d ? M : V;
        u.nsplit[d] = umma_nsplit(cdiv(R, BM), cdiv(L, KS), nsm);
    }
    u.partial.ensure((size_t)std::max(u.nsplit[0] * M, u.nsplit[1] * V) * 64 * sizeof(float));
    u.cmax.ensure((size_t)SHO_TC_MAX_COILS * sizeof(unsigned));
    u.err = device_error_ptr();
    static bool attrs = false;
    if (!attrs) {
        MMR_CUDA(cudaFuncSetAttribute(sho_umma_kernel<false, 16>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_bytes(16)));
        MMR_CUDA(cudaFuncSetAttribute(sho_umma_kernel<false, 32>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_bytes(32)));
        MMR_CUDA(cudaFuncSetAttribute(sho_umma_kernel<false, 64>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_bytes(64)));
        MMR_CUDA(cudaFuncSetAttribute(sho_umma_kernel<true, 16>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_bytes(16)));
        MMR_CUDA(cudaFuncSetAttribute(sho_umma_kernel<true, 32>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_bytes(32)));
        MMR_CUDA(cudaFuncSetAttribute(sho_umma_kernel<true, 64>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_bytes(64)));
        attrs = true;
    }
    u.ok = true;
    return true;
}

template <bool ADJ, int N0>
static void umma_group(ShoUmma& u, long long V, long long M, const float2* in, float2* out, long long nb, int c0,
                       cudaStream_t st, const int* active) {
    using namespace umma;
    const long long R = ADJ ? V : M, L = ADJ ? M : V;
    const long long Q = cdiv(L, KS);
    const int nsplit = u.nsplit[ADJ ? 1 : 0];
    const long long nitems = cdiv(R, BM) * nsplit;
    const unsigned* cm = u.cmax.as<unsigned>();
    __half* b = u.b.as<__half>();
    sho_umma_prep_kernel<ADJ, N0><<<dim3((unsigned)cdiv(Q * KS, 256), N0 / 2), 256, 0, st>>>(in, L, Q * KS, (int)nb,
                                                                                              c0, cm, b, active);
    check_launch("sho_umma_prep");
    const unsigned grid = (unsigned)std::min<long long>(nitems, device_sm_count());
    sho_umma_kernel<ADJ, N0><<<grid, nthreads(N0), smem_bytes(N0), st>>>(ADJ ? u.map_adj : u.map_fwd, b,
                                                                          u.partial.as<float>(), R, Q, nsplit, nitems,
                                                                          u.err, active);
    check_launch("sho_umma");
    // 1/sqrt(V) (sampHighOrder.m:387) and the 2^-11 of the A operand's fixed-point high parts
    const float scale = (float)(1.0 / std::sqrt((double)V) / 2048.0);
    sho_umma_reduce_kernel<N0><<<dim3((unsigned)cdiv(R, 256), N0 / 2), 256, 0, st>>>(
        u.partial.as<float>(), nsplit, R, (int)nb, c0, cm, scale, out, active);
    check_launch("sho_umma_reduce");
}

template <bool ADJ>
static void umma_apply(ShoUmma& u, long long V, long long M, const float2* in, float2* out, long long nb,
                       cudaStream_t st, const int* active) {
    MMR_REQUIRE(u.ok, "tcgen05 encoding not prepared");
    MMR_REQUIRE(nb >= 1 && nb <= SHO_TC_MAX_COILS, "tensor-core encoding handles 1..%lld columns", SHO_TC_MAX_COILS);
    const long long L = ADJ ? M : V;
    MMR_CUDA(cudaMemsetAsync(u.cmax.p, 0, (size_t)nb * sizeof(unsigned), st));
    sho_umma_colmax_kernel<<<dim3((unsigned)std::min<long long>(cdiv(L, 256), 256), (unsigned)nb), 256, 0, st>>>(
        in, L, (int)nb, u.cmax.as<unsigned>(), active);
    check_launch("sho_umma_colmax");
    if (nb <= 8) {
        umma_group<ADJ, 16>(u, V, M, in, out, nb, 0, st, active);
    } else if (nb <= 16) {
        umma_group<ADJ, 32>(u, V, M, in, out, nb, 0, st, active);
    } else {
        for (long long c0 = 0; c0 < nb; c0 += 32) umma_group<ADJ, 64>(u, V, M, in, out, nb, (int)c0, st, active);
    }
}

void sho_umma_forward(ShoUmma& u, long long V, long long M, const float2* x, float2* y, long long nb, cudaStream_t st,
                      const int* active) {
    umma_apply<false>(u, V, M, x, y, nb, st, active);
}

void sho_umma_adjoint(ShoUmma& u, long long V, long long M, const float2* y, float2* x, long long nb, cudaStream_t st,
                      const int* active) {
    umma_apply<true>(u, V, M, y, x, nb, st, active);
}

}  // namespace mmr
