// sampHighOrder encoding on the 5th-generation tensor cores (tcgen05.mma, TMEM
// accumulators, bulk-copied B operand, L2-prefetched phase table).
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
// integer, exact in FP16) and lo = 2^11 v - hi (|lo| <= 1/2, FP16); the
// column-normalised coil data in floating point, hi = FP16(b), lo = FP16(2^11
// (b - hi)).  TMEM accumulators take hi*hi (main), hi*lo_b (corr1) and
// lo_a*hi (corr2) in FP32, combined as main + corr1 / 2^11 + corr2 (about
// 22-bit operands).  The phase comes from a blocked copy of the table in
// radians, so the producers feed it straight to the SFU.  Every
// accumulation in TMEM covers 64 inputs; the epilogue adds the accumulation
// sets in FP32 registers and the split-K partials are summed in FP64 in a
// fixed order by a second kernel.
//
// One persistent CTA per SM walks (row tile, K split) work items (whole 128-input
// phase blocks, so every item has an even number of 32-input stages, taken in
// chunks of two); warp roles (16 producer warps for up to 16 coils per pass, 8
// for 32):
//   producers   per stage (32 inputs x 128 rows) load their phases straight
//               from global memory one stage ahead into registers (thread 0
//               also issues a bulk L2 prefetch of the phase block quarter
//               sixteen stages ahead), evaluate sincos on the SFU, split to
//               FP16 hi/lo and store the A operand, 128-byte swizzled, into a
//               6-deep ring (4 for 32-coil groups); once per chunk they hand
//               the previous chunk to the MMA thread (a proxy fence, then one
//               arrival per warp) and wait for the chunk that last used their
//               slots;
//   B loader    one bulk copy per chunk of the pre-split coil data into a
//               2-chunk ring, completing on the chunk slot's mbarrier;
//   MMA warp    one thread: per chunk it probes three barriers (accumulation
//               set free, A stored, B landed) with back-to-back test_waits,
//               issues 16 tcgen05.mma (kind::f16, M 128, K 16) behind one
//               tcgen05 fence, and commits twice: the chunk's A and B slots,
//               and its accumulation set to the epilogue.  An mbarrier wait or
//               a tcgen05 fence costs this thread a few hundred cycles, about
//               the issue time of six MMAs, so there is one of each per 16
//               MMAs.  The warp owns the TMEM allocation (all 512 columns);
//   4 epilogue warps: per chunk (64 inputs) the MMA warp moves on to the next
//               accumulation set of a TMEM ring, and the epilogue warps (each
//               its 32-lane quarter) wait for the set's commit, read it with
//               tcgen05.ld and add it to FP32 register totals, which they
//               store as the item's partial sums at its end.
// The A ring is as deep as shared memory allows: the producers run up to three
// chunks ahead of the tensor pipe.  Generic stores into an A slot are followed
// by a fence.proxy.async before the hand-off; without it, adjoint rows came
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

#include <cuda_fp16.h>

#include "nufft.cuh"
#include "sho_tc.cuh"
#include "umma.cuh"

namespace mmr {

namespace umma {

constexpr int BM = 128;                      // output rows per work item (TMEM lanes)
constexpr int KS = 32;                       // inputs per pipeline stage
constexpr int SB = 4;                        // B operand ring depth
constexpr int PS = 2;                        // stages per TMEM accumulation set (64 inputs)
constexpr int PF = 16;                       // L2 prefetch distance of the phase tiles, in stages
constexpr int MAX_SA = 6;
constexpr int QUARTER_BYTES = BM * KS * 4;   // one stage's phases: a quarter of a 128 x 128 block (16 KB)
static_assert(BM == 4 * KS, "a phase block holds four stages along the input dimension");
constexpr int LA = 1;                        // stages of phases each producer thread keeps in flight
// Operands in the 128-byte-swizzled K-major layout: rows of 128 bytes, 16-byte chunk c of row r at
// chunk position c ^ (r & 7), 8-row groups 1 KB apart.  An A stage is two 128-row regions, the
// cos region holding [hi (32 inputs, 64 B) | lo (64 B)] per row and the sin region the same; a B
// stage is 2 N0 rows (hi rows, then lo rows) of [cos part (64 B) | sin part (64 B)].  The MMAs
// step through the 16-input halves by advancing the descriptor start 32 bytes within the row.
constexpr int A_REGION = BM * 128;           // 16 KB: the cos region, then the sin region
constexpr int A_BYTES = 2 * A_REGION;
constexpr int TMEM_COLS = 512;
constexpr int MAX_SETS = 16;
constexpr float HI_SCALE = 2048.f;           // A: fixed-point high parts in units of 2^-11
constexpr float LO_SCALE = 2048.f;           // B: low parts scaled by 2^11
constexpr float ROUND_MAGIC = 12582912.f;    // 1.5 * 2^23: x + m - m rounds |x| < 2^22 to an integer
// warps 0 .. NPW-1 producers, NPW the MMA warp, NPW+1 the B loader, NPW+2 .. NPW+5 the epilogue
__host__ __device__ constexpr int nprod_warps(int N0) { return N0 <= 32 ? 16 : 8; }
__host__ __device__ constexpr int nthreads(int N0) { return (nprod_warps(N0) + 6) * 32; }
// A operand ring depth: as many 32 KB stages as shared memory leaves beside the B ring, so that
// the producers run several stages ahead of the tensor pipe
__host__ __device__ constexpr int n_a_stages(int N0) { return N0 <= 32 ? 6 : 4; }   // even: whole chunks
// B operand of one stage: 2 N0 rows of 128 bytes
__host__ __device__ constexpr int b_bytes(int N0) { return 2 * N0 * 128; }
// TMEM accumulation sets: SET_W(N0) columns each, main at 0, corr1 at N0, corr2 at 2 N0
__host__ __device__ constexpr int set_w(int N0) { return 4 * N0; }
__host__ __device__ constexpr int nsets(int N0) {
    return TMEM_COLS / set_w(N0) < MAX_SETS ? TMEM_COLS / set_w(N0) : MAX_SETS;
}

// offsets in the 1024-aligned dynamic shared memory: A stages from 0, then B stages, then barriers
__host__ __device__ constexpr int off_b(int N0) { return n_a_stages(N0) * A_BYTES; }
__host__ __device__ constexpr int bar_off(int N0) { return off_b(N0) + SB * b_bytes(N0); }
// barriers: cfull[4] (of MAX_SA) bfull[SB] setfull[MAX_SETS] setempty[MAX_SETS] drain chunk[4], then
// the TMEM address slot.  Per chunk (two stages) the MMA thread waits once (cfull: both stages' A and
// B in place) and commits twice: chunk[c & 3] frees the chunk's A and B slots, setfull its
// accumulation set for the epilogue.  (Each mbarrier wait or tcgen05 fence costs the single issuing
// thread a few hundred cycles of latency, so they are kept to one per 16 MMAs.)
__host__ __device__ constexpr int nbars() { return MAX_SA + SB + 2 * MAX_SETS + 5; }
static_assert(bar_off(16) + nbars() * 8 + 16 + 1024 <= 232448, "shared memory (16 columns)");
static_assert(bar_off(32) + nbars() * 8 + 16 + 1024 <= 232448, "shared memory (32 columns)");
static_assert(bar_off(64) + nbars() * 8 + 16 + 1024 <= 232448, "shared memory (64 columns)");
__host__ __device__ constexpr int smem_bytes(int N0) { return bar_off(N0) + nbars() * 8 + 16 + 1024; }


// Work item w -> row tile and the stage range of its K split: a balanced integer split of the
// phase blocks (four stages each), so that an item reads whole 64 KB blocks.
__host__ __device__ __forceinline__ void item_range(long long w, int nsplit, long long Q, long long& rt,
                                                    long long& sp, long long& qa, long long& qb) {
    const long long Qb = (Q + 3) >> 2;
    rt = w / nsplit;
    sp = w - rt * nsplit;
    qa = std::min(Q, 4 * (sp * Qb / nsplit));
    qb = std::min(Q, 4 * ((sp + 1) * Qb / nsplit));
}

// Walks a CTA's stages in order: items blockIdx.x, + gridDim.x, ..., each from qa to qb - 1.
struct Cursor {
    int w, rt, q, qb;
    bool valid;
    __device__ __forceinline__ void enter(long long nitems, int nsplit, long long Q) {
        valid = w < nitems;
        if (valid) {
            long long rt_, sp_, qa_, qb_;
            item_range(w, nsplit, Q, rt_, sp_, qa_, qb_);
            rt = (int)rt_;
            q = (int)qa_;
            qb = (int)qb_;
        }
    }
    __device__ __forceinline__ void next(long long nitems, int nsplit, long long Q) {
        if (++q >= qb) {
            w += gridDim.x;
            enter(nitems, nsplit, Q);
        }
    }
};

}  // namespace umma

// partial[sp][row][N0] for every work item.  tblk: the phase table in radians in 128 x 128 blocks
// ([V / 128][M / 128][128 voxels][128 samples], zero-padded; mblk blocks along M).  bglob: the B
// operand in per-stage blocks laid out as in shared memory.
template <bool ADJ, int N0>
__global__ void __launch_bounds__(umma::nthreads(N0), 1)
    sho_umma_kernel(const float* __restrict__ tblk, long long V, long long M, long long mblk,
                    const __half* __restrict__ bglob, float* __restrict__ partial, long long Q, int nsplit,
                    long long nitems, int* err, const int* active) {
    using namespace umma;
    constexpr int NS = nsets(N0);
    constexpr int SW = set_w(N0);
    constexpr int NPW = nprod_warps(N0), NPROD = NPW * 32;
    constexpr int WARP_MMA = NPW, WARP_B = NPW + 1;
    constexpr int SA = n_a_stages(N0);
    constexpr int OFF_A = 0, OFF_B = off_b(N0);
    const long long R = ADJ ? V : M;
    constexpr int CPT = (BM * KS / 8) / NPROD;     // 8-input chunks per producer thread and stage
    if (active && *active) return;
    extern __shared__ uint8_t smem_raw[];
    uint8_t* sm = smem_raw + ((1024u - (su32(smem_raw) & 1023u)) & 1023u);
    const uint32_t s0 = su32(sm);
    const uint32_t bars = s0 + bar_off(N0);
    auto cfull = [&](int i) { return bars + 8u * i; };     // chunk c's operands ready: cfull[c & 3]
    auto bfull = [&](int i) { return bars + 8u * (MAX_SA + i); };
    constexpr int SET0 = MAX_SA + SB;
    auto setfull = [&](int i) { return bars + 8u * (SET0 + i); };
    auto setempty = [&](int i) { return bars + 8u * (SET0 + MAX_SETS + i); };
    const uint32_t drain = bars + 8u * (SET0 + 2 * MAX_SETS);
    auto chunkbar = [&](int i) { return bars + 8u * (SET0 + 2 * MAX_SETS + 1 + i); };
    uint32_t* tslot = reinterpret_cast<uint32_t*>(sm + bar_off(N0) + nbars() * 8);
    __shared__ volatile int abort_flag;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (tid == 0) {
        abort_flag = 0;
        // per chunk: one arrival per producer warp
        for (int i = 0; i < 4; ++i) bar_init(cfull(i), NPW);
        for (int i = 0; i < SB / 2; ++i) bar_init(bfull(i), 1);   // per B chunk slot (two stages)
        for (int i = 0; i < NS; ++i) {
            bar_init(setfull(i), 1);
            bar_init(setempty(i), 4);          // one arrival per epilogue warp
        }
        bar_init(drain, 1);
        for (int i = 0; i < 4; ++i) bar_init(chunkbar(i), 1);
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
        // most 2048, exact in FP16) and a low part lo = 2^11 v - hi (|lo| <= 1/2): the MMAs then give
        // 2^11 times the sums, which the reduce kernel scales back.  Each thread loads
        // its phases of the next stage into registers while it works on this one; thread 0 keeps the
        // L2 prefetches PF stages ahead of those loads.
        // (row, 8-input chunk) pairs of a stage: 128 x 4, CPT per thread.  Forward: lanes run along
        // the rows (samples, contiguous in the table); adjoint: four lanes share a row (a voxel's 32
        // samples, 128 contiguous bytes), so that a warp's loads touch 8 lines instead of 32.
        auto row_of = [&](int j) { return ADJ ? (tid + j * NPROD) >> 2 : tid & (BM - 1); };
        auto chunk_of = [&](int j) { return ADJ ? (tid + j * NPROD) & 3 : (tid >> 7) + j * (NPROD / BM); };
        // out-of-range phases read as 0: their B rows are zero, or their output rows are dropped
        // stage q of row tile rt: block (q / 4, rt) forward, (rt, q / 4) adjoint, inputs 32 (q % 4) ..
        auto stage_block = [&](const Cursor& cs) {
            const long long qb4 = cs.q >> 2;
            return tblk + (ADJ ? (long long)cs.rt * mblk + qb4 : qb4 * mblk + cs.rt) * (BM * BM);
        };
        auto load_stage = [&](const Cursor& cs, float (&t)[CPT][8]) {
            const float* blk = stage_block(cs);
            const int sub = (cs.q & 3) * KS;
#pragma unroll
            for (int j = 0; j < CPT; ++j) {
                const int r = row_of(j), kc = chunk_of(j);
                if (ADJ) {
                    // row r = voxel: 8 consecutive samples, 32 bytes
                    const float4* p = reinterpret_cast<const float4*>(blk + r * BM + sub + kc * 8);
                    const float4 lo4 = __ldcs(p), hi4 = __ldcs(p + 1);
                    t[j][0] = lo4.x; t[j][1] = lo4.y; t[j][2] = lo4.z; t[j][3] = lo4.w;
                    t[j][4] = hi4.x; t[j][5] = hi4.y; t[j][6] = hi4.z; t[j][7] = hi4.w;
                } else {
                    // row r = sample, 8 voxels: each warp load is 128 consecutive bytes of one voxel row
                    const float* p = blk + (sub + kc * 8) * BM + r;
#pragma unroll
                    for (int e = 0; e < 8; ++e) t[j][e] = __ldcs(p + e * BM);
                }
            }
        };
        // this CTA's stage count
        long long nst = 0;
        for (long long w = blockIdx.x; w < nitems; w += gridDim.x) {
            long long rt, sp, qa, qb;
            item_range(w, nsplit, Q, rt, sp, qa, qb);
            nst += qb - qa;
        }
        Cursor ld, pre;       // the next stage to load, the next stage to prefetch into L2
        ld.w = blockIdx.x;
        ld.enter(nitems, nsplit, Q);
        pre = ld;
        // one 16 KB quarter of a block per stage: over a block's four stages the whole block is
        // fetched, PF stages before it is read
        auto prefetch = [&]() {
            const float* q4 = stage_block(pre) + (pre.q & 3) * (BM * KS);
            asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(q4), "n"(QUARTER_BYTES) : "memory");
            pre.next(nitems, nsplit, Q);
        };
        if (tid == 0)
            for (int k = 0; k < PF && pre.valid; ++k) prefetch();
        // register ring: while stage g is split and stored, stages g + 1 .. g + LA are in flight
        float tr[LA + 1][CPT][8];
        int as = 0;            // A slot of stage g
#pragma unroll
        for (int u = 0; u < LA; ++u)
            if (ld.valid) {
                load_stage(ld, tr[u]);
                ld.next(nitems, nsplit, Q);
            }
        for (long long g0 = 0; g0 < nst && !abort_flag; g0 += LA + 1) {
#pragma unroll
            for (int slot = 0; slot < LA + 1; ++slot) {
                const long long g = g0 + slot;
                if (g >= nst) break;
                if (ld.valid) {
                    load_stage(ld, tr[(slot + LA) % (LA + 1)]);
                    ld.next(nitems, nsplit, Q);
                }
                if (tid == 0 && pre.valid) prefetch();
                float (&t)[CPT][8] = tr[slot];
                // cos hi, cos lo, sin hi, sin lo of this thread's 8-input chunks, as FP16 pairs
                uint32_t pk[CPT][4][4];
#pragma unroll
                for (int j = 0; j < CPT; ++j) {
#pragma unroll
                    for (int e = 0; e < 4; ++e) {
                        float chv[2], shv[2], clv[2], slv[2];
#pragma unroll
                        for (int u = 0; u < 2; ++u) {
                            float sv, cv;
                            __sincosf(t[j][2 * e + u], &sv, &cv);
                            // hi = round(2^11 v) in one rounding of the exact 2^11 v + 1.5 2^23; the
                            // residual 2^11 v - hi is exact in one FMA
                            chv[u] = __fsub_rn(__fmaf_rn(cv, HI_SCALE, ROUND_MAGIC), ROUND_MAGIC);
                            shv[u] = __fsub_rn(__fmaf_rn(sv, HI_SCALE, ROUND_MAGIC), ROUND_MAGIC);
                            clv[u] = __fmaf_rn(cv, HI_SCALE, -chv[u]);
                            slv[u] = __fmaf_rn(sv, HI_SCALE, -shv[u]);
                        }
                        pk[j][0][e] = h2bits(__floats2half2_rn(chv[0], chv[1]));
                        pk[j][1][e] = h2bits(__floats2half2_rn(clv[0], clv[1]));
                        pk[j][2][e] = h2bits(__floats2half2_rn(shv[0], shv[1]));
                        pk[j][3][e] = h2bits(__floats2half2_rn(slv[0], slv[1]));
                    }
                }
                // Once per chunk (two stages), at its first stage: the previous chunk's stores, issued
                // before this stage's sincos, have drained by now: order them before the async
                // proxy's reads and hand that chunk to the MMA thread; then wait until the chunk that
                // last used this chunk's two A slots (SA is even) has completed.  Lane 0 waits, the
                // warp follows it (one poller per warp on the barrier).
                if ((g & 1) == 0) {
                    if (g > 0) {
                        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                        __syncwarp();
                        if (lane == 0) bar_arrive(cfull((int)(((g >> 1) - 1) & 3)));
                    }
                    if (g >= SA) {
                        const long long k = (g - SA) >> 1;
                        int okw = 1;
                        if (lane == 0)
                            okw = bar_wait(chunkbar((int)(k & 3)), (uint32_t)((k >> 2) & 1), &abort_flag, err);
                        __syncwarp();
                        if (!__shfl_sync(0xffffffffu, okw, 0)) break;
                    }
                }
                uint8_t* a = sm + OFF_A + as * A_BYTES;
#pragma unroll
                for (int j = 0; j < CPT; ++j) {
                    const int r = row_of(j), kc = chunk_of(j);
                    // row r of each region; hi in chunk kc, lo in chunk 4 + kc, swizzled by r & 7
                    uint8_t* rc = a + r * 128;
                    uint8_t* rs = rc + A_REGION;
                    const int sw = r & 7;
                    *reinterpret_cast<uint4*>(rc + ((kc ^ sw) << 4)) = make_uint4(pk[j][0][0], pk[j][0][1], pk[j][0][2], pk[j][0][3]);
                    *reinterpret_cast<uint4*>(rc + (((4 + kc) ^ sw) << 4)) = make_uint4(pk[j][1][0], pk[j][1][1], pk[j][1][2], pk[j][1][3]);
                    *reinterpret_cast<uint4*>(rs + ((kc ^ sw) << 4)) = make_uint4(pk[j][2][0], pk[j][2][1], pk[j][2][2], pk[j][2][3]);
                    *reinterpret_cast<uint4*>(rs + (((4 + kc) ^ sw) << 4)) = make_uint4(pk[j][3][0], pk[j][3][1], pk[j][3][2], pk[j][3][3]);
                }
                if (++as == SA) as = 0;
            }
        }
        // the last chunk's hand-off
        if (nst > 0 && !abort_flag) {
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            __syncwarp();
            if (lane == 0) bar_arrive(cfull((int)(((nst - 1) >> 1) & 3)));
        }
    } else if (warp == WARP_B) {
        // -------------------------------------------------------------- B loader --
        // a chunk's B operand (coil data, FP16 hi / lo, both parts, two stages: adjacent in global
        // and in shared memory) by one bulk copy into a ring of SB / 2 chunk slots, completing on the
        // slot's bfull; slot reuse waits for the completion of the chunk that last read it
        constexpr int NBC = SB / 2;
        long long c = 0;   // chunk copies issued
        if (lane == 0) {
            bool ok = true;
            for (long long w = blockIdx.x; w < nitems && ok && !abort_flag; w += gridDim.x) {
                long long rt, sp, qa, qb;
                item_range(w, nsplit, Q, rt, sp, qa, qb);
                for (long long q = qa; q < qb; q += PS) {
                    const int bc = (int)(c % NBC);
                    const long long k = c - NBC;
                    if (c >= NBC && !bar_wait(chunkbar((int)(k & 3)), (uint32_t)((k >> 2) & 1), &abort_flag, err)) {
                        ok = false;
                        break;
                    }
                    bar_expect(bfull(bc), (uint32_t)(PS * b_bytes(N0)));
                    asm volatile(
                        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                            s0 + OFF_B + bc * (PS * b_bytes(N0))),
                        "l"(bglob + (size_t)q * (b_bytes(N0) / 2)), "r"((uint32_t)(PS * b_bytes(N0))), "r"(bfull(bc))
                        : "memory");
                    ++c;
                }
            }
            if (abort_flag) {   // the copies in flight land before the CTA exits
                for (long long k = std::max<long long>(0, c - NBC); k < c; ++k)
                    bar_wait(bfull((int)(k % NBC)), (uint32_t)((k / NBC) & 1), &abort_flag, err, true);
            }
        }
        __syncwarp();
    } else if (warp == WARP_MMA) {
        // ------------------------------------------------------------------ MMA --
        if (lane == 0) {
            constexpr uint32_t ID2 = idesc(BM, 2 * N0), ID1 = idesc(BM, N0);
            // descriptors of A slot 0 / B slot 0 as 32-bit words
            const uint64_t da0 = sdesc_sw128(s0 + OFF_A), db0 = sdesc_sw128(s0 + OFF_B);
            const uint32_t da_lo = (uint32_t)da0, da_hi = (uint32_t)(da0 >> 32);
            const uint32_t db_lo = (uint32_t)db0, db_hi = (uint32_t)(db0 >> 32);
            long long c = 0;
            int as = 0, bs = 0;          // operand slots of the current stage
            bool ok = true;
            for (long long w = blockIdx.x; w < nitems && ok && !abort_flag; w += gridDim.x) {
                long long rt, sp, qa, qb;
                item_range(w, nsplit, Q, rt, sp, qa, qb);
                for (long long q0 = qa; q0 < qb; q0 += PS, ++c) {   // chunks of two stages
                    const int set = (int)(c % NS);
                    const uint32_t se = setempty(set), se_ph = (uint32_t)(((c / NS) + 1) & 1);
                    const uint32_t cf = cfull((int)(c & 3)), cf_ph = (uint32_t)((c >> 2) & 1);
                    const uint32_t bf = bfull((int)(c % (SB / 2))), bf_ph = (uint32_t)((c / (SB / 2)) & 1);
                    // the set free, the A stages stored, the B chunk landed: three probes issued back to
                    // back, a bounded wait only for those not yet complete
                    const uint32_t t1 = c >= NS ? bar_test(se, se_ph) : 1u;
                    const uint32_t t2 = bar_test(cf, cf_ph);
                    const uint32_t t3 = bar_test(bf, bf_ph);
                    if ((!t1 && !bar_wait(se, se_ph, &abort_flag, err)) || (!t2 && !bar_wait(cf, cf_ph, &abort_flag, err)) ||
                        (!t3 && !bar_wait(bf, bf_ph, &abort_flag, err))) {
                        ok = false;
                        break;
                    }
                    fence_after();
                    const uint32_t dset = tmem + (uint32_t)(set * SW);
#pragma unroll
                    for (int h = 0; h < PS; ++h) {
                        // descriptor low words of this stage's A and B slots; offsets below in 16-byte units
                        const uint32_t alo = da_lo + (uint32_t)(as * (A_BYTES >> 4));
                        const uint32_t blo = db_lo + (uint32_t)(bs * (b_bytes(N0) >> 4));
#pragma unroll
                        for (int j = 0; j < KS / 16; ++j) {
                            const uint32_t ko = (uint32_t)j * (32 >> 4);   // 16 inputs = 32 bytes along the row
                            const uint32_t acc = (h == 0 && j == 0) ? 0u : 1u;
                            constexpr uint32_t LO = 64 >> 4, SIN = A_REGION >> 4;
                            // [main | corr1] += cos_hi x [Bc_hi; Bc_lo];  corr2 += cos_lo x Bc_hi; then the sin parts
                            mma2(dset, alo + ko, da_hi, blo + ko, db_hi, ID2, acc);
                            mma2(dset + 2 * N0, alo + LO + ko, da_hi, blo + ko, db_hi, ID1, acc);
                            mma2(dset, alo + SIN + ko, da_hi, blo + LO + ko, db_hi, ID2, 1u);
                            mma2(dset + 2 * N0, alo + SIN + LO + ko, da_hi, blo + LO + ko, db_hi, ID1, 1u);
                        }
                        if (++as == SA) as = 0;
                        if (++bs == SB) bs = 0;
                    }
                    commit(chunkbar((int)(c & 3)));   // the chunk's A and B slots
                    commit(setfull(set));              // its accumulation set, for the epilogue
                }
            }
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
                // lane 0 waits (acquire), the warp reconverges behind it before the warp-collective
                // tcgen05.ld; a wait that ran out stops the whole warp
                int got = 1;
                if (lane == 0) got = bar_wait(setfull(set), (uint32_t)((c / NS) & 1), &abort_flag, err);
                __syncwarp();
                if (!__shfl_sync(0xffffffffu, got, 0)) {
                    ok = false;
                    break;
                }
                fence_after();
                const uint32_t ts = tq + (uint32_t)(set * SW);
#pragma unroll
                for (int cb = 0; cb < N0; cb += 16) {
                    float mv[16], cv[16];
                    tmem_ld16x2(ts + N0 + cb, ts + 2 * N0 + cb, mv, cv);     // corr1 (B lo x 2^11), corr2
#pragma unroll
                    for (int k = 0; k < 16; ++k) cv[k] = __fmaf_rn(mv[k], 1.f / LO_SCALE, cv[k]);
                    tmem_ld16(ts + cb, mv);                                  // main
#pragma unroll
                    for (int k = 0; k < 16; ++k) tot[cb + k] += mv[k] + cv[k];
                }
                fence_before();
                __syncwarp();
                if (lane == 0) bar_arrive(setempty(set));
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

// The [V][M] phase table (turns) as radians, FP32(2 pi t), in 128 x 128 blocks: block (vb, mb) at
// (vb mblk + mb) 128^2, voxel-major inside, zero beyond V and M.  One CTA per block.
__global__ void sho_umma_block_kernel(const float* __restrict__ turn, long long V, long long M, long long mblk,
                                      float* __restrict__ tblk) {
    using namespace umma;
    const long long blk = blockIdx.x;
    const long long vb = blk / mblk, mb = blk - vb * mblk;
    float* dst = tblk + blk * (BM * BM);
    for (int i = threadIdx.x; i < BM * BM; i += blockDim.x) {
        const long long v = vb * BM + (i >> 7), m = mb * BM + (i & (BM - 1));
        dst[i] = (v < V && m < M) ? __fmul_rn(6.28318530717958647692f, turn[v * M + m]) : 0.f;
    }
}

// Per-column max |re|, |im| of in[L, nb] as float bits (cmax zeroed by the caller): a block
// reduction, one atomic per block and column.
__global__ void sho_umma_colmax_kernel(const float2* __restrict__ in, long long L, int nb,
                                       unsigned* __restrict__ cmax, const int* active) {
    if (active && *active) return;
    __shared__ float red[32];
    const int c = blockIdx.y;
    float m = 0.f;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < L; i += (long long)gridDim.x * blockDim.x) {
        const float2 v = in[i + L * c];
        m = fmaxf(m, fmaxf(fabsf(v.x), fabsf(v.y)));
    }
    for (int o = 16; o; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x < 32) {
        m = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.f;
        for (int o = 16; o; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
        if (threadIdx.x == 0) atomicMax(cmax + c, __float_as_uint(m));
    }
}

// B operand of coils c0 .. c0 + N0/2 - 1 in per-stage blocks of 2 N0 rows x 128 bytes (the swizzled
// layout of the kernel's shared memory): rows 0 .. N0 - 1 the FP16 high parts of the N0 output columns
// (real parts of the coils, then imaginary parts), rows N0 .. 2 N0 - 1 the low parts scaled by 2^11;
// per row the 32 inputs of the cos part, then of the sin part; inputs >= L and coils >= nb are zero.
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
    const int ch = k >> 3;   // 16-byte chunk of the cos part; the sin part's is 4 + ch
    auto at = [&](int row, int c) { return blk + row * 64 + ((c ^ (row & 7)) << 3) + (k & 7); };
    auto put = [&](int sub, int n, float v) {
        const __half h = __float2half_rn(v);
        const __half l = __float2half_rn((v - __half2float(h)) * LO_SCALE);
        *at(n, 4 * sub + ch) = h;
        *at(N0 + n, 4 * sub + ch) = l;
    };
    put(0, cl, bc0);
    put(0, N0 / 2 + cl, bc1);
    put(1, cl, bs0);
    put(1, N0 / 2 + cl, bs1);
}

// out[row + R c] = scale * max|in_c| * (sum_sp partial[sp][row][cl] + i partial[sp][row][N0/2 + cl]),
// summed over the splits in a fixed order (FP64).  A block takes 32 rows: it reads their partial rows
// contiguously (N0 floats each) and writes each coil's 32 outputs contiguously, through a transposing
// shared-memory tile.
template <int N0>
__global__ void __launch_bounds__(256) sho_umma_reduce_kernel(const float* __restrict__ partial, int nsplit, long long R,
                                                               int nb, int c0, const unsigned* __restrict__ cmax,
                                                               float scale, float2* __restrict__ out, const int* active) {
    if (active && *active) return;
    constexpr int RB = 32;
    __shared__ float tile[N0][RB + 1];
    const long long row0 = (long long)blockIdx.x * RB;
    for (int e = threadIdx.x; e < RB * N0; e += blockDim.x) {
        const int i = e / N0, col = e - i * N0;    // consecutive threads: consecutive columns of a row
        const long long row = row0 + i;
        double acc = 0.0;
        if (row < R)
            for (int sp = 0; sp < nsplit; ++sp) acc += partial[((size_t)sp * R + row) * N0 + col];
        tile[col][i] = (float)acc;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < RB * (N0 / 2); e += blockDim.x) {
        const int cl = e / RB, i = e - cl * RB;    // consecutive threads: consecutive rows of a coil
        const int c = c0 + cl;
        const long long row = row0 + i;
        if (row >= R || c >= nb) continue;
        const float f = scale * __uint_as_float(cmax[c]);
        out[row + R * c] = make_float2(tile[cl][i] * f, tile[N0 / 2 + cl][i] * f);
    }
}

// ------------------------------------------------------------------------ host --
// K split per row tile (in whole phase blocks): the persistent CTAs get equal numbers of equal
// items, items as long as the balance allows.
static int umma_nsplit(long long rtiles, long long Q, int nsm) {
    const long long Qb = cdiv(Q, 4);
    int best = 1;
    double best_cost = 1e300;
    for (int ns = 1; ns <= std::min<long long>(Qb, 128); ++ns) {
        const long long items = rtiles * ns;
        const long long per_cta = cdiv(items, std::min<long long>(items, nsm));
        const double cost = (double)per_cta * (4.0 * (double)cdiv(Qb, ns) + 2.0);
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
    if (V > (1LL << 30) || M > (1LL << 30)) return false;   // tile coordinates fit int
    int major = 0, dev = 0;
    MMR_CUDA(cudaGetDevice(&dev));
    MMR_CUDA(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev));
    if (major != 10) return false;
    // the blocked copy of the table, when it fits in half of the free memory
    const long long vblk = cdiv(V, BM), mblk = cdiv(M, BM);
    const size_t tb_bytes = (size_t)vblk * (size_t)mblk * BM * BM * sizeof(float);
    size_t fr = 0, tot = 0;
    MMR_CUDA(cudaMemGetInfo(&fr, &tot));
    if (tb_bytes > fr / 2) return false;
    u.tblk.ensure(tb_bytes);
    u.mblk = mblk;
    sho_umma_block_kernel<<<(unsigned)(vblk * mblk), 256>>>(turn, V, M, mblk, u.tblk.as<float>());
    check_launch("sho_umma_block");
    const int nsm = device_sm_count();
    u.lpad = cdiv(std::max(V, M), BM) * BM;   // inputs padded to whole phase blocks (4 stages)
    u.b.ensure((size_t)(u.lpad / KS) * b_bytes(64));
    for (int d = 0; d < 2; ++d) {
        const long long R = d ? V : M, L = d ? M : V;
        u.nsplit[d] = umma_nsplit(cdiv(R, BM), 4 * cdiv(L, BM), nsm);
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
    const long long Q = 4 * cdiv(L, BM);   // stages, padded to whole phase blocks: every item has an even count
    const int nsplit = u.nsplit[ADJ ? 1 : 0];
    const long long nitems = cdiv(R, BM) * nsplit;
    const unsigned* cm = u.cmax.as<unsigned>();
    __half* b = u.b.as<__half>();
    sho_umma_prep_kernel<ADJ, N0><<<dim3((unsigned)cdiv(Q * KS, 256), N0 / 2), 256, 0, st>>>(in, L, Q * KS, (int)nb,
                                                                                              c0, cm, b, active);
    check_launch("sho_umma_prep");
    const unsigned grid = (unsigned)std::min<long long>(nitems, device_sm_count());
    sho_umma_kernel<ADJ, N0><<<grid, nthreads(N0), smem_bytes(N0), st>>>(
        u.tblk.as<float>(), V, M, u.mblk, b, u.partial.as<float>(), Q, nsplit, nitems, u.err, active);
    check_launch("sho_umma");
    // 1/sqrt(V) (sampHighOrder.m:387) and the 2^-11 of the A operand's fixed-point high parts
    const float scale = (float)(1.0 / std::sqrt((double)V) / 2048.0);
    sho_umma_reduce_kernel<N0><<<(unsigned)cdiv(R, 32), 256, 0, st>>>(
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
    sho_umma_colmax_kernel<<<dim3((unsigned)std::min<long long>(cdiv(L, 1024), 64), (unsigned)nb), 256, 0, st>>>(
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
