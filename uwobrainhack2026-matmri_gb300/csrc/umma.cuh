// Device helpers of the tcgen05 kernels (sho_umma.cu, gram_umma.cu): mbarriers with bounded waits,
// shared-memory matrix and instruction descriptors, tcgen05.mma / commit / fences, TMEM loads.
#pragma once

#include <cstdint>

#include <cuda_fp16.h>

namespace mmr {
namespace umma {

// mbarrier waits: each try_wait may suspend the thread for up to SUSPEND_NS (it resumes as soon as
// the phase completes), so that waiting warps take few issue slots from the working ones; at most
// WAIT_POLLS polls (about a second) before a wait counts as timed out
constexpr uint32_t SUSPEND_NS = 500;
constexpr uint32_t WAIT_POLLS = 1u << 21;

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
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done)
            : "r"(bar), "r"(parity), "n"(SUSPEND_NS)
            : "memory");
        if (done) return true;
        if (!drain && (it & 63u) == 63u && *abort_flag) return false;
    }
    *abort_flag = 1;
    atomicExch(err, 1);
    return false;
}
// Non-blocking test of a phase's completion (no suspension): several can be issued back to back
// so that their latencies overlap.
__device__ __forceinline__ uint32_t bar_test(uint32_t bar, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    return done;
}

// Shared-memory matrix descriptor, K-major with 128-byte swizzle: start address >> 4 in bits 0-13,
// the leading offset (unused by this layout; 16 bytes) in bits 16-29, the 8-row group stride (1 KB)
// >> 4 in bits 32-45, descriptor version 1 at bit 46, layout type 2 (128-byte swizzle) in bits 61-63.
__device__ __forceinline__ uint64_t sdesc_sw128(uint32_t saddr) {
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) |
           ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
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
// The same with each descriptor given as its two 32-bit words: the start address (bits 0-13 of the
// low word, byte address >> 4) of a descriptor advances by a plain 32-bit add, which cannot carry
// into the offset field above it because shared-memory addresses stay below 2^18.
__device__ __forceinline__ void mma2(uint32_t d, uint32_t alo, uint32_t ahi, uint32_t blo, uint32_t bhi, uint32_t id,
                                     uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t.reg .b64 da, db;\n\t"
        "mov.b64 da, {%1, %2};\n\tmov.b64 db, {%3, %4};\n\tsetp.ne.b32 p, %6, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], da, db, %5, p;\n\t}\n" ::"r"(d),
        "r"(alo), "r"(ahi), "r"(blo), "r"(bhi), "r"(id), "r"(acc));
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

// Shared-memory matrix descriptor, K-major with 64-byte swizzle (rows of 64 bytes, 16-byte chunk c
// of row r at c ^ ((r >> 1) & 3), 8-row groups 512 bytes apart): layout type 4 in bits 61-63.
__device__ __forceinline__ uint64_t sdesc_sw64(uint32_t saddr) {
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)1 << 16) | ((uint64_t)(512 >> 4) << 32) |
           ((uint64_t)1 << 46) | ((uint64_t)4 << 61);
}

}  // namespace umma
}  // namespace mmr
