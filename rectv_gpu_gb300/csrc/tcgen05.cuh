// Inline-PTX helpers for the fifth-generation tensor cores (tcgen05) of
// sm_103a: tensor-memory (TMEM) allocation, shared-memory matrix descriptors,
// MMA issue and completion tracking through an mbarrier, and TMEM loads.
//
// Conventions used by every kernel of this library:
//  * operands are K-major without swizzle: 8-row x 16-byte core matrices
//    stored as 128 contiguous bytes; `lbo` is the byte distance between core
//    matrices adjacent in K, `sbo` between core matrices adjacent in M (or N);
//  * D is FP32 in TMEM, M = 128: row i of D is TMEM lane i, column j is TMEM
//    column (base + j);
//  * the tensor core reads a TF32 operand from the top 19 bits of each FP32
//    word (the low 13 mantissa bits are ignored, i.e. truncated), so an FP32
//    array is its own TF32 "high" part and x - trunc13(x) is the exact rest.
//  * every wait is bounded by a clock limit; on expiry the caller records an
//    error and carries on through its barriers.  A thread whose wait has
//    expired once passes healthy = false to its later waits, which then give
//    up after kWaitShort cycles instead of kWaitLong: a lost arrival costs
//    one long wait per thread plus short ones, so a persistent block that
//    waits thousands of times still ends promptly, and the short waits still
//    let copies that are merely late land before the block moves on.
#pragma once

#include <cstdint>

namespace rectv {
namespace tc {

__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// x with the 13 low mantissa bits cleared: the TF32 value the tensor core uses.
__device__ __forceinline__ float trunc_tf32(float x) { return __uint_as_float(__float_as_uint(x) & 0xffffe000u); }

// Shared-memory matrix descriptor (K-major, no swizzle, descriptor version 1).
__device__ __forceinline__ uint64_t sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | ((uint64_t)1 << 46);
}

// Instruction descriptor: D FP32; A and B of format fmt (kind::tf32: 2 = TF32;
// kind::f16: 1 = BF16), both K-major, dense; N >> 3 at bit 17, M >> 4 at bit 24.
__host__ __device__ constexpr uint32_t idesc(uint32_t fmt, int M, int N) {
    return (1u << 4) | (fmt << 7) | (fmt << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}
constexpr uint32_t kFmtBF16 = 1;
constexpr uint32_t kFmtTF32 = 2;

// D (+)= A B^T with A [M x 8] TF32, B [N x 8] TF32 (one K step).
__device__ __forceinline__ void mma_tf32(uint32_t d, uint64_t a, uint64_t b, uint32_t id, uint32_t acc) {
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
        "l"(a), "l"(b), "r"(id), "r"(acc)
        : "memory");
}

// D (+)= A B^T with A [M x 16] BF16, B [N x 16] BF16 (one K step).
__device__ __forceinline__ void mma_bf16(uint32_t d, uint64_t a, uint64_t b, uint32_t id, uint32_t acc) {
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
        "l"(a), "l"(b), "r"(id), "r"(acc)
        : "memory");
}

// Arrive once on the mbarrier when all MMAs issued so far by this thread are done.
__device__ __forceinline__ void commit(void *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                     smem_addr(bar))
                 : "memory");
}

__device__ __forceinline__ void mbar_init(void *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}

// One-thread 1D bulk copy (TMA engine) of `bytes` (a multiple of 16, both
// addresses 16-byte aligned) from global to shared memory; completion is
// counted on the mbarrier as transaction bytes (one arrival per copy).
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, void *bar) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
            smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}

// Wait limits in SM clock cycles: about one second, and about 0.1 ms.
constexpr long long kWaitLong = 2000000000LL;
constexpr long long kWaitShort = 200000LL;

// Wait for phase `parity` of the mbarrier; false when it has not completed
// within kWaitLong cycles (kWaitShort when `healthy` is false, i.e. after an
// earlier wait of this thread gave up), or within `limit` cycles if given.
__device__ __forceinline__ bool mbar_wait(void *bar, uint32_t parity, bool healthy = true, long long limit = 0) {
    const uint32_t a = smem_addr(bar);
    if (limit <= 0) limit = healthy ? kWaitLong : kWaitShort;
    const long long t0 = clock64();
    for (;;) {
        uint32_t done;
        asm volatile(
            "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
        if (clock64() - t0 > limit) return false;
    }
}

// Order this thread's generic-proxy shared-memory writes before later
// tensor-core (async-proxy) reads of them.
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }
__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }

// Whole-warp TMEM allocation of ncols columns (power of two >= 32); the base
// address is written to *slot.
__device__ __forceinline__ void alloc(uint32_t *slot, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_addr(slot)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
}
__device__ __forceinline__ void dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(taddr), "r"(ncols) : "memory");
}

// Whole-warp load of 32 consecutive FP32 columns of this warp's 32 TMEM lanes
// (warp w of the block may address lanes 32 (w % 4) .. 32 (w % 4) + 31).
__device__ __forceinline__ void ld32(uint32_t taddr, float (&v)[32]) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
        : "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]),
          "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]),
          "=r"(r[30]), "=r"(r[31])
        : "r"(taddr + 16));
    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// Whole-warp load of 8 consecutive FP32 columns of this warp's 32 TMEM lanes.
__device__ __forceinline__ void ld8(uint32_t taddr, float (&v)[8]) {
    uint32_t r[8];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
    for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
}

}  // namespace tc
}  // namespace rectv
