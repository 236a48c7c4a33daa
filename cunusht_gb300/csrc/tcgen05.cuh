// tcgen05 / TMA-bulk / mbarrier helpers (inline PTX) and the integer-digit
// split shared by the tensor-core Legendre kernels (legendre_tc.cu,
// legendre_tc_adj.cu).  sm_100a-family only.
#pragma once
#include <cstdint>

namespace cunusht {

// ---------------------------------------------------------------- tcgen05 / mbarrier helpers
constexpr int MBAR_SPIN_LIMIT = 1 << 22;

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor, no swizzle, descriptor version 1.
// K-major operand: core matrices of 8 rows x 16 bytes (8 elements along K,
// rows 16 bytes apart); lbo = byte distance between core matrices adjacent in
// K, sbo = between 8-row groups.  MN-major operand (transpose bit of the
// instruction descriptor set): core matrices of 8 K-rows x 16 bytes (8
// elements along M / N); lbo = between core matrices adjacent in K, sbo =
// between core matrices adjacent in M / N (checked by the self test).
__device__ __forceinline__ uint64_t sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::f16: D f32 (bits 4-5 = 1), A and B bf16
// (bits 7-9, 10-12 = 1), both K-major, N >> 3 at bit 17, M >> 4 at bit 24.
__host__ __device__ constexpr uint32_t idesc_bf16_f32(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void tc_mma(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
        ::"r"(d_tmem), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc)
        : "memory");
}

__device__ __forceinline__ void tc_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// generic-proxy shared-memory writes made visible to the tensor cores
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_init_fence() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

// Wait for the completion of the barrier phase with the given parity; false
// when the iteration limit runs out first.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, int limit = MBAR_SPIN_LIMIT) {
    for (int it = 0; it < limit; ++it) {
        uint32_t ok;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(ok)
            : "r"(bar), "r"(parity)
            : "memory");
        if (ok) return true;
    }
    return false;
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

// bytes from global to shared memory by the bulk-copy engine, completion counted on bar
// (both addresses 16-byte aligned, bytes a multiple of 16)
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void *src, uint32_t bytes, uint32_t bar) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                 "l"(src), "r"(bytes), "r"(bar)
                 : "memory");
}

// named barrier id over nthr threads (a multiple of 32) and its OR-reduction
__device__ __forceinline__ void bar_sync_n(int id, int nthr) {
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthr) : "memory");
}
__device__ __forceinline__ int bar_or_n(int id, int nthr, int v) {
    uint32_t r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\t"
        "setp.ne.u32 q, %1, 0;\n\t"
        "bar.red.or.pred p, %3, %2, q;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(r)
        : "r"(v), "r"(nthr), "r"(id)
        : "memory");
    return (int)r;
}

// barrier 1 over the first nthr threads of the block (the others never wait on it)
__device__ __forceinline__ void bar_sync_1(int nthr) { asm volatile("bar.sync 1, %0;" ::"r"(nthr) : "memory"); }
// barrier 1 that also returns whether any participating thread passed v != 0
__device__ __forceinline__ int bar_or_1(int nthr, int v) {
    uint32_t r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\t"
        "setp.ne.u32 q, %1, 0;\n\t"
        "bar.red.or.pred p, 1, %2, q;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(r)
        : "r"(v), "r"(nthr)
        : "memory");
    return (int)r;
}

// one warp, converged
__device__ __forceinline__ void tmem_alloc(uint32_t dst_smem, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(dst_smem), "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// 16 consecutive 32-bit columns of the calling thread's lane (warp-collective)
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float (&v)[8]) {
    uint32_t r[8];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr)
                 : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
}

// ---------------------------------------------------------------- digit split
// x = (h + l) sc for a power of two sc (|h sc| <= 128) as d0 + d1/256 +
// d2/256^2 + d3/256^3 + O(2^-25), integer digits |d_i| <= 128.  The integer
// part of h sc by one FMA with the rounding constant 1.5 x 2^23, its exact
// remainder by another; l sc (l below half an ulp of h) is added to the
// remainder, which stays within 0.5 (plus an ulp), so the next digit rounds to
// at most 128 in magnitude.
__device__ __forceinline__ void digits4s(float h, float l, float sc, float (&d)[4]) {
    const float RND = 12582912.f;
    d[0] = __fsub_rn(__fmaf_rn(h, sc, RND), RND);
    float r = __fmaf_rn(l, sc, __fmaf_rn(h, sc, -d[0]));
#pragma unroll
    for (int k = 1; k < 4; ++k) {
        d[k] = __fsub_rn(__fmaf_rn(r, 256.f, RND), RND);
        r = __fmaf_rn(r, 256.f, -d[k]);
    }
}

// two integer-valued floats (|v| <= 256) as packed bf16 (exact: their low 16 bits are zero)
__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    return __byte_perm(__float_as_uint(lo), __float_as_uint(hi), 0x7632);
}

__device__ __forceinline__ float pow2f(int e) { return __int_as_float((127 + e) << 23); }  // -126 <= e <= 127
// 2^e, or 0 below the normal range (terms scaled that low are below 2^-102 of the sums)
__device__ __forceinline__ float pow2f_or0(int e) { return e < -126 ? 0.f : pow2f(e); }

}  // namespace cunusht
