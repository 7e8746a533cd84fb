// Fifth-generation tensor core (tcgen05) building blocks for sm_103a:
// BF16 x BF16 -> FP32 tiles with the accumulator in tensor memory (TMEM).
//
// Operands live in shared memory in the K-major, no-swizzle canonical
// layout: an R x K tile (R a multiple of 8, K a multiple of 16) is a grid of
// 8-row x 8-element "core matrices" of 128 contiguous bytes (row stride 16 B);
// core matrix (rb, kb) sits at byte (rb * K/8 + kb) * 128.  In the matrix
// descriptor the leading-dimension byte offset (LBO) is therefore the step
// between K-adjacent core matrices (128 B) and the stride-dimension byte
// offset (SBO) the step between 8-row groups (K * 16 B).  One
// tcgen05.mma of shape M=128 x N x K=16 consumes two core-matrix columns, so
// K step s starts 256 * s bytes into the tile.
//
// The D accumulator (M = 128, cta_group::1) maps row i to TMEM lane i and
// column j to TMEM column j; warp w of the CTA reads lanes 32w..32w+31 with
// tcgen05.ld.32x32b.
//
// Every wait on an mbarrier is bounded: on timeout the caller records an
// error and leaves without touching the accumulator further.
#pragma once
#include <cstdint>

namespace ertgb {
namespace umma {

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

// byte offset of element (r, k) of an R x K bf16 tile in the canonical layout
__device__ __forceinline__ uint32_t kmajor_offset(int r, int k, int K) {
    return ((uint32_t)(((r >> 3) * (K >> 3) + (k >> 3))) << 7) + ((uint32_t)(r & 7) << 4) + ((uint32_t)(k & 7) << 1);
}

// byte offset of the 16-byte chunk (r, 8c .. 8c+7)
__device__ __forceinline__ uint32_t kmajor_chunk(int r, int c, int K) {
    return ((uint32_t)(((r >> 3) * (K >> 3) + c)) << 7) + ((uint32_t)(r & 7) << 4);
}

__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = (uint64_t)((addr & 0x3FFFFu) >> 4);
    d |= (uint64_t)((lbo & 0x3FFFFu) >> 4) << 16;
    d |= (uint64_t)((sbo & 0x3FFFFu) >> 4) << 32;
    d |= (uint64_t)1 << 46;  // descriptor version of tcgen05
    return d;                 // base offset 0, relative LBO, no swizzle
}

// instruction descriptor of kind::f16: A, B bf16 (K-major), D fp32
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void fence_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void fence_before() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// whole warp; writes the TMEM base address to *dst
__device__ __forceinline__ void tmem_alloc(uint32_t *dst, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
// whole warp
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void mbar_init(uint64_t *mbar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(mbar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// bounded wait for the phase with the given parity to complete
__device__ __forceinline__ bool mbar_wait(uint64_t *mbar, uint32_t parity, uint32_t limit) {
    const uint32_t a = smem_u32(mbar);
    for (uint32_t it = 0; it < limit; ++it) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.b32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

// one elected thread: D (+)= A * B^T over one K=16 step
__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

// one elected thread: arrive on mbar when all earlier MMAs of this thread finish
__device__ __forceinline__ void mma_commit(uint64_t *mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                     smem_u32(mbar))
                 : "memory");
}

// Issue the K loop of an M=128 x N tile: A is 128 x K, B is N x K, both in the
// canonical layout at smem byte addresses a_addr / b_addr.
__device__ __forceinline__ void mma_tile(uint32_t tmem_d, uint32_t a_addr, uint32_t b_addr, int N, int K,
                                         bool accumulate) {
    const uint32_t idesc = idesc_bf16(128, N);
    const uint32_t sbo = (uint32_t)K * 16u;
    for (int s = 0; s < K / 16; ++s) {
        const uint64_t ad = smem_desc(a_addr + 256u * s, 128u, sbo);
        const uint64_t bd = smem_desc(b_addr + 256u * s, 128u, sbo);
        mma_bf16(tmem_d, ad, bd, idesc, (accumulate || s > 0) ? 1u : 0u);
    }
}

// 32 consecutive fp32 columns of this thread's lane (row)
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float *v) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

}  // namespace umma
}  // namespace ertgb
