// tc.cuh -- the tcgen05 building blocks of the radiance-cache MLP: shared
// memory operand layout, matrix and instruction descriptors, TMEM
// allocation, one CTA-wide GEMM step (M = 128 rows) and the accumulator
// read-back.
//
// Operands are bf16 in shared memory, K-major without swizzle: an M x K
// (or N x K) matrix is cut into 8-row x 8-element core matrices of 128
// contiguous bytes; the next core matrix along K is 128 bytes further (the
// descriptor's leading byte offset), the next 8-row group K/8 * 128 bytes
// further (stride byte offset). One tcgen05.mma of kind::f16 consumes 16
// elements of K, so a K = 64 product is four MMAs whose operand start
// addresses advance 256 bytes each. The fp32 accumulator lives in TMEM:
// row r of the 128-row tile is TMEM lane r, column j is TMEM column j; warp w
// reads lanes 32w..32w+31 with tcgen05.ld.
#pragma once
#include <cuda_bf16.h>
#include <cstdint>

namespace pm {

constexpr uint32_t kMbarSpin = 1u << 24;  // bound on an mbarrier wait

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

// Byte offset of element (row, k) in the K-major core-matrix layout.
__device__ __forceinline__ uint32_t core_offset(int row, int k, int K) {
    return (uint32_t)((((row >> 3) * (K >> 3) + (k >> 3)) << 7) + ((row & 7) << 4) + ((k & 7) << 1));
}

__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((saddr >> 4) & 0x3FFF) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | (1ull << 46);
}

// kind::f16 instruction descriptor: fp32 accumulate, bf16 A and B, M x N;
// a_mn / b_mn select the MN-major (transposed) form of an operand. For an
// MN-major operand without swizzle the 8 x 16-byte core matrix runs along
// M (or N); the descriptor's leading byte offset is then the distance
// between core matrices adjacent in K and the stride byte offset the
// distance between core matrices adjacent in M (N).
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N, int a_mn = 0, int b_mn = 0) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)a_mn << 15) | ((uint32_t)b_mn << 16) |
           ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mbar_init(uint64_t *mbar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(mbar)));
    asm volatile("fence.mbarrier_init.release.cluster;");
}

// Waits for the given phase, polling at most `polls` times; false when the
// bound runs out.
__device__ __forceinline__ bool mbar_wait(uint64_t *mbar, uint32_t phase, uint32_t polls = kMbarSpin) {
    uint32_t done = 0;
    for (uint32_t it = 0; it < polls && !done; ++it) {
        asm volatile(
            "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(smem_addr(mbar)), "r"(phase));
    }
    return done != 0;
}

// A wait whose first bound is `polls`: when that runs out the caller is
// told (false), and the wait goes on under the default bound so that the
// copy or MMA it waits for is no longer in flight when the caller stops.
__device__ __forceinline__ bool mbar_wait_drain(uint64_t *mbar, uint32_t phase, uint32_t polls) {
    if (mbar_wait(mbar, phase, polls)) return true;
    mbar_wait(mbar, phase, kMbarSpin);
    return false;
}

// Warp-collective: allocates `cols` TMEM columns and writes their address
// to *dst (shared memory).
__device__ __forceinline__ void tmem_alloc(uint32_t *dst, uint32_t cols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(dst)),
                 "r"(cols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
}

__device__ __forceinline__ void tmem_free(uint32_t taddr, uint32_t cols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(cols));
}

// Makes this thread's generic shared-memory writes visible to the tensor
// core's async proxy and orders them before a CTA barrier.
__device__ __forceinline__ void publish_smem() {
    asm volatile("fence.proxy.async.shared::cta;");
    asm volatile("tcgen05.fence::before_thread_sync;");
}
__device__ __forceinline__ void after_sync() { asm volatile("tcgen05.fence::after_thread_sync;"); }

// Bulk copy of `bytes` (a multiple of 16, both addresses 16-byte aligned)
// from global to shared memory, completing on mbar: the calling thread
// arms mbar with the byte count, the copy engine completes the phase.
__device__ __forceinline__ void bulk_load(void *dst_smem, const void *src_gmem, uint32_t bytes,
                                          uint64_t *mbar) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(mbar)),
                 "r"(bytes)
                 : "memory");
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dst_smem)),
        "l"(src_gmem), "r"(bytes), "r"(smem_addr(mbar))
        : "memory");
}

// Barrier over the `count` threads of named barrier `id` (1..15).
__device__ __forceinline__ void named_sync(uint32_t id, uint32_t count) {
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(count) : "memory");
}

// One tcgen05.mma of kind::f16 (K = 16): D (TMEM) = A * B^T, or D += A * B^T
// when accumulate is set.
__device__ __forceinline__ void mma_bf16(uint32_t taddr, uint64_t adesc, uint64_t bdesc,
                                         uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(taddr),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
}

// Arrives on mbar once every tcgen05.mma this thread issued has completed.
__device__ __forceinline__ void mma_commit(uint64_t *mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
        smem_addr(mbar)));
}

// D[128 x N] (TMEM at taddr) = A[128 x K] * B[N x K]^T, issued by one
// thread; completion arrives on mbar.
__device__ __forceinline__ void mma_issue(uint32_t taddr, uint32_t a, uint32_t b, int K, int N,
                                          uint64_t *mbar) {
    const uint32_t idesc = idesc_bf16(128, N);
    const uint32_t sbo = (uint32_t)(K >> 3) << 7;
    for (int s = 0; s < (K >> 4); ++s) {
        const uint64_t ad = smem_desc(a + s * 256, 128, sbo);
        const uint64_t bd = smem_desc(b + s * 256, 128, sbo);
        const uint32_t acc = s > 0 ? 1u : 0u;
        asm volatile(
            "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(taddr),
            "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
    }
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
        smem_addr(mbar)));
}

// This thread's accumulator row, 16 columns from col. A warp reaches the
// TMEM lanes of its quarter of the SM sub-partitions: lanes 32 * (warp % 4)
// onward, so thread t of a 128-thread group reads row t % 128.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, int col, float *v) {
    const uint32_t warp = (threadIdx.x >> 5) & 3u;
    const uint32_t a = taddr + ((warp * 32u) << 16) + (uint32_t)col;
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
          "=r"(r[14]), "=r"(r[15])
        : "r"(a));
    asm volatile("tcgen05.wait::ld.sync.aligned;");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

}  // namespace pm
