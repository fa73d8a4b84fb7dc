// to_tc.cuh - fifth-generation tensor core (tcgen05) primitives for sm_103a:
// shared-memory matrix descriptors, instruction descriptors, TMEM
// allocation, MMA issue/commit, bounded mbarrier waits and TMEM loads.
//
// Operand tiles are K-major with no swizzle: the tile is cut into "core
// matrices" of 8 rows x 16 bytes (128 contiguous bytes, row r at 16*r).
// Core matrix (row group g, K chunk c) sits at g*SBO + c*LBO; here LBO =
// 128 (K chunks of a row group adjacent) and SBO = 8 * (bytes of K per row),
// one full row group.  One MMA consumes 32 bytes of K (16 bf16 or 8 tf32
// elements), so K step s starts 2*LBO*s = 256*s bytes into the tile.
#pragma once
#include <cstdint>

namespace to_tc {

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// byte offset of element (r, k) in a K-major tile with kbytes bytes of K
// per row (a multiple of 16); es = element bytes
__device__ __forceinline__ uint32_t kmaj_off(int r, int k, int kbytes, int es) {
    const int kb = k * es;
    return (uint32_t)((r >> 3) * (kbytes * 8) + (kb >> 4) * 128 + (r & 7) * 16 + (kb & 15));
}

// tcgen05 shared memory descriptor, no swizzle (layout type 0), version 1
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((saddr & 0x3FFFF) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | (1ull << 46);
}

// instruction descriptor: FP32 accumulate, K-major A and B, M x N
// ab = 1: bf16 operands (kind::f16); ab = 2: tf32 operands (kind::tf32)
__host__ __device__ constexpr uint32_t idesc(uint32_t ab, int M, int N) {
    return (1u << 4) | (ab << 7) | (ab << 10) | ((uint32_t)(N >> 3) << 17) |
           ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t ad, uint64_t bd,
                                         uint32_t id, uint32_t accumulate) {
    asm volatile("{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
                 "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}"
                 :: "r"(tmem_d), "l"(ad), "l"(bd), "r"(id), "r"(accumulate));
}

__device__ __forceinline__ void mma_tf32(uint32_t tmem_d, uint64_t ad, uint64_t bd,
                                         uint32_t id, uint32_t accumulate) {
    asm volatile("{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
                 "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}"
                 :: "r"(tmem_d), "l"(ad), "l"(bd), "r"(id), "r"(accumulate));
}

// arrive on the mbarrier once every MMA this thread issued has completed
__device__ __forceinline__ void commit(void* mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                 :: "r"(smem_u32(mbar)) : "memory");
}

__device__ __forceinline__ void mbar_init(void* mbar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(smem_u32(mbar)), "r"(count));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Wait for phase `parity` of the mbarrier to complete.  Bounded: gives up
// after about 0.2 s of global time and returns false.
// bounded wait on a phase of an mbarrier: gives up after limit_ns of global
// time (or 2^24 polls) and returns false
__device__ __forceinline__ bool mbar_wait_limit(void* mbar, uint32_t parity, uint64_t limit_ns) {
    const uint32_t addr = smem_u32(mbar);
    uint64_t t0;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
    for (int it = 0; it < (1 << 24); ++it) {
        uint32_t done;
        asm volatile("{\n.reg .pred P1;\nmbarrier.try_wait.parity.shared::cta.b64 P1, [%1], %2;\n"
                     "selp.b32 %0, 1, 0, P1;\n}"
                     : "=r"(done) : "r"(addr), "r"(parity) : "memory");
        if (done) return true;
        uint64_t t1;
        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t1));
        if (t1 - t0 > limit_ns) return false;
    }
    return false;
}
__device__ __forceinline__ bool mbar_wait(void* mbar, uint32_t parity) {
    return mbar_wait_limit(mbar, parity, 200000000ull);
}

// generic-proxy smem writes -> visible to the tensor core (async proxy)
__device__ __forceinline__ void fence_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void fence_before_sync() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after_sync() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// TMEM allocation by one full warp; the column base is written to *slot
template <int NCOLS>
__device__ __forceinline__ void tmem_alloc(uint32_t* slot) {
    static_assert(NCOLS >= 32 && NCOLS <= 512 && (NCOLS & (NCOLS - 1)) == 0, "TMEM columns");
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                 :: "r"(smem_u32(slot)), "r"(NCOLS) : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
template <int NCOLS>
__device__ __forceinline__ void tmem_free(uint32_t base) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;"
                 :: "r"(base), "r"(NCOLS) : "memory");
}

// 16 consecutive FP32 columns of this thread's TMEM lane (warp w of the
// warpgroup reads lanes 32w..32w+31): taddr = base + (32w << 16) + col
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
    uint32_t r[16];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 "
                 "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]),
                   "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]),
                   "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int j = 0; j < 16; ++j) v[j] = __uint_as_float(r[j]);
}

__device__ __forceinline__ uint32_t lane_addr(uint32_t base, int warp_in_group, int col) {
    return base + ((uint32_t)(warp_in_group * 32) << 16) + (uint32_t)col;
}

}  // namespace to_tc
