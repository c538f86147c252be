// tc.cuh -- Blackwell tensor-core building blocks used by the convolution kernels: tcgen05
// MMA descriptors, TMEM allocation and loads, mbarrier waits with iteration limits, cp.async.
//
// Operand layout in shared memory (K-major, no swizzle): an R x K BF16 operand is a grid of
// "core matrices" of 8 rows x 8 elements (8 x 16 bytes, stored contiguously, row by row);
// core matrix (r/8, k/8) starts at ((r/8) * (K/8) + k/8) * 128 bytes.  Core matrices adjacent
// in K are 128 bytes apart (leading byte offset), those adjacent in R are K/8 * 128 bytes
// apart (stride byte offset).  One tcgen05.mma of kind::f16 consumes K = 16.
#pragma once

#include <cstdint>

#include <cuda_bf16.h>

namespace scihpc {
namespace tc {

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// shared-memory matrix descriptor: start address, leading / stride byte offsets, the
// descriptor version bit (46) and no swizzling
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= uint64_t((saddr & 0x3FFFF) >> 4);
    d |= uint64_t((lbo & 0x3FFFF) >> 4) << 16;
    d |= uint64_t((sbo & 0x3FFFF) >> 4) << 32;
    d |= uint64_t(1) << 46;
    return d;
}

// instruction descriptor, kind::f16: FP32 accumulator, BF16 A and B, both K-major, M x N
__host__ __device__ constexpr uint32_t idesc_bf16(int m, int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | (uint32_t(n >> 3) << 17) | (uint32_t(m >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void commit(uint64_t *mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(mbar))
                 : "memory");
}

__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// make generic-proxy shared-memory writes (st.shared, cp.async) visible to the tensor core
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// one warp allocates ncols (power of two, >= 32) TMEM columns; the address lands in *dst
__device__ __forceinline__ void tmem_alloc(uint32_t *dst, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)), "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_free(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// 8 consecutive FP32 columns of this thread's TMEM lane (warp w reads lanes 32w .. 32w+31)
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float (&v)[8]) {
    uint32_t r[8];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int q = 0; q < 8; ++q) v[q] = __uint_as_float(r[q]);
}

__device__ __forceinline__ void mbar_init(uint64_t *mbar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(mbar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Wait until the barrier completes the phase of the given parity.  Gives up after `limit`
// polls (returns false) so that a lost arrival ends in an error status, not a hang.
__device__ __forceinline__ bool mbar_wait(uint64_t *mbar, uint32_t parity, int limit = 1 << 24) {
    uint32_t done = 0;
    for (int it = 0; it < limit; ++it) {
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(smem_u32(mbar)), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

// the next phase of the barrier completes after one arrival and `bytes` of transaction data
__device__ __forceinline__ void mbar_expect_tx(uint64_t *mbar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(mbar)), "r"(bytes)
                 : "memory");
}

// TMA: one box of a 3D tensor map (x innermost) into shared memory, completing on `mbar`.
// The box may start at negative or out-of-range coordinates (zero fill there); x times the
// element size must be a multiple of 16 bytes.
__device__ __forceinline__ void tma_load_3d(void *smem, const void *tmap, int x, int y, int z, uint64_t *mbar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(
            smem_u32(smem)),
        "l"(tmap), "r"(x), "r"(y), "r"(z), "r"(smem_u32(mbar))
        : "memory");
}

// 16-byte asynchronous copy global -> shared; src_bytes 0 zero-fills the destination
__device__ __forceinline__ void cp16(void *smem, const void *gmem, uint32_t src_bytes) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(smem_u32(smem)), "l"(gmem), "r"(src_bytes)
                 : "memory");
}
// 4-byte asynchronous copy global -> shared (no alignment beyond the element's)
__device__ __forceinline__ void cp4(void *smem, const void *gmem) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(smem_u32(smem)), "l"(gmem) : "memory");
}
// 8-byte asynchronous copy global -> shared (both 8-byte aligned)
__device__ __forceinline__ void cp8(void *smem, const void *gmem) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(smem_u32(smem)), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

}  // namespace tc
}  // namespace scihpc
