// tcgen05 building blocks shared by the tensor-core kernels: shared-memory
// matrix descriptors for the canonical no-swizzle and the 128-byte swizzled
// K-major layouts, the kind::f16 instruction descriptor, MMA issue and
// commit, bounded mbarrier waits, the tcgen05 fences and TMEM loads.
//
// Layout: a K-major operand of R rows and a K chunk of KC 16-bit elements is
// stored as 8-row x 16-byte core matrices; core matrix (r / 8, k / 8) sits at
// ((r / 8) * (KC / 8) + k / 8) * 128 bytes, row r % 8 at 16 bytes each. So the
// core matrices adjacent in K are 128 bytes apart (the descriptor's leading
// byte offset) and adjacent 8-row groups KC * 16 bytes apart (its stride byte
// offset). One MMA consumes K = 16 (two core matrices): the K step s starts
// 256 * s bytes into the operand.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace rv {
namespace tc {

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Byte offset of element (r, k) in a K-major operand with a K chunk of kc.
__device__ __forceinline__ uint32_t core_offset(uint32_t r, uint32_t k, uint32_t kc) {
    return ((r >> 3) * (kc >> 3) + (k >> 3)) * 128u + (r & 7u) * 16u + (k & 7u) * 2u;
}

// Shared-memory matrix descriptor (version 1, no swizzle, base offset 0).
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t sbo_bytes) {
    return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)(128u >> 4) << 16) |
           ((uint64_t)((sbo_bytes >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// The 128-byte swizzled K-major layout for a K chunk of 64 16-bit elements
// (one 128-byte row per operand row): row r at r * 128 bytes, its sixteen-
// byte piece j stored at piece j ^ (r % 8). Eight-row groups are 1024 bytes
// apart (the stride byte offset); an operand must start on a 1024-byte
// boundary, and the K step s of an MMA starts 32 * s bytes in.
__device__ __host__ __forceinline__ uint32_t sw128_offset(uint32_t r, uint32_t k) {
    return r * 128u + ((((k >> 3) ^ r) & 7u) << 4) + (k & 7u) * 2u;
}

// Shared-memory matrix descriptor (version 1) for the 128-byte swizzled
// K-major layout: stride byte offset 1024, leading byte offset unused (1).
__device__ __forceinline__ uint64_t smem_desc_sw128(uint32_t addr) {
    return (uint64_t)((addr >> 4) & 0x3FFFu) | (1ull << 16) | ((uint64_t)(1024u >> 4) << 32) | (1ull << 46) |
           (2ull << 61);
}

// kind::f16 instruction descriptor: FP32 accumulator, A and B of type
// `ab` (0 = FP16, 1 = BF16) both K-major, shape m x n.
__host__ __device__ constexpr uint32_t instr_desc_f16(uint32_t ab, uint32_t m, uint32_t n) {
    return (1u << 4) | (ab << 7) | (ab << 10) | ((n >> 3) << 17) | ((m >> 4) << 24);
}

__device__ __forceinline__ void mma_f16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate));
}

// The mbarrier at `mbar` completes one phase when every MMA this thread has
// issued so far has finished.
__device__ __forceinline__ void commit(uint32_t mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar) : "memory");
}

__device__ __forceinline__ void mbar_init(uint32_t mbar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(mbar), "r"(count));
}

__device__ __forceinline__ void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

// Polls the phase with parity `parity` at most `limit` times; false when the
// limit ran out first.
__device__ __forceinline__ bool wait_parity(uint32_t mbar, uint32_t parity, uint32_t limit) {
    for (uint32_t i = 0; i < limit; ++i) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(mbar), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// Generic-proxy writes to shared memory become visible to the tensor cores.
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// Warp-wide: `cols` TMEM columns (a power of two >= 32) allocated, address
// written to shared memory at `slot`.
__device__ __forceinline__ void tmem_alloc(uint32_t slot, uint32_t cols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(slot), "r"(cols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t tmem, uint32_t cols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(cols));
}

// Warp-wide: 16 consecutive FP32 columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

}  // namespace tc
}  // namespace rv
