// Fifth-generation tensor-core (tcgen05) building blocks for sm_103a, as inline PTX:
// tensor-memory (TMEM) allocation, shared-memory matrix descriptors, the single-thread MMA
// issue, completion through an mbarrier, and TMEM -> register loads.
//
// Operand layout.  Operands live in shared memory without swizzling, as "core matrices" of 8 rows
// x 16 bytes (8 x 8 16-bit elements, 128 contiguous bytes).  For a K-major operand a core matrix
// holds 8 rows (M or N) x 8 consecutive K values; for an MN-major operand it holds 8 consecutive K
// values as rows, each row 8 consecutive M (or N) values.  The descriptor gives the byte distance
// between core matrices adjacent along K (leading-dimension offset, LBO) and along M / N
// (stride-dimension offset, SBO).  The helpers k_major_offset / mn_major_offset below place an
// element in the layouts every kernel here uses.
//
// Accumulators: an M = 128 MMA writes row i of D to TMEM lane i, column j of D to TMEM column
// base + j (FP32).  A warp may read only the 32 lanes of its quarter (warp id % 4).
//
// Every wait on an mbarrier is bounded: a kernel that gives up records an error and still
// releases its TMEM, so a fault in the pipeline ends the launch instead of hanging the GPU.
#pragma once

#include <cstdint>

namespace uwg {
namespace tc {

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// 64-bit shared-memory matrix descriptor (no swizzle): start address, LBO and SBO in 16-byte
// units, descriptor version 1 at bits 46-47, layout type 0 (no swizzle) at bits 61-63.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo_bytes, uint32_t sbo_bytes) {
    uint64_t d = (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)((lbo_bytes & 0x3FFFFu) >> 4) << 16;
    d |= (uint64_t)((sbo_bytes & 0x3FFFFu) >> 4) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

// 32-bit instruction descriptor of kind::f16: D in FP32 (bits 4-5 = 1), A and B of format `fmt`
// (0 = FP16, 1 = BF16; bits 7-9 and 10-12), A / B major (bit 15 / 16: 0 = K-major, 1 = MN-major),
// N >> 3 at bits 17-22, M >> 4 at bits 24-28.
__host__ __device__ constexpr uint32_t idesc_f16(int M, int N, int fmt, int a_mn, int b_mn) {
    return (1u << 4) | ((uint32_t)fmt << 7) | ((uint32_t)fmt << 10) | ((uint32_t)a_mn << 15) |
           ((uint32_t)b_mn << 16) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}
constexpr int kFmtF16 = 0;
constexpr int kFmtBF16 = 1;

// Byte offset of element (r, k) (r along M / N, k along K) of a K-major operand of `kdim` K values
// per row: core matrices adjacent along K are 128 bytes apart (LBO = 128), row groups of 8 are
// kdim * 16 bytes apart (SBO = kdim * 16).
__host__ __device__ constexpr uint32_t k_major_offset(int r, int k, int kdim) {
    return (uint32_t)((r >> 3) * (kdim * 16) + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2);
}
// Byte offset of element (r, k) of an MN-major operand of `rdim` rows (M or N): core matrices
// adjacent along M / N are 128 bytes apart (SBO = 128), K groups of 8 are rdim * 16 bytes apart
// (LBO = rdim * 16).
__host__ __device__ constexpr uint32_t mn_major_offset(int r, int k, int rdim) {
    return (uint32_t)((k >> 3) * (rdim * 16) + (r >> 3) * 128 + (k & 7) * 16 + (r & 7) * 2);
}
// Descriptors of the K step s (K values 16 s .. 16 s + 15) of an operand laid out as above.
__device__ __forceinline__ uint64_t k_major_desc(uint32_t base, int s, int kdim) {
    return smem_desc(base + (uint32_t)s * 256u, 128u, (uint32_t)kdim * 16u);
}
__device__ __forceinline__ uint64_t mn_major_desc(uint32_t base, int s, int rdim) {
    return smem_desc(base + (uint32_t)s * 2u * (uint32_t)rdim * 16u, (uint32_t)rdim * 16u, 128u);
}

// ---- TMEM allocation (one whole warp executes these) ----
__device__ __forceinline__ void tmem_alloc(uint32_t* smem_dst, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(smem_dst)),
                 "r"(ncols)
                 : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// ---- ordering ----
__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// generic-proxy shared-memory writes made visible to the tensor core (async proxy)
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// ---- mbarrier ----
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Waits for the phase with parity `parity` to complete; false after `limit` polls (each poll
// suspends for a bounded, implementation-defined time).
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, uint32_t limit = (1u << 22)) {
    for (uint32_t i = 0; i < limit; ++i)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// ---- MMA: D[tmem] (+)= A[smem] * B[smem]^T, issued by one thread ----
__device__ __forceinline__ void mma_f16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                        uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
        "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
        : "memory");
}
// The mbarrier receives one arrival when every MMA issued so far by this thread has completed.
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

// ---- TMEM -> registers: this thread's lane, 8 / 16 consecutive 32-bit columns ----
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, uint32_t r[8]) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr)
                 : "memory");
}
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t r[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// TMEM address of lane `lane`, column `col` relative to an allocation at `base`
__device__ __forceinline__ uint32_t tmem_addr(uint32_t base, int lane, int col) {
    return base + ((uint32_t)lane << 16) + (uint32_t)col;
}

// Smallest power of two >= n and >= 32 (TMEM allocations are 32..512 columns, powers of two).
__host__ __device__ constexpr uint32_t tmem_cols(int n) {
    return n <= 32 ? 32u : n <= 64 ? 64u : n <= 128 ? 128u : n <= 256 ? 256u : 512u;
}

}  // namespace tc
}  // namespace uwg
