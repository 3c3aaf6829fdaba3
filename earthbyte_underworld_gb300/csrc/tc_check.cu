// Self-check of the tcgen05 building blocks (tc.cuh): one 128 x N x K product D = A B^T computed
// by a single CTA on the tensor core and returned to the host, for the operand layouts the
// library's tensor-core kernels use.  A test compares it with a host product; the library's
// convolution and element-contraction kernels rely on exactly these descriptors.
#include <cstring>
#include <vector>

#include "internal.cuh"
#include "tc.cuh"

namespace uwg {
namespace {

constexpr int kRegion = 64 * 1024;   // shared-memory bytes reserved per operand

// layout: 0 = both K-major, 2 = both MN-major, 4 = A K-major and B MN-major;
// layout + 1 swaps the LBO / SBO fields of the descriptors (a diagnostic of the field order)
__global__ void __launch_bounds__(128) k_tc_check(int layout, int fmt, int N, int K, const uint16_t* __restrict__ A,
                                                  const uint16_t* __restrict__ B, float* __restrict__ D,
                                                  uint32_t* __restrict__ err) {
    extern __shared__ __align__(1024) unsigned char smem[];
    __shared__ uint64_t bar;
    __shared__ uint32_t tbase;
    const int M = 128;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const bool swap = layout & 1;
    const bool a_mn = (layout & ~1) == 2, b_mn = (layout & ~1) >= 2;
    const uint32_t ncols = tc::tmem_cols(N);
    if (warp == 0) {
        tc::tmem_alloc(&tbase, ncols);
        tc::tmem_relinquish();
    }
    if (threadIdx.x == 0) tc::mbar_init(&bar, 1);
    for (int i = threadIdx.x; i < 2 * kRegion / 16; i += blockDim.x) reinterpret_cast<uint4*>(smem)[i] = make_uint4(0, 0, 0, 0);
    __syncthreads();
    for (int i = threadIdx.x; i < M * K; i += blockDim.x) {
        const int r = i / K, k = i % K;
        const uint32_t off = a_mn ? tc::mn_major_offset(r, k, M) : tc::k_major_offset(r, k, K);
        *reinterpret_cast<uint16_t*>(smem + off) = A[i];
    }
    for (int i = threadIdx.x; i < N * K; i += blockDim.x) {
        const int r = i / K, k = i % K;
        const uint32_t off = b_mn ? tc::mn_major_offset(r, k, N) : tc::k_major_offset(r, k, K);
        *reinterpret_cast<uint16_t*>(smem + kRegion + off) = B[i];
    }
    tc::fence_proxy_async();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t taddr = tbase;
    if (threadIdx.x == 0) {
        const uint32_t idesc = tc::idesc_f16(M, N, fmt, a_mn ? 1 : 0, b_mn ? 1 : 0);
        const uint32_t sa = tc::smem_u32(smem), sb = tc::smem_u32(smem + kRegion);
        for (int s = 0; s < K / 16; ++s) {
            uint64_t da = a_mn ? tc::mn_major_desc(sa, s, M) : tc::k_major_desc(sa, s, K);
            uint64_t db = b_mn ? tc::mn_major_desc(sb, s, N) : tc::k_major_desc(sb, s, K);
            if (swap) {
                // exchange the 14-bit LBO (bits 16-29) and SBO (bits 32-45) fields
                const uint64_t la = (da >> 16) & 0x3FFF, sa_ = (da >> 32) & 0x3FFF;
                const uint64_t lb = (db >> 16) & 0x3FFF, sb_ = (db >> 32) & 0x3FFF;
                da = (da & ~((0x3FFFull << 16) | (0x3FFFull << 32))) | (sa_ << 16) | (la << 32);
                db = (db & ~((0x3FFFull << 16) | (0x3FFFull << 32))) | (sb_ << 16) | (lb << 32);
            }
            tc::mma_f16(taddr, da, db, idesc, s > 0 ? 1u : 0u);
        }
        tc::mma_commit(&bar);
    }
    const bool ok = tc::mbar_wait(&bar, 0);
    if (!ok && lane == 0) atomicOr(err, 1u);
    tc::fence_after_sync();
    if (ok) {
        const int row = 32 * warp + lane;
        for (int c = 0; c < N; c += 8) {
            uint32_t r[8];
            tc::tmem_ld8(tc::tmem_addr(taddr, 32 * warp, c), r);
            tc::tmem_wait_ld();
#pragma unroll
            for (int j = 0; j < 8; ++j) D[(int64_t)row * N + c + j] = __uint_as_float(r[j]);
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) {
        tc::fence_after_sync();
        tc::tmem_dealloc(taddr, ncols);
    }
}

// Largest byte offset (exclusive) an operand of `rows` x K read through the descriptors of
// `layout` can touch: the K steps' start addresses plus the span of one step's core matrices,
// with the stride fields as the descriptor carries them.
int64_t reach(bool mn, bool swap, int rows, int K) {
    const int64_t step = mn ? 2LL * rows * 16 : 256;                 // start advance per K step
    int64_t lbo = mn ? (int64_t)rows * 16 : 128, sbo = mn ? 128 : (int64_t)K * 16;
    if (swap) std::swap(lbo, sbo);
    return (int64_t)(K / 16 - 1) * step + lbo + (int64_t)(rows / 8 - 1) * sbo + 128;
}

}  // namespace

int tc_check(int layout, int fmt, int N, int K, const uint16_t* A, const uint16_t* B, float* D) {
    const int M = 128;
    UWG_REQUIRE(layout >= 0 && layout <= 5 && (fmt == tc::kFmtF16 || fmt == tc::kFmtBF16), UWGPU_ERR_ARGUMENT,
                "tc_check: bad layout or format");
    UWG_REQUIRE(N >= 16 && N <= 256 && N % 16 == 0 && K >= 16 && K <= 256 && K % 16 == 0, UWGPU_ERR_ARGUMENT,
                "tc_check: N must be 16..256 and K 16..256, multiples of 16");
    const bool swap = layout & 1, a_mn = (layout & ~1) == 2, b_mn = (layout & ~1) >= 2;
    // every read stays inside its operand's region, whatever the field order
    UWG_REQUIRE(reach(a_mn, swap, M, K) <= kRegion && reach(b_mn, swap, N, K) <= kRegion &&
                    (int64_t)M * K * 2 <= kRegion && (int64_t)N * K * 2 <= kRegion,
                UWGPU_ERR_ARGUMENT, "tc_check: operands exceed the shared-memory regions");
    DArray<uint16_t> dA, dB;
    DArray<float> dD;
    DArray<uint32_t> dErr;
    dA.ensure((size_t)M * K);
    dB.ensure((size_t)N * K);
    dD.ensure((size_t)M * N);
    dErr.ensure(1);
    UWG_CUDA(cudaMemcpy(dA.p, A, sizeof(uint16_t) * M * K, cudaMemcpyHostToDevice));
    UWG_CUDA(cudaMemcpy(dB.p, B, sizeof(uint16_t) * N * K, cudaMemcpyHostToDevice));
    UWG_CUDA(cudaMemset(dD.p, 0, sizeof(float) * M * N));
    UWG_CUDA(cudaMemset(dErr.p, 0, sizeof(uint32_t)));
    UWG_CUDA(cudaFuncSetAttribute(k_tc_check, cudaFuncAttributeMaxDynamicSharedMemorySize, 2 * kRegion));
    k_tc_check<<<1, 128, 2 * kRegion>>>(layout, fmt, N, K, dA.p, dB.p, dD.p, dErr.p);
    check_launch("k_tc_check");
    UWG_CUDA(cudaDeviceSynchronize());
    uint32_t err = 0;
    UWG_CUDA(cudaMemcpy(&err, dErr.p, sizeof(uint32_t), cudaMemcpyDeviceToHost));
    UWG_CUDA(cudaMemcpy(D, dD.p, sizeof(float) * M * N, cudaMemcpyDeviceToHost));
    UWG_REQUIRE(err == 0, UWGPU_ERR_CUDA, "tc_check: the MMA did not complete in time");
    return UWGPU_OK;
}

}  // namespace uwg
