// Tensor-core (tcgen05) building blocks of the large-cell contraction, and a one-tile
// self-check of the MMA operand layouts against the host.
//
// Operands are BF16 in shared memory, in 8 x 16-byte core matrices without swizzle; FP32
// values are split x = hi + lo (two BF16) and a product is formed as hi*hi + hi*lo + lo*hi
// in the FP32 accumulator in tensor memory (about 16 significant bits per operand).
#include <cuda_bf16.h>

#include "tc_common.cuh"
#include "tdg_internal.cuh"

namespace tdg {

namespace {

// Byte offset of element (mn, k) in a tile of core matrices; core (mn/8, k/8) starts at
// (mn/8)*c_mn + (k/8)*c_k. MN-major: the 8 rows of a core are 8 k, each row 8 consecutive mn.
// K-major: the rows are 8 mn, each row 8 consecutive k.
__device__ __forceinline__ uint32_t core_off(int mn, int k, uint32_t c_mn, uint32_t c_k, bool k_major) {
    const uint32_t base = (uint32_t)(mn >> 3) * c_mn + (uint32_t)(k >> 3) * c_k;
    return k_major ? base + (mn & 7) * 16 + (k & 7) * 2 : base + (k & 7) * 16 + (mn & 7) * 2;
}

constexpr long long kWaitCycles = 2000000000LL;  // about 1 s at 2 GHz

// One 128 x n x 16 tile: D = A B with A 128 x 16 (row-major floats), B 16 x n. variant bit 0
// swaps the roles of the leading/stride byte offsets, bit 1 selects K-major operands.
// Every offset either reading of the descriptor can form stays inside the 227 KB of
// dynamic shared memory this kernel is launched with.
__global__ void __launch_bounds__(128) k_mma_check(int variant, int n, const float *A, const float *B, float *D,
                                                   int *status) {
    extern __shared__ __align__(1024) unsigned char sm[];
    __shared__ uint64_t mbar;
    __shared__ uint32_t tbase;
    unsigned char *a_hi = sm, *a_lo = sm + 32768, *b_hi = sm + 65536, *b_lo = sm + 73728;
    const bool swap = variant & 1, kmaj = (variant & 2) != 0;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    constexpr int M = 128, K = 16;
    const uint32_t a_cmn = 128, a_ck = (M / 8) * 128;
    const uint32_t b_cmn = 128, b_ck = (uint32_t)(n / 8) * 128;
    if (warp == 0) tc::tmem_alloc(&tbase, 256);
    for (int i = tid; i < M * K; i += blockDim.x) {
        const int m = i / K, k = i % K;
        unsigned short h, l;
        tc::split_bf16(A[i], h, l);
        const uint32_t o = core_off(m, k, a_cmn, a_ck, kmaj);
        *(unsigned short *)(a_hi + o) = h;
        *(unsigned short *)(a_lo + o) = l;
    }
    for (int i = tid; i < K * n; i += blockDim.x) {
        const int k = i / n, c = i % n;
        unsigned short h, l;
        tc::split_bf16(B[i], h, l);
        const uint32_t o = core_off(c, k, b_cmn, b_ck, kmaj);
        *(unsigned short *)(b_hi + o) = h;
        *(unsigned short *)(b_lo + o) = l;
    }
    if (tid == 0) {
        tc::mbar_init(&mbar, 1);
        tc::fence_mbar_init();
    }
    tc::fence_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t taddr = tbase;
    if (tid == 0) {
        const uint32_t idesc = tc::idesc_bf16_f32(M, n, !kmaj, !kmaj);
        const uint32_t ua[3] = {tc::smem_u32(a_hi), tc::smem_u32(a_hi), tc::smem_u32(a_lo)};
        const uint32_t ub[3] = {tc::smem_u32(b_hi), tc::smem_u32(b_lo), tc::smem_u32(b_hi)};
        for (int j = 0; j < 3; ++j) {
            const uint64_t ad = swap ? tc::smem_desc(ua[j], a_cmn, a_ck) : tc::smem_desc(ua[j], a_ck, a_cmn);
            const uint64_t bd = swap ? tc::smem_desc(ub[j], b_cmn, b_ck) : tc::smem_desc(ub[j], b_ck, b_cmn);
            tc::mma_bf16(taddr, ad, bd, idesc, j > 0 ? 1u : 0u);
        }
        tc::mma_commit(&mbar);
    }
    const bool ok = tc::mbar_wait(&mbar, 0, kWaitCycles);
    if (!ok && lane == 0) atomicExch(status, 1);
    tc::fence_after_sync();
    for (int c = 0; c < n; c += 8) {
        float v[8];
        tc::tmem_ld8(taddr + ((uint32_t)(32 * warp) << 16) + (uint32_t)c, v);
        for (int i = 0; i < 8; ++i) D[(size_t)(32 * warp + lane) * n + c + i] = v[i];
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(taddr, 256);
}

}  // namespace

cudaError_t launch_mma_check(int variant, int n, const float *a, const float *b, float *d, int *status,
                             cudaStream_t s) {
    if (n < 16 || n > 256 || n % 16 != 0) return cudaErrorInvalidValue;
    const int smem = 220 * 1024;
    cudaError_t e = cudaFuncSetAttribute(k_mma_check, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    k_mma_check<<<1, 128, smem, s>>>(variant, n, a, b, d, status);
    return cudaGetLastError();
}

}  // namespace tdg
