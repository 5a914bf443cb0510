// kifi_tc_gemm.cu -- BF16 GEMM on the 5th-generation tensor cores (tcgen05)
// with FP32 accumulation in TMEM, the building block of the pose proposer's
// forward and backward passes:
//
//   C[m][n] (+)= sum_k A[m][k] * B[n][k]      A: M x K, B: N x K (both BF16,
//                                             K contiguous), C: FP32
//
// A CTA of 4 warps owns a 128 x BN tile of C.  For each 64-deep chunk of K
// all threads stage A's 128 x 64 and B's BN x 64 slices in shared memory in
// the canonical no-swizzle K-major layout (kifi_tc.cuh), one thread issues
// four 128 x BN x 16 MMAs into the TMEM accumulator and commits them to an
// mbarrier, and the CTA waits on it before restaging.  Warp w then reads
// TMEM lanes 32w..32w+31 (rows of the tile) with tcgen05.ld and writes C,
// or adds into C atomically when K is split across blockIdx.z.  Every wait is
// bounded; a wait that gives up raises bit 1 of *status.
//
// K, the leading dimensions and the split size must be multiples of 8 (one
// 16-byte chunk never straddles the end of K) and A, B 16-byte aligned.
#include <cuda_bf16.h>

#include "kifi_internal.h"
#include "kifi_tc.cuh"

namespace kifi {
namespace {

constexpr int kBM = 128, kBK = 64;
constexpr uint32_t kLBO = 128;              // K-adjacent core matrices
constexpr uint32_t kSBO = (kBK / 8) * 128;  // next group of 8 rows
constexpr uint32_t kMaxPolls = 1u << 24;

template <int BN>
__global__ void __launch_bounds__(128) k_gemm_bf16(const __nv_bfloat16* __restrict__ A,
                                                   const __nv_bfloat16* __restrict__ B, float* __restrict__ C,
                                                   int M, int N, int K, int lda, int ldb, int ldc, int k_split,
                                                   int atomic, unsigned int* __restrict__ status) {
    __shared__ __align__(1024) unsigned char sA[kBM * kBK * 2];
    __shared__ __align__(1024) unsigned char sB[BN * kBK * 2];
    __shared__ __align__(8) uint64_t bar;
    __shared__ uint32_t tslot;
    constexpr uint32_t kCols = BN < 32 ? 32 : BN;
    constexpr uint32_t kIdesc = tc::idesc_bf16_f32(kBM, BN);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int m0 = blockIdx.x * kBM, n0 = blockIdx.y * BN;
    const int kb = blockIdx.z * k_split;
    const int ke = min(K, kb + k_split);
    if (warp == 0) tc::tmem_alloc(&tslot, kCols);
    if (tid == 0) {
        tc::mbar_init(&bar, 1);
        tc::fence_async_smem();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = tslot;
    const uint32_t a_base = tc::smem_u32(sA), b_base = tc::smem_u32(sB);
    uint32_t phase = 0;
    bool ok = true;
    for (int k0 = kb; k0 < ke; k0 += kBK) {
        // 16-byte chunks: chunk c = (row r, k group g), 8 chunks per row
        for (int c = tid; c < kBM * 8; c += 128) {
            const int r = c >> 3, g = c & 7, gm = m0 + r, gk = k0 + 8 * g;
            uint4 v = make_uint4(0u, 0u, 0u, 0u);
            if (gm < M && gk < ke) v = *reinterpret_cast<const uint4*>(A + (size_t)gm * lda + gk);
            *reinterpret_cast<uint4*>(sA + (r >> 3) * kSBO + g * kLBO + (r & 7) * 16) = v;
        }
        for (int c = tid; c < BN * 8; c += 128) {
            const int r = c >> 3, g = c & 7, gn = n0 + r, gk = k0 + 8 * g;
            uint4 v = make_uint4(0u, 0u, 0u, 0u);
            if (gn < N && gk < ke) v = *reinterpret_cast<const uint4*>(B + (size_t)gn * ldb + gk);
            *reinterpret_cast<uint4*>(sB + (r >> 3) * kSBO + g * kLBO + (r & 7) * 16) = v;
        }
        tc::fence_async_smem();
        __syncthreads();
        if (tid == 0) {
            tc::fence_after_sync();
#pragma unroll
            for (int s = 0; s < kBK / 16; ++s)
                tc::mma_bf16(tmem, tc::smem_desc(a_base + s * 2 * kLBO, kLBO, kSBO),
                             tc::smem_desc(b_base + s * 2 * kLBO, kLBO, kSBO), kIdesc, k0 > kb || s > 0);
            tc::mma_commit(&bar);
        }
        const bool waited = tc::mbar_wait(&bar, phase, kMaxPolls);
        // one decision for the whole CTA (the barrier also guards restaging)
        if (__syncthreads_or(!waited)) {
            tc::mbar_wait(&bar, phase, kMaxPolls);  // give the MMAs in flight a last bounded chance
            ok = false;
            break;
        }
        phase ^= 1u;
    }
    if (!ok) {
        if (tid == 0 && status) atomicOr(status, 2u);
    } else if (kb < ke) {
        tc::fence_after_sync();
        const int row = m0 + warp * 32 + lane;
#pragma unroll
        for (int c0 = 0; c0 < BN; c0 += 16) {
            float v[16];
            tc::tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
            if (row < M) {
                float* out = C + (size_t)row * ldc + n0 + c0;
#pragma unroll
                for (int j = 0; j < 16; ++j)
                    if (n0 + c0 + j < N) {
                        if (atomic) atomicAdd(out + j, v[j]);
                        else out[j] = v[j];
                    }
            }
        }
    } else if (!atomic) {  // empty K range: C = 0
        const int row = m0 + warp * 32 + lane;
        if (row < M)
            for (int j = 0; j < BN && n0 + j < N; ++j) C[(size_t)row * ldc + n0 + j] = 0.0f;
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, kCols);
}

}  // namespace

cudaError_t gemm_bf16_enqueue(const void* A, const void* B, float* C, int M, int N, int K, int lda, int ldb,
                              int ldc, int k_split, bool atomic, unsigned int* status, cudaStream_t st) {
    if (k_split <= 0) k_split = K;
    const int zs = (K + k_split - 1) / k_split;
    const dim3 grid_m((M + kBM - 1) / kBM, 1, zs > 0 ? zs : 1);
    const __nv_bfloat16* a = (const __nv_bfloat16*)A;
    const __nv_bfloat16* b = (const __nv_bfloat16*)B;
    if (N <= 16) {
        k_gemm_bf16<16><<<grid_m, 128, 0, st>>>(a, b, C, M, N, K, lda, ldb, ldc, k_split, atomic, status);
    } else if (N <= 32) {
        k_gemm_bf16<32><<<grid_m, 128, 0, st>>>(a, b, C, M, N, K, lda, ldb, ldc, k_split, atomic, status);
    } else if (N <= 64) {
        k_gemm_bf16<64><<<grid_m, 128, 0, st>>>(a, b, C, M, N, K, lda, ldb, ldc, k_split, atomic, status);
    } else {
        dim3 g = grid_m;
        g.y = (N + 127) / 128;
        k_gemm_bf16<128><<<g, 128, 0, st>>>(a, b, C, M, N, K, lda, ldb, ldc, k_split, atomic, status);
    }
    return cudaGetLastError();
}

}  // namespace kifi
