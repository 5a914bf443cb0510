// kifi_tc_gemm.cu -- BF16 GEMMs on the 5th-generation tensor cores (tcgen05)
// with FP32 accumulation in TMEM, the building blocks of the pose proposer's
// forward and backward passes:
//
//   C[m][n] (+)= sum_k A[m][k] * B[n][k]      A: M x K, B: N x K (both BF16,
//                                             K contiguous), C: FP32
//
// and the same product with A the implicit im2col matrix of a 3x3 / stride 2
// / pad 1 convolution over an NHWC BF16 input (A is never materialised).
//
// One persistent, warp-specialised kernel serves both.  A CTA of six warps
// walks 128 x BN tiles of C (grid-strided):
//   warp 0     one thread issues the TMA loads of each 64-deep K chunk of A
//              (and of B, unless all of B stays resident in shared memory:
//              one N tile, no K split, B small) into a ring of shared-memory
//              stages, each completing on its `full` mbarrier by transaction
//              bytes;
//   warp 1     one thread waits for a full stage, issues four 128 x BN x 16
//              tcgen05.mma into one of two TMEM accumulators and commits them
//              to the stage's `empty` mbarrier (the producer reuses the stage
//              once the MMAs that read it are done), and after a tile's last
//              chunk commits to the accumulator's `acc_full` mbarrier;
//   warps 2-5  the epilogue: wait for a finished accumulator, read TMEM lanes
//              32(w%4)..+31 with tcgen05.ld, write C (plain, atomically when
//              K is split across tiles, or as BF16 after bias and ReLU), then
//              release the accumulator through `acc_empty`.
// Loads of the next chunks and the next tile's MMAs therefore overlap the
// current MMAs and epilogue.  The host sizes the ring: two CTAs per SM where
// four stages fit in half the SM's shared memory, else one CTA with up to
// eight stages.
//
// A and B stages are written by TMA with 128-byte swizzle (rows of 64 BF16).
// The convolution's A chunk is one tap (Cin = 64: 128-byte rows) or two taps
// (Cin = 32: two 64-byte-row halves with 64-byte swizzle) of the 3x3 window:
// a 4-D tensor map over the input (C, W, H, N) with element strides
// (1, 2, 2, 1) reads, for output pixels (oy, ox) of the tile, the input
// pixels (2 oy - 1 + ky, 2 ox - 1 + kx); coordinates outside the input read
// as zeros, which is the convolution's padding.  A tile covers `th` output
// rows of one image, or `nb` whole images, so its rows are consecutive rows
// of the output matrix.
//
// Every wait is bounded.  A wait that gives up raises a CTA-wide abort flag
// that ends the other roles' waits, waits (bounded) for the copies and MMAs
// in flight, frees TMEM and raises bit 1 of *status.
//
// The leading dimensions must be multiples of 8 (tensor-map strides are
// multiples of 16 bytes), A and B 16-byte aligned.
#include <cuda.h>
#include <cuda_bf16.h>

#include <mutex>

#include "kifi_internal.h"
#include "kifi_tc.cuh"

namespace kifi {
namespace {

constexpr int kBM = 128, kBK = 64, kMaxStages = 8;
constexpr int kGemmThreads = 192;
constexpr uint32_t kMaxPolls = 1u << 24;
constexpr uint32_t kATile = kBM * kBK * 2;  // 16 KB

struct Epilogue {
    float* C;                // FP32 output (row stride ldc), unless out_bf is set
    int ldc;
    int atomic;              // add into C
    const float* bias;       // per column, or null
    int relu;
    __nv_bfloat16* out_bf;   // BF16 output bf16(relu?(acc + bias)), row stride ldc
};

// the tiles of one launch
struct Tiles {
    int M, N, K;
    int mt, nt, zs, k_split;  // plain GEMM: M tiles, N tiles, K splits
    // convolution: output rows Ho x Wo per image, th rows per tile (nb = 1)
    // or nb whole images per tile (th = Ho); tiles per image (nb = 1)
    int conv, Ho, Wo, th, nb, tpi, taps_per_chunk;
    uint32_t a_tap_bytes;  // bytes of one tap's box
    // pipeline: ring stages; B resident in shared memory (all nk_b chunks,
    // loaded once) or staged with A in every stage
    int stages, b_res, nk_b;
};

struct TileAt {
    int m0, n0, kb, ke;
    int b0, oy0;   // convolution: first image and output row
    int rows;      // tile rows that are output rows (the rest are not written)
};

__device__ __forceinline__ TileAt tile_at(const Tiles& T, int t) {
    TileAt a;
    if (T.conv) {
        a.n0 = 0;
        a.kb = 0;
        a.ke = T.K;
        if (T.nb > 1) {
            a.b0 = t * T.nb;
            a.oy0 = 0;
            a.m0 = a.b0 * T.Ho * T.Wo;
            a.rows = min(T.nb * T.Ho * T.Wo, T.M - a.m0);
        } else {
            a.b0 = t / T.tpi;
            a.oy0 = (t - a.b0 * T.tpi) * T.th;
            a.m0 = (a.b0 * T.Ho + a.oy0) * T.Wo;
            a.rows = min(T.th, T.Ho - a.oy0) * T.Wo;
        }
    } else {
        const int per_z = T.mt * T.nt;
        const int z = t / per_z, r = t - z * per_z;
        const int nti = r / T.mt;
        a.m0 = (r - nti * T.mt) * kBM;
        a.n0 = nti;  // scaled by BN by the caller
        a.kb = z * T.k_split;
        a.ke = min(T.K, a.kb + T.k_split);
        a.b0 = a.oy0 = 0;
        a.rows = min(kBM, T.M - a.m0);
    }
    return a;
}

// bounded wait that also ends when another role has given up
__device__ __forceinline__ bool wait_bar(uint64_t* bar, uint32_t parity, volatile int* abort) {
    for (uint32_t i = 0; i < kMaxPolls; ++i) {
        if (tc::mbar_try_wait(bar, parity)) return true;
        if (*abort) return false;
    }
    *abort = 1;
    return false;
}

__device__ __forceinline__ uint64_t smem_desc_sw64(uint32_t start) {
    // 64-byte swizzle: rows of 64 bytes, 8-row groups 512 bytes apart, layout type 4
    return (uint64_t)((start >> 4) & 0x3fffu) | ((uint64_t)1 << 16) | ((uint64_t)(512 >> 4) << 32) |
           ((uint64_t)1 << 46) | ((uint64_t)4 << 61);
}

template <int BN>
__device__ __forceinline__ void epilogue_store(const Epilogue& ep, const float (&v)[16], long long row, int col,
                                               int N) {
    float w[16];
#pragma unroll
    for (int j = 0; j < 16; ++j) {
        float x = v[j];
        if (ep.bias && col + j < N) x = x + ep.bias[col + j];
        if (ep.relu) x = fmaxf(x, 0.0f);
        w[j] = x;
    }
    const bool full = col + 16 <= N;
    if (ep.out_bf) {
        __nv_bfloat16* o = ep.out_bf + row * ep.ldc + col;
        if (full && ((reinterpret_cast<uintptr_t>(o) & 15u) == 0)) {
            uint4 p[2];
            uint32_t* pw = reinterpret_cast<uint32_t*>(p);
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const __nv_bfloat162 h = __floats2bfloat162_rn(w[2 * j], w[2 * j + 1]);
                pw[j] = *reinterpret_cast<const uint32_t*>(&h);
            }
            reinterpret_cast<uint4*>(o)[0] = p[0];
            reinterpret_cast<uint4*>(o)[1] = p[1];
        } else {
#pragma unroll
            for (int j = 0; j < 16; ++j)
                if (col + j < N) o[j] = __float2bfloat16_rn(w[j]);
        }
        return;
    }
    float* o = ep.C + row * ep.ldc + col;
    if (ep.atomic) {
#pragma unroll
        for (int j = 0; j < 16; ++j)
            if (col + j < N) atomicAdd(o + j, w[j]);
    } else if (full && ((reinterpret_cast<uintptr_t>(o) & 15u) == 0)) {
#pragma unroll
        for (int j = 0; j < 4; ++j)
            reinterpret_cast<float4*>(o)[j] = make_float4(w[4 * j], w[4 * j + 1], w[4 * j + 2], w[4 * j + 3]);
    } else {
#pragma unroll
        for (int j = 0; j < 16; ++j)
            if (col + j < N) o[j] = w[j];
    }
}

template <int BN>
__global__ void __launch_bounds__(kGemmThreads, 1) k_gemm_bf16_tma(const __grid_constant__ CUtensorMap tmA,
                                                                   const __grid_constant__ CUtensorMap tmB,
                                                                   const Tiles T, const Epilogue ep,
                                                                   unsigned int* __restrict__ status) {
    constexpr uint32_t kBTile = BN * kBK * 2;  // a multiple of 1024, like kATile
    constexpr uint32_t kCols = 2 * BN < 32 ? 32 : 2 * BN;
    constexpr uint32_t kIdesc = tc::idesc_bf16_f32(kBM, BN);
    extern __shared__ unsigned char gemm_mem[];
    __shared__ __align__(8) uint64_t full[kMaxStages], empty[kMaxStages], acc_full[2], acc_empty[2], b_full, drain;
    __shared__ uint32_t tslot, n_issued, n_consumed;
    __shared__ int abort_flag;
    // [resident B: nk_b chunks][stages x (A, plus B unless resident)], 1024-byte aligned
    const uint32_t base = (tc::smem_u32(gemm_mem) + 1023u) & ~1023u;
    const uint32_t ring = base + (T.b_res ? (uint32_t)T.nk_b * kBTile : 0u);
    const uint32_t stage_bytes = kATile + (T.b_res ? 0u : kBTile);
    const int S = T.stages;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int tiles = T.conv ? (T.nb > 1 ? (T.M / (T.Ho * T.Wo) + T.nb - 1) / T.nb
                                         : (T.M / (T.Ho * T.Wo)) * T.tpi)
                             : T.mt * T.nt * T.zs;
    if (warp == 0) tc::tmem_alloc(&tslot, kCols);
    if (threadIdx.x == 32) {
        for (int s = 0; s < S; ++s) {
            tc::mbar_init(&full[s], 1);
            tc::mbar_init(&empty[s], 1);
        }
        tc::mbar_init(&b_full, 1);
        for (int a = 0; a < 2; ++a) {
            tc::mbar_init(&acc_full[a], 1);
            tc::mbar_init(&acc_empty[a], 4);
        }
        tc::mbar_init(&drain, 1);
        n_issued = n_consumed = 0;
        abort_flag = 0;
        tc::fence_mbar_init();
        tc::fence_async_smem();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = tslot;
    volatile int* abort = &abort_flag;

    if (warp == 0) {
        if (lane == 0) {  // TMA producer
            uint32_t s = 0, ph = 0, issued = 0;
            if (T.b_res) {  // all of B once (a single N tile, K not split)
                tc::mbar_arrive_expect_tx(&b_full, (uint32_t)T.nk_b * kBTile);
                for (int kc = 0; kc < T.nk_b; ++kc) tc::tma_load_2d(base + kc * kBTile, &tmB, kc * kBK, 0, &b_full);
            }
            for (int t = blockIdx.x; t < tiles; t += gridDim.x) {
                const TileAt at = tile_at(T, t);
                const int nk = (at.ke - at.kb + kBK - 1) / kBK;
                for (int kc = 0; kc < nk; ++kc) {
                    if (!wait_bar(&empty[s], ph ^ 1u, abort)) goto produced;
                    const uint32_t a_dst = ring + s * stage_bytes, b_dst = a_dst + kATile;
                    const int k0 = at.kb + kc * kBK;
                    if (T.conv) {
                        uint32_t bytes = T.b_res ? 0u : kBTile;
                        int taps = 0;
                        for (int j = 0; j < T.taps_per_chunk; ++j)
                            if (kc * T.taps_per_chunk + j < 9) ++taps;
                        bytes += taps * T.a_tap_bytes;
                        tc::mbar_arrive_expect_tx(&full[s], bytes);
                        for (int j = 0; j < taps; ++j) {
                            const int tap = kc * T.taps_per_chunk + j, ky = tap / 3, kx = tap - 3 * ky;
                            tc::tma_load_4d(a_dst + j * (kATile / T.taps_per_chunk), &tmA, 0, kx - 1,
                                            2 * at.oy0 - 1 + ky, at.b0, &full[s]);
                        }
                    } else {
                        tc::mbar_arrive_expect_tx(&full[s], stage_bytes);
                        tc::tma_load_2d(a_dst, &tmA, k0, at.m0, &full[s]);
                    }
                    if (!T.b_res) tc::tma_load_2d(b_dst, &tmB, k0, at.n0 * BN, &full[s]);
                    ++issued;
                    if (++s == (uint32_t)S) {
                        s = 0;
                        ph ^= 1u;
                    }
                }
            }
        produced:
            n_issued = issued;
        }
    } else if (warp == 1) {
        if (lane == 0) {  // MMA issuer
            uint32_t s = 0, ph = 0, consumed = 0;
            int j = 0;
            const bool b_ok = !T.b_res || wait_bar(&b_full, 0, abort);
            for (int t = blockIdx.x; b_ok && t < tiles; t += gridDim.x, ++j) {
                const TileAt at = tile_at(T, t);
                const int nk = (at.ke - at.kb + kBK - 1) / kBK;
                const uint32_t acc = j & 1, aph = (j >> 1) & 1;
                if (!wait_bar(&acc_empty[acc], aph ^ 1u, abort)) break;
                tc::fence_after_sync();
                const uint32_t d = tmem + acc * BN;
                bool ok = true;
                for (int kc = 0; kc < nk; ++kc) {
                    if (!wait_bar(&full[s], ph, abort)) {
                        ok = false;
                        break;
                    }
                    ++consumed;
                    tc::fence_after_sync();
                    const uint32_t a = ring + s * stage_bytes;
                    const uint32_t b = T.b_res ? base + kc * kBTile : a + kATile;
#pragma unroll
                    for (int kk = 0; kk < kBK / 16; ++kk) {
                        uint64_t adesc;
                        if (T.conv && T.taps_per_chunk == 2) {
                            // two 64-byte-row halves, one tap each; a missing ninth-plus tap is skipped
                            if (kc * 2 + (kk >> 1) >= 9) continue;
                            adesc = smem_desc_sw64(a + (kk >> 1) * (kATile / 2) + (kk & 1) * 32);
                        } else {
                            adesc = tc::smem_desc_sw128(a + kk * 32);
                        }
                        tc::mma_bf16(d, adesc, tc::smem_desc_sw128(b + kk * 32), kIdesc, kc > 0 || kk > 0);
                    }
                    tc::mma_commit(&empty[s]);
                    if (++s == (uint32_t)S) {
                        s = 0;
                        ph ^= 1u;
                    }
                }
                if (!ok) break;
                tc::mma_commit(&acc_full[acc]);
            }
            n_consumed = consumed;
        }
    } else {  // epilogue, warps 2-5: TMEM lanes 32 (warp % 4) ..
        const int q = warp & 3;
        int j = 0;
        for (int t = blockIdx.x; t < tiles; t += gridDim.x, ++j) {
            const TileAt at = tile_at(T, t);
            const uint32_t acc = j & 1, aph = (j >> 1) & 1;
            // one decision per warp: tcgen05.ld below is warp-collective
            if (!__all_sync(0xffffffffu, wait_bar(&acc_full[acc], aph, abort))) break;
            tc::fence_after_sync();
            const int r = q * 32 + lane;
            const bool row_ok = r < at.rows;
            const long long row = (long long)at.m0 + r;
            const int n0 = at.n0 * BN;
#pragma unroll
            for (int c0 = 0; c0 < BN; c0 += 16) {
                float v[16];
                tc::tmem_ld16(tmem + ((uint32_t)(q * 32) << 16) + acc * BN + (uint32_t)c0, v);
                if (row_ok && n0 + c0 < T.N) epilogue_store<BN>(ep, v, row, n0 + c0, T.N);
            }
            tc::fence_before_sync();
            __syncwarp();
            if (lane == 0) tc::mbar_arrive(&acc_empty[acc]);
        }
    }

    __syncthreads();
    if (abort_flag) {
        if (threadIdx.x == 0) {
            // copies issued but never consumed: wait (bounded) for them to land
            for (uint32_t g = n_consumed; g < n_issued; ++g)
                tc::mbar_wait(&full[g % S], (g / S) & 1u, kMaxPolls);
            if (T.b_res) tc::mbar_wait(&b_full, 0, kMaxPolls);
            if (status) atomicOr(status, 2u);
        }
        if (threadIdx.x == 32) {  // MMAs in flight
            tc::mma_commit(&drain);
            tc::mbar_wait(&drain, 0, kMaxPolls);
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, kCols);
}

// ------------------------------------------------------------------ host

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encoder() {
    static EncodeTiledFn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (EncodeTiledFn)p;
    });
    return fn;
}

bool encode(CUtensorMap* map, const void* ptr, int rank, const cuuint64_t* dims, const cuuint64_t* strides,
            const cuuint32_t* box, const cuuint32_t* estr, CUtensorMapSwizzle sw) {
    EncodeTiledFn fn = encoder();
    if (!fn) return false;
    return fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, (cuuint32_t)rank, const_cast<void*>(ptr), dims, strides, box,
              estr, CU_TENSOR_MAP_INTERLEAVE_NONE, sw, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// rows x K (row stride ld elements), boxes of 64 x box_rows, 128-byte swizzle
bool matrix_map(CUtensorMap* map, const void* ptr, int rows, int K, int ld, int box_rows) {
    const cuuint64_t dims[2] = {(cuuint64_t)K, (cuuint64_t)rows};
    const cuuint64_t strides[1] = {(cuuint64_t)ld * 2};
    const cuuint32_t box[2] = {(cuuint32_t)kBK, (cuuint32_t)box_rows};
    const cuuint32_t estr[2] = {1, 1};
    return encode(map, ptr, 2, dims, strides, box, estr, CU_TENSOR_MAP_SWIZZLE_128B);
}

// per device: shared memory per SM and per block, reserved per block, SMs
struct DeviceLimits {
    int per_sm = 0, per_block = 0, reserved = 0, sms = 0;
};

cudaError_t device_limits(DeviceLimits* out) {
    constexpr int kMaxDevices = 64;
    static DeviceLimits cache[kMaxDevices];
    static std::once_flag once[kMaxDevices];
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    static cudaError_t err[kMaxDevices];
    std::call_once(once[dev], [&] {
        DeviceLimits& L = cache[dev];
        cudaError_t x = cudaDeviceGetAttribute(&L.per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
        if (!x) x = cudaDeviceGetAttribute(&L.per_block, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        if (!x) x = cudaDeviceGetAttribute(&L.reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev);
        if (!x) x = cudaDeviceGetAttribute(&L.sms, cudaDevAttrMultiProcessorCount, dev);
        err[dev] = x;
    });
    *out = cache[dev];
    return err[dev];
}

template <int BN>
cudaError_t launch(const CUtensorMap& a, const CUtensorMap& b, Tiles T, int tiles, const Epilogue& ep,
                   unsigned int* status, cudaStream_t st) {
    constexpr uint32_t kBTile = BN * kBK * 2;
    // the kernel's static shared memory (its barriers), the same on every device
    static size_t static_smem = 0;
    static std::once_flag once;
    static cudaError_t fa_err = cudaSuccess;
    std::call_once(once, [] {
        cudaFuncAttributes fa;
        fa_err = cudaFuncGetAttributes(&fa, k_gemm_bf16_tma<BN>);
        if (!fa_err) static_smem = fa.sharedSizeBytes;
    });
    if (fa_err) return fa_err;
    DeviceLimits L;
    cudaError_t e = device_limits(&L);
    if (e) return e;
    // per-CTA shared memory budget at `occ` CTAs per SM (1024 bytes for the alignment of the ring)
    auto budget = [&](int occ) -> long long {
        const long long x = std::min<long long>((long long)L.per_sm / occ - L.reserved, L.per_block);
        return x - (long long)static_smem - 1024;
    };
    // B stays resident when the launch has one N tile, K is not split and B
    // fits beside four stages of A with two CTAs per SM; otherwise B is staged
    // with A.  Two CTAs per SM where four stages fit, else one with a deeper ring.
    const int chunks = (T.k_split + kBK - 1) / kBK;
    T.b_res = (T.nt == 1 && T.zs == 1 && (long long)chunks * kBTile + 4ll * kATile <= budget(2)) ? 1 : 0;
    T.nk_b = T.b_res ? chunks : 0;
    const size_t fixed = (size_t)T.nk_b * kBTile;
    const size_t stage = kATile + (T.b_res ? 0 : kBTile);
    int occ = 2;
    if ((long long)(fixed + 4 * stage) > budget(2)) occ = 1;
    const long long fit = (budget(occ) - (long long)fixed) / (long long)stage;
    if (fit < 2) return cudaErrorInvalidValue;
    T.stages = (int)std::min<long long>(kMaxStages, fit);
    const size_t smem = fixed + (size_t)T.stages * stage + 1024;
    e = cudaFuncSetAttribute(k_gemm_bf16_tma<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    // the whole unified L1 as shared memory, so that `occ` CTAs share an SM
    if (!e)
        e = cudaFuncSetAttribute(k_gemm_bf16_tma<BN>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                 (int)cudaSharedmemCarveoutMaxShared);
    if (e) return e;
    const int grid = std::min(tiles, std::max(L.sms, 1) * occ);
    k_gemm_bf16_tma<BN><<<grid, kGemmThreads, smem, st>>>(a, b, T, ep, status);
    return cudaGetLastError();
}

template <int BN>
cudaError_t run(const void* A, const void* B, int M, int N, int K, int lda, int ldb, const Tiles& T0,
                const Epilogue& ep, unsigned int* status, cudaStream_t st) {
    CUtensorMap a, b;
    if (!matrix_map(&a, A, M, K, lda, kBM) || !matrix_map(&b, B, N, K, ldb, BN)) return cudaErrorInvalidValue;
    Tiles T = T0;
    T.nt = (N + BN - 1) / BN;
    return launch<BN>(a, b, T, T.mt * T.nt * T.zs, ep, status, st);
}

}  // namespace

cudaError_t gemm_bf16_enqueue(const void* A, const void* B, float* C, int M, int N, int K, int lda, int ldb,
                              int ldc, int k_split, bool atomic, unsigned int* status, cudaStream_t st,
                              const GemmEpilogue* epi) {
    if (M <= 0 || N <= 0) return cudaSuccess;
    Epilogue ep{C, ldc, atomic ? 1 : 0, nullptr, 0, nullptr};
    if (epi) {
        ep.bias = epi->bias;
        ep.relu = epi->relu ? 1 : 0;
        ep.out_bf = (__nv_bfloat16*)epi->out_bf16;
    }
    if (K <= 0) {  // an empty sum: C = 0 (or unchanged when accumulating)
        if (atomic || ep.out_bf || ep.bias) return atomic ? cudaSuccess : cudaErrorInvalidValue;
        return cudaMemset2DAsync(C, (size_t)ldc * 4, 0, (size_t)N * 4, M, st);
    }
    // K splits start on chunk boundaries, so a chunk never reads past its split
    if (k_split <= 0 || k_split >= K) k_split = K;
    else k_split = (k_split + kBK - 1) / kBK * kBK;
    Tiles T{};
    T.M = M;
    T.N = N;
    T.K = K;
    T.mt = (M + kBM - 1) / kBM;
    T.zs = (K + k_split - 1) / k_split;
    T.k_split = k_split;
    if (T.zs > 1 && !atomic) return cudaErrorInvalidValue;
    if (N <= 16) return run<16>(A, B, M, N, K, lda, ldb, T, ep, status, st);
    if (N <= 32) return run<32>(A, B, M, N, K, lda, ldb, T, ep, status, st);
    if (N <= 64) return run<64>(A, B, M, N, K, lda, ldb, T, ep, status, st);
    return run<128>(A, B, M, N, K, lda, ldb, T, ep, status, st);
}

cudaError_t conv3x3s2_bf16_enqueue(const void* x, int batch, int H, int W, int Cin, const void* Wt, int Co, int Kp,
                                   const float* bias, bool relu, void* out_bf16, unsigned int* status,
                                   cudaStream_t st) {
    if (batch <= 0) return cudaSuccess;
    if ((Cin != 32 && Cin != 64) || Kp < 9 * Cin || Kp % 8 || (Co != 64 && Co != 128))
        return cudaErrorInvalidValue;
    Tiles T{};
    T.conv = 1;
    T.Ho = (H + 1) / 2;
    T.Wo = (W + 1) / 2;
    T.M = batch * T.Ho * T.Wo;
    T.N = Co;
    T.K = 9 * Cin;
    T.mt = T.nt = T.zs = 1;
    T.k_split = T.K;
    T.taps_per_chunk = kBK / Cin;
    const int per_image = T.Ho * T.Wo;
    if (T.Wo > kBM) return cudaErrorInvalidValue;
    if (per_image <= kBM / 2) {  // several whole images per tile
        T.th = T.Ho;
        T.nb = kBM / per_image;
        T.tpi = 1;
    } else {
        T.nb = 1;
        T.th = std::min(T.Ho, kBM / T.Wo);
        T.tpi = (T.Ho + T.th - 1) / T.th;
    }
    T.a_tap_bytes = (uint32_t)(T.nb * T.th * T.Wo * Cin * 2);
    // the input (C, W, H, N) read with element strides 2 along W and H
    CUtensorMap a, b;
    const cuuint64_t dims[4] = {(cuuint64_t)Cin, (cuuint64_t)W, (cuuint64_t)H, (cuuint64_t)batch};
    const cuuint64_t strides[3] = {(cuuint64_t)Cin * 2, (cuuint64_t)W * Cin * 2, (cuuint64_t)H * W * Cin * 2};
    const cuuint32_t box[4] = {(cuuint32_t)Cin, (cuuint32_t)(2 * T.Wo), (cuuint32_t)(2 * T.th), (cuuint32_t)T.nb};
    const cuuint32_t estr[4] = {1, 2, 2, 1};
    if (!encode(&a, x, 4, dims, strides, box, estr,
                Cin == 64 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_64B))
        return cudaErrorInvalidValue;
    Epilogue ep{nullptr, Co, 0, bias, relu ? 1 : 0, (__nv_bfloat16*)out_bf16};
    const int tiles = T.nb > 1 ? (batch + T.nb - 1) / T.nb : batch * T.tpi;
    if (Co == 64) {
        if (!matrix_map(&b, Wt, Co, Kp, Kp, 64)) return cudaErrorInvalidValue;
        return launch<64>(a, b, T, tiles, ep, status, st);
    }
    if (!matrix_map(&b, Wt, Co, Kp, Kp, 128)) return cudaErrorInvalidValue;
    return launch<128>(a, b, T, tiles, ep, status, st);
}

}  // namespace kifi
