// kifi_integrate.cu -- one Integrator::Integrate (KinectFission/kifi/
// Integrator.cpp:26-71) on sm_103a, as four kernels on one stream:
//
//  k_frame_setup   derive eyeToWorld / worldToClip and the projection
//                  constants from the pose (Integrator.cpp:41-42), reset the
//                  per-frame counters (k_frame_setup_sort for 30-bit keys also
//                  prepares the sort's digit histograms and tile counters).
//  k_splat_emit    DepthMap2PointCloud (Integrator.cpp:76-183) fused with
//                  ExpandChunks (:186-250) and the de-duplication of
//                  std::unique (:50-55): every valid pixel's voxel key and its
//                  seven {0,1}^3 neighbours are tested against the volume's
//                  occupancy bitmap (one bit per voxel of the res^3 grid); the
//                  thread whose atomicOr flips a bit owns that key and appends
//                  it to the frame's list of keys NEW to the volume.
//                  For 30-bit keys (k_splat_emit_hist) it also counts the
//                  three 10-bit digits of every key it stores.
//  (radix sort)    the new keys are sorted (kifi_sort.cu): three 10-bit
//                  digit passes for 30-bit keys.
//  k_merge_update  flat_map::insert (flat_map.h:164-197) as a merge-path
//                  merge of the sorted resident keys with the sorted new keys
//                  into the other half of the ping-pong buffers, fused with
//                  UpdateVoxels (Integrator.cpp:253-358): every output voxel is
//                  projected into the frame and its (distance-sum, weight)
//                  updated before it is written -- one read and one write of
//                  the volume per frame.
//
// Batches (kifi_api_batch.cu) run the same bodies on many volumes: one
// launch per stage whose CTAs are shared out by block maps, or k_fuse_queue,
// one persistent launch whose CTAs walk a device work queue of (stage,
// scene, chunk) items.
//
// Set semantics.  The reference dilates the sorted unique splat keys U with
// three set unions: S2 = U + {0, dz, dy, dy+dz}, then the +x step adds s+1
// for every s in S2 except the largest (its loop never emits the successor of
// the last key).  Keys never carry between fields because a valid splat has
// every coordinate <= res-2 (Integrator.cpp:151-154), so the dilated set is
// exactly U + {0,1}^3 minus the single key max(U) + pack(1,1,1).  The emit
// kernel records that key (an atomicMax over the splats); if it turns out to
// be new it is the largest new key, and k_merge_update drops it and clears
// its bit.
//
// Resident voxels keep their value in the union, new ones start at
// Voxel() = (0, 0) (Integrator.cpp:60-63).  The update visits the first
// n/4*4 voxels of the merged volume only -- the reference's 4-wide loop drops
// the n%4 tail (Integrator.cpp:269) -- which the merge kernel can apply
// directly because the merged size n = N0 + #new is known before it runs.
#include <algorithm>

#include "kifi_internal.h"
#include "kifi_sort_body.cuh"

namespace kifi {
namespace {

constexpr int kEmitThreads = 256;
constexpr int kMergeThreads = 256;
constexpr int kMergeItems = 8;                            // outputs per thread
constexpr int kMergeTile = kMergeThreads * kMergeItems;   // 2048 outputs per tile (30-bit keys)
// outputs per merge tile: 64-bit keys halve it to stay within 48 KB of shared memory
template <typename K>
__host__ __device__ constexpr int merge_tile() { return sizeof(K) == 4 ? kMergeTile : kMergeTile / 2; }
constexpr uint16_t kFromB = 0x8000u;

__global__ void k_frame_setup(DeviceCtl* ctl) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        ctl->n_new = 0u;
        ctl->excluded_key = 0ull;
    }
}

// The same for 30-bit keys, plus the set-up of the frame's sort: its digit
// histograms (filled by the splat) zeroed, its passes' tile counters at the
// first tile and a new look-back generation.
__global__ void k_frame_setup_sort(DeviceCtl* ctl, SortScratch ss) {
    for (int i = threadIdx.x; i < kSortHistWords; i += blockDim.x) ss.hist[i] = 0u;
    if (threadIdx.x < kFrameSortPasses) ss.tile_counter[threadIdx.x] = ss.first_tile;
    if (threadIdx.x == 0) {
        ctl->n_new = 0u;
        ctl->excluded_key = 0ull;
        *ss.epoch += 1ull;
    }
}

__device__ __forceinline__ float load_depth(const void* depth, size_t i, bool u16) {
    // DepthStream::NextFrame converts 16-bit millimetres with value * 0.001f
    // (DepthStream.cpp:89-90)
    if (u16) return fmul((float)(unsigned int)__ldg((const unsigned short*)depth + i), 0.001f);
    return __ldg((const float*)depth + i);
}

// The occupancy bitmap is laid out in 4x4x4 bricks: one 64-bit word per
// brick (bricks x-fastest, then y, then z), bit (x&3) | (y&3)<<2 | (z&3)<<4
// within it.  A voxel's {0,1}^3 dilation then lies in one word unless it
// crosses a brick face (1.95 words on average instead of four x-rows), and
// a 32-byte sector covers 16 x 4 x 4 voxels of a surface instead of one row.
__host__ __device__ constexpr int bitmap_res(int res) { return res < 4 ? 4 : res; }

__device__ __forceinline__ size_t brick_word(uint32_t x, uint32_t y, uint32_t z, int res) {
    const size_t nb = (size_t)(bitmap_res(res) >> 2);
    return (size_t)(x >> 2) + nb * ((size_t)(y >> 2) + nb * (size_t)(z >> 2));
}

// bit position of a key in the bitmap (as 32-bit words: b >> 5, bit b & 31)
template <typename K>
__device__ __forceinline__ size_t bit_index(K key, const Codec<K>& cd, int res) {
    const uint32_t x = cd.x(key), y = cd.y(key), z = cd.z(key);
    return brick_word(x, y, z, res) * 64 + ((x & 3u) | (y & 3u) << 2 | (z & 3u) << 4);
}

// the bits of coordinates [c, c+1] of one axis inside brick `side` (0: c's
// brick, 1: the next one when c is the brick's last coordinate), as a 4-bit set
__device__ __forceinline__ uint32_t pair_bits(uint32_t c, int side) {
    const uint32_t l = c & 3u;
    if (l != 3u) return side ? 0u : 3u << l;
    return side ? 1u : 8u;
}
// {0..3} bit set -> spread by `stride` (4 for y rows, 16 for z planes)
__device__ __forceinline__ uint64_t spread(uint32_t set4, int stride) {
    uint64_t r = 0;
#pragma unroll
    for (int i = 0; i < 4; ++i)
        if (set4 >> i & 1u) r |= 1ull << (i * stride);
    return r;
}

// maximum over the warp
__device__ __forceinline__ uint32_t warp_max(uint32_t v) { return __reduce_max_sync(0xffffffffu, v); }
__device__ __forceinline__ uint64_t warp_max(uint64_t v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const uint64_t w = __shfl_xor_sync(0xffffffffu, v, o);
        v = w > v ? w : v;
    }
    return v;
}

// Splat of one pixel (Integrator.cpp:121-154 for one SSE lane).
template <typename K>
__device__ __forceinline__ bool splat_pixel(const FrameConst& fc, const float (&e2w)[16],
                                            const Geom& g, const Codec<K>& cd, int u, int v, float d, K* key) {
    if (!(d > 0.0f)) return false;
    float p[4];
    // point = (u, -v, -1, 0) + 0; point * flInv + ppOverFl; point * depth + (0,0,0,1)
    p[0] = fadd(fmul(fadd(fmul((float)u, fc.fl_inv_x), fc.pp_x), d), 0.0f);
    p[1] = fadd(fmul(fadd(fmul(fadd(0.0f, -(float)v), fc.fl_inv_y), fc.pp_y), d), 0.0f);
    p[2] = fadd(fmul(fadd(fmul(-1.0f, 1.0f), 0.0f), d), 0.0f);
    p[3] = fadd(fmul(fadd(fmul(0.0f, 1.0f), 0.0f), d), 1.0f);
    float w[4];
    mat_vec(e2w, p, w);
    // VoxelIndex(world) - 0.5 (Volume.cpp:90-93); the w lane uses (1, 0)
    float ix = fsub(fadd(fmul(w[0], g.vlen_inv), g.index_off), 0.5f);
    float iy = fsub(fadd(fmul(w[1], g.vlen_inv), g.index_off), 0.5f);
    float iz = fsub(fadd(fmul(w[2], g.vlen_inv), g.index_off), 0.5f);
    float iw = fsub(fadd(fmul(w[3], 1.0f), 0.0f), 0.5f);
    const float mx = fc.max_index;
    if (!(ix >= 0.0f && ix < mx && iy >= 0.0f && iy < mx && iz >= 0.0f && iz < mx && iw >= 0.0f &&
          iw < mx))
        return false;
    *key = cd.pack((uint32_t)ix, (uint32_t)iy, (uint32_t)iz);
    return true;
}

// Splat + dilation + new-key emission of one frame; `blk` / `nblk` are the
// CTA's index and the CTA count working on this frame (the launch's own, or
// a share of a batched launch over several volumes).  With kHist (30-bit
// keys) the CTA also counts the three 10-bit digits of every key it stores,
// in shared memory, and adds its counts to the sort's histograms `hist`.
constexpr int kEmitWarps = kEmitThreads / 32;
struct SplatSmem {
    unsigned long long ex;
    unsigned int wtot[kEmitWarps], wpre[kEmitWarps], base;
};
template <bool kHist>
struct SplatSmemHist : SplatSmem {
    unsigned int counts[kHist ? kSortHistWords : 1];
};
template <bool kU16, typename K, bool kHist = false>
__device__ __forceinline__ void splat_emit_body(DeviceCtl* __restrict__ ctl, const Geom& g,
                                                const void* __restrict__ depth, uint32_t* __restrict__ bitmap,
                                                K* __restrict__ new_keys, unsigned int new_cap,
                                                const FrameConst& fc, unsigned int blk, unsigned int nblk,
                                                SplatSmemHist<kHist>& sm, unsigned int* __restrict__ hist = nullptr) {
    static_assert(!kHist || sizeof(K) == 4, "digit counts of 30-bit keys");
    unsigned int* s_hist = nullptr;
    if constexpr (kHist) {
        // a CTA without pixels has nothing to count
        if ((size_t)blk * kEmitThreads >= (size_t)fc.width * fc.height) return;
        s_hist = sm.counts;
        for (int i = threadIdx.x; i < kSortHistWords; i += blockDim.x) s_hist[i] = 0u;
        __syncthreads();
    }
    const Codec<K> cd(g.kb);
    const int W = fc.width, H = fc.height;
    const size_t P = (size_t)W * H;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    float e2w[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) e2w[i] = fc.eye_to_world.m[i];
    // Per-frame counters are shared by every CTA: the excluded key's maximum
    // and the new-key count take one global atomic per CTA (one per warp
    // queued thousands of same-address atomics at one L2 slice).
    unsigned long long& s_ex = sm.ex;
    unsigned int(&s_wtot)[kEmitWarps] = sm.wtot;
    unsigned int(&s_wpre)[kEmitWarps] = sm.wpre;
    unsigned int& s_base = sm.base;
    if (threadIdx.x == 0) s_ex = 0ull;
    __syncthreads();
    const size_t stride = (size_t)nblk * kEmitThreads;
    // CTA-uniform trip count: the append's barriers are reached by every thread
    for (size_t c0 = (size_t)blk * kEmitThreads; c0 < P; c0 += stride) {
        const size_t i = c0 + threadIdx.x;
        K key = 0;
        bool valid = false;
        if (i < P) {
            // frames hold at most 2^26 pixels: a 32-bit division, not a 64-bit one
            const unsigned int iu = (unsigned int)i;
            const int v = (int)(iu / (unsigned int)W), u = (int)(iu - (unsigned int)v * (unsigned int)W);
            valid = splat_pixel<K>(fc, e2w, g, cd, u, v, load_depth(depth, i, kU16), &key);
        }
        // the excluded key of the dilation: max splat + pack(1,1,1)
        const K ex = warp_max(valid ? (K)(key + cd.pack(1, 1, 1)) : (K)0);
        if (lane == 0 && ex) atomicMax(&s_ex, (unsigned long long)ex);
        // neighbouring pixels often land in one voxel: one emitter per key
        unsigned int peers = __match_any_sync(0xffffffffu, valid ? key : ~(K)0);
        const bool emitter = valid && (lane == __ffs(peers) - 1);
        // The dilation's 8 keys lie in the brick words of the bitmap: one
        // word, or 2, 4 or 8 where the cube crosses brick faces.  All probes
        // are issued before any decision; atomics only for bits still clear.
        // A thread owns the bits its atomicOr flipped.
        uint64_t got[8];     // per word slot: the bits this thread flipped
        uint32_t wbase[3];   // the first brick's coordinates
        if (emitter) {
            const uint32_t x = cd.x(key), y = cd.y(key), z = cd.z(key);
            wbase[0] = x >> 2; wbase[1] = y >> 2; wbase[2] = z >> 2;
            const size_t nb = (size_t)(bitmap_res(g.res) >> 2);
            unsigned long long* words = (unsigned long long*)bitmap;
            const size_t w0 = brick_word(x, y, z, g.res);
            uint64_t mask[8], pre[8];
#pragma unroll
            for (int o = 0; o < 8; ++o) {
                const int i = o & 1, j = (o >> 1) & 1, k = o >> 2;
                const uint32_t xm = pair_bits(x, i), ym = pair_bits(y, j), zm = pair_bits(z, k);
                // xm < 16 and the spreads leave room: the products do not carry
                mask[o] = (uint64_t)xm * spread(ym, 4) * spread(zm, 16);
                pre[o] = mask[o] ? __ldcg(words + w0 + i + nb * (j + nb * k)) : ~0ull;
            }
#pragma unroll
            for (int o = 0; o < 8; ++o) {
                const int i = o & 1, j = (o >> 1) & 1, k = o >> 2;
                const uint64_t need = mask[o] & ~pre[o];
                got[o] = need ? need & ~(uint64_t)atomicOr(words + w0 + i + nb * (j + nb * k),
                                                           (unsigned long long)need)
                              : 0ull;
            }
        } else {
#pragma unroll
            for (int o = 0; o < 8; ++o) got[o] = 0ull;
            wbase[0] = wbase[1] = wbase[2] = 0u;
        }
        // append: each thread's keys follow the keys of the lanes before it
        unsigned int cnt = 0;
#pragma unroll
        for (int o = 0; o < 8; ++o) cnt += __popcll(got[o]);
        unsigned int incl = cnt;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const unsigned int y = __shfl_up_sync(0xffffffffu, incl, d);
            if (lane >= d) incl += y;
        }
        // the CTA's keys take one range of the list: warp totals, their
        // prefix and one atomic by thread 0
        if (lane == 31) s_wtot[warp] = incl;
        __syncthreads();
        if (threadIdx.x == 0) {
            unsigned int run = 0;
#pragma unroll
            for (int w = 0; w < kEmitWarps; ++w) {
                s_wpre[w] = run;
                run += s_wtot[w];
            }
            s_base = run ? atomicAdd(&ctl->n_new, run) : 0u;
        }
        __syncthreads();
        if (cnt) {
            unsigned int at = s_base + s_wpre[warp] + incl - cnt;
#pragma unroll
            for (int o = 0; o < 8; ++o) {
                uint64_t m = got[o];
                const uint32_t bx = (wbase[0] + (o & 1)) << 2, by = (wbase[1] + ((o >> 1) & 1)) << 2,
                               bz = (wbase[2] + (o >> 2)) << 2;
                while (m) {
                    const uint32_t b = (uint32_t)__ffsll((long long)m) - 1u;
                    m &= m - 1ull;
                    if (at < new_cap) {
                        const K key_out = cd.pack(bx + (b & 3u), by + ((b >> 2) & 3u), bz + (b >> 4));
                        new_keys[at] = key_out;
                        if constexpr (kHist) {
                            const uint32_t ku = (uint32_t)key_out;
                            atomicAdd(&s_hist[ku & (kFrameRadix - 1)], 1u);
                            atomicAdd(&s_hist[kFrameRadix + ((ku >> kFrameDigitBits) & (kFrameRadix - 1))], 1u);
                            atomicAdd(&s_hist[2 * kFrameRadix + (ku >> (2 * kFrameDigitBits))], 1u);
                        }
                    } else {
                        atomicOr(&ctl->status, KIFI_DEV_ERR_CAPACITY);
                    }
                    ++at;
                }
            }
        }
    }
    __syncthreads();
    if (threadIdx.x == 0 && s_ex) atomicMax(&ctl->excluded_key, s_ex);
    if constexpr (kHist) {
        for (int i = threadIdx.x; i < kSortHistWords; i += blockDim.x) {
            const unsigned int c = s_hist[i];
            if (c) atomicAdd(&hist[i], c);
        }
    }
}

template <bool kU16, typename K>
__global__ void __launch_bounds__(kEmitThreads) k_splat_emit(DeviceCtl* __restrict__ ctl, Geom g,
                                                             const void* __restrict__ depth,
                                                             uint32_t* __restrict__ bitmap,
                                                             K* __restrict__ new_keys,
                                                             unsigned int new_cap,
                                                             const FrameConst fc) {
    __shared__ SplatSmemHist<false> sm;
    splat_emit_body<kU16, K>(ctl, g, depth, bitmap, new_keys, new_cap, fc, blockIdx.x, gridDim.x, sm);
}

// 30-bit keys: the splat also fills the frame sort's digit histograms
template <bool kU16>
__global__ void __launch_bounds__(kEmitThreads) k_splat_emit_hist(DeviceCtl* __restrict__ ctl, Geom g,
                                                                  const void* __restrict__ depth,
                                                                  uint32_t* __restrict__ bitmap,
                                                                  uint32_t* __restrict__ new_keys,
                                                                  unsigned int new_cap, const FrameConst fc,
                                                                  unsigned int* __restrict__ hist) {
    __shared__ SplatSmemHist<true> sm;
    splat_emit_body<kU16, uint32_t, true>(ctl, g, depth, bitmap, new_keys, new_cap, fc, blockIdx.x, gridDim.x,
                                          sm, hist);
}

// Packed float pairs (f32x2): one instruction, each half rounded as the
// scalar __fmul_rn / __fadd_rn of that half.  A product is fma(a, b, -0)
// with the -0 a runtime value: the rounded product for every input, and
// not fused by ptxas into the add that consumes it (a packed multiply
// would be).
__device__ __forceinline__ unsigned long long f2(float lo, float hi) {
    unsigned long long d;
    asm("mov.b64 %0, {%1, %2};" : "=l"(d) : "f"(lo), "f"(hi));
    return d;
}
__device__ __forceinline__ void unf2(unsigned long long v, float& lo, float& hi) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
__device__ __forceinline__ unsigned long long f2_mul(unsigned long long a, unsigned long long b,
                                                     unsigned long long neg_zero) {
    unsigned long long d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(neg_zero));
    return d;
}
__device__ __forceinline__ unsigned long long f2_add(unsigned long long a, unsigned long long b) {
    unsigned long long d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}

// UpdateVoxels for one voxel (Integrator.cpp:273-322 for one SSE lane),
// split in two: the projection and range tests give the depth pixel the
// voxel reads (or -1 when it is not updated) and its clip w; apply_depth
// then folds that pixel's depth into the voxel.  Callers project several
// voxels before reading any depth, so the reads are in flight together.
//
// The projection of VoxelCenter(index) (Volume.cpp:75-78) through
// worldToClip: rows 0, 1 and 3 in mat_vec's order for two voxels at once
// (f32x2); row 2 is formed per voxel only when needed (pixel_of_clip).
// The w lane of the centre is 1 * 1 + 0 = 1, and w2c[12 + i] * 1 is
// w2c[12 + i] exactly.
template <typename K>
__device__ __forceinline__ void clip_pair(K ka, K kb, const float (&w2c)[16], const Geom& g,
                                          unsigned long long nz, float (&c)[2][3], float (&xyw)[2][3]) {
    const Codec<K> cd(g.kb);
    const unsigned long long vlen = f2(g.vlen, g.vlen), off = f2(g.center_off, g.center_off);
    unsigned long long cc[3];
    cc[0] = f2_add(f2_mul(f2((float)cd.x(ka), (float)cd.x(kb)), vlen, nz), off);
    cc[1] = f2_add(f2_mul(f2((float)cd.y(ka), (float)cd.y(kb)), vlen, nz), off);
    cc[2] = f2_add(f2_mul(f2((float)cd.z(ka), (float)cd.z(kb)), vlen, nz), off);
#pragma unroll
    for (int j = 0; j < 3; ++j) unf2(cc[j], c[0][j], c[1][j]);
    const int rows[3] = {0, 1, 3};
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        const int i = rows[r];
        const unsigned long long a = f2_add(f2_mul(f2(w2c[i], w2c[i]), cc[0], nz),
                                            f2_mul(f2(w2c[4 + i], w2c[4 + i]), cc[1], nz));
        const unsigned long long b =
            f2_add(f2_mul(f2(w2c[8 + i], w2c[8 + i]), cc[2], nz), f2(w2c[12 + i], w2c[12 + i]));
        unf2(f2_add(a, b), xyw[0][r], xyw[1][r]);
    }
}

// The depth pixel a voxel reads (or -1) from its clip x, y, w (and its
// centre c, for row 2 when needed).
__device__ __forceinline__ int pixel_of_clip(float x, float y, float w, const float (&c)[3], const FrameConst& fc,
                                             const float (&w2c)[16], float& w_out) {
    // lane w: (w/w) * 0 + 0 lies in [-FLT_MAX, FLT_MAX) iff w/w is finite,
    // i.e. iff w is finite and non-zero (w/w is then exactly 1).
    if (!(isfinite(w) && w != 0.0f)) return -1;
    // lane z: (z/w) * 0 + 0 lies in [-1, 1) iff z/w is finite.  When the
    // host has bounded |z| by 1e18 over the whole volume (fc.z_bounded), any
    // |w| >= 1e-18 keeps the quotient finite and z need not be formed.
    if (!(fc.z_bounded && fabsf(w) >= 1e-18f)) {
        const float z = fadd(fadd(fmul(w2c[2], c[0]), fmul(w2c[6], c[1])), fadd(fmul(w2c[10], c[2]), w2c[14]));
        if (!isfinite(z)) return -1;
        if (!(fabsf(z) <= 1e18f && fabsf(w) >= 1e-18f) && !isfinite(fdiv(z, w))) return -1;
    }
    // u = (x/w) * W/2 + W/2 and v likewise, IEEE-exact.  Only floor(u),
    // floor(v) and the range tests use them, so first try a fast reciprocal
    // (__fdividef: at most 2 ulp).  For frames up to 4096 pixels on a side
    // the approximate u' differs from u by less than 2.5e-3 wherever
    // u' lies in [-0.5, W + 0.5] (relative error of x * rcp(w) against the
    // rounded x/w at most 3.6e-7 + 6e-8, times |u - W/2| <= 4097, plus the
    // roundings of the two remaining operations), so when u' is at least
    // 1/256 away from every integer, floor(u') = floor(u) and every range test
    // agrees; otherwise the exact division decides.
    if (!fc.fast_uv) {
        const float u = fadd(fmul(fdiv(x, w), fc.half_w), fc.half_w);
        const float v = fadd(fmul(fdiv(y, w), fc.half_h), fc.half_h);
        if (!(u >= 0.0f && u < (float)fc.width && v >= 0.0f && v < (float)fc.height)) return -1;
        w_out = w;
        return (fc.height - 1 - (int)(uint32_t)v) * fc.width + (int)(uint32_t)u;
    }
    const float rw = __fdividef(1.0f, w);
    const float ua = fadd(fmul(fmul(x, rw), fc.half_w), fc.half_w);
    const float va = fadd(fmul(fmul(y, rw), fc.half_h), fc.half_h);
    const float Wf = (float)fc.width, Hf = (float)fc.height;
    if (!(ua >= -0.5f && ua <= Wf + 0.5f && va >= -0.5f && va <= Hf + 0.5f)) return -1;
    constexpr float kE = 1.0f / 256.0f;
    float u, v;
    {
        const float fu = floorf(ua), fv = floorf(va);
        const bool su = ua - fu >= kE && fu + 1.0f - ua >= kE;
        const bool sv = va - fv >= kE && fv + 1.0f - va >= kE;
        u = su ? fu + 0.5f : fadd(fmul(fdiv(x, w), fc.half_w), fc.half_w);
        v = sv ? fv + 0.5f : fadd(fmul(fdiv(y, w), fc.half_h), fc.half_h);
    }
    if (!(u >= 0.0f && u < Wf && v >= 0.0f && v < Hf)) return -1;
    w_out = w;
    return (fc.height - 1 - (int)(uint32_t)v) * fc.width + (int)(uint32_t)u;
}

// depth d at the voxel's pixel, w its clip w: signedDist = d - w, updated
// when the depth is valid and signedDist >= -trunc,
// Voxel::Update(std::min(signedDist, trunc)) (Voxel.h:53-57)
__device__ __forceinline__ void apply_depth(float2& val, float d, float w, const Geom& g) {
    const float sd = fsub(d, w);
    if (d > 0.0f && sd >= -g.trunc) {
        val.x = fadd(val.x, (g.trunc < sd) ? g.trunc : sd);
        val.y = fadd(val.y, 1.0f);
    }
}

// The TSDF update of four output voxels: the voxels at positions >= upd_end
// (outside the reference's update range, or no voxel) keep their values.
template <bool kU16, typename K>
__device__ __forceinline__ void update4(const K (&key)[4], float2 (&val)[4],
                                        const unsigned long long (&pos)[4], unsigned long long upd_end,
                                        const FrameConst& fc, const float (&w2c)[16], const Geom& g,
                                        const void* depth) {
    int ix[4];
    float w[4], d[4];
    const unsigned long long nz = f2(fc.neg_zero, fc.neg_zero);
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        float c[2][3], xyw[2][3];
        clip_pair<K>(key[2 * h], key[2 * h + 1], w2c, g, nz, c, xyw);
#pragma unroll
        for (int j = 0; j < 2; ++j) {
            const int q = 2 * h + j;
            w[q] = 0.0f;
            ix[q] = pos[q] < upd_end ? pixel_of_clip(xyw[j][0], xyw[j][1], xyw[j][2], c[j], fc, w2c, w[q]) : -1;
        }
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) d[q] = ix[q] >= 0 ? load_depth(depth, (size_t)ix[q], kU16) : 0.0f;
#pragma unroll
    for (int q = 0; q < 4; ++q)
        if (ix[q] >= 0) apply_depth(val[q], d[q], w[q], g);
}

// number of A elements among the first d outputs of merge(A, B); A and B
// are sorted and disjoint.
template <typename K>
__device__ __forceinline__ unsigned long long merge_path(const K* __restrict__ A,
                                                         unsigned long long na,
                                                         const K* __restrict__ B,
                                                         unsigned long long nb,
                                                         unsigned long long d) {
    unsigned long long lo = d > nb ? d - nb : 0, hi = d < na ? d : na;
    while (lo < hi) {
        unsigned long long mid = (lo + hi) >> 1;
        if (A[mid] < B[d - 1 - mid]) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

template <typename K>
struct MergeInputs {
    const K* b_keys;          // sorted new keys
    const uint32_t* b_index;  // optional: b's position in b_vals (inserts)
    const float2* b_vals;     // optional values of new keys; null = Voxel()
    const unsigned int* b_count;
    bool update;              // run UpdateVoxels on the merged volume
};

struct PartitionSmem {
    unsigned long long e, n1;
    int ok;
};

// Merge set-up and partition.  Thread 0 settles the merge: drops the
// dilation's excluded key when it is the largest new key (clearing its
// occupancy bit), checks the capacity and publishes (e, N1).  Every thread t
// then computes the merge-path split of output tile t: the number of resident
// keys among the first t*kMergeTile outputs.  The binary searches of all
// tiles run in parallel here instead of serialising the merge kernel's tiles.
template <typename K>
__device__ __forceinline__ void merge_partition_body(DeviceCtl* __restrict__ ctl, const Geom& g,
                                                     const VolumeBuffers& vb, const MergeInputs<K>& in,
                                                     unsigned long long* __restrict__ splits,
                                                     unsigned int max_tiles, unsigned int blk, unsigned int nblk,
                                                     PartitionSmem& sm) {
    constexpr int kTile = merge_tile<K>();
    const Codec<K> cd(g.kb);
    unsigned long long& s_e = sm.e;
    unsigned long long& s_n1 = sm.n1;
    int& s_ok = sm.ok;
    const unsigned int cur = ctl->cur;
    const unsigned long long N0 = ctl->n[cur];
    // select rather than index: a runtime index into a parameter array
    // would force the array into local memory
    const K* __restrict__ A = (const K*)(cur ? vb.keys[1] : vb.keys[0]);
    const K* __restrict__ B = in.b_keys;
    // a sort that gave up on a bounded wait leaves its keys unordered: the
    // volume stays as it was (the host rebuilds the occupancy bits)
    const bool timed_out = (ctl->status & KIFI_DEV_ERR_TIMEOUT) != 0u;
    if (threadIdx.x == 0) {
        unsigned long long e = *in.b_count;
        const K excluded = (K)ctl->excluded_key;
        const bool drop = !timed_out && e > 0 && excluded != 0 && B[e - 1] == excluded;
        if (drop) --e;
        const bool ok = !timed_out && N0 + e <= vb.cap;
        s_e = e;
        s_n1 = N0 + e;
        s_ok = ok;
        if (blk == 0) {
            ctl->merge_e = e;
            ctl->merge_n1 = N0 + e;
            ctl->merge_ok = ok ? 1u : 0u;
            if (drop) {
                size_t b = bit_index(excluded, cd, g.res);
                atomicAnd(vb.bitmap + (b >> 5), ~(1u << (b & 31)));
            }
            if (!ok && !timed_out) atomicOr(&ctl->status, KIFI_DEV_ERR_CAPACITY);
        }
    }
    __syncthreads();
    const unsigned long long e = s_e, N1 = s_n1;
    if (!s_ok) {
        if (timed_out) return;
        // no room: leave the volume as it was and take the new keys back out
        // of the occupancy bitmap; the host grows the buffers and retries.
        for (unsigned long long i = (unsigned long long)blk * blockDim.x + threadIdx.x; i < e;
             i += (unsigned long long)nblk * blockDim.x) {
            size_t b = bit_index(B[i], cd, g.res);
            atomicAnd(vb.bitmap + (b >> 5), ~(1u << (b & 31)));
        }
        return;
    }
    const unsigned long long n_tiles = (N1 + kTile - 1) / kTile;
    for (unsigned long long t = (unsigned long long)blk * blockDim.x + threadIdx.x;
         t <= n_tiles && t < max_tiles; t += (unsigned long long)nblk * blockDim.x) {
        const unsigned long long d = t * kTile < N1 ? t * kTile : N1;
        splits[t] = merge_path(A, N0, B, e, d);
    }
}

template <typename K>
__global__ void __launch_bounds__(256) k_merge_partition(DeviceCtl* __restrict__ ctl, Geom g,
                                                          VolumeBuffers vb, MergeInputs<K> in,
                                                          unsigned long long* __restrict__ splits,
                                                          unsigned int max_tiles) {
    __shared__ PartitionSmem sm;
    merge_partition_body<K>(ctl, g, vb, in, splits, max_tiles, blockIdx.x, gridDim.x, sm);
}

// four consecutive keys, streamed (p 16-byte aligned for 32-bit keys,
// 32-byte aligned for 64-bit keys)
__device__ __forceinline__ void ld4(const uint32_t* p, uint32_t (&k)[4]) {
    const uint4 v = __ldcs((const uint4*)p);
    k[0] = v.x; k[1] = v.y; k[2] = v.z; k[3] = v.w;
}
__device__ __forceinline__ void ld4(const uint64_t* p, uint64_t (&k)[4]) {
    const ulonglong2 a = __ldcs((const ulonglong2*)p), b = __ldcs((const ulonglong2*)(p + 2));
    k[0] = a.x; k[1] = a.y; k[2] = b.x; k[3] = b.y;
}
__device__ __forceinline__ void st4(uint32_t* p, const uint32_t (&k)[4]) {
    __stcs((uint4*)p, make_uint4(k[0], k[1], k[2], k[3]));
}
__device__ __forceinline__ void st4(uint64_t* p, const uint64_t (&k)[4]) {
    __stcs((ulonglong2*)p, make_ulonglong2(k[0], k[1]));
    __stcs((ulonglong2*)(p + 2), make_ulonglong2(k[2], k[3]));
}

template <typename K>
struct MergeSmem {
    alignas(16) K sA_k[merge_tile<K>() + 8];
    float2 sA_v[merge_tile<K>() + 4];
    K sB_k[merge_tile<K>()];
    uint16_t sSrc[merge_tile<K>()];
};

template <bool kU16, typename K>
__device__ __forceinline__ void merge_update_body(DeviceCtl* __restrict__ ctl, const Geom& g,
                                                  const VolumeBuffers& vb, const MergeInputs<K>& in,
                                                  const void* __restrict__ depth,
                                                  const unsigned long long* __restrict__ splits,
                                                  const FrameConst& fc, unsigned int blk, unsigned int nblk,
                                                  MergeSmem<K>& sm) {
    constexpr int kTile = merge_tile<K>();
    constexpr int kItems = kTile / kMergeThreads;
    K* const sA_k = sm.sA_k;
    float2* const sA_v = sm.sA_v;
    K* const sB_k = sm.sB_k;
    uint16_t* const sSrc = sm.sSrc;

    if (!ctl->merge_ok) return;
    const unsigned int cur = ctl->cur, out = cur ^ 1u;
    const unsigned long long N0 = ctl->n[cur];
    const unsigned long long e = ctl->merge_e;
    const unsigned long long N1 = ctl->merge_n1;
    const K* __restrict__ A = (const K*)(cur ? vb.keys[1] : vb.keys[0]);
    const float2* __restrict__ Av = cur ? vb.vals[1] : vb.vals[0];
    const K* __restrict__ B = in.b_keys;
    const unsigned long long upd_end = in.update ? (N1 / 4 * 4) : 0ull;
    K* __restrict__ outK = (K*)(out ? vb.keys[1] : vb.keys[0]);
    float2* __restrict__ outV = out ? vb.vals[1] : vb.vals[0];
    const unsigned long long n_tiles = (N1 + kTile - 1) / kTile;
    float w2c[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) w2c[i] = fc.world_to_clip.m[i];

    for (unsigned long long t = blk; t < n_tiles; t += nblk) {
        const unsigned long long d0 = t * kTile;
        const unsigned long long d1 = (d0 + kTile < N1) ? d0 + kTile : N1;
        const int len = (int)(d1 - d0);
        const unsigned long long a0 = splits[t], a1 = splits[t + 1];
        const int na = (int)(a1 - a0), nb = len - na;
        if (nb == 0) {
            // only resident voxels in this tile: straight streaming, no
            // barrier.  Each thread loads all its groups of four first, then
            // projects them, reads their depth pixels together and stores.
            constexpr int kGroups = kItems / 4;
            const bool vec = (a0 & 3ull) == 0;
            K kk[kGroups][4];
            float2 vv[kGroups][4];
#pragma unroll
            for (int r = 0; r < kGroups; ++r) {
                const int j0 = threadIdx.x * 4 + r * kMergeThreads * 4;
                const unsigned long long ia = a0 + j0;
                if (j0 >= len) {
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        kk[r][q] = (K)0;
                        vv[r][q] = make_float2(0.0f, 0.0f);
                    }
                } else if (vec && j0 + 4 <= len) {
                    ld4(A + ia, kk[r]);
                    const float4 va = __ldcs((const float4*)(Av + ia));
                    const float4 vb4 = __ldcs((const float4*)(Av + ia + 2));
                    vv[r][0] = make_float2(va.x, va.y); vv[r][1] = make_float2(va.z, va.w);
                    vv[r][2] = make_float2(vb4.x, vb4.y); vv[r][3] = make_float2(vb4.z, vb4.w);
                } else {
                    const int m = len - j0;
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        kk[r][q] = q < m ? __ldcs(A + ia + q) : (K)0;
                        vv[r][q] = q < m ? __ldcs(Av + ia + q) : make_float2(0.0f, 0.0f);
                    }
                }
            }
#pragma unroll
            for (int r = 0; r < kGroups; ++r) {
                const int j0 = threadIdx.x * 4 + r * kMergeThreads * 4;
                if (j0 >= len) break;
                const unsigned long long p = d0 + j0;
                // positions past the tile are past the update range too
                // (only the last tile is ragged, and upd_end <= N1)
                const unsigned long long pos[4] = {p, p + 1, p + 2, p + 3};
                update4<kU16, K>(kk[r], vv[r], pos, upd_end, fc, w2c, g, depth);
                if (j0 + 4 <= len) {
                    st4(outK + p, kk[r]);
                    __stcs((float4*)(outV + p), make_float4(vv[r][0].x, vv[r][0].y, vv[r][1].x, vv[r][1].y));
                    __stcs((float4*)(outV + p + 2), make_float4(vv[r][2].x, vv[r][2].y, vv[r][3].x, vv[r][3].y));
                } else {
                    const int m = len - j0;
#pragma unroll
                    for (int q = 0; q < 4; ++q)
                        if (q < m) {
                            outK[p + q] = kk[r][q];
                            outV[p + q] = vv[r][q];
                        }
                }
            }
            continue;
        }
        if (nb <= kMergeThreads && (int)(a0 & 3ull) + na <= kTile) {
            // Few new keys (the common mixed tile: a median of 16-25 per
            // 2048 outputs).  Each thread keeps its resident entries in
            // registers (aligned 128-bit loads from a0 rounded down to 4) and
            // places each at its A index plus the number of new keys below
            // it, found in the tile's staged new keys; a new key goes to its
            // B index plus the number of resident keys below it.  Resident
            // keys are staged too, for that second search.
            const unsigned long long ka = a0 & ~3ull;
            const int koff = (int)(a0 - ka);
            const unsigned long long b0 = d0 - a0;
            if ((int)threadIdx.x < nb) sB_k[threadIdx.x] = B[b0 + threadIdx.x];
            K kk[2][4];
            float2 vv[2][4];
            int li0[2];
#pragma unroll
            for (int r = 0; r < 2; ++r) {
                const int ls = (int)threadIdx.x * 4 + r * kMergeThreads * 4;
                li0[r] = ls - koff;
                if (ka + (unsigned long long)ls < a1) {  // reads at most 3 entries past a1 (array padding)
                    ld4(A + ka + ls, kk[r]);
                    const float4 x0 = __ldcs((const float4*)(Av + ka + ls));
                    const float4 x1 = __ldcs((const float4*)(Av + ka + ls + 2));
                    vv[r][0] = make_float2(x0.x, x0.y); vv[r][1] = make_float2(x0.z, x0.w);
                    vv[r][2] = make_float2(x1.x, x1.y); vv[r][3] = make_float2(x1.z, x1.w);
                } else {
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        kk[r][q] = (K)0;
                        vv[r][q] = make_float2(0.0f, 0.0f);
                    }
                }
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const int li = li0[r] + q;
                    if (li >= 0 && li < na) sA_k[li] = kk[r][q];
                }
            }
            __syncthreads();
#pragma unroll
            for (int r = 0; r < 2; ++r) {
                unsigned long long pos[4];
                int rank = -1;  // new keys below the current resident key
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const int li = li0[r] + q;
                    pos[q] = ~0ull;  // not this tile's: never updated or stored
                    if (li >= 0 && li < na) {
                        const K a = kk[r][q];
                        if (rank < 0) {
                            int lo = 0, hi = nb;
                            while (lo < hi) {
                                const int mid = (lo + hi) >> 1;
                                if (sB_k[mid] < a) lo = mid + 1;
                                else hi = mid;
                            }
                            rank = lo;
                        } else {
                            while (rank < nb && sB_k[rank] < a) ++rank;
                        }
                        pos[q] = d0 + (unsigned long long)(li + rank);
                    }
                }
                update4<kU16, K>(kk[r], vv[r], pos, upd_end, fc, w2c, g, depth);
#pragma unroll
                for (int q = 0; q < 4; ++q)
                    if (pos[q] != ~0ull) {
                        __stcs(outK + pos[q], kk[r][q]);
                        __stcs(outV + pos[q], vv[r][q]);
                    }
            }
            if ((int)threadIdx.x < nb) {
                const int j = (int)threadIdx.x;
                K key[4] = {sB_k[j], (K)0, (K)0, (K)0};
                float2 val[4] = {make_float2(0.0f, 0.0f), make_float2(0.0f, 0.0f), make_float2(0.0f, 0.0f),
                                 make_float2(0.0f, 0.0f)};
                if (in.b_vals) val[0] = in.b_vals[in.b_index ? in.b_index[b0 + j] : b0 + j];
                int lo = 0, hi = na;
                while (lo < hi) {
                    const int mid = (lo + hi) >> 1;
                    if (sA_k[mid] < key[0]) lo = mid + 1;
                    else hi = mid;
                }
                const unsigned long long pos[4] = {d0 + (unsigned long long)(j + lo), ~0ull, ~0ull, ~0ull};
                update4<kU16, K>(key, val, pos, upd_end, fc, w2c, g, depth);
                __stcs(outK + pos[0], key[0]);
                __stcs(outV + pos[0], val[0]);
            }
            __syncthreads();
            continue;
        }
        // mixed tile with many new keys: stage both ranges in shared memory and merge there
        const unsigned long long b0 = d0 - a0;
        const unsigned long long ka = a0 & ~3ull;
        const int koff = (int)(a0 - ka);
        for (int i = threadIdx.x * 4; i < koff + na; i += kMergeThreads * 4) {
            K kk[4];
            ld4(A + ka + i, kk);
            sA_k[i] = kk[0]; sA_k[i + 1] = kk[1]; sA_k[i + 2] = kk[2]; sA_k[i + 3] = kk[3];
        }
        const unsigned long long va = a0 & ~1ull;
        const int voff = (int)(a0 - va);
        for (int i = threadIdx.x * 2; i < voff + na; i += kMergeThreads * 2)
            *(float4*)&sA_v[i] = __ldcs((const float4*)(Av + va + i));
        for (int i = threadIdx.x; i < nb; i += kMergeThreads) sB_k[i] = B[b0 + i];
        __syncthreads();
        {
            const int dd = threadIdx.x * kItems;
            if (dd < len) {
                int lo = dd > nb ? dd - nb : 0, hi = dd < na ? dd : na;
                while (lo < hi) {
                    int mid = (lo + hi) >> 1;
                    if (sA_k[koff + mid] < sB_k[dd - 1 - mid]) lo = mid + 1;
                    else hi = mid;
                }
                int ia = lo, ib = dd - lo;
                const int end = dd + kItems < len ? dd + kItems : len;
                for (int j = dd; j < end; ++j) {
                    bool takeA = ib >= nb || (ia < na && sA_k[koff + ia] < sB_k[ib]);
                    sSrc[j] = takeA ? (uint16_t)ia++ : (uint16_t)(kFromB | ib++);
                }
            }
        }
        __syncthreads();
        // outputs j, j + 256, j + 512, j + 768 of the tile per group of four
        for (int j0 = threadIdx.x; j0 < len; j0 += 4 * kMergeThreads) {
            K key[4];
            float2 val[4];
            unsigned long long pos[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int j = j0 + q * kMergeThreads;
                key[q] = (K)0;
                val[q] = make_float2(0.0f, 0.0f);
                pos[q] = ~0ull;  // no voxel: never updated
                if (j < len) {
                    const uint16_t src = sSrc[j];
                    pos[q] = d0 + j;
                    if (!(src & kFromB)) {
                        key[q] = sA_k[koff + src];
                        val[q] = sA_v[voff + src];
                    } else {
                        const int ib = src & ~kFromB;
                        key[q] = sB_k[ib];
                        if (in.b_vals) val[q] = in.b_vals[in.b_index ? in.b_index[b0 + ib] : b0 + ib];
                    }
                }
            }
            update4<kU16, K>(key, val, pos, upd_end, fc, w2c, g, depth);
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int j = j0 + q * kMergeThreads;
                if (j < len) {
                    __stcs(outK + d0 + j, key[q]);
                    __stcs(outV + d0 + j, val[q]);
                }
            }
        }
        __syncthreads();
    }
    // the last CTA to finish publishes the new volume
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        unsigned int prev = atomicAdd(&ctl->tile_counter[7], 1u);
        if (prev == nblk - 1) {
            ctl->n[out] = N1;
            ctl->cur = out;
            ctl->tile_counter[7] = 0u;
            const unsigned int slot = (unsigned int)(ctl->frames % kFrameLog);
            ctl->log_n0[slot] = N0;
            ctl->log_new[slot] = e;
            ctl->log_n1[slot] = N1;
            ctl->frames += 1ull;
            __threadfence();
        }
    }
}

// Two builds of the same merge: beside tracking, 76 registers and 3 CTAs
// per SM, so that fewer SMs are held when the next ICP step starts; alone,
// capped at 64 registers for a fourth CTA per SM (a few spilled words, in
// L1).  Measured at ~21 M voxels, 10-frame runs: alone 122 -> 113 us; in the
// pipeline the capped build gave 2000 against 2036 frames/s.
template <bool kU16, typename K>
__global__ void __launch_bounds__(kMergeThreads) k_merge_update(DeviceCtl* __restrict__ ctl, Geom g,
                                                                VolumeBuffers vb, MergeInputs<K> in,
                                                                const void* __restrict__ depth,
                                                                const unsigned long long* __restrict__ splits,
                                                                const FrameConst fc) {
    __shared__ MergeSmem<K> sm;
    merge_update_body<kU16, K>(ctl, g, vb, in, depth, splits, fc, blockIdx.x, gridDim.x, sm);
}
template <bool kU16, typename K>
__global__ void __launch_bounds__(kMergeThreads, 4) k_merge_update_alone(DeviceCtl* __restrict__ ctl, Geom g,
                                                                         VolumeBuffers vb, MergeInputs<K> in,
                                                                         const void* __restrict__ depth,
                                                                         const unsigned long long* __restrict__ splits,
                                                                         const FrameConst fc) {
    __shared__ MergeSmem<K> sm;
    merge_update_body<kU16, K>(ctl, g, vb, in, depth, splits, fc, blockIdx.x, gridDim.x, sm);
}

// inserts: keep keys not yet in the volume (flat_map::insert keeps resident
// values), appending (key, position) pairs for the sort.
template <typename K>
__global__ void k_insert_filter(DeviceCtl* ctl, Geom g, uint32_t* bitmap, const K* keys,
                                const unsigned int* n_ptr, K* out_keys, uint32_t* out_idx) {
    const Codec<K> cd(g.kb);
    const unsigned int n = *n_ptr;
    const int lane = threadIdx.x & 31;
    const unsigned int n_round = (n + 31) / 32 * 32;
    for (unsigned int i = blockIdx.x * blockDim.x + threadIdx.x; i < n_round;
         i += gridDim.x * blockDim.x) {
        bool mine = false;
        K k = 0;
        if (i < n) {
            k = keys[i];
            size_t b = bit_index(k, cd, g.res);
            uint32_t mask = 1u << (b & 31);
            mine = !(atomicOr(bitmap + (b >> 5), mask) & mask);
        }
        unsigned int ballot = __ballot_sync(0xffffffffu, mine);
        if (!ballot) continue;
        unsigned int base = 0;
        if (lane == __ffs(ballot) - 1) base = atomicAdd(&ctl->n_new, (unsigned int)__popc(ballot));
        base = __shfl_sync(0xffffffffu, base, __ffs(ballot) - 1);
        if (mine) {
            unsigned int at = base + __popc(ballot & ((1u << lane) - 1u));
            out_keys[at] = k;
            out_idx[at] = i;
        }
    }
}

// the occupancy bits of the resident keys (after the bitmap was cleared)
template <typename K>
__global__ void k_bitmap_from_keys(const DeviceCtl* __restrict__ ctl, Geom g, VolumeBuffers vb) {
    const Codec<K> cd(g.kb);
    const unsigned int cur = ctl->cur;
    const unsigned long long n = ctl->n[cur];
    const K* __restrict__ keys = (const K*)(cur ? vb.keys[1] : vb.keys[0]);
    for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (unsigned long long)gridDim.x * blockDim.x) {
        const size_t b = bit_index(keys[i], cd, g.res);
        atomicOr(vb.bitmap + (b >> 5), 1u << (b & 31));
    }
}

// ---- batched: one frame for each volume of a batch, one launch per stage;
// each volume's CTAs run the single-volume kernel body on its arguments
__global__ void k_frame_setup_batch(const FuseJob* __restrict__ jobs, int n) {
    if ((int)blockIdx.x < n && threadIdx.x == 0) {
        DeviceCtl* ctl = jobs[blockIdx.x].ctl;
        ctl->n_new = 0u;
        ctl->excluded_key = 0ull;
    }
}

template <typename K>
__global__ void __launch_bounds__(kEmitThreads) k_splat_emit_batch(const FuseJob* __restrict__ jobs, BlockMap m) {
    const int v = block_owner(m, blockIdx.x);
    const FuseJob& j = jobs[v];
    const unsigned int b0 = m.first[v];
    __shared__ SplatSmemHist<false> sm;
    splat_emit_body<true, K>(j.ctl, j.g, j.depth, j.vb.bitmap, (K*)j.vb.new_keys, (unsigned int)j.vb.new_cap, j.fc,
                             blockIdx.x - b0, m.first[v + 1] - b0, sm);
}

template <typename K>
__global__ void __launch_bounds__(256) k_merge_partition_batch(const FuseJob* __restrict__ jobs, BlockMap m) {
    const int v = block_owner(m, blockIdx.x);
    const FuseJob& j = jobs[v];
    const unsigned int b0 = m.first[v];
    const MergeInputs<K> in{(const K*)j.vb.new_keys, nullptr, nullptr, &j.ctl->n_new, true};
    __shared__ PartitionSmem sm;
    merge_partition_body<K>(j.ctl, j.g, j.vb, in, j.vb.splits, j.max_tiles, blockIdx.x - b0, m.first[v + 1] - b0,
                            sm);
}

template <typename K>
__global__ void __launch_bounds__(kMergeThreads) k_merge_update_batch(const FuseJob* __restrict__ jobs, BlockMap m) {
    const int v = block_owner(m, blockIdx.x);
    const FuseJob& j = jobs[v];
    const unsigned int b0 = m.first[v];
    const MergeInputs<K> in{(const K*)j.vb.new_keys, nullptr, nullptr, &j.ctl->n_new, true};
    __shared__ MergeSmem<K> sm;
    merge_update_body<true, K>(j.ctl, j.g, j.vb, in, j.depth, j.vb.splits, j.fc, blockIdx.x - b0,
                               m.first[v + 1] - b0, sm);
}

// ---- batched fusion as one persistent launch over a device work queue
//
// The items of a step are (stage, scene, chunk): the frame set-up, the
// splat chunks, the histogram chunks, each digit pass's chunks, the
// partition chunks and the merge chunks of every scene, numbered stage by
// stage (a stage's chunks per scene are its block map's shares).  CTAs take
// item numbers from one counter.  Before its body an item waits until every
// item of the scene's previous stage has finished; those items have smaller
// numbers, so they were handed out before it, to CTAs that are running: the
// wait always ends, whatever CTAs are resident.  A wait is bounded: past the
// limit the scene's status takes KIFI_DEV_ERR_TIMEOUT, the item is skipped
// (the partition then leaves the volume as it was) and still counts as done.
template <typename K>
union QueueSmem {
    SplatSmemHist<false> splat;
    sort_detail::SortHistSmem hist;
    sort_detail::SortPassSmem<8> pass;
    PartitionSmem part;
    MergeSmem<K> merge;
};

__device__ __forceinline__ unsigned int ld_acquire_u32(const unsigned int* p) {
    unsigned int v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// chunks of stage k for scene v (stage 0, the set-up: one)
__device__ __forceinline__ unsigned int stage_chunks(const FuseQueuePlan& q, int k, int v) {
    if (k == 0) return 1u;
    const BlockMap& m = q.maps[fuse_stage_map(k, q.passes)];
    return m.first[v + 1] - m.first[v];
}

template <typename K>
__global__ void __launch_bounds__(kMergeThreads) k_fuse_queue(const FuseJob* __restrict__ jobs, FuseQueuePlan q,
                                                               unsigned int* __restrict__ next,
                                                               unsigned int* __restrict__ done,
                                                               unsigned long long spin_limit) {
    __shared__ QueueSmem<K> sm;
    __shared__ unsigned int s_item;
    __shared__ int s_go;
    const unsigned int total = q.first[q.stages];
    for (;;) {
        if (threadIdx.x == 0) s_item = atomicAdd(next, 1u);
        __syncthreads();
        const unsigned int i = s_item;
        __syncthreads();  // read by every thread before thread 0 takes the next item
        if (i >= total) break;
        int k = 0;
        while (i >= q.first[k + 1]) ++k;
        const unsigned int local = i - q.first[k];
        int v;
        unsigned int c, nb;
        if (k == 0) {
            v = (int)local;
            c = 0u;
            nb = 1u;
        } else {
            const BlockMap& m = q.maps[fuse_stage_map(k, q.passes)];
            v = block_owner(m, local);
            c = local - m.first[v];
            nb = m.first[v + 1] - m.first[v];
        }
        const FuseJob& j = jobs[v];
        if (k > 0) {
            if (threadIdx.x == 0) {
                const unsigned int want = stage_chunks(q, k - 1, v);
                const unsigned int* d = done + (size_t)v * q.stages + (k - 1);
                unsigned long long spins = 0;
                bool ok = true;
                while (ld_acquire_u32(d) < want) {
                    if (++spins > spin_limit) {
                        ok = false;
                        atomicOr(&j.ctl->status, KIFI_DEV_ERR_TIMEOUT);
                        break;
                    }
                    __nanosleep(64);
                }
                s_go = ok;
            }
            __syncthreads();
        }
        if (k == 0 || s_go) {
            const int pass = k - 3;
            if (k == 0) {
                if (threadIdx.x == 0) {
                    j.ctl->n_new = 0u;
                    j.ctl->excluded_key = 0ull;
                }
                sort_detail::sort_prepare_body(j.ss, q.passes);
            } else if (k == 1) {
                splat_emit_body<true, K>(j.ctl, j.g, j.depth, j.vb.bitmap, (K*)j.vb.new_keys,
                                         (unsigned int)j.vb.new_cap, j.fc, c, nb, sm.splat);
            } else if (k == 2) {
                sort_detail::sort_histogram_body<K>((const K*)j.vb.new_keys, &j.ctl->n_new, j.ss, q.passes, c, nb,
                                                    sm.hist);
            } else if (pass < q.passes) {
                K* keys = (K*)j.vb.new_keys;
                K* alt = (K*)j.ss.alt_keys;
                sort_detail::sort_pass_body<false, K, 8>(pass & 1 ? alt : keys, pass & 1 ? keys : alt, nullptr,
                                                         nullptr, &j.ctl->n_new, j.ss, pass, c, sm.pass);
            } else {
                const MergeInputs<K> in{(const K*)j.vb.new_keys, nullptr, nullptr, &j.ctl->n_new, true};
                if (pass == q.passes)
                    merge_partition_body<K>(j.ctl, j.g, j.vb, in, j.vb.splits, j.max_tiles, c, nb, sm.part);
                else
                    merge_update_body<true, K>(j.ctl, j.g, j.vb, in, j.depth, j.vb.splits, j.fc, c, nb, sm.merge);
            }
        }
        __syncthreads();  // the item's stores are done
        if (threadIdx.x == 0) {
            __threadfence();
            atomicAdd(done + (size_t)v * q.stages + k, 1u);
        }
    }
}

__global__ void k_reset_new(DeviceCtl* ctl) {
    ctl->n_new = 0u;
    ctl->excluded_key = 0ull;
}

}  // namespace

int merge_blocks_per_sm() {
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_merge_update_alone<true, uint32_t>, kMergeThreads, 0) !=
            cudaSuccess ||
        n < 1)
        n = 4;
    return n;
}

template <typename K>
static unsigned int max_tiles_of(const VolumeBuffers& vb) {
    return (unsigned int)((vb.cap + merge_tile<K>() - 1) / merge_tile<K>() + 2);
}

size_t merge_max_tiles(const VolumeBuffers& vb, size_t cap) {
    const int tile = vb.key_bytes == 8 ? merge_tile<uint64_t>() : merge_tile<uint32_t>();
    return (cap + tile - 1) / tile + 2;
}

template <typename K>
static cudaError_t merge_enqueue(DeviceCtl* ctl, const Geom& g, VolumeBuffers& vb,
                                 const MergeInputs<K>& in, const void* depth, bool u16,
                                 const FrameConst& fc, const LaunchShape& ls, cudaStream_t st,
                                 cudaEvent_t after_partition = nullptr) {
    const unsigned int mt = max_tiles_of<K>(vb);
    k_merge_partition<K><<<(mt + 255) / 256, 256, 0, st>>>(ctl, g, vb, in, vb.splits, mt);
    if (after_partition) cudaEventRecord(after_partition, st);
    if (ls.beside_tracking) {
        if (u16)
            k_merge_update<true, K><<<ls.merge_ctas, kMergeThreads, 0, st>>>(ctl, g, vb, in, depth, vb.splits, fc);
        else
            k_merge_update<false, K><<<ls.merge_ctas, kMergeThreads, 0, st>>>(ctl, g, vb, in, depth, vb.splits, fc);
    } else {
        if (u16)
            k_merge_update_alone<true, K><<<ls.merge_ctas, kMergeThreads, 0, st>>>(ctl, g, vb, in, depth, vb.splits,
                                                                                   fc);
        else
            k_merge_update_alone<false, K><<<ls.merge_ctas, kMergeThreads, 0, st>>>(ctl, g, vb, in, depth, vb.splits,
                                                                                    fc);
    }
    return cudaGetLastError();
}

template <typename K>
static cudaError_t integrate_enqueue_t(DeviceCtl* ctl, const Geom& g, VolumeBuffers& vb, SortScratch& ss,
                                       const void* depth_dev, bool depth_u16, const kifi_camera& cam,
                                       const Mat4& world_to_eye, const LaunchShape& ls, cudaStream_t st,
                                       cudaEvent_t* events) {
    // frame constants on the host, in the reference's float order
    FrameConst fc = make_frame_const(cam, world_to_eye, g.res);
    fc.z_bounded = clip_z_bounded(fc.world_to_clip, g.side);
    if (events) cudaEventRecord(events[0], st);
    const unsigned int new_cap = (unsigned int)vb.new_cap;
    K* nk = (K*)vb.new_keys;
    const K* sorted = nk;
    cudaError_t e;
    if constexpr (sizeof(K) == 4) {
        // 30-bit keys: set-up and digit counts ride on the set-up and splat
        // kernels; the sort is its three digit passes.  The splat takes at
        // most one CTA per kEmitThreads pixels (a CTA without pixels would
        // only launch and leave).
        const size_t pix_ctas = ((size_t)cam.width * cam.height + kEmitThreads - 1) / kEmitThreads;
        const int splat_ctas = (int)std::min<size_t>((size_t)ls.splat_ctas, std::max<size_t>(pix_ctas, 1));
        sort_limits(&ss);
        k_frame_setup_sort<<<1, 256, 0, st>>>(ctl, ss);
        if (depth_u16)
            k_splat_emit_hist<true><<<splat_ctas, kEmitThreads, 0, st>>>(ctl, g, depth_dev, vb.bitmap, nk, new_cap,
                                                                          fc, ss.hist);
        else
            k_splat_emit_hist<false><<<splat_ctas, kEmitThreads, 0, st>>>(ctl, g, depth_dev, vb.bitmap, nk, new_cap,
                                                                           fc, ss.hist);
        if (events) cudaEventRecord(events[1], st);
        e = sort_frame_keys(nk, &ctl->n_new, ss, &ctl->status, ls.sort_ctas, st, &sorted);
    } else {
        k_frame_setup<<<1, 32, 0, st>>>(ctl);
        if (depth_u16)
            k_splat_emit<true, K><<<ls.splat_ctas, kEmitThreads, 0, st>>>(ctl, g, depth_dev, vb.bitmap, nk, new_cap,
                                                                          fc);
        else
            k_splat_emit<false, K><<<ls.splat_ctas, kEmitThreads, 0, st>>>(ctl, g, depth_dev, vb.bitmap, nk,
                                                                           new_cap, fc);
        if (events) cudaEventRecord(events[1], st);
        e = sort_keys(vb.new_keys, sizeof(K), 3 * g.kb, nullptr, &ctl->n_new, ss, &ctl->status, ls.sort_ctas, st);
    }
    if (e != cudaSuccess) return e;
    if (events) cudaEventRecord(events[2], st);
    MergeInputs<K> in{sorted, nullptr, nullptr, &ctl->n_new, true};
    e = merge_enqueue<K>(ctl, g, vb, in, depth_dev, depth_u16, fc, ls, st, events ? events[3] : nullptr);
    if (events) cudaEventRecord(events[4], st);
    return e;
}

cudaError_t integrate_enqueue(DeviceCtl* ctl, const Geom& g, VolumeBuffers& vb, SortScratch& ss,
                              const void* depth_dev, bool depth_u16, const kifi_camera& cam,
                              const Mat4& world_to_eye, const LaunchShape& ls, cudaStream_t st,
                              cudaEvent_t* events) {
    if (vb.key_bytes == 8)
        return integrate_enqueue_t<uint64_t>(ctl, g, vb, ss, depth_dev, depth_u16, cam, world_to_eye, ls, st,
                                             events);
    return integrate_enqueue_t<uint32_t>(ctl, g, vb, ss, depth_dev, depth_u16, cam, world_to_eye, ls, st, events);
}

template <typename K>
static cudaError_t integrate_batch_t(const FuseJob* jobs, int n, int passes, const FuseMaps& m, cudaStream_t st) {
    k_frame_setup_batch<<<n, 32, 0, st>>>(jobs, n);
    k_splat_emit_batch<K><<<m.splat.grid, kEmitThreads, 0, st>>>(jobs, m.splat);
    cudaError_t e = sort_batch_enqueue(jobs, n, sizeof(K), passes, m.hist, m.pass, st);
    if (e != cudaSuccess) return e;
    k_merge_partition_batch<K><<<m.partition.grid, 256, 0, st>>>(jobs, m.partition);
    k_merge_update_batch<K><<<m.merge.grid, kMergeThreads, 0, st>>>(jobs, m.merge);
    return cudaGetLastError();
}

cudaError_t integrate_batch_enqueue(const FuseJob* jobs, int n, int key_bytes, int passes, const FuseMaps& maps,
                                    cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    if (key_bytes == 8) return integrate_batch_t<uint64_t>(jobs, n, passes, maps, st);
    return integrate_batch_t<uint32_t>(jobs, n, passes, maps, st);
}

cudaError_t integrate_queue_enqueue(const FuseJob* jobs, int key_bytes, const FuseQueuePlan& plan,
                                    unsigned int* next, unsigned int* done, int ctas, cudaStream_t st) {
    if (plan.n <= 0) return cudaSuccess;
    unsigned long long limit = 0;
    {
        SortScratch probe{};
        sort_limits(&probe);
        limit = probe.spin_limit;
    }
    if (key_bytes == 8)
        k_fuse_queue<uint64_t><<<ctas, kMergeThreads, 0, st>>>(jobs, plan, next, done, limit);
    else
        k_fuse_queue<uint32_t><<<ctas, kMergeThreads, 0, st>>>(jobs, plan, next, done, limit);
    return cudaGetLastError();
}

cudaError_t bitmap_rebuild_enqueue(const DeviceCtl* ctl, const Geom& g, const VolumeBuffers& vb,
                                   const LaunchShape& ls, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(vb.bitmap, 0, vb.bitmap_words * 4, st);
    if (e) return e;
    if (vb.key_bytes == 8) k_bitmap_from_keys<uint64_t><<<ls.sms * 8, 256, 0, st>>>(ctl, g, vb);
    else k_bitmap_from_keys<uint32_t><<<ls.sms * 8, 256, 0, st>>>(ctl, g, vb);
    return cudaGetLastError();
}

cudaError_t insert_filter_enqueue(DeviceCtl* ctl, const Geom& g, VolumeBuffers& vb, const void* keys_dev,
                                  const unsigned int* n_dev, const LaunchShape& ls, cudaStream_t st) {
    k_reset_new<<<1, 1, 0, st>>>(ctl);
    if (vb.key_bytes == 8)
        k_insert_filter<uint64_t><<<ls.splat_ctas, 256, 0, st>>>(ctl, g, vb.bitmap, (const uint64_t*)keys_dev, n_dev,
                                                                (uint64_t*)vb.new_keys, vb.new_idx);
    else
        k_insert_filter<uint32_t><<<ls.splat_ctas, 256, 0, st>>>(ctl, g, vb.bitmap, (const uint32_t*)keys_dev, n_dev,
                                                                (uint32_t*)vb.new_keys, vb.new_idx);
    return cudaGetLastError();
}

// Merge of the filtered, (key, index)-sorted insert keys; values are taken
// from vals_dev[index], or Voxel() when vals_dev is null.
cudaError_t insert_merge_enqueue(DeviceCtl* ctl, const Geom& g, VolumeBuffers& vb,
                                 const float2* vals_dev, const LaunchShape& ls, cudaStream_t st) {
    FrameConst fc{};
    if (vb.key_bytes == 8) {
        MergeInputs<uint64_t> in{(const uint64_t*)vb.new_keys, vb.new_idx, vals_dev, &ctl->n_new, false};
        return merge_enqueue<uint64_t>(ctl, g, vb, in, nullptr, false, fc, ls, st);
    }
    MergeInputs<uint32_t> in{(const uint32_t*)vb.new_keys, vb.new_idx, vals_dev, &ctl->n_new, false};
    return merge_enqueue<uint32_t>(ctl, g, vb, in, nullptr, false, fc, ls, st);
}

}  // namespace kifi
