// kifi_integrate.cu -- one Integrator::Integrate (KinectFission/kifi/
// Integrator.cpp:26-71) on sm_103a, as four kernels on one stream:
//
//  k_frame_setup   derive eyeToWorld / worldToClip and the projection
//                  constants from the pose (Integrator.cpp:41-42), reset the
//                  per-frame counters.
//  k_splat_emit    DepthMap2PointCloud (Integrator.cpp:76-183) fused with
//                  ExpandChunks (:186-250) and the de-duplication of
//                  std::unique (:50-55): every valid pixel's voxel key and its
//                  seven {0,1}^3 neighbours are tested against the volume's
//                  occupancy bitmap (one bit per voxel of the res^3 grid); the
//                  thread whose atomicOr flips a bit owns that key and appends
//                  it to the frame's list of keys NEW to the volume.
//  (radix sort)    the new keys are sorted (kifi_sort.cu).
//  k_merge_update  flat_map::insert (flat_map.h:164-197) as a merge-path
//                  merge of the sorted resident keys with the sorted new keys
//                  into the other half of the ping-pong buffers, fused with
//                  UpdateVoxels (Integrator.cpp:253-358): every output voxel is
//                  projected into the frame and its (distance-sum, weight)
//                  updated before it is written -- one read and one write of
//                  the volume per frame.
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
#include "kifi_internal.h"

namespace kifi {
namespace {

constexpr int kEmitThreads = 256;
constexpr int kMergeThreads = 256;
constexpr int kMergeItems = 8;                            // outputs per thread
constexpr int kMergeTile = kMergeThreads * kMergeItems;   // 2048 outputs per tile
constexpr uint16_t kFromB = 0x8000u;

__global__ void k_frame_setup(DeviceCtl* ctl) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        ctl->n_new = 0u;
        ctl->excluded_key = 0u;
    }
}

__device__ __forceinline__ float load_depth(const void* depth, size_t i, bool u16) {
    // DepthStream::NextFrame converts 16-bit millimetres with value * 0.001f
    // (DepthStream.cpp:89-90)
    if (u16) return fmul((float)(unsigned int)__ldg((const unsigned short*)depth + i), 0.001f);
    return __ldg((const float*)depth + i);
}

__device__ __forceinline__ size_t bit_index(uint32_t key, int res) {
    return (size_t)key_x(key) + (size_t)res * ((size_t)key_y(key) + (size_t)res * key_z(key));
}

// Splat of one pixel (Integrator.cpp:121-154 for one SSE lane).
__device__ __forceinline__ bool splat_pixel(const FrameConst& fc, const float (&e2w)[16],
                                            const Geom& g, int u, int v, float d, uint32_t* key) {
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
    *key = pack30((uint32_t)ix, (uint32_t)iy, (uint32_t)iz);
    return true;
}

template <bool kU16>
__global__ void __launch_bounds__(kEmitThreads) k_splat_emit(DeviceCtl* __restrict__ ctl, Geom g,
                                                             const void* __restrict__ depth,
                                                             uint32_t* __restrict__ bitmap,
                                                             uint32_t* __restrict__ new_keys,
                                                             unsigned int new_cap,
                                                             const FrameConst fc) {
    const int W = fc.width, H = fc.height;
    const size_t P = (size_t)W * H;
    const int lane = threadIdx.x & 31;
    float e2w[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) e2w[i] = fc.eye_to_world.m[i];
    const size_t stride = (size_t)gridDim.x * kEmitThreads;
    const size_t P_round = (P + 31) / 32 * 32;  // warp-uniform trip count
    for (size_t i = (size_t)blockIdx.x * kEmitThreads + threadIdx.x; i < P_round; i += stride) {
        uint32_t key = 0;
        bool valid = false;
        if (i < P) {
            int u = (int)(i % (size_t)W), v = (int)(i / (size_t)W);
            valid = splat_pixel(fc, e2w, g, u, v, load_depth(depth, i, kU16), &key);
        }
        // the excluded key of the dilation: max splat + pack(1,1,1)
        unsigned int ex = __reduce_max_sync(0xffffffffu, valid ? key + pack30(1, 1, 1) : 0u);
        if (lane == 0 && ex) atomicMax(&ctl->excluded_key, ex);
        // neighbouring pixels often land in one voxel: one emitter per key
        unsigned int peers = __match_any_sync(0xffffffffu, valid ? key : 0xffffffffu);
        const bool emitter = valid && (lane == __ffs(peers) - 1);
        // The dilation's 8 keys are 4 (y, z) rows of an (x, x+1) pair.  The
        // pair's bits are adjacent in the bitmap, so one word probe covers
        // both unless x is the last bit of its word.  All probes are issued
        // before any decision; atomics only for bits still clear.
        uint32_t got[4] = {0u, 0u, 0u, 0u};   // bit 0: key + dx=0 new, bit 1: dx=1 new
        if (emitter) {
            uint32_t* wp[4];
            uint32_t* wq[4];
            uint32_t m0[4], m1[4], pre0[4], pre1[4];
#pragma unroll
            for (int o = 0; o < 4; ++o) {
                const uint32_t k0 = key + pack30(0, o & 1, o >> 1);
                const size_t b = bit_index(k0, g.res);
                const uint32_t sh = (uint32_t)(b & 31);
                wp[o] = bitmap + (b >> 5);
                wq[o] = bitmap + ((b + 1) >> 5);
                m0[o] = sh == 31 ? 0x80000000u : (3u << sh);
                m1[o] = sh == 31 ? 1u : 0u;
                pre0[o] = __ldcg(wp[o]);
                pre1[o] = sh == 31 ? __ldcg(wq[o]) : 0u;
            }
#pragma unroll
            for (int o = 0; o < 4; ++o) {
                const uint32_t sh = m0[o] == 0x80000000u && m1[o] ? 31u : (uint32_t)(__ffs(m0[o]) - 1);
                uint32_t need0 = m0[o] & ~pre0[o];
                uint32_t need1 = m1[o] & ~pre1[o];
                uint32_t flipped0 = 0u, flipped1 = 0u;
                if (need0) flipped0 = need0 & ~atomicOr(wp[o], need0);
                if (need1) flipped1 = need1 & ~atomicOr(wq[o], need1);
                // dx = 0 is bit sh of word 0; dx = 1 is bit sh+1 of word 0, or bit 0 of word 1
                const uint32_t n0 = (flipped0 >> sh) & 1u;
                const uint32_t n1 = m1[o] ? (flipped1 & 1u) : ((flipped0 >> (sh + 1)) & 1u);
                got[o] = n0 | (n1 << 1);
            }
        }
        // warp-aggregated append: one atomic per warp
        const unsigned int cnt = __popc(got[0] | (got[1] << 2) | (got[2] << 4) | (got[3] << 6));
        unsigned int incl = cnt;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const unsigned int y = __shfl_up_sync(0xffffffffu, incl, d);
            if (lane >= d) incl += y;
        }
        const unsigned int total = __shfl_sync(0xffffffffu, incl, 31);
        if (total) {
            unsigned int base = 0;
            if (lane == 31) base = atomicAdd(&ctl->n_new, total);
            base = __shfl_sync(0xffffffffu, base, 31);
            unsigned int at = base + incl - cnt;
#pragma unroll
            for (int o = 0; o < 4; ++o) {
                const uint32_t k0 = key + pack30(0, o & 1, o >> 1);
#pragma unroll
                for (int dx = 0; dx < 2; ++dx) {
                    if (!((got[o] >> dx) & 1u)) continue;
                    if (at < new_cap) new_keys[at] = k0 + (uint32_t)dx;
                    else atomicOr(&ctl->status, KIFI_DEV_ERR_CAPACITY);
                    ++at;
                }
            }
        }
    }
}

// UpdateVoxels for one voxel (Integrator.cpp:273-322 for one SSE lane).
template <bool kU16>
__device__ __forceinline__ void update_voxel(uint32_t key, float2& val, const FrameConst& fc,
                                             const float (&w2c)[16], const Geom& g,
                                             const void* depth) {
    // VoxelCenter: index * (vlen, vlen, vlen, 1) + (off, off, off, 0)
    float c[4];
    c[0] = fadd(fmul((float)key_x(key), g.vlen), g.center_off);
    c[1] = fadd(fmul((float)key_y(key), g.vlen), g.center_off);
    c[2] = fadd(fmul((float)key_z(key), g.vlen), g.center_off);
    c[3] = 1.0f;  // 1 * 1 + 0
    // rows 0, 1, 3 of worldToClip * c (mat_vec's order); row 2 below
    auto row = [&](int i) {
        return fadd(fadd(fmul(w2c[i], c[0]), fmul(w2c[4 + i], c[1])),
                    fadd(fmul(w2c[8 + i], c[2]), fmul(w2c[12 + i], c[3])));
    };
    const float x = row(0), y = row(1), w = row(3);
    // lane w: (w/w) * 0 + 0 lies in [-FLT_MAX, FLT_MAX) iff w/w is finite,
    // i.e. iff w is finite and non-zero (w/w is then exactly 1).
    if (!(isfinite(w) && w != 0.0f)) return;
    // lane z: (z/w) * 0 + 0 lies in [-1, 1) iff z/w is finite.  When the
    // host has bounded |z| by 1e18 over the whole volume (fc.z_bounded), any
    // |w| >= 1e-18 keeps the quotient finite and z need not be formed.
    if (!(fc.z_bounded && fabsf(w) >= 1e-18f)) {
        const float z = row(2);
        if (!isfinite(z)) return;
        if (!(fabsf(z) <= 1e18f && fabsf(w) >= 1e-18f) && !isfinite(fdiv(z, w))) return;
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
        if (!(u >= 0.0f && u < (float)fc.width && v >= 0.0f && v < (float)fc.height)) return;
        const size_t px = (uint32_t)u;
        const size_t py = (size_t)fc.height - (uint32_t)v - 1;
        const float d = load_depth(depth, py * (size_t)fc.width + px, kU16);
        const float sd = fsub(d, w);
        if (d > 0.0f && sd >= -g.trunc) {
            val.x = fadd(val.x, (g.trunc < sd) ? g.trunc : sd);
            val.y = fadd(val.y, 1.0f);
        }
        return;
    }
    const float rw = __fdividef(1.0f, w);
    const float ua = fadd(fmul(fmul(x, rw), fc.half_w), fc.half_w);
    const float va = fadd(fmul(fmul(y, rw), fc.half_h), fc.half_h);
    const float Wf = (float)fc.width, Hf = (float)fc.height;
    if (!(ua >= -0.5f && ua <= Wf + 0.5f && va >= -0.5f && va <= Hf + 0.5f)) return;
    constexpr float kE = 1.0f / 256.0f;
    float u, v;
    {
        const float fu = floorf(ua), fv = floorf(va);
        const bool su = ua - fu >= kE && fu + 1.0f - ua >= kE;
        const bool sv = va - fv >= kE && fv + 1.0f - va >= kE;
        u = su ? fu + 0.5f : fadd(fmul(fdiv(x, w), fc.half_w), fc.half_w);
        v = sv ? fv + 0.5f : fadd(fmul(fdiv(y, w), fc.half_h), fc.half_h);
    }
    if (!(u >= 0.0f && u < Wf && v >= 0.0f && v < Hf)) return;
    const size_t px = (uint32_t)u;
    const size_t py = (size_t)fc.height - (uint32_t)v - 1;
    const float d = load_depth(depth, py * (size_t)fc.width + px, kU16);
    const float sd = fsub(d, w);
    if (d > 0.0f && sd >= -g.trunc) {
        // Voxel::Update(std::min(signedDist, trunc)) (Voxel.h:53-57)
        val.x = fadd(val.x, (g.trunc < sd) ? g.trunc : sd);
        val.y = fadd(val.y, 1.0f);
    }
}

// number of A elements among the first d outputs of merge(A, B); A and B
// are sorted and disjoint.
__device__ __forceinline__ unsigned long long merge_path(const uint32_t* __restrict__ A,
                                                         unsigned long long na,
                                                         const uint32_t* __restrict__ B,
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

struct MergeInputs {
    const uint32_t* b_keys;   // sorted new keys
    const uint32_t* b_index;  // optional: b's position in b_vals (inserts)
    const float2* b_vals;     // optional values of new keys; null = Voxel()
    const unsigned int* b_count;
    bool update;              // run UpdateVoxels on the merged volume
};

// Merge set-up and partition.  Thread 0 settles the merge: drops the
// dilation's excluded key when it is the largest new key (clearing its
// occupancy bit), checks the capacity and publishes (e, N1).  Every thread t
// then computes the merge-path split of output tile t: the number of resident
// keys among the first t*kMergeTile outputs.  The binary searches of all
// tiles run in parallel here instead of serialising the merge kernel's tiles.
__global__ void __launch_bounds__(256) k_merge_partition(DeviceCtl* __restrict__ ctl, Geom g,
                                                          VolumeBuffers vb, MergeInputs in,
                                                          unsigned long long* __restrict__ splits,
                                                          unsigned int max_tiles) {
    __shared__ unsigned long long s_e, s_n1;
    __shared__ int s_ok;
    const unsigned int cur = ctl->cur;
    const unsigned long long N0 = ctl->n[cur];
    // select rather than index: a runtime index into a parameter array
    // would force the array into local memory
    const uint32_t* __restrict__ A = cur ? vb.keys[1] : vb.keys[0];
    const uint32_t* __restrict__ B = in.b_keys;
    if (threadIdx.x == 0) {
        unsigned long long e = *in.b_count;
        const uint32_t excluded = ctl->excluded_key;
        const bool drop = e > 0 && excluded != 0u && B[e - 1] == excluded;
        if (drop) --e;
        const bool ok = N0 + e <= vb.cap;
        s_e = e;
        s_n1 = N0 + e;
        s_ok = ok;
        if (blockIdx.x == 0) {
            ctl->merge_e = e;
            ctl->merge_n1 = N0 + e;
            ctl->merge_ok = ok ? 1u : 0u;
            if (drop) {
                size_t b = bit_index(excluded, g.res);
                atomicAnd(vb.bitmap + (b >> 5), ~(1u << (b & 31)));
            }
            if (!ok) atomicOr(&ctl->status, KIFI_DEV_ERR_CAPACITY);
        }
    }
    __syncthreads();
    const unsigned long long e = s_e, N1 = s_n1;
    if (!s_ok) {
        // no room: leave the volume as it was and take the new keys back out
        // of the occupancy bitmap; the host grows the buffers and retries.
        for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < e;
             i += (unsigned long long)gridDim.x * blockDim.x) {
            size_t b = bit_index(B[i], g.res);
            atomicAnd(vb.bitmap + (b >> 5), ~(1u << (b & 31)));
        }
        return;
    }
    const unsigned long long n_tiles = (N1 + kMergeTile - 1) / kMergeTile;
    for (unsigned long long t = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
         t <= n_tiles && t < max_tiles; t += (unsigned long long)gridDim.x * blockDim.x) {
        const unsigned long long d = t * kMergeTile < N1 ? t * kMergeTile : N1;
        splits[t] = merge_path(A, N0, B, e, d);
    }
}

// One output voxel: value from A or Voxel(), TSDF update when inside the
// reference's update range.
template <bool kU16>
__device__ __forceinline__ void finish_voxel(uint32_t key, float2& val, unsigned long long pos,
                                             unsigned long long upd_end, const FrameConst& fc,
                                             const float (&w2c)[16], const Geom& g,
                                             const void* depth) {
    if (pos < upd_end) update_voxel<kU16>(key, val, fc, w2c, g, depth);
}

template <bool kU16>
__global__ void __launch_bounds__(kMergeThreads) k_merge_update(DeviceCtl* __restrict__ ctl, Geom g,
                                                                VolumeBuffers vb, MergeInputs in,
                                                                const void* __restrict__ depth,
                                                                const unsigned long long* __restrict__ splits,
                                                                const FrameConst fc) {
    __shared__ uint32_t sA_k[kMergeTile + 8];
    __shared__ float2 sA_v[kMergeTile + 4];
    __shared__ uint32_t sB_k[kMergeTile];
    __shared__ uint16_t sSrc[kMergeTile];

    if (!ctl->merge_ok) return;
    const unsigned int cur = ctl->cur, out = cur ^ 1u;
    const unsigned long long N0 = ctl->n[cur];
    const unsigned long long e = ctl->merge_e;
    const unsigned long long N1 = ctl->merge_n1;
    const uint32_t* __restrict__ A = cur ? vb.keys[1] : vb.keys[0];
    const float2* __restrict__ Av = cur ? vb.vals[1] : vb.vals[0];
    const uint32_t* __restrict__ B = in.b_keys;
    const unsigned long long upd_end = in.update ? (N1 / 4 * 4) : 0ull;
    uint32_t* __restrict__ outK = out ? vb.keys[1] : vb.keys[0];
    float2* __restrict__ outV = out ? vb.vals[1] : vb.vals[0];
    const unsigned long long n_tiles = (N1 + kMergeTile - 1) / kMergeTile;
    float w2c[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) w2c[i] = fc.world_to_clip.m[i];

    for (unsigned long long t = blockIdx.x; t < n_tiles; t += gridDim.x) {
        const unsigned long long d0 = t * kMergeTile;
        const unsigned long long d1 = (d0 + kMergeTile < N1) ? d0 + kMergeTile : N1;
        const int len = (int)(d1 - d0);
        const unsigned long long a0 = splits[t], a1 = splits[t + 1];
        const int na = (int)(a1 - a0), nb = len - na;
        if (nb == 0) {
            // only resident voxels in this tile: straight streaming, no barrier
            const bool vec = (a0 & 3ull) == 0;
#pragma unroll
            for (int r = 0; r < kMergeItems / 4; ++r) {
                const int j0 = threadIdx.x * 4 + r * kMergeThreads * 4;
                if (j0 >= len) break;
                uint32_t k0, k1, k2, k3;
                float2 v0, v1, v2, v3;
                const unsigned long long ia = a0 + j0;
                if (vec && j0 + 4 <= len) {
                    const uint4 kk = __ldcs((const uint4*)(A + ia));
                    const float4 va = __ldcs((const float4*)(Av + ia));
                    const float4 vb4 = __ldcs((const float4*)(Av + ia + 2));
                    k0 = kk.x; k1 = kk.y; k2 = kk.z; k3 = kk.w;
                    v0 = make_float2(va.x, va.y); v1 = make_float2(va.z, va.w);
                    v2 = make_float2(vb4.x, vb4.y); v3 = make_float2(vb4.z, vb4.w);
                } else {
                    const int m = len - j0;
                    k0 = __ldcs(A + ia); v0 = __ldcs(Av + ia);
                    k1 = m > 1 ? __ldcs(A + ia + 1) : 0u; v1 = m > 1 ? __ldcs(Av + ia + 1) : v0;
                    k2 = m > 2 ? __ldcs(A + ia + 2) : 0u; v2 = m > 2 ? __ldcs(Av + ia + 2) : v0;
                    k3 = m > 3 ? __ldcs(A + ia + 3) : 0u; v3 = m > 3 ? __ldcs(Av + ia + 3) : v0;
                }
                const unsigned long long p = d0 + j0;
                finish_voxel<kU16>(k0, v0, p, upd_end, fc, w2c, g, depth);
                finish_voxel<kU16>(k1, v1, p + 1, upd_end, fc, w2c, g, depth);
                finish_voxel<kU16>(k2, v2, p + 2, upd_end, fc, w2c, g, depth);
                finish_voxel<kU16>(k3, v3, p + 3, upd_end, fc, w2c, g, depth);
                if (j0 + 4 <= len) {
                    __stcs((uint4*)(outK + p), make_uint4(k0, k1, k2, k3));
                    __stcs((float4*)(outV + p), make_float4(v0.x, v0.y, v1.x, v1.y));
                    __stcs((float4*)(outV + p + 2), make_float4(v2.x, v2.y, v3.x, v3.y));
                } else {
                    const int m = len - j0;
                    outK[p] = k0; outV[p] = v0;
                    if (m > 1) { outK[p + 1] = k1; outV[p + 1] = v1; }
                    if (m > 2) { outK[p + 2] = k2; outV[p + 2] = v2; }
                }
            }
            continue;
        }
        // mixed tile: stage both ranges in shared memory and merge there
        const unsigned long long b0 = d0 - a0;
        const unsigned long long ka = a0 & ~3ull;
        const int koff = (int)(a0 - ka);
        for (int i = threadIdx.x * 4; i < koff + na; i += kMergeThreads * 4)
            *(uint4*)&sA_k[i] = __ldcs((const uint4*)(A + ka + i));
        const unsigned long long va = a0 & ~1ull;
        const int voff = (int)(a0 - va);
        for (int i = threadIdx.x * 2; i < voff + na; i += kMergeThreads * 2)
            *(float4*)&sA_v[i] = __ldcs((const float4*)(Av + va + i));
        for (int i = threadIdx.x; i < nb; i += kMergeThreads) sB_k[i] = B[b0 + i];
        __syncthreads();
        {
            const int dd = threadIdx.x * kMergeItems;
            if (dd < len) {
                int lo = dd > nb ? dd - nb : 0, hi = dd < na ? dd : na;
                while (lo < hi) {
                    int mid = (lo + hi) >> 1;
                    if (sA_k[koff + mid] < sB_k[dd - 1 - mid]) lo = mid + 1;
                    else hi = mid;
                }
                int ia = lo, ib = dd - lo;
                const int end = dd + kMergeItems < len ? dd + kMergeItems : len;
                for (int j = dd; j < end; ++j) {
                    bool takeA = ib >= nb || (ia < na && sA_k[koff + ia] < sB_k[ib]);
                    sSrc[j] = takeA ? (uint16_t)ia++ : (uint16_t)(kFromB | ib++);
                }
            }
        }
        __syncthreads();
        for (int j = threadIdx.x; j < len; j += kMergeThreads) {
            const uint16_t src = sSrc[j];
            uint32_t key;
            float2 val;
            if (!(src & kFromB)) {
                key = sA_k[koff + src];
                val = sA_v[voff + src];
            } else {
                const int ib = src & ~kFromB;
                key = sB_k[ib];
                if (in.b_vals) val = in.b_vals[in.b_index ? in.b_index[b0 + ib] : b0 + ib];
                else val = make_float2(0.0f, 0.0f);
            }
            finish_voxel<kU16>(key, val, d0 + j, upd_end, fc, w2c, g, depth);
            __stcs(outK + d0 + j, key);
            __stcs(outV + d0 + j, val);
        }
        __syncthreads();
    }
    // the last CTA to finish publishes the new volume
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        unsigned int prev = atomicAdd(&ctl->tile_counter[7], 1u);
        if (prev == gridDim.x - 1) {
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

// inserts: keep keys not yet in the volume (flat_map::insert keeps resident
// values), appending (key, position) pairs for the sort.
__global__ void k_insert_filter(DeviceCtl* ctl, Geom g, uint32_t* bitmap, const uint32_t* keys,
                                const unsigned int* n_ptr, uint32_t* out_keys, uint32_t* out_idx) {
    const unsigned int n = *n_ptr;
    const int lane = threadIdx.x & 31;
    const unsigned int n_round = (n + 31) / 32 * 32;
    for (unsigned int i = blockIdx.x * blockDim.x + threadIdx.x; i < n_round;
         i += gridDim.x * blockDim.x) {
        bool mine = false;
        uint32_t k = 0;
        if (i < n) {
            k = keys[i];
            size_t b = bit_index(k, g.res);
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

__global__ void k_reset_new(DeviceCtl* ctl) {
    ctl->n_new = 0u;
    ctl->excluded_key = 0u;
}

}  // namespace

int merge_blocks_per_sm() {
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_merge_update<true>, kMergeThreads, 0) !=
            cudaSuccess ||
        n < 1)
        n = 4;
    return n;
}

static unsigned int max_tiles_of(const VolumeBuffers& vb) {
    return (unsigned int)((vb.cap + kMergeTile - 1) / kMergeTile + 2);
}

static cudaError_t merge_enqueue(DeviceCtl* ctl, const Geom& g, VolumeBuffers& vb,
                                 const MergeInputs& in, const void* depth, bool u16,
                                 const FrameConst& fc, const LaunchShape& ls, cudaStream_t st,
                                 cudaEvent_t after_partition = nullptr) {
    const unsigned int mt = max_tiles_of(vb);
    k_merge_partition<<<(mt + 255) / 256, 256, 0, st>>>(ctl, g, vb, in, vb.splits, mt);
    if (after_partition) cudaEventRecord(after_partition, st);
    if (u16)
        k_merge_update<true><<<ls.merge_ctas, kMergeThreads, 0, st>>>(ctl, g, vb, in, depth,
                                                                     vb.splits, fc);
    else
        k_merge_update<false><<<ls.merge_ctas, kMergeThreads, 0, st>>>(ctl, g, vb, in, depth,
                                                                      vb.splits, fc);
    return cudaGetLastError();
}

cudaError_t integrate_enqueue(DeviceCtl* ctl, const Geom& g, VolumeBuffers& vb, SortScratch& ss,
                              const void* depth_dev, bool depth_u16, const kifi_camera& cam,
                              const Mat4& world_to_eye, const LaunchShape& ls, cudaStream_t st,
                              cudaEvent_t* events) {
    // frame constants on the host, in the reference's float order
    FrameConst fc = make_frame_const(cam, world_to_eye, g.res);
    fc.z_bounded = clip_z_bounded(fc.world_to_clip, g.side);
    if (events) cudaEventRecord(events[0], st);
    k_frame_setup<<<1, 32, 0, st>>>(ctl);
    const unsigned int new_cap = (unsigned int)vb.new_cap;
    if (depth_u16)
        k_splat_emit<true><<<ls.splat_ctas, kEmitThreads, 0, st>>>(ctl, g, depth_dev, vb.bitmap,
                                                                   vb.new_keys, new_cap, fc);
    else
        k_splat_emit<false><<<ls.splat_ctas, kEmitThreads, 0, st>>>(ctl, g, depth_dev, vb.bitmap,
                                                                    vb.new_keys, new_cap, fc);
    if (events) cudaEventRecord(events[1], st);
    cudaError_t e = sort_u32(vb.new_keys, nullptr, &ctl->n_new, ss, &ctl->status, ls.sort_ctas, st);
    if (e != cudaSuccess) return e;
    if (events) cudaEventRecord(events[2], st);
    MergeInputs in{vb.new_keys, nullptr, nullptr, &ctl->n_new, true};
    e = merge_enqueue(ctl, g, vb, in, depth_dev, depth_u16, fc, ls, st, events ? events[3] : nullptr);
    if (events) cudaEventRecord(events[4], st);
    return e;
}

cudaError_t insert_filter_enqueue(DeviceCtl* ctl, const Geom& g, VolumeBuffers& vb,
                                  const uint32_t* keys_dev, const unsigned int* n_dev,
                                  const LaunchShape& ls, cudaStream_t st) {
    k_reset_new<<<1, 1, 0, st>>>(ctl);
    k_insert_filter<<<ls.splat_ctas, 256, 0, st>>>(ctl, g, vb.bitmap, keys_dev, n_dev, vb.new_keys,
                                                   vb.new_idx);
    return cudaGetLastError();
}

// Merge of the filtered, (key, index)-sorted insert keys; values are taken
// from vals_dev[index], or Voxel() when vals_dev is null.
cudaError_t insert_merge_enqueue(DeviceCtl* ctl, const Geom& g, VolumeBuffers& vb,
                                 const float2* vals_dev, const LaunchShape& ls, cudaStream_t st) {
    MergeInputs in{vb.new_keys, vb.new_idx, vals_dev, &ctl->n_new, false};
    FrameConst fc{};
    return merge_enqueue(ctl, g, vb, in, nullptr, false, fc, ls, st);
}

}  // namespace kifi
