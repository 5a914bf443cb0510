// kifi_mesh.cu -- sparse marching cubes over the sorted voxel keys on
// sm_103a: kifi::Mesher::Mesh (KinectFission/kifi/Mesher.cpp:14-45) and
// Mesher::Generate<bool> (:85-229).
//
// The reference walks the sorted volume backwards (voxels n-2 .. 0) with
// three neighbour pointers (+y, +z, +yz) that start at n-2 and only move down.
// After the walk for voxel i each pointer sits at
//     min(n-2, upper_bound(keys, key_i + delta) - 1),
// a closed form that depends on voxel i alone, so every voxel is handled by
// its own thread:
//
//  k_row_directory  start index of every (y, z) key row (key >> b, b key bits
//                   per axis); a neighbour search then only scans one row,
//                   starting where the searching voxel sits in its own row.
//  k_mesh_tile_ranges  per tile of 1024 voxels and neighbour offset, the
//                   ranges of positions its voxels' lookups fall in.
//  k_mesh_status    one status byte per voxel (weight, distance sign).
//  k_mesh_classify_tiled  per voxel i in [0, n-2] with weight > 0: which of its
//                   +x/+y/+z edges carry a vertex (Mesher.cpp:140-168) and,
//                   for Mesh(verts, indices), the cube's marching-cubes case
//                   and triangle count (:172-226); a voxel with any output
//                   keeps its +y, +z and +yz lookups for emission.  Per tile
//                   it also scans the vertex and index counts (a voxel's
//                   first vertex within the tile goes into its flags, its
//                   first index beside its lookups), lists the tile's voxels
//                   with output and writes the tile's packed (index, vertex)
//                   totals.
//  k_scan_tile_sums one CTA turns the tile totals into tile offsets.
//  k_mesh_emit      per tile, over its list of voxels with output: writes the
//                   vertices (by the voxel's lane) and the triangle indices
//                   (spread over the warp's lanes).
//
// Output order equals the reference's:
//  * Mesh(verts): vertices in generation order -- voxels descending, axes
//    x, y, z -- so voxel i's vertices start after those of all voxels j > i.
//  * Mesh(verts, indices): vertices sorted by id 3*key+axis (Mesher.cpp:25-26),
//    which is ascending voxel order; triangles in generation order (voxels
//    descending, table order), each index mapped to its vertex's rank
//    (:28-44).  That mapping walk stops at the first index id that has no
//    vertex; every index id at or above it keeps its raw id.  k_mesh_emit
//    reproduces this: its first pass records the smallest missing id, and a
//    second pass reads that bound on the device and rewrites the indices at
//    or above it (it returns at once when no id was missing).
#include "kifi_internal.h"
#include "mc_table.cuh"

namespace kifi {
namespace {

constexpr int kThreads = 256;

template <typename K>
__device__ __forceinline__ unsigned long long lower_bound_key(const K* __restrict__ k, unsigned long long n, K t) {
    unsigned long long lo = 0, hi = n;
    while (lo < hi) {
        unsigned long long mid = (lo + hi) >> 1;
        if (k[mid] < t) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// row_start[r] = first index whose (z, y) row (key >> b) >= r, for r in [0, 2^2b]
template <typename K>
__global__ void k_row_directory(const K* __restrict__ keys, const unsigned int* __restrict__ n_dev, int b,
                                unsigned int* __restrict__ row_start) {
    const unsigned long long n = *n_dev;
    const unsigned int rows = 1u << (2 * b);
    for (unsigned int r = blockIdx.x * blockDim.x + threadIdx.x; r <= rows; r += gridDim.x * blockDim.x)
        row_start[r] = (unsigned int)lower_bound_key<K>(keys, n, (K)r << b);
}

// upper_bound(keys, t) using the row directory: keys of t's row lie in
// [row_start[r], row_start[r+1]) sorted by x.  `hint` is where t probably
// sits within its row -- the searching voxel's own offset within its row,
// since neighbouring rows of a surface hold similar runs of x.  Two probes
// around the guess settle most lookups; otherwise a binary search of the
// side the probes leave.  The result does not depend on the hint.
template <typename K>
__device__ __forceinline__ unsigned int upper_bound_row(const K* __restrict__ keys,
                                                        const unsigned int* __restrict__ rs,
                                                        K t, unsigned int n, const Codec<K>& cd,
                                                        unsigned int hint) {
    const unsigned long long r = cd.row(t);
    // a neighbour of a voxel on the last z slice lies past every key
    if (r >= (1ull << (2 * cd.b))) return n;
    unsigned int lo = rs[r], hi = rs[r + 1];
    if (lo == hi) return lo;
    const unsigned int g = hint < hi - lo ? lo + hint : hi;
    const bool right = g < hi && keys[g] <= t;   // the answer lies above g
    const bool left = g > lo && keys[g - 1] > t;  // ... or below g
    if (right) lo = g + 1;
    else if (left) hi = g - 1;  // keys[g - 1] > t: the answer is at most g - 1
    else return g;
    while (lo < hi) {
        unsigned int mid = (lo + hi) >> 1;
        if (keys[mid] <= t) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// neighbour pointer position after the reference's walk (see file comment)
template <typename K>
__device__ __forceinline__ unsigned int walk_ptr(const K* keys, const unsigned int* rs, K t, unsigned int n,
                                                 const Codec<K>& cd, unsigned int hint) {
    unsigned int p = upper_bound_row<K>(keys, rs, t, n, cd, hint) - 1u;
    return p < n - 2 ? p : n - 2;
}

__device__ __forceinline__ float vdist(float2 v) { return fdiv(v.x, v.y); }  // Voxel::Distance

// Packed per-voxel flags: bits 0-2 the vertex axes, 3-5 the triangle count,
// 6-13 the marching-cubes case, 14-24 the voxel's first vertex within its
// classification tile (at most 3 x 1024 = 3072).
__device__ __forceinline__ unsigned int f_axes(unsigned int f) { return f & 7u; }
__device__ __forceinline__ unsigned int f_tris(unsigned int f) { return (f >> 3) & 7u; }
__device__ __forceinline__ unsigned int f_case(unsigned int f) { return (f >> 6) & 0xffu; }
__device__ __forceinline__ unsigned int f_vofs(unsigned int f) { return f >> 14; }

// exclusive scan of one 64-bit value per thread over a CTA of kT threads;
// the CTA's total to *total
template <int kT, bool kTrailingSync = true>
__device__ __forceinline__ unsigned long long block_exclusive_scan(unsigned long long x,
                                                                   unsigned long long* total) {
    __shared__ unsigned long long warp_sums[kT / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned long long inc = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        unsigned long long y = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += y;
    }
    if (lane == 31) warp_sums[warp] = inc;
    __syncthreads();
    unsigned long long before = 0, all = 0;
#pragma unroll
    for (int w = 0; w < kT / 32; ++w) {
        if (w < warp) before += warp_sums[w];
        all += warp_sums[w];
    }
    if (kTrailingSync) __syncthreads();  // warp_sums may be rewritten next
    *total = all;
    return before + inc - x;
}

struct Cube {
    unsigned int idx[8];  // voxel index of each corner (valid where found)
    float2 val[8];        // Voxel() = (0,0) where not found
};

// Corner lookups of Mesher.cpp:122-132 (corners 0,1,2,4) and, when
// kTris, :174-181 (corners 3,5,6,7).  Corner c = (c&1, c>>1&1, c>>2) in the
// reference's voxels[] numbering: self, +x, +y, +xy, +z, +xz, +yz, +xyz.
template <bool kTris, typename K>
__device__ __forceinline__ void load_cube(const K* __restrict__ keys,
                                          const float2* __restrict__ vals,
                                          const unsigned int* __restrict__ rs, unsigned int n,
                                          unsigned int i, Cube& c, const Codec<K>& cd) {
    const K key = keys[i];
    const float2 zero = make_float2(0.0f, 0.0f);
    // this voxel's offset within its row, where its neighbours likely sit in theirs
    const unsigned int hint = i - rs[cd.row(key)];
    c.idx[0] = i;
    c.val[0] = vals[i];
    c.idx[1] = i + 1;
    c.val[1] = keys[i + 1] == key + cd.pack(1, 0, 0) ? vals[i + 1] : zero;
    const unsigned int iTop = walk_ptr<K>(keys, rs, key + cd.pack(0, 1, 0), n, cd, hint);
    const unsigned int iFront = walk_ptr<K>(keys, rs, key + cd.pack(0, 0, 1), n, cd, hint);
    c.idx[2] = iTop;
    c.val[2] = keys[iTop] == key + cd.pack(0, 1, 0) ? vals[iTop] : zero;
    c.idx[4] = iFront;
    c.val[4] = keys[iFront] == key + cd.pack(0, 0, 1) ? vals[iFront] : zero;
    if (kTris) {
        const unsigned int iFT = walk_ptr<K>(keys, rs, key + cd.pack(0, 1, 1), n, cd, hint);
        c.idx[6] = iFT;
        c.val[6] = keys[iFT] == key + cd.pack(0, 1, 1) ? vals[iFT] : zero;
        c.idx[3] = iTop + 1;
        c.val[3] = keys[iTop + 1] == key + cd.pack(1, 1, 0) ? vals[iTop + 1] : zero;
        c.idx[5] = iFront + 1;
        c.val[5] = keys[iFront + 1] == key + cd.pack(1, 0, 1) ? vals[iFront + 1] : zero;
        c.idx[7] = iFT + 1;
        c.val[7] = keys[iFT + 1] == key + cd.pack(1, 1, 1) ? vals[iFT + 1] : zero;
    }
}

// vertex axes of a voxel: bit a set when edge +a carries a vertex
// Mesher.cpp:140-168's test Distance(self) * Distance(neighbour) <= 0
// without the divisions where its outcome is certain: for 2^-30 <= |x|, |w|
// <= 2^30 (both voxels) each quotient x / w is a float of magnitude in
// [2^-60, 2^60], so their product is a normal non-zero float (magnitude in
// [2^-120, 2^120]) whose sign is the product of the four operand signs; it
// is <= 0 exactly when the two quotients differ in sign.  Zeros, NaNs,
// infinities and the rest of the range take the reference's divisions.
__device__ __forceinline__ bool in_sign_range(float2 v) {
    const float ax = fabsf(v.x), aw = fabsf(v.y);
    return ax >= 0x1p-30f && ax <= 0x1p30f && aw >= 0x1p-30f && aw <= 0x1p30f;
}
// Voxel::Distance(v) < 0 without the division where its sign is certain:
// for 2^-100 <= |x| and 2^-100 <= |w| <= 2^24 the quotient x / w is a
// normal non-zero float (|x / w| >= 2^-124), so it is negative exactly when
// x and w differ in sign.  Zeros, NaNs, infinities and the rest of the
// range take the reference's division.
__device__ __forceinline__ bool dist_negative(float2 v) {
    const float ax = fabsf(v.x), aw = fabsf(v.y);
    if (ax >= 0x1p-100f && aw >= 0x1p-100f && aw <= 0x1p24f) return (v.x < 0.0f) != (v.y < 0.0f);
    return vdist(v) < 0.0f;
}

// Classification reads a voxel through one status byte, computed once per
// staged voxel: E weight != 0 (the reference's skip test, :172-181), P
// weight > 0 (the vertex test's neighbour condition, :140-168), N
// Distance() < 0 (the case bit, :191-199, exact through dist_negative), R
// operands in in_sign_range, S the quotient's sign (x < 0 != w < 0).  A
// voxel that is not found reads as status 0, as Voxel() = (0, 0) does.
constexpr unsigned int kStE = 1, kStP = 2, kStN = 4, kStR = 8, kStS = 16;
__device__ __forceinline__ unsigned int voxel_status(float2 v) {
    unsigned int s = 0;
    if (v.y != 0.0f) s |= kStE;
    if (v.y > 0.0f) s |= kStP;
    if (dist_negative(v)) s |= kStN;
    if (in_sign_range(v)) s |= kStR;
    if ((v.x < 0.0f) != (v.y < 0.0f)) s |= kStS;
    return s;
}

// the status of every voxel (one byte each, four per 32-bit store)
__global__ void __launch_bounds__(kThreads) k_mesh_status(const float2* __restrict__ vals,
                                                          const unsigned int* __restrict__ n_dev,
                                                          unsigned int* __restrict__ status4) {
    const unsigned int n = *n_dev;
    const float4* v2 = reinterpret_cast<const float4*>(vals);  // two voxels per vector
    for (unsigned int q = blockIdx.x * blockDim.x + threadIdx.x; q < (n + 3u) / 4u; q += gridDim.x * blockDim.x) {
        const unsigned int i = 4u * q;
        unsigned int word = 0;
        if (i + 4u <= n) {
            const float4 a = __ldg(v2 + 2 * q), b = __ldg(v2 + 2 * q + 1);
            word = voxel_status(make_float2(a.x, a.y)) | voxel_status(make_float2(a.z, a.w)) << 8 |
                   voxel_status(make_float2(b.x, b.y)) << 16 | voxel_status(make_float2(b.z, b.w)) << 24;
        } else {
            for (unsigned int k = 0; i + k < n; ++k) word |= voxel_status(vals[i + k]) << (8u * k);
        }
        status4[q] = word;
    }
}

// One live voxel's flags without the tile offset -- vertex axes, triangle
// count, case -- from its corners' statuses st and indices idx (corner c =
// (c&1, c>>1&1, c>>2): self, +x, +y, +xy, +z, +xz, +yz, +xyz).  A vertex
// test whose operands are out of in_sign_range takes the reference's
// divisions on the voxels themselves.
template <bool kTris>
__device__ __forceinline__ unsigned int classify_status(const unsigned int (&st)[8], const unsigned int (&idx)[8],
                                                        const float2* __restrict__ vals, const uint64_t* s_mc) {
    unsigned int f = 0;
    const unsigned int s0 = st[0];
    const int nb[3] = {1, 2, 4};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const unsigned int o = st[nb[a]];
        if (!(o & kStP)) continue;
        bool cross;
        if (s0 & o & kStR) cross = ((s0 ^ o) & kStS) != 0u;
        else cross = fmul(vdist(vals[idx[0]]), vdist(vals[idx[nb[a]]])) <= 0.0f;
        if (cross) f |= 1u << a;
    }
    if (kTris) {
        const unsigned int all = st[1] & st[2] & st[3] & st[4] & st[5] & st[6] & st[7];
        if (all & kStE) {
            // the reference's corner bit order (Mesher.cpp:191-199)
            auto neg = [&](int q) { return (st[q] & kStN) ? 1u : 0u; };
            const unsigned int lut = neg(0) << 2 | neg(1) << 3 | neg(2) << 6 | neg(3) << 7 | neg(4) << 1 |
                                     neg(5) << 0 | neg(6) << 5 | neg(7) << 4;
            const unsigned int tris = mc_tri_count_of(s_mc[lut]);
            if (tris) f |= tris << 3 | lut << 6;
        }
    }
    return f;
}

// Classification by tiles of kClassTile consecutive voxels.  For a
// neighbour offset d (+y, +z, +yz) the lookup positions walk_ptr(key_i + d)
// are non-decreasing in i, so the positions of a run of voxels all lie
// between those of its first and last voxel.  The +y positions start at the
// voxel itself, so the tile and its +y lookups are one region (A) from the
// tile's first voxel on; the +yz positions start at or after the +z ones,
// so those two offsets share region B.  A tile that spans two z slices gets
// region B in two ranges, one per slice, since the lookups of the two parts
// land a whole slice apart.  k_mesh_tile_ranges finds the regions of every
// tile at once (one thread per tile, searches through the row directory).
// The classification stages both regions in shared memory with independent
// coalesced loads -- keys, and the status byte k_mesh_status wrote per voxel
// in place of its value -- and builds every cube from the staging: one
// search in the staged keys for a thread's first voxel in a range, a
// forward walk for its next.  A tile whose regions are longer than the
// staging holds searches per voxel (load_cube).  Results are identical.
constexpr int kClassItems = 4;
constexpr int kClassTile = kThreads * kClassItems;  // 1024 voxels
constexpr int kStageA = 2048, kStageB = 2048;        // staged keys per region
// One staging buffer: keys of region A, keys of region B (two ranges), then
// the status bytes alike.  Copies start on 16-byte boundaries, so each part
// has room for the alignment shifts and round-ups; every part starts on a
// 16-byte boundary.  Two buffers: the next tile's copies land in one while
// the current tile is classified from the other.
constexpr int kKeyA = kStageA + 8, kKeyB = kStageB + 16, kStA = kStageA + 32, kStB = kStageB + 64;
template <typename K>
__host__ __device__ constexpr size_t class_buf_bytes() {
    return (size_t)(kKeyA + kKeyB) * sizeof(K) + kStA + kStB;
}
template <typename K>
__host__ __device__ constexpr size_t class_smem() {
    return 2 * class_buf_bytes<K>();
}
static_assert(class_buf_bytes<uint32_t>() % 16 == 0 && class_buf_bytes<uint64_t>() % 16 == 0, "16-byte parts");
static_assert((kKeyA * 4) % 16 == 0 && (kKeyA * 8) % 16 == 0 && kStA % 16 == 0, "16-byte parts");

constexpr unsigned int kStageSpinLimit = 1u << 24;  // polls before a staging wait gives up

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init1(uint64_t* bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(bar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ bool mbar_try(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity) {
    for (unsigned int i = 0; i < kStageSpinLimit; ++i)
        if (mbar_try(bar, parity)) return true;
    return false;
}
// `bytes` (a multiple of 16) from global `src` to shared `dst`, both 16-byte
// aligned, completing on `bar` by transaction bytes
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(dst)),
                 "l"(src), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}

// Where a tile's staged regions sit in its buffer: per part, the element
// offset of the aligned copy's start and of the range's first element.
struct StagedTile {
    unsigned int ka0, ka;        // region A keys
    unsigned int sa0, sa;        // region A statuses
    unsigned int kb0[2], kb[2];  // region B keys, per range
    unsigned int sb0[2], sb[2];  // region B statuses, per range
};
__device__ __forceinline__ unsigned int up_to(unsigned int x, unsigned int m) { return (x + m - 1) / m * m; }
template <typename K>
__device__ __forceinline__ StagedTile staged_tile(const MeshTileRange& r, unsigned int i0) {
    constexpr unsigned int kv = 16 / sizeof(K);  // keys per 16 bytes
    StagedTile L;
    L.ka0 = 0;
    L.ka = i0 % kv;
    L.sa0 = 0;
    L.sa = i0 % 16u;
    unsigned int ko = 0, so = 0;
#pragma unroll
    for (int sg = 0; sg < 2; ++sg) {
        L.kb0[sg] = ko;
        L.kb[sg] = ko + r.b_lo[sg] % kv;
        L.sb0[sg] = so;
        L.sb[sg] = so + r.b_lo[sg] % 16u;
        if (r.b_len[sg]) {
            ko = up_to(L.kb[sg] + r.b_len[sg], kv);
            so = up_to(L.sb[sg] + r.b_len[sg], 16u);
        }
    }
    return L;
}
// thread 0: the copies of tile (r, i0) into buffer `buf`, announced on `bar`
template <typename K>
__device__ __forceinline__ void stage_tile_async(unsigned char* buf, const K* keys, const unsigned char* status,
                                                 const MeshTileRange& r, unsigned int i0, uint64_t* bar) {
    const StagedTile L = staged_tile<K>(r, i0);
    K* kA = (K*)buf;
    K* kB = kA + kKeyA;
    unsigned char* sA = (unsigned char*)(kB + kKeyB);
    unsigned char* sB = sA + kStA;
    // the buffer's earlier contents were read through the generic proxy
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    const uint32_t bka = up_to((L.ka + r.a_len) * (unsigned int)sizeof(K), 16u);
    const uint32_t bsa = up_to(L.sa + r.a_len, 16u);
    uint32_t bkb[2], bsb[2];
    uint32_t total = bka + bsa;
#pragma unroll
    for (int sg = 0; sg < 2; ++sg) {
        bkb[sg] = r.b_len[sg] ? up_to((L.kb[sg] - L.kb0[sg] + r.b_len[sg]) * (unsigned int)sizeof(K), 16u) : 0u;
        bsb[sg] = r.b_len[sg] ? up_to(L.sb[sg] - L.sb0[sg] + r.b_len[sg], 16u) : 0u;
        total += bkb[sg] + bsb[sg];
    }
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(total)
                 : "memory");
    bulk_g2s(kA + L.ka0, keys + (i0 - L.ka), bka, bar);
    bulk_g2s(sA + L.sa0, status + (i0 - L.sa), bsa, bar);
#pragma unroll
    for (int sg = 0; sg < 2; ++sg)
        if (r.b_len[sg]) {
            const unsigned int lo = r.b_lo[sg];
            bulk_g2s(kB + L.kb0[sg], keys + (lo - (L.kb[sg] - L.kb0[sg])), bkb[sg], bar);
            bulk_g2s(sB + L.sb0[sg], status + (lo - (L.sb[sg] - L.sb0[sg])), bsb[sg], bar);
        }
}
__device__ __forceinline__ bool tile_fits(const MeshTileRange& r) {
    return r.a_len <= (unsigned int)kStageA && r.b_len[0] + r.b_len[1] <= (unsigned int)kStageB;
}

typedef MeshTileRange TileRange;

// Eight lanes per tile.  The z-slice split needs no search: the first key of
// slice z0 + 1 starts row (z0 + 1) << b of the row directory.  The tile's up
// to seven neighbour searches are independent and run one per lane.
constexpr int kRangeLanes = 8;

template <typename K>
__global__ void k_mesh_tile_ranges(const K* __restrict__ keys, int kb, const unsigned int* __restrict__ rs,
                                   const unsigned int* __restrict__ n_dev, int with_yz,
                                   TileRange* __restrict__ ranges, unsigned int max_tiles) {
    const unsigned int n = *n_dev;
    const unsigned int tiles = min((n + kClassTile - 1) / kClassTile, max_tiles);
    const Codec<K> cd(kb);
    const K dy = cd.pack(0, 1, 0), dz = cd.pack(0, 0, 1), dyz = cd.pack(0, 1, 1);
    const unsigned int lane = threadIdx.x & (kRangeLanes - 1);
    const unsigned int gmask = 0xFFu << ((threadIdx.x & 31u) & ~(unsigned int)(kRangeLanes - 1));
    const unsigned int groups = gridDim.x * blockDim.x / kRangeLanes;
    for (unsigned int t = (blockIdx.x * blockDim.x + threadIdx.x) / kRangeLanes; t < tiles; t += groups) {
        const unsigned int i0 = t * kClassTile;
        const unsigned int last = min(min(i0 + (unsigned int)kClassTile, n), n - 1u);  // voxels with a cube: < last
        TileRange r;
        r.b_lo[0] = r.b_lo[1] = r.b_len[0] = r.b_len[1] = 0u;
        // region A: the tile and the one after, and every +y position plus one
        r.a_len = min(i0 + (unsigned int)kClassTile + 1u, n) - i0;
        r.split = last;
        if (last > i0) {
            const K k0 = keys[i0], kl = keys[last - 1];
            unsigned int split = last;
            const unsigned int z0 = cd.z(k0), zl = cd.z(kl);
            if (z0 != zl) {  // a range per z slice when the tile spans exactly two
                const unsigned int a = rs[cd.row(cd.pack(0, 0, z0 + 1))];  // keys[i0] < keys[a] <= keys[last - 1]
                if (cd.z(keys[a]) == zl) split = a;
            }
            const bool two = split < last;
            // region B per slice: from the first +z position (clamped) to the
            // last +z or +yz position plus one
            K q = kl + dy;
            bool active = true;
            switch (lane) {
                case 1: q = k0 + dz; break;
                case 2: q = keys[split - 1] + dz; break;
                case 3: q = keys[split - 1] + dyz; active = with_yz; break;
                case 4: q = keys[split] + dz; active = two; break;
                case 5: q = kl + dz; active = two; break;
                case 6: q = kl + dyz; active = two && with_yz; break;
                case 7: active = false; break;
                default: break;
            }
            const unsigned int p = active ? upper_bound_row<K>(keys, rs, q, n, cd, 0u) - 1u : 0u;
            unsigned int w[7];
#pragma unroll
            for (int j = 0; j < 7; ++j) w[j] = __shfl_sync(gmask, p, j, kRangeLanes);
            r.a_len = max(r.a_len, min(w[0] + 1u, n - 1u) + 1u - i0);
            r.b_lo[0] = min(w[1], n - 2u);
            r.b_len[0] = min((with_yz ? max(w[2], w[3]) : w[2]) + 1u, n - 1u) - r.b_lo[0] + 1u;
            if (two) {
                r.b_lo[1] = min(w[4], n - 2u);
                r.b_len[1] = min((with_yz ? max(w[5], w[6]) : w[5]) + 1u, n - 1u) - r.b_lo[1] + 1u;
            }
            r.split = split;
        }
        if (lane == 0) ranges[t] = r;
    }
}

template <bool kTris, typename K>
__global__ void __launch_bounds__(kThreads, 4) k_mesh_classify_tiled(const K* __restrict__ keys, int kb,
                                                                     const float2* __restrict__ vals,
                                                                     const unsigned char* __restrict__ status,
                                                                     const unsigned int* __restrict__ rs,
                                                                     const unsigned int* __restrict__ n_dev,
                                                                     const TileRange* __restrict__ ranges,
                                                                     unsigned int max_tiles,
                                                                     unsigned int* __restrict__ flags,
                                                                     unsigned long long* __restrict__ tile_sums,
                                                                     unsigned int* __restrict__ tile_nflag,
                                                                     unsigned int* __restrict__ flagged,
                                                                     uint4* __restrict__ corners,
                                                                     unsigned long long* __restrict__ error) {
    constexpr int kD = kTris ? 3 : 2;  // offsets looked up: +y, +z (and +yz)
    extern __shared__ __align__(16) unsigned char class_mem[];
    __shared__ __align__(8) uint64_t s_bar[2];  // a staging buffer's copies have landed
    __shared__ int s_fail;
    __shared__ uint64_t s_mc[256];
    if (kTris) mc_table_to_shared(s_mc);
    const unsigned int n = *n_dev;
    const Codec<K> cd(kb);
    const K delta[3] = {cd.pack(0, 1, 0), cd.pack(0, 0, 1), cd.pack(0, 1, 1)};
    const unsigned int tiles = min((n + kClassTile - 1) / kClassTile, max_tiles);
    unsigned int issued0 = 0u, issued1 = 0u;  // thread 0: batches of copies issued per buffer
    if (threadIdx.x == 0) {
        mbar_init1(&s_bar[0]);
        mbar_init1(&s_bar[1]);
        s_fail = 0;
        // the first tile's copies
        if (blockIdx.x < tiles && tile_fits(ranges[blockIdx.x])) {
            stage_tile_async<K>(class_mem, keys, status, ranges[blockIdx.x], blockIdx.x * kClassTile, &s_bar[0]);
            ++issued0;
        }
    }
    __syncthreads();
    uint32_t phase0 = 0u, phase1 = 0u;  // per buffer: the parity of its next batch of copies
    unsigned int it = 0;
    for (unsigned int t = blockIdx.x; t < tiles; t += gridDim.x, ++it) {
        const unsigned int i0 = t * kClassTile;
        const unsigned int i1 = min(i0 + (unsigned int)kClassTile, n);
        const TileRange r = ranges[t];
        const bool fits = tile_fits(r);
        const unsigned int b = it & 1u;
        unsigned char* buf = class_mem + b * class_buf_bytes<K>();
        // the next tile's copies into the other buffer (free: every thread has
        // passed the previous tile's closing barrier)
        const unsigned int tn = t + gridDim.x;
        if (threadIdx.x == 0 && tn < tiles) {
            const TileRange rn = ranges[tn];
            if (tile_fits(rn)) {
                stage_tile_async<K>(class_mem + (b ^ 1u) * class_buf_bytes<K>(), keys, status, rn, tn * kClassTile,
                                    &s_bar[b ^ 1u]);
                if (b) ++issued0;
                else ++issued1;
            }
        }
        if (fits) {
            const bool ok = mbar_wait_bounded(&s_bar[b], b ? phase1 : phase0);
            if (!ok) s_fail = 1;
            if (b) phase1 ^= 1u;
            else phase0 ^= 1u;
        }
        if (__syncthreads_or(s_fail)) break;  // a wait gave up: leave the tile loop (reported below)
        const StagedTile L = staged_tile<K>(r, i0);
        const K* s_ka = (const K*)buf + L.ka;                                   // key i0 of region A
        const unsigned char* s_sa = buf + (kKeyA + kKeyB) * sizeof(K) + L.sa;   // its status
        const K* kbase = (const K*)buf + kKeyA;
        const unsigned char* sbase = buf + (kKeyA + kKeyB) * sizeof(K) + kStA;
        const unsigned int tb = threadIdx.x * kClassItems;  // this thread's first voxel in the tile
        unsigned int pos[kD], seg[kD];  // running count of a range's staged keys <= key + d; its range
#pragma unroll
        for (int d = 0; d < kD; ++d) {
            pos[d] = 0u;
            seg[d] = 2u;  // none yet: search
        }
        unsigned int fl[kClassItems];
        uint3 look[kClassItems];  // the +y, +z, +yz lookups, kept for emission
#pragma unroll
        for (int j = 0; j < kClassItems; ++j) {
            fl[j] = 0u;
            look[j] = make_uint3(0u, 0u, 0u);
        }
#pragma unroll
        for (int j = 0; j < kClassItems; ++j) {
            const unsigned int i = i0 + tb + j;
            if (i >= i1) break;
            unsigned int st[8], idx[8];
            bool live;
            if (!fits) {
                live = i + 1 < n && vals[i].y != 0.0f;
                if (live) {
                    Cube c;
                    load_cube<kTris, K>(keys, vals, rs, n, i, c, cd);
#pragma unroll
                    for (int q = 0; q < 8; ++q) {
                        idx[q] = c.idx[q];
                        st[q] = (kTris || q == 0 || q == 1 || q == 2 || q == 4) ? voxel_status(c.val[q]) : 0u;
                    }
                }
            } else {
                const unsigned int s0 = s_sa[tb + j];
                live = i + 1 < n && (s0 & kStE);
                if (live) {
                    const K key = s_ka[tb + j];
                    idx[0] = i;
                    st[0] = s0;
                    idx[1] = i + 1;
                    st[1] = s_ka[tb + j + 1] == key + cd.pack(1, 0, 0) ? s_sa[tb + j + 1] : 0u;
                    unsigned int w[kD];  // each lookup's position within its staged range
                    // region B's range of this voxel (+z, +yz): its keys and statuses
                    const unsigned int sgb = i >= r.split ? 1u : 0u;
                    const K* s_kbr = kbase + (sgb ? L.kb[1] : L.kb[0]);
                    const unsigned char* s_sbr = sbase + (sgb ? L.sb[1] : L.sb[0]);
#pragma unroll
                    for (int d = 0; d < kD; ++d) {
                        // region A for +y (one range, from i0); region B for +z, +yz
                        const unsigned int sg = d == 0 ? 0u : sgb;
                        const unsigned int Ln = d == 0 ? r.a_len : (sg ? r.b_len[1] : r.b_len[0]);
                        const unsigned int lod = d == 0 ? i0 : (sg ? r.b_lo[1] : r.b_lo[0]);
                        const K* sk = d == 0 ? s_ka : s_kbr;
                        const K tk = key + delta[d];
                        unsigned int p = pos[d];
                        if (seg[d] != sg) {  // the thread's first live voxel in this range: search
                            unsigned int a = 0, e = Ln;
                            while (a < e) {
                                const unsigned int mid = (a + e) >> 1;
                                if (sk[mid] <= tk) a = mid + 1;
                                else e = mid;
                            }
                            p = a;
                            seg[d] = sg;
                        } else {  // later voxels: the positions only move forward
                            while (p < Ln && sk[p] <= tk) ++p;
                        }
                        pos[d] = p;
                        // walk_ptr = min(n - 2, upper_bound - 1), upper_bound = lo + p
                        const unsigned int gp = min(lod + p - 1u, n - 2u);
                        idx[d == 0 ? 2 : (d == 1 ? 4 : 6)] = gp;
                        w[d] = gp - lod;
                    }
                    // corners: +y, +z (+yz) at the lookups, +xy, +xz (+xyz) one past
                    st[2] = s_ka[w[0]] == key + delta[0] ? s_sa[w[0]] : 0u;
                    st[4] = s_kbr[w[1]] == key + delta[1] ? s_sbr[w[1]] : 0u;
                    idx[3] = idx[2] + 1;
                    idx[5] = idx[4] + 1;
                    if (kTris) {
                        st[6] = s_kbr[w[2]] == key + delta[2] ? s_sbr[w[2]] : 0u;
                        idx[7] = idx[6] + 1;
                        st[3] = s_ka[w[0] + 1] == key + cd.pack(1, 1, 0) ? s_sa[w[0] + 1] : 0u;
                        st[5] = s_kbr[w[1] + 1] == key + cd.pack(1, 0, 1) ? s_sbr[w[1] + 1] : 0u;
                        st[7] = s_kbr[w[2] + 1] == key + cd.pack(1, 1, 1) ? s_sbr[w[2] + 1] : 0u;
                    } else {
                        idx[6] = idx[7] = 0u;
                        st[3] = st[5] = st[6] = st[7] = 0u;
                    }
                }
            }
            if (live) {
                fl[j] = classify_status<kTris>(st, idx, vals, s_mc);
                look[j] = make_uint3(idx[2], idx[4], kTris ? idx[6] : 0u);
            }
        }
        // in-tile offsets of the vertices (into the flags), of the indices
        // (beside the lookups) and of the voxels with output (their list),
        // one CTA scan of (output voxels << 48 | indices << 24 | vertices)
        unsigned int nv = 0, ni = 0, nf = 0;
#pragma unroll
        for (int j = 0; j < kClassItems; ++j) {
            nv += __popc(f_axes(fl[j]));
            ni += 3u * f_tris(fl[j]);
            nf += fl[j] ? 1u : 0u;
        }
        unsigned long long total;
        // (no trailing barrier: the next tile's first barrier orders the reuse)
        const unsigned long long ex = block_exclusive_scan<kThreads, false>(
            (unsigned long long)nf << 48 | (unsigned long long)ni << 24 | nv, &total);
        unsigned int vo = (unsigned int)(ex & 0xffffffu), io = (unsigned int)((ex >> 24) & 0xffffffu);
        unsigned int fo = (unsigned int)(ex >> 48);
#pragma unroll
        for (int j = 0; j < kClassItems; ++j) {
            const unsigned int i = i0 + tb + j;
            if (i < i1) {
                flags[i] = fl[j] | vo << 14;
                if (fl[j]) {
                    // emission reuses the lookups instead of searching again
                    corners[i] = make_uint4(look[j].x, look[j].y, look[j].z, io);
                    flagged[i0 + fo] = i;
                    ++fo;
                }
            }
            vo += __popc(f_axes(fl[j]));
            io += 3u * f_tris(fl[j]);
        }
        if (threadIdx.x == 0) {
            tile_sums[t] = (total >> 24 & 0xffffffull) << 32 | (total & 0xffffffull);
            tile_nflag[t] = (unsigned int)(total >> 48);
        }
    }
    if (s_fail && threadIdx.x == 0) {
        // a staging wait gave up: report it (the mesh is not emitted) and wait,
        // bounded, for the copies still in flight before the CTA exits
        atomicExch(error, 1ull);
        if (issued0) mbar_wait_bounded(&s_bar[0], (issued0 - 1u) & 1u);
        if (issued1) mbar_wait_bounded(&s_bar[1], (issued1 - 1u) & 1u);
    }
}

// The corners of a flagged voxel from its stored lookups: +x, +xy, +xz and
// +xyz sit one index past self, +y, +z and +yz (load_cube's walk).  Values
// are loaded where emission reads them.
__device__ __forceinline__ void stored_cube(unsigned int i, uint4 cr, unsigned int* idx) {
    idx[0] = i;
    idx[1] = i + 1;
    idx[2] = cr.x;
    idx[3] = cr.x + 1;
    idx[4] = cr.y;
    idx[5] = cr.y + 1;
    idx[6] = cr.z;
    idx[7] = cr.z + 1;
}

// edge e of the cube -> (corner, axis), from localToGlobal (Mesher.cpp:206-218):
// corners {4, 0, 0, 1, 6, 2, 2, 3, 5, 4, 0, 1} (4 bits each) and axes
// {0, 2, 0, 2, 0, 2, 0, 2, 1, 1, 1, 1} (2 bits each), decoded in registers
constexpr unsigned long long kEdgeCorners = 0x104532261004ull;
constexpr unsigned int kEdgeAxes = 0x558888u;
__device__ __forceinline__ int edge_corner(int e) { return (int)((kEdgeCorners >> (4 * e)) & 15u); }
__device__ __forceinline__ int edge_axis(int e) { return (int)((kEdgeAxes >> (2 * e)) & 3u); }

// Emission over the voxels with output in ascending order (the tiles'
// lists end to end), 32 per warp step.  A voxel's first vertex is its
// tile's vertex offset plus the in-tile offset in its flags, its first index
// slot its tile's index offset plus the in-tile offset kept beside its
// lookups.
template <bool kTris, typename K>
__global__ void __launch_bounds__(kThreads) k_mesh_emit(const K* __restrict__ keys, int kb,
                                                        const float2* __restrict__ vals,
                                                        const unsigned int* __restrict__ n_dev, Geom g,
                                                        const unsigned int* __restrict__ flags,
                                                        const uint4* __restrict__ corners,
                                                        const unsigned long long* __restrict__ tile_ofs,
                                                        const unsigned int* __restrict__ tile_nflag,
                                                        const unsigned int* __restrict__ flagged,
                                                        MeshCounts* __restrict__ mc,
                                                        unsigned long long vert_cap,
                                                        unsigned long long idx_cap,
                                                        unsigned long long missing_bound,
                                                        const unsigned long long* __restrict__ missing_bound_dev,
                                                        float* __restrict__ verts,
                                                        uint32_t* __restrict__ idx,
                                                        unsigned long long* __restrict__ missing_min) {
    __shared__ uint64_t s_mc[256];
    if (kTris) {
        mc_table_to_shared(s_mc);
        __syncthreads();
    }
    const unsigned int n = *n_dev;
    const Codec<K> cd(kb);
    // the counts of the counting passes; outputs that do not fit are not written
    // (every CTA sees the same counts and returns alike; the host grows and re-emits)
    const unsigned long long n_verts = mc->n_verts, n_idx = mc->n_idx;
    if (mc->error) return;  // the classification gave up: nothing to emit (the host reports it)
    const bool overflow = n_verts > vert_cap || (kTris && n_idx > idx_cap);
    // the flag describes this emission (an earlier one into smaller buffers may have set it)
    if (blockIdx.x == 0 && threadIdx.x == 0) mc->overflow = overflow ? 1ull : 0ull;
    if (overflow) return;
    // a re-run for the index mapping's stop rule takes its bound from the first run, and only
    // when that run found a missing vertex
    if (missing_bound_dev) {
        missing_bound = *missing_bound_dev;
        if (missing_bound == ~0ull) return;
    }
    // Indices are emitted warp-cooperatively: the warp's 32 voxels stage their
    // case word, corner indices and first output slot in shared memory, and
    // all lanes walk the warp's indices together (a lane finds its voxel by a
    // search over the prefix of the voxels' index counts), so a warp does
    // not wait on its lane with the most triangles.
    constexpr int kWarps = kThreads / 32;
    __shared__ unsigned int s_cidx[kWarps][8][32];  // corner voxel
    __shared__ unsigned int s_cvb[kWarps][8][32];   // corner voxel's first vertex
    __shared__ unsigned char s_cax[kWarps][8][32];  // corner voxel's vertex axes
    __shared__ uint64_t s_mcw[kWarps][32];
    __shared__ unsigned int s_first[kWarps][32];
    __shared__ unsigned int s_excl[kWarps][33];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const unsigned int warps = gridDim.x * kWarps;
    const unsigned int tiles = (n + kClassTile - 1) / kClassTile;
    // The voxels with output, counted across tiles (tile_nflag holds each tile's
    // first position), are cut into chunks of 32; each warp takes a contiguous
    // run of chunks and finds the tile of each position by walking forward.
    const unsigned int n_out = (unsigned int)mc->n_flagged;
    const unsigned int chunks = (n_out + 31u) / 32u;
    const unsigned int wid = blockIdx.x * kWarps + warp;
    const unsigned int cbeg = (unsigned int)((unsigned long long)chunks * wid / warps);
    const unsigned int cend = (unsigned int)((unsigned long long)chunks * (wid + 1) / warps);
    unsigned int tile = 0;
    if (cbeg < cend) {  // the warp's first tile: the last with a first position <= 32 cbeg
        unsigned int a = 0, b = tiles;
        while (a + 1 < b) {
            const unsigned int mid = (a + b) >> 1;
            if (tile_nflag[mid] <= 32u * cbeg) a = mid;
            else b = mid;
        }
        tile = a;
    }
    for (unsigned int ch = cbeg; ch < cend; ++ch) {
        const unsigned int gpos = 32u * ch + lane;
        const bool valid = gpos < n_out;
        unsigned int tl = tile;
        if (valid)
            while (tile_nflag[tl + 1] <= gpos) ++tl;  // tile_nflag[tiles] = n_out > gpos
        tile = __shfl_sync(0xffffffffu, tl, 31);      // positions only move forward
        const unsigned int i = valid ? flagged[tl * kClassTile + (gpos - tile_nflag[tl])] : 0u;
        const unsigned int f = valid ? flags[i] : 0u;
        const unsigned long long tofs = valid ? tile_ofs[tl] : 0ull;
        unsigned int cidx[8];
        uint4 cr = make_uint4(0u, 0u, 0u, 0u);
        if (f) {
            cr = corners[i];
            stored_cube(i, cr, cidx);
        }
        const unsigned int axes = f_axes(f);
        // vertices (Mesher.cpp:134-168): at most three per voxel, by the voxel's lane
        if (axes) {
            const K key = keys[i];
            const unsigned int vbase = (unsigned int)(tofs & 0xffffffffu) + f_vofs(f);
            const unsigned int nv = __popc(axes);
            const unsigned long long first =
                kTris ? vbase : n_verts - vbase - nv;  // ascending ids / generation order
            const float cx = fadd(fmul((float)(int)cd.x(key), g.vlen), g.center_off);
            const float cy = fadd(fmul((float)(int)cd.y(key), g.vlen), g.center_off);
            const float cz = fadd(fmul((float)(int)cd.z(key), g.vlen), g.center_off);
            const float dself = vdist(vals[i]);
            const int nb[3] = {1, 2, 4};
            unsigned int r = 0;
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                if (!(axes >> a & 1u)) continue;
                const float dn = vdist(vals[cidx[nb[a]]]);  // a flagged axis: the neighbour exists
                const float t = fmul(fdiv(fabsf(dself), fadd(fabsf(dself), fabsf(dn))), g.vlen);
                float p[3] = {cx, cy, cz};
                p[a] = fadd(p[a], t);
                float* o = verts + 3 * (first + r);
                o[0] = p[0];
                o[1] = p[1];
                o[2] = p[2];
                ++r;
            }
        }
        if constexpr (kTris) {
            const unsigned int ni = 3u * f_tris(f);
            unsigned int inc = ni;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const unsigned int y = __shfl_up_sync(0xffffffffu, inc, o);
                if (lane >= o) inc += y;
            }
            const unsigned int total = __shfl_sync(0xffffffffu, inc, 31);
            if (total == 0u) continue;  // warp-uniform
            __syncwarp();  // the previous round's readers are done with the staging
            s_excl[warp][lane] = inc - ni;
            if (lane == 31) s_excl[warp][32] = inc;
            if (ni) {
                s_mcw[warp][lane] = s_mc[f_case(f)];  // the case's triangle edges
                // generation order: voxels descending
                s_first[warp][lane] = (unsigned int)(n_idx - ((tofs >> 32) + cr.w) - ni);
                // each corner voxel's vertex axes and first vertex: independent loads
                unsigned int cf[8];
                unsigned long long co[8];
#pragma unroll
                for (int k = 0; k < 8; ++k) {
                    cf[k] = flags[cidx[k]];
                    co[k] = tile_ofs[cidx[k] / kClassTile];
                }
#pragma unroll
                for (int k = 0; k < 8; ++k) {
                    s_cidx[warp][k][lane] = cidx[k];
                    s_cax[warp][k][lane] = (unsigned char)f_axes(cf[k]);
                    s_cvb[warp][k][lane] = (unsigned int)(co[k] & 0xffffffffu) + f_vofs(cf[k]);
                }
            }
            __syncwarp();
            unsigned long long local_min = ~0ull;
            for (unsigned int j = lane; j < total; j += 32u) {
                // v = the last voxel whose exclusive prefix is <= j (it has ni > 0)
                int v = 0;
#pragma unroll
                for (int step = 16; step > 0; step >>= 1)
                    if (s_excl[warp][v + step] <= j) v += step;
                const unsigned int t = j - s_excl[warp][v];
                const int e = mc_tri_edge_of(s_mcw[warp][v], (int)t);
                const int corner = edge_corner(e), axis = edge_axis(e);
                const unsigned int cax = s_cax[warp][corner][v];
                const bool has = (cax >> axis & 1u) != 0u;
                // the edge id 3 * key + axis, needed for a missing vertex and on the
                // stop rule's re-run: 32 bits wide for 30-bit keys (as in the reference);
                // for 64-bit keys the stop rule compares full ids and an id written in
                // place of a missing vertex keeps its low 32 bits
                const bool need_id = !has || missing_bound != ~0ull;
                const unsigned long long id =
                    need_id ? 3ull * (unsigned long long)keys[s_cidx[warp][corner][v]] + (unsigned long long)axis
                            : 0ull;
                uint32_t outv;
                if (has) {
                    outv = s_cvb[warp][corner][v] + __popc(cax & ((1u << axis) - 1u));
                } else {
                    outv = (uint32_t)id;
                    local_min = min(local_min, id);
                }
                if (need_id && id >= missing_bound) outv = (uint32_t)id;
                idx[(unsigned long long)s_first[warp][v] + t] = outv;
            }
            if (local_min != ~0ull && missing_min) atomicMin(missing_min, local_min);
        }
    }
}

// single CTA: exclusive scans (in place) of the classification tiles' packed
// (index count << 32 | vertex count) and of their counts of voxels with
// output (the total after the last), the totals to *counts; the packed
// halves stay below 2^32 for volumes under 2^28 voxels
constexpr int kSumThreads = 1024, kSumItems = 8, kSumRound = kSumThreads * kSumItems;
// dynamic shared memory of k_scan_tile_sums: one round of both arrays
constexpr size_t kSumSmem = (size_t)kSumRound * (sizeof(unsigned long long) + sizeof(unsigned int));
__global__ void __launch_bounds__(kSumThreads) k_scan_tile_sums(unsigned long long* __restrict__ sums,
                                                                unsigned int* __restrict__ nflag,
                                                                const unsigned int* __restrict__ n_dev,
                                                                MeshCounts* __restrict__ counts) {
    extern __shared__ __align__(16) unsigned char sum_mem[];
    unsigned long long* s_v = (unsigned long long*)sum_mem;  // [kSumRound]
    unsigned int* s_f = (unsigned int*)(s_v + kSumRound);    // [kSumRound]
    const unsigned int n_tiles = (*n_dev + kClassTile - 1) / kClassTile;
    unsigned long long carry = 0, fcarry = 0;
    for (unsigned int b = 0; b < n_tiles; b += kSumRound) {
        // coalesced loads of the round into shared memory, then each thread
        // takes kSumItems consecutive entries from there
        for (unsigned int j = threadIdx.x; j < (unsigned int)kSumRound; j += kSumThreads) {
            const bool in = b + j < n_tiles;
            s_v[j] = in ? sums[b + j] : 0ull;
            s_f[j] = in ? nflag[b + j] : 0u;
        }
        __syncthreads();
        const unsigned int l0 = threadIdx.x * kSumItems;
        unsigned long long v[kSumItems], s = 0, fs = 0;
        unsigned int fv[kSumItems];
#pragma unroll
        for (int q = 0; q < kSumItems; ++q) {
            v[q] = s_v[l0 + q];
            fv[q] = s_f[l0 + q];
            s += v[q];
            fs += fv[q];
        }
        unsigned long long total, ftotal;
        unsigned long long run = carry + block_exclusive_scan<kSumThreads>(s, &total);
        unsigned long long frun = fcarry + block_exclusive_scan<kSumThreads>(fs, &ftotal);
#pragma unroll
        for (int q = 0; q < kSumItems; ++q) {
            s_v[l0 + q] = run;
            s_f[l0 + q] = (unsigned int)frun;
            run += v[q];
            frun += fv[q];
        }
        __syncthreads();
        for (unsigned int j = threadIdx.x; j < (unsigned int)kSumRound; j += kSumThreads)
            if (b + j < n_tiles) {
                sums[b + j] = s_v[j];
                nflag[b + j] = s_f[j];
            }
        carry += total;
        fcarry += ftotal;
        __syncthreads();  // the staging is reused by the next round
    }
    if (threadIdx.x == 0) {
        nflag[n_tiles] = (unsigned int)fcarry;
        counts->n_verts = carry & 0xffffffffull;
        counts->n_idx = carry >> 32;
        counts->missing_min = ~0ull;
        counts->overflow = 0ull;
        counts->n_flagged = fcarry;
    }
}

}  // namespace

cudaError_t mesh_scratch_reserve(MeshScratch* m, size_t n, int kb) {
    const size_t rows = ((size_t)1 << (2 * kb)) + 1;
    if (m->cap >= n && m->vflags && m->rows_cap >= rows) return cudaSuccess;
    if (n < m->cap) n = m->cap;
    mesh_scratch_free(m);
    size_t cap = n < 1024 ? 1024 : n;
    const size_t tiles = (cap + kClassTile - 1) / kClassTile + 1;
    cudaError_t e;
    if ((e = cudaMalloc(&m->vflags, cap * sizeof(unsigned int)))) return e;
    if ((e = cudaMalloc(&m->vstatus, (cap + 4) / 4 * 4 + 32))) return e;  // 16-byte copies read past the end
    if ((e = cudaMalloc(&m->corners, cap * sizeof(uint4)))) return e;
    if ((e = cudaMalloc(&m->tile_sums, tiles * sizeof(unsigned long long)))) return e;
    if ((e = cudaMalloc(&m->tile_nflag, tiles * sizeof(unsigned int)))) return e;
    if ((e = cudaMalloc(&m->flagged, tiles * kClassTile * sizeof(unsigned int)))) return e;
    if ((e = cudaMalloc(&m->rows, rows * sizeof(unsigned int)))) return e;
    if ((e = cudaMalloc(&m->tile_ranges, tiles * sizeof(MeshTileRange)))) return e;
    m->rows_cap = rows;
    if ((e = cudaMalloc(&m->counts, sizeof(MeshCounts)))) return e;
    if ((e = cudaMalloc(&m->n_dev, sizeof(unsigned int)))) return e;
    m->cap = cap;
    return cudaSuccess;
}

void mesh_scratch_free(MeshScratch* m) {
    cudaFree(m->vflags);
    cudaFree(m->vstatus);
    cudaFree(m->corners);
    cudaFree(m->tile_sums);
    cudaFree(m->tile_nflag);
    cudaFree(m->flagged);
    cudaFree(m->rows);
    cudaFree(m->tile_ranges);
    cudaFree(m->counts);
    cudaFree(m->n_dev);
    *m = MeshScratch{};
}

static int grid_for(size_t n, int sms) {
    size_t b = (n + kThreads - 1) / kThreads;
    size_t cap = (size_t)sms * 8;
    return (int)(b < 1 ? 1 : (b > cap ? cap : b));
}

// The voxel count is read on the device from ms.n_dev (<= n_cap, which sizes
// the grids), so the passes can be enqueued before the count is known.
template <typename K>
static void mesh_count_t(const K* keys, const float2* vals, size_t n_cap, int kb, int with_indices, MeshScratch& ms,
                         int sms, cudaStream_t st, cudaEvent_t* stage_events) {
    cudaMemsetAsync(&ms.counts->error, 0, sizeof(unsigned long long), st);  // set by a staging wait that gives up
    k_row_directory<K><<<grid_for(((size_t)1 << (2 * kb)) + 1, sms), kThreads, 0, st>>>(keys, ms.n_dev, kb, ms.rows);
    if (stage_events) cudaEventRecord(stage_events[0], st);
    // tile ranges, then the classification (its grid: up to 8 CTAs per SM, each walking tiles)
    const unsigned int max_tiles = (unsigned int)((n_cap + kClassTile - 1) / kClassTile);
    k_mesh_tile_ranges<K><<<grid_for((size_t)max_tiles * kRangeLanes, sms), kThreads, 0, st>>>(
        keys, kb, ms.rows, ms.n_dev, with_indices, ms.tile_ranges, max_tiles);
    const int class_grid = (int)(max_tiles < (unsigned int)(sms * 8) ? (max_tiles ? max_tiles : 1) : sms * 8);
    k_mesh_status<<<grid_for((n_cap + 3) / 4, sms), kThreads, 0, st>>>(vals, ms.n_dev, (unsigned int*)ms.vstatus);
    if (with_indices) {
        const size_t smem = class_smem<K>();
        cudaFuncSetAttribute(k_mesh_classify_tiled<true, K>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k_mesh_classify_tiled<true, K><<<class_grid, kThreads, smem, st>>>(keys, kb, vals, ms.vstatus, ms.rows, ms.n_dev,
                                                                          ms.tile_ranges, max_tiles, ms.vflags,
                                                                          ms.tile_sums, ms.tile_nflag, ms.flagged,
                                                                          ms.corners, &ms.counts->error);
    } else {
        const size_t smem = class_smem<K>();
        cudaFuncSetAttribute(k_mesh_classify_tiled<false, K>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k_mesh_classify_tiled<false, K><<<class_grid, kThreads, smem, st>>>(keys, kb, vals, ms.vstatus, ms.rows, ms.n_dev,
                                                                           ms.tile_ranges, max_tiles, ms.vflags,
                                                                           ms.tile_sums, ms.tile_nflag, ms.flagged,
                                                                           ms.corners, &ms.counts->error);
    }
    if (stage_events) cudaEventRecord(stage_events[1], st);
    cudaFuncSetAttribute(k_scan_tile_sums, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSumSmem);
    k_scan_tile_sums<<<1, kSumThreads, kSumSmem, st>>>(ms.tile_sums, ms.tile_nflag, ms.n_dev, ms.counts);
}

cudaError_t mesh_count_enqueue(const void* keys, int key_bytes, const float2* vals, size_t n_cap, int kb,
                               int with_indices, MeshScratch& ms, int sms, cudaStream_t st, cudaEvent_t* stage_events) {
    if (key_bytes == 8)
        mesh_count_t<uint64_t>((const uint64_t*)keys, vals, n_cap, kb, with_indices, ms, sms, st, stage_events);
    else mesh_count_t<uint32_t>((const uint32_t*)keys, vals, n_cap, 10, with_indices, ms, sms, st, stage_events);
    return cudaGetLastError();
}

// Both emit passes: the first records the smallest edge id without a vertex
// in ms.counts->missing_min; the second (the index mapping's stop rule)
// re-emits with that bound and does nothing when the first found none.
template <typename K>
static void mesh_emit_t(const Geom& g, const K* keys, const float2* vals, size_t n_cap, int with_indices,
                        MeshScratch& ms, size_t vert_cap, size_t idx_cap, float* verts_dev, uint32_t* idx_dev,
                        int sms, cudaStream_t st) {
    unsigned long long* mm = &ms.counts->missing_min;
    const int kb = sizeof(K) == 4 ? 10 : g.kb;
    const int grid = grid_for(n_cap, sms);
    if (with_indices) {
        k_mesh_emit<true, K><<<grid, kThreads, 0, st>>>(keys, kb, vals, ms.n_dev, g, ms.vflags, ms.corners,
                                                          ms.tile_sums, ms.tile_nflag, ms.flagged, ms.counts, vert_cap, idx_cap, ~0ull, nullptr,
                                                          verts_dev, idx_dev, mm);
        k_mesh_emit<true, K><<<grid, kThreads, 0, st>>>(keys, kb, vals, ms.n_dev, g, ms.vflags, ms.corners,
                                                          ms.tile_sums, ms.tile_nflag, ms.flagged, ms.counts, vert_cap, idx_cap, 0ull, mm,
                                                          verts_dev, idx_dev, nullptr);
    } else {
        k_mesh_emit<false, K><<<grid, kThreads, 0, st>>>(keys, kb, vals, ms.n_dev, g, ms.vflags, ms.corners,
                                                           ms.tile_sums, ms.tile_nflag, ms.flagged, ms.counts, vert_cap, idx_cap, ~0ull, nullptr,
                                                           verts_dev, idx_dev, mm);
    }
}

cudaError_t mesh_emit_enqueue(const Geom& g, const void* keys, int key_bytes, const float2* vals, size_t n_cap,
                              int with_indices, MeshScratch& ms, size_t vert_cap, size_t idx_cap,
                              float* verts_dev, uint32_t* idx_dev, int sms, cudaStream_t st) {
    if (key_bytes == 8)
        mesh_emit_t<uint64_t>(g, (const uint64_t*)keys, vals, n_cap, with_indices, ms, vert_cap, idx_cap, verts_dev,
                              idx_dev, sms, st);
    else
        mesh_emit_t<uint32_t>(g, (const uint32_t*)keys, vals, n_cap, with_indices, ms, vert_cap, idx_cap, verts_dev,
                              idx_dev, sms, st);
    return cudaGetLastError();
}

// Copy of the resident voxels (buffer ctl->cur, ctl->n[cur] of them) for a
// mesh that runs while fusion goes on; the count goes to *n_dev.  16-byte
// loads (four 32-bit or two 64-bit keys, two voxels), four in flight per
// thread, streaming past L1; the buffers are cudaMalloc'd (256-byte aligned).
template <typename K>
__global__ void __launch_bounds__(256) k_mesh_snapshot(const DeviceCtl* __restrict__ ctl, VolumeBuffers vb,
                                                       K* __restrict__ keys, float2* __restrict__ vals,
                                                       unsigned long long cap, unsigned int* __restrict__ n_dev) {
    constexpr unsigned int kPerVec = 16 / sizeof(K);  // keys per 16 bytes
    const unsigned int cur = ctl->cur;
    unsigned long long n = ctl->n[cur];
    if (n > cap) n = cap;
    const K* sk = (const K*)(cur ? vb.keys[1] : vb.keys[0]);
    const float2* sv = cur ? vb.vals[1] : vb.vals[0];
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    const unsigned long long t0 = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
    // keys: n / kPerVec vectors, then the tail
    const unsigned long long nk = n / kPerVec;
    const uint4* ks = reinterpret_cast<const uint4*>(sk);
    uint4* kd = reinterpret_cast<uint4*>(keys);
    for (unsigned long long i = t0; i < nk; i += 4 * stride) {
        uint4 v[4];
#pragma unroll
        for (int u = 0; u < 4; ++u)
            if (i + u * stride < nk) v[u] = __ldcs(ks + i + u * stride);
#pragma unroll
        for (int u = 0; u < 4; ++u)
            if (i + u * stride < nk) kd[i + u * stride] = v[u];
    }
    for (unsigned long long i = nk * kPerVec + t0; i < n; i += stride) keys[i] = __ldcs(sk + i);
    // voxels: two per vector
    const unsigned long long nv = n / 2;
    const float4* vs = reinterpret_cast<const float4*>(sv);
    float4* vd = reinterpret_cast<float4*>(vals);
    for (unsigned long long i = t0; i < nv; i += 4 * stride) {
        float4 v[4];
#pragma unroll
        for (int u = 0; u < 4; ++u)
            if (i + u * stride < nv) v[u] = __ldcs(vs + i + u * stride);
#pragma unroll
        for (int u = 0; u < 4; ++u)
            if (i + u * stride < nv) vd[i + u * stride] = v[u];
    }
    if ((n & 1) && t0 == 0) vals[n - 1] = __ldcs(sv + n - 1);
    if (blockIdx.x == 0 && threadIdx.x == 0) *n_dev = (unsigned int)n;
}

cudaError_t mesh_snapshot_enqueue(const DeviceCtl* ctl, const VolumeBuffers& vb, void* keys, float2* vals,
                                  size_t cap, unsigned int* n_dev, int sms, cudaStream_t st) {
    if (vb.key_bytes == 8)
        k_mesh_snapshot<uint64_t><<<sms * 4, 256, 0, st>>>(ctl, vb, (uint64_t*)keys, vals, cap, n_dev);
    else
        k_mesh_snapshot<uint32_t><<<sms * 4, 256, 0, st>>>(ctl, vb, (uint32_t*)keys, vals, cap, n_dev);
    return cudaGetLastError();
}

}  // namespace kifi
