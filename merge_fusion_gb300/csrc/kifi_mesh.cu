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
//  k_mesh_tile_ranges  per tile of 512 voxels and neighbour offset, the
//                   range of positions its voxels' lookups fall in.
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
// classification tile (at most 3 x 512 = 1536).
__device__ __forceinline__ unsigned int f_axes(unsigned int f) { return f & 7u; }
__device__ __forceinline__ unsigned int f_tris(unsigned int f) { return (f >> 3) & 7u; }
__device__ __forceinline__ unsigned int f_case(unsigned int f) { return (f >> 6) & 0xffu; }
__device__ __forceinline__ unsigned int f_vofs(unsigned int f) { return f >> 14; }

// exclusive scan of one 64-bit value per thread over a CTA of kT threads;
// the CTA's total to *total
template <int kT>
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
    __syncthreads();
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
__device__ __forceinline__ unsigned int vertex_axes(const Cube& c) {
    const float2 sv = c.val[0];
    const bool s_ok = in_sign_range(sv);
    const bool s_neg = (sv.x < 0.0f) != (sv.y < 0.0f);
    unsigned int axes = 0;
    const int nb[3] = {1, 2, 4};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const float2 o = c.val[nb[a]];
        if (!(o.y > 0.0f)) continue;
        bool crosses;
        if (s_ok && in_sign_range(o)) crosses = s_neg != ((o.x < 0.0f) != (o.y < 0.0f));
        else crosses = fmul(vdist(sv), vdist(o)) <= 0.0f;
        if (crosses) axes |= 1u << a;
    }
    return axes;
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

// marching-cubes case with the reference's corner bit order (Mesher.cpp:191-199)
__device__ __forceinline__ int cube_case(const Cube& c) {
    return dist_negative(c.val[0]) << 2 | dist_negative(c.val[1]) << 3 |
           dist_negative(c.val[2]) << 6 | dist_negative(c.val[3]) << 7 |
           dist_negative(c.val[4]) << 1 | dist_negative(c.val[5]) << 0 |
           dist_negative(c.val[6]) << 5 | dist_negative(c.val[7]) << 4;
}

// One voxel's classification from its cube (live: the voxel is in [0, n-2]
// with a non-zero weight, and c holds its corners): its flags without the
// tile offset -- vertex axes, triangle count, case.
template <bool kTris>
__device__ __forceinline__ unsigned int classify_voxel(const Cube& c, bool live, const uint64_t* s_mc) {
    unsigned int f = 0;
    if (live) {
        f = vertex_axes(c);
        if (kTris) {
            bool skip = false;
#pragma unroll
            for (int q = 1; q < 8; ++q) skip |= (0.0f == c.val[q].y);
            if (!skip) {
                const int lut = cube_case(c);
                const unsigned int tris = mc_tri_count_of(s_mc[lut]);
                if (tris) f |= tris << 3 | (unsigned int)lut << 6;
            }
        }
    }
    return f;
}

// Classification by tiles of kClassTile consecutive voxels.  For a
// neighbour offset d (+y, +z, +yz) the lookup positions walk_ptr(key_i + d)
// are non-decreasing in i, so the tile's positions all lie between those of
// its first and last voxel.  k_mesh_tile_ranges finds those bounds for every
// tile at once (six row-directory searches per tile, one thread each); the
// classification then stages the tile's keys and voxels and each offset's
// range in shared memory with independent coalesced loads and builds every
// cube from the staging: one search in the staged keys for a thread's first
// voxel, a forward walk for its next.  A tile whose ranges are longer than
// the staging holds searches per voxel (load_cube).  Results are identical.
constexpr int kClassItems = 2;
constexpr int kClassTile = kThreads * kClassItems;  // 512 voxels
constexpr int kClassStage = 1024;                    // staged keys per offset
// dynamic shared memory of k_mesh_classify_tiled: per offset a staged range
// of keys and voxels, the tile's own keys and voxels (plus the one after)
template <typename K>
__host__ __device__ constexpr size_t class_smem(int n_offsets) {
    return ((size_t)n_offsets * kClassStage + kClassTile + 1) * (sizeof(K) + sizeof(float2));
}

// per tile and offset d: the first staged position and the range length
// (length 0: nothing to stage; longer than kClassStage: search per voxel)
template <typename K>
__global__ void k_mesh_tile_ranges(const K* __restrict__ keys, int kb, const unsigned int* __restrict__ rs,
                                   const unsigned int* __restrict__ n_dev, int n_offsets,
                                   uint2* __restrict__ ranges, unsigned int max_tiles) {
    const unsigned int n = *n_dev;
    const unsigned int tiles = min((n + kClassTile - 1) / kClassTile, max_tiles);
    const Codec<K> cd(kb);
    const K delta[3] = {cd.pack(0, 1, 0), cd.pack(0, 0, 1), cd.pack(0, 1, 1)};
    for (unsigned int q = blockIdx.x * blockDim.x + threadIdx.x; q < tiles * n_offsets;
         q += gridDim.x * blockDim.x) {
        const unsigned int t = q / n_offsets;
        const int d = (int)(q - t * n_offsets);
        const unsigned int i0 = t * kClassTile;
        const unsigned int last = min(min(i0 + (unsigned int)kClassTile, n), n - 1u);  // voxels with a cube: < last
        uint2 r = make_uint2(0u, 0u);
        if (last > i0) {
            // walk positions (unclamped) of the first and last voxel; the range
            // [min(p0, n-2), min(p1 + 1, n - 1)] holds every position and the one after
            const unsigned int p0 = upper_bound_row<K>(keys, rs, keys[i0] + delta[d], n, cd, 0u) - 1u;
            const unsigned int p1 = upper_bound_row<K>(keys, rs, keys[last - 1] + delta[d], n, cd, 0u) - 1u;
            const unsigned int lo = min(p0, n - 2u);
            r = make_uint2(lo, min(p1 + 1u, n - 1u) - lo + 1u);
        }
        ranges[(size_t)t * 3 + d] = r;
    }
}

template <bool kTris, typename K>
__global__ void __launch_bounds__(kThreads) k_mesh_classify_tiled(const K* __restrict__ keys, int kb,
                                                                  const float2* __restrict__ vals,
                                                                  const unsigned int* __restrict__ rs,
                                                                  const unsigned int* __restrict__ n_dev,
                                                                  const uint2* __restrict__ ranges,
                                                                  unsigned int max_tiles,
                                                                  unsigned int* __restrict__ flags,
                                                                  unsigned long long* __restrict__ tile_sums,
                                                                  unsigned int* __restrict__ tile_nflag,
                                                                  unsigned int* __restrict__ flagged,
                                                                  uint4* __restrict__ corners) {
    constexpr int kD = kTris ? 3 : 2;  // offsets looked up: +y, +z (and +yz)
    constexpr int kStage = kClassStage;
    extern __shared__ __align__(16) unsigned char class_mem[];
    float2* s_val = (float2*)class_mem;                           // [kD][kStage]
    float2* s_tval = s_val + kD * kStage;                          // [kClassTile + 1]
    K* s_key = (K*)(s_tval + kClassTile + 1);                     // [kD][kStage]
    K* s_tkey = s_key + kD * kStage;                              // [kClassTile + 1]
    __shared__ uint64_t s_mc[256];
    if (kTris) mc_table_to_shared(s_mc);
    const unsigned int n = *n_dev;
    const Codec<K> cd(kb);
    const K delta[3] = {cd.pack(0, 1, 0), cd.pack(0, 0, 1), cd.pack(0, 1, 1)};
    const float2 zero = make_float2(0.0f, 0.0f);
    const unsigned int tiles = min((n + kClassTile - 1) / kClassTile, max_tiles);
    for (unsigned int t = blockIdx.x; t < tiles; t += gridDim.x) {
        const unsigned int i0 = t * kClassTile;
        const unsigned int i1 = min(i0 + (unsigned int)kClassTile, n);
        unsigned int lo[kD], len[kD];
        bool fits = true;
#pragma unroll
        for (int d = 0; d < kD; ++d) {
            const uint2 r = ranges[(size_t)t * 3 + d];
            lo[d] = r.x;
            len[d] = r.y;
            fits &= r.y <= (unsigned int)kStage;
        }
        __syncthreads();  // the previous tile is done with the staging
        if (fits) {
            // independent loads: the tile's own keys and voxels (and the one
            // after), then each offset's range
            for (unsigned int j = threadIdx.x; j <= (unsigned int)kClassTile; j += kThreads)
                if (i0 + j < n) {
                    s_tkey[j] = keys[i0 + j];
                    s_tval[j] = vals[i0 + j];
                }
#pragma unroll
            for (int d = 0; d < kD; ++d)
                for (unsigned int j = threadIdx.x; j < len[d]; j += kThreads) {
                    s_key[d * kStage + j] = keys[lo[d] + j];
                    s_val[d * kStage + j] = vals[lo[d] + j];
                }
        }
        __syncthreads();
        const unsigned int tb = threadIdx.x * kClassItems;  // this thread's first voxel in the tile
        unsigned int pos[kD];  // running count of staged keys <= key + d
#pragma unroll
        for (int d = 0; d < kD; ++d) pos[d] = 0xffffffffu;
        unsigned int fl[kClassItems];
        uint3 look[kClassItems];  // the +y, +z, +yz lookups, kept for emission
#pragma unroll
        for (int j = 0; j < kClassItems; ++j) fl[j] = 0u;
#pragma unroll
        for (int j = 0; j < kClassItems; ++j) {
            const unsigned int i = i0 + tb + j;
            if (i >= i1) break;
            Cube c;
            bool live;
            if (!fits) {
                live = i + 1 < n && vals[i].y != 0.0f;
                if (live) load_cube<kTris, K>(keys, vals, rs, n, i, c, cd);
            } else {
                const float2 v0 = s_tval[tb + j];
                live = i + 1 < n && v0.y != 0.0f;
                if (live) {
                    const K key = s_tkey[tb + j];
                    c.idx[0] = i;
                    c.val[0] = v0;
                    c.idx[1] = i + 1;
                    c.val[1] = s_tkey[tb + j + 1] == key + cd.pack(1, 0, 0) ? s_tval[tb + j + 1] : zero;
                    unsigned int w[kD];
#pragma unroll
                    for (int d = 0; d < kD; ++d) {
                        const K tk = key + delta[d];
                        const K* sk = s_key + d * kStage;
                        unsigned int p = pos[d];
                        if (p == 0xffffffffu) {  // the thread's first live voxel: search
                            unsigned int a = 0, b = len[d];
                            while (a < b) {
                                const unsigned int mid = (a + b) >> 1;
                                if (sk[mid] <= tk) a = mid + 1;
                                else b = mid;
                            }
                            p = a;
                        } else {  // later voxels: the positions only move forward
                            while (p < len[d] && sk[p] <= tk) ++p;
                        }
                        pos[d] = p;
                        // walk_ptr = min(n - 2, upper_bound - 1), upper_bound = lo + p;
                        // w[d] is the staged index of that position
                        w[d] = min(lo[d] + p - 1u, n - 2u) - lo[d];
                    }
                    // corners: self, +x, +y, +xy, +z, +xz, +yz, +xyz (Mesher.cpp:122-132, 174-181)
                    const K* ky = s_key;
                    const K* kz = s_key + kStage;
                    const float2* vy = s_val;
                    const float2* vz = s_val + kStage;
                    c.idx[2] = lo[0] + w[0];
                    c.val[2] = ky[w[0]] == key + delta[0] ? vy[w[0]] : zero;
                    c.idx[4] = lo[1] + w[1];
                    c.val[4] = kz[w[1]] == key + delta[1] ? vz[w[1]] : zero;
                    if (kTris) {
                        const K* kyz = s_key + (kD - 1) * kStage;
                        const float2* vyz = s_val + (kD - 1) * kStage;
                        const unsigned int wy = w[kD - 1];
                        c.idx[6] = lo[kD - 1] + wy;
                        c.val[6] = kyz[wy] == key + delta[2] ? vyz[wy] : zero;
                        c.idx[3] = c.idx[2] + 1;
                        c.val[3] = ky[w[0] + 1] == key + cd.pack(1, 1, 0) ? vy[w[0] + 1] : zero;
                        c.idx[5] = c.idx[4] + 1;
                        c.val[5] = kz[w[1] + 1] == key + cd.pack(1, 0, 1) ? vz[w[1] + 1] : zero;
                        c.idx[7] = c.idx[6] + 1;
                        c.val[7] = kyz[wy + 1] == key + cd.pack(1, 1, 1) ? vyz[wy + 1] : zero;
                    }
                }
            }
            fl[j] = classify_voxel<kTris>(c, live, s_mc);
            look[j] = make_uint3(c.idx[2], c.idx[4], kTris ? c.idx[6] : 0u);
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
        const unsigned long long ex = block_exclusive_scan<kThreads>(
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

// Emission: each warp takes the voxels with output of one classification
// tile (their list, ascending), 32 at a time.  A voxel's first vertex is its
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
    __shared__ unsigned int s_cidx[kWarps][8][32];
    __shared__ uint64_t s_mcw[kWarps][32];
    __shared__ unsigned int s_first[kWarps][32];
    __shared__ unsigned int s_excl[kWarps][33];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const unsigned int warps = gridDim.x * kWarps;
    const unsigned int tiles = (n + kClassTile - 1) / kClassTile;
    // each warp takes a tile's voxels with output, 32 at a time
    for (unsigned int tile = blockIdx.x * kWarps + warp; tile < tiles; tile += warps)
    for (unsigned int c0 = 0, cnt = tile_nflag[tile]; c0 < cnt; c0 += 32u) {
        const unsigned long long tofs = tile_ofs[tile];
        const unsigned int k = c0 + lane;
        const unsigned int i = k < cnt ? flagged[tile * kClassTile + k] : 0u;
        const unsigned int f = k < cnt ? flags[i] : 0u;
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
#pragma unroll
                for (int k = 0; k < 8; ++k) s_cidx[warp][k][lane] = cidx[k];
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
                const unsigned int ci = s_cidx[warp][corner][v];
                const unsigned int cf = flags[ci];
                const bool has = (cf >> axis & 1u) != 0u;
                // the edge id 3 * key + axis, needed for a missing vertex and on the
                // stop rule's re-run: 32 bits wide for 30-bit keys (as in the reference);
                // for 64-bit keys the stop rule compares full ids and an id written in
                // place of a missing vertex keeps its low 32 bits
                const bool need_id = !has || missing_bound != ~0ull;
                const unsigned long long id =
                    need_id ? 3ull * (unsigned long long)keys[ci] + (unsigned long long)axis : 0ull;
                uint32_t outv;
                if (has) {
                    outv = (unsigned int)(tile_ofs[ci / kClassTile] & 0xffffffffu) + f_vofs(cf) +
                           __popc(f_axes(cf) & ((1u << axis) - 1u));
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

// single CTA: exclusive scan (in place) of the classification tiles' packed
// (index count << 32 | vertex count), the totals to *counts; both halves stay
// below 2^32 for volumes under 2^28 voxels
constexpr int kSumThreads = 1024, kSumItems = 8;
__global__ void __launch_bounds__(kSumThreads) k_scan_tile_sums(unsigned long long* __restrict__ sums,
                                                                const unsigned int* __restrict__ n_dev,
                                                                MeshCounts* __restrict__ counts) {
    const unsigned int n_tiles = (*n_dev + kClassTile - 1) / kClassTile;
    unsigned long long carry = 0;
    for (unsigned int b = 0; b < n_tiles; b += kSumThreads * kSumItems) {
        const unsigned int i0 = b + threadIdx.x * kSumItems;
        unsigned long long v[kSumItems], s = 0;
#pragma unroll
        for (int q = 0; q < kSumItems; ++q) {
            v[q] = i0 + q < n_tiles ? sums[i0 + q] : 0ull;
            s += v[q];
        }
        unsigned long long total;
        unsigned long long run = carry + block_exclusive_scan<kSumThreads>(s, &total);
#pragma unroll
        for (int q = 0; q < kSumItems; ++q) {
            if (i0 + q < n_tiles) sums[i0 + q] = run;
            run += v[q];
        }
        carry += total;
    }
    if (threadIdx.x == 0) {
        counts->n_verts = carry & 0xffffffffull;
        counts->n_idx = carry >> 32;
        counts->missing_min = ~0ull;
        counts->overflow = 0ull;
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
    if ((e = cudaMalloc(&m->corners, cap * sizeof(uint4)))) return e;
    if ((e = cudaMalloc(&m->tile_sums, tiles * sizeof(unsigned long long)))) return e;
    if ((e = cudaMalloc(&m->tile_nflag, tiles * sizeof(unsigned int)))) return e;
    if ((e = cudaMalloc(&m->flagged, tiles * kClassTile * sizeof(unsigned int)))) return e;
    if ((e = cudaMalloc(&m->rows, rows * sizeof(unsigned int)))) return e;
    if ((e = cudaMalloc(&m->tile_ranges, tiles * 3 * sizeof(uint2)))) return e;
    m->rows_cap = rows;
    if ((e = cudaMalloc(&m->counts, sizeof(MeshCounts)))) return e;
    if ((e = cudaMalloc(&m->n_dev, sizeof(unsigned int)))) return e;
    m->cap = cap;
    return cudaSuccess;
}

void mesh_scratch_free(MeshScratch* m) {
    cudaFree(m->vflags);
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
    k_row_directory<K><<<grid_for(((size_t)1 << (2 * kb)) + 1, sms), kThreads, 0, st>>>(keys, ms.n_dev, kb, ms.rows);
    if (stage_events) cudaEventRecord(stage_events[0], st);
    // tile ranges, then the classification (its grid: up to 8 CTAs per SM, each walking tiles)
    const unsigned int max_tiles = (unsigned int)((n_cap + kClassTile - 1) / kClassTile);
    const int offsets = with_indices ? 3 : 2;
    k_mesh_tile_ranges<K><<<grid_for((size_t)max_tiles * offsets, sms), kThreads, 0, st>>>(
        keys, kb, ms.rows, ms.n_dev, offsets, ms.tile_ranges, max_tiles);
    const int class_grid = (int)(max_tiles < (unsigned int)(sms * 8) ? (max_tiles ? max_tiles : 1) : sms * 8);
    if (with_indices) {
        const size_t smem = class_smem<K>(3);
        cudaFuncSetAttribute(k_mesh_classify_tiled<true, K>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k_mesh_classify_tiled<true, K><<<class_grid, kThreads, smem, st>>>(keys, kb, vals, ms.rows, ms.n_dev,
                                                                          ms.tile_ranges, max_tiles, ms.vflags,
                                                                          ms.tile_sums, ms.tile_nflag, ms.flagged,
                                                                          ms.corners);
    } else {
        const size_t smem = class_smem<K>(2);
        cudaFuncSetAttribute(k_mesh_classify_tiled<false, K>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k_mesh_classify_tiled<false, K><<<class_grid, kThreads, smem, st>>>(keys, kb, vals, ms.rows, ms.n_dev,
                                                                           ms.tile_ranges, max_tiles, ms.vflags,
                                                                           ms.tile_sums, ms.tile_nflag, ms.flagged,
                                                                           ms.corners);
    }
    if (stage_events) cudaEventRecord(stage_events[1], st);
    k_scan_tile_sums<<<1, kSumThreads, 0, st>>>(ms.tile_sums, ms.n_dev, ms.counts);
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
