/*
 * kifi_oracle.c -- CPU restatement of the reference's per-frame depth-fusion
 * path (denniskb/merge_fusion, KinectFission/kifi).
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker: the parity tests,
 * __graft_entry__.smoke() and the cpu_baseline leg of bench.py call it to
 * produce expected results.  The shipped library never links, loads or calls
 * it, and no product code path falls back to it.
 *
 * Parity is pinned: tests/test_oracle_pinned.py checks this file
 * bit-for-bit against the reference's own code compiled by
 * oracle/build_ref.py, and tests/golden/ holds fixtures generated from the
 * reference (tests/golden/make_golden.py).
 *
 * Every float expression follows the reference's operation order; build it
 * with -O2 -ffp-contract=off and without fast-math so that no multiply/add
 * is fused and every division is correctly rounded, exactly like the
 * reference's SSE1 code.  All matrices are 16 floats in kifi's float4x4
 * memory order (four columns, KinectFission/kifi/util/math.h:59-61).
 */
#include <float.h>
#include <limits.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "kifi_oracle.h"

/* ------------------------------------------------------------------ math */

/* float4x4 * float4: (c0*x + c1*y) + (c2*z + c3*w), lane by lane.
 * KinectFission/kifi/util/math.h:362-365 (float4 form) and :381-397 (SSE
 * form) -- both evaluate the same expression tree. */
void or_mat_vec(const float* m, const float* v, float* out) {
    float r[4];
    for (int i = 0; i < 4; ++i) {
        float a = m[0 + i] * v[0];
        float b = m[4 + i] * v[1];
        float c = m[8 + i] * v[2];
        float d = m[12 + i] * v[3];
        r[i] = (a + b) + (c + d);
    }
    memcpy(out, r, 16);
}

/* float4x4 * float4x4, column by column -- math.h:367-377 */
void or_mat_mul(const float* a, const float* b, float* out) {
    float r[16];
    for (int c = 0; c < 4; ++c) or_mat_vec(a, b + 4 * c, r + 4 * c);
    memcpy(out, r, 64);
}

/* util::invert_transform (rigid inverse) -- math.h:615-625 */
void or_invert_transform(const float* in, float* out) {
    float m[16];
    memcpy(m, in, 64);
    float t[4] = {-m[12], -m[13], -m[14], 1.0f};
    m[12] = 0.0f; m[13] = 0.0f; m[14] = 0.0f; m[15] = 1.0f;
    float s;
    s = m[1]; m[1] = m[4]; m[4] = s;   /* col0.y <-> col1.x */
    s = m[2]; m[2] = m[8]; m[8] = s;   /* col0.z <-> col2.x */
    s = m[6]; m[6] = m[9]; m[9] = s;   /* col1.z <-> col2.y */
    float c3[4];
    or_mat_vec(m, t, c3);
    memcpy(m + 12, c3, 16);
    memcpy(out, m, 64);
}


/* DepthSensorParams::EyeToClipRH -- DepthSensorParams.cpp:47-63 */
void or_eye_to_clip(const or_camera* c, float* out) {
    float m[16];
    memset(m, 0, 64);
    m[0 + 4 * 0] = 2.0f * c->fx / (float)c->width;
    m[0 + 4 * 2] = (float)c->width - 2.0f * c->cx;
    m[1 + 4 * 1] = 2.0f * c->fy / (float)c->height;
    m[1 + 4 * 2] = (float)c->height - 2.0f * c->cy;
    m[2 + 4 * 2] = -(c->zfar + c->znear) / (c->zfar - c->znear);
    m[2 + 4 * 3] = -2.0f * c->zfar * c->znear / (c->zfar - c->znear);
    m[3 + 4 * 2] = -1.0f;
    memcpy(out, m, 64);
}

/* --------------------------------------------------------------- volume */


void or_geom_init(or_geom* g, int res, float side, float trunc) {
    g->res = res;
    g->side = side;
    g->trunc = trunc;
    float mn = -0.5f * side; /* Volume::Minimum, Volume.cpp:63-66 */
    g->vlen = side / (float)res;
    g->center_off = g->vlen * 0.5f + mn;
    g->vlen_inv = 1.0f / g->vlen;
    g->index_off = g->vlen_inv * -mn;
}

/* util::pack / unpack -- math.h:442-457 (30-bit linear keys) */
static inline uint32_t pack30(uint32_t x, uint32_t y, uint32_t z) { return z << 20 | y << 10 | x; }

/* ---------------------------------------------------------------- splat */

/* Integrator::DepthMap2PointCloud -- Integrator.cpp:76-183.
 * One key per pixel with depth > 0 whose voxel index (after the -0.5 shift)
 * lies in [0, res-1) on all three axes; row-major pixel order. */
size_t or_splat(const or_geom* g, const float* depth, const or_camera* cam,
                const float* world_to_eye, uint32_t* out) {
    float e2w[16];
    or_invert_transform(world_to_eye, e2w);
    float fl_inv_x = 1.0f / cam->fx, fl_inv_y = 1.0f / cam->fy;
    float pp_x = (0.5f - cam->cx) * fl_inv_x;
    float pp_y = (cam->cy - 0.5f) * fl_inv_y;
    float max_index = (float)(g->res - 1);
    size_t n = 0;
    for (int v = 0; v < cam->height; ++v) {
        float row = 0.0f + -(float)v;
        for (int u = 0; u < cam->width; ++u) {
            float d = depth[(size_t)v * cam->width + u];
            if (!(d > 0.0f)) continue;
            float p[4];
            p[0] = ((float)u * fl_inv_x + pp_x) * d + 0.0f;
            p[1] = (row * fl_inv_y + pp_y) * d + 0.0f;
            p[2] = (-1.0f * 1.0f + 0.0f) * d + 0.0f;
            p[3] = (0.0f * 1.0f + 0.0f) * d + 1.0f;
            float w[4];
            or_mat_vec(e2w, p, w);
            float ix = (w[0] * g->vlen_inv + g->index_off) - 0.5f;
            float iy = (w[1] * g->vlen_inv + g->index_off) - 0.5f;
            float iz = (w[2] * g->vlen_inv + g->index_off) - 0.5f;
            /* lane w: (w*1 + 0) - 0.5 = 0.5, always inside [0, res-1) for res >= 2 */
            if (ix >= 0.0f && ix < max_index && iy >= 0.0f && iy < max_index && iz >= 0.0f &&
                iz < max_index)
                out[n++] = pack30((uint32_t)ix, (uint32_t)iy, (uint32_t)iz);
        }
    }
    return n;
}

/* ------------------------------------------------------- sort / unique */

/* util::radix_sort keys only: LSD, four stable 8-bit passes with an
 * exclusive scan of the 256 counts -- algorithm.h:63-91, numeric.h:78-108 */
void or_radix_sort_u32(uint32_t* keys, size_t n) {
    uint32_t* tmp = (uint32_t*)malloc(n * 4 + 4);
    uint32_t *src = keys, *dst = tmp;
    for (int shift = 0; shift != 32; shift += 8) {
        size_t cnt[256] = {0};
        for (size_t i = 0; i < n; ++i) ++cnt[(src[i] >> shift) & 0xff];
        size_t acc = 0;
        for (int b = 0; b < 256; ++b) { size_t t = cnt[b]; cnt[b] = acc; acc += t; }
        for (size_t i = 0; i < n; ++i) dst[cnt[(src[i] >> shift) & 0xff]++] = src[i];
        uint32_t* s = src; src = dst; dst = s;
    }
    /* four passes: the result is back in keys */
    free(tmp);
}

/* util::radix_sort key/value pairs (algorithm.h:93-134); values are 32-bit. */
void or_radix_sort_pairs_u32(uint32_t* keys, uint32_t* vals, size_t n) {
    uint32_t* tk = (uint32_t*)malloc(n * 4 + 4);
    uint32_t* tv = (uint32_t*)malloc(n * 4 + 4);
    uint32_t *sk = keys, *sv = vals, *dk = tk, *dv = tv;
    for (int shift = 0; shift != 32; shift += 8) {
        size_t cnt[256] = {0};
        for (size_t i = 0; i < n; ++i) ++cnt[(sk[i] >> shift) & 0xff];
        size_t acc = 0;
        for (int b = 0; b < 256; ++b) { size_t t = cnt[b]; cnt[b] = acc; acc += t; }
        for (size_t i = 0; i < n; ++i) {
            size_t d = cnt[(sk[i] >> shift) & 0xff]++;
            dk[d] = sk[i];
            dv[d] = sv[i];
        }
        uint32_t* s;
        s = sk; sk = dk; dk = s;
        s = sv; sv = dv; dv = s;
    }
    free(tk);
    free(tv);
}

/* std::unique on a sorted range -- Integrator.cpp:50-55 */
size_t or_unique_u32(uint32_t* keys, size_t n) {
    if (n == 0) return 0;
    size_t m = 1;
    for (size_t i = 1; i < n; ++i)
        if (keys[i] != keys[m - 1]) keys[m++] = keys[i];
    return m;
}

/* sorted set union of two sorted unique u32 ranges (std::set_union) */
static size_t set_union_u32(const uint32_t* a, size_t na, const uint32_t* b, size_t nb,
                            uint32_t* out) {
    size_t i = 0, j = 0, k = 0;
    while (i < na && j < nb) {
        if (a[i] < b[j]) out[k++] = a[i++];
        else if (b[j] < a[i]) out[k++] = b[j++];
        else { out[k++] = a[i++]; ++j; }
    }
    while (i < na) out[k++] = a[i++];
    while (j < nb) out[k++] = b[j++];
    return k;
}

/* Integrator::ExpandChunks / ExpandChunksHelper -- Integrator.cpp:186-250.
 * keys: sorted unique; out must hold 8*n.  The z and y steps are set unions
 * with the shifted copy; the x step walks the list once and, as in the
 * reference, never adds the successor of the last key. */
size_t or_expand(const uint32_t* keys, size_t n, uint32_t* out) {
    if (n == 0) return 0;
    uint32_t* a = (uint32_t*)malloc(8 * n * 4);
    uint32_t* b = (uint32_t*)malloc(8 * n * 4);
    uint32_t* sh = (uint32_t*)malloc(8 * n * 4);
    memcpy(a, keys, n * 4);
    size_t m = n;
    const uint32_t deltas[2] = {pack30(0, 0, 1), pack30(0, 1, 0)};
    for (int s = 0; s < 2; ++s) {
        for (size_t i = 0; i < m; ++i) sh[i] = a[i] + deltas[s];
        m = set_union_u32(a, m, sh, m, b);
        uint32_t* t = a; a = b; b = t;
    }
    size_t dst = 0;
    uint32_t prev = a[0];
    for (size_t i = 0; i < m; ++i) {
        uint32_t x = a[i];
        out[dst] = prev;
        dst += (x != prev);
        out[dst++] = x;
        prev = x + 1;
    }
    free(a);
    free(b);
    free(sh);
    return dst;
}

/* util::set_union with values (algorithm.h:138-198): ties take side 1. */
size_t or_set_union_i32(const int32_t* k1, const int32_t* v1, size_t n1, const int32_t* k2,
                        const int32_t* v2, size_t n2, int32_t* ko, int32_t* vo) {
    size_t i = 0, j = 0, k = 0;
    while (i < n1 && j < n2) {
        if (k1[i] < k2[j]) { ko[k] = k1[i]; vo[k++] = v1[i++]; }
        else if (k2[j] < k1[i]) { ko[k] = k2[j]; vo[k++] = v2[j++]; }
        else { ko[k] = k1[i]; vo[k++] = v1[i++]; ++j; }
    }
    while (i < n1) { ko[k] = k1[i]; vo[k++] = v1[i++]; }
    while (j < n2) { ko[k] = k2[j]; vo[k++] = v2[j++]; }
    return k;
}

/* ----------------------------------------------------- merge + update */

/* flat_map::insert (flat_map.h:164-197): union of the resident map with the
 * new keys; resident voxels keep their value, new ones get Voxel() = (0,0)
 * (Integrator.cpp:60-63).  vals are (distance-sum, weight) pairs. */
size_t or_insert(const uint32_t* rk, const float* rv, size_t nr, const uint32_t* nk, size_t nn,
                 uint32_t* ok, float* ov) {
    size_t i = 0, j = 0, k = 0;
    while (i < nr && j < nn) {
        if (rk[i] < nk[j]) { ok[k] = rk[i]; ov[2 * k] = rv[2 * i]; ov[2 * k + 1] = rv[2 * i + 1]; ++k; ++i; }
        else if (nk[j] < rk[i]) { ok[k] = nk[j]; ov[2 * k] = 0.0f; ov[2 * k + 1] = 0.0f; ++k; ++j; }
        else { ok[k] = rk[i]; ov[2 * k] = rv[2 * i]; ov[2 * k + 1] = rv[2 * i + 1]; ++k; ++i; ++j; }
    }
    while (i < nr) { ok[k] = rk[i]; ov[2 * k] = rv[2 * i]; ov[2 * k + 1] = rv[2 * i + 1]; ++k; ++i; }
    while (j < nn) { ok[k] = nk[j]; ov[2 * k] = 0.0f; ov[2 * k + 1] = 0.0f; ++k; ++j; }
    return k;
}

/* Integrator::UpdateVoxels -- Integrator.cpp:253-358 with Volume::VoxelCenter
 * (Volume.cpp:75-78) and Voxel::Update (Voxel.h:53-57).
 *
 * Only indices [0, n/4*4) are visited (the reference's 4-wide loop drops the
 * n%4 tail).  The z and w lanes of the projected point are multiplied by the
 * zero z/w components of ndcToUV, so their range test only rejects
 * non-finite values. */
void or_update(const or_geom* g, const uint32_t* keys, float* vals, size_t n, const float* depth,
               int width, int height, const float* world_to_clip) {
    float hw = (float)width * 0.5f, hh = (float)height * 0.5f;
    size_t end = n / 4 * 4;
    for (size_t i = 0; i < end; ++i) {
        uint32_t k = keys[i];
        float p[4] = {(float)(k & 0x3ffu), (float)(k >> 10 & 0x3ffu), (float)(k >> 20), 1.0f};
        float c[4];
        c[0] = p[0] * g->vlen + g->center_off;
        c[1] = p[1] * g->vlen + g->center_off;
        c[2] = p[2] * g->vlen + g->center_off;
        c[3] = p[3] * 1.0f + 0.0f;
        float cl[4];
        or_mat_vec(world_to_clip, c, cl);
        float dist = cl[3];
        float q0 = cl[0] / cl[3], q1 = cl[1] / cl[3], q2 = cl[2] / cl[3], q3 = cl[3] / cl[3];
        float u = q0 * hw + hw;
        float v = q1 * hh + hh;
        float z = q2 * 0.0f + 0.0f;
        float w = q3 * 0.0f + 0.0f;
        if (!(u >= 0.0f && u < (float)width && v >= 0.0f && v < (float)height && z >= -1.0f &&
              z < 1.0f && w >= -FLT_MAX && w < FLT_MAX))
            continue;
        size_t px = (uint32_t)u;
        size_t py = (size_t)height - (uint32_t)v - 1;
        float d = depth[py * (size_t)width + px];
        float sd = d - dist;
        if (d > 0.0f && sd >= -g->trunc) {
            float upd = (g->trunc < sd) ? g->trunc : sd; /* std::min(sd, trunc) */
            vals[2 * i] += upd;
            vals[2 * i + 1] += 1.0f;
        }
    }
}

/* Integrator::Integrate -- Integrator.cpp:26-71: splat, radix sort, unique,
 * expand, flat_map insert, update.  (rk, rv, nr) is the resident volume;
 * the new volume goes to (ok, ov) which must hold nr + 8*w*h entries.
 * Returns the new size. */
size_t or_integrate(const or_geom* g, const float* depth, const or_camera* cam,
                    const float* world_to_eye, const uint32_t* rk, const float* rv, size_t nr,
                    uint32_t* ok, float* ov) {
    size_t P = (size_t)cam->width * cam->height;
    uint32_t* pc = (uint32_t*)malloc(P * 4 + 4);
    uint32_t* ex = (uint32_t*)malloc(8 * P * 4 + 4);
    size_t n = or_splat(g, depth, cam, world_to_eye, pc);
    or_radix_sort_u32(pc, n);
    n = or_unique_u32(pc, n);
    size_t e = or_expand(pc, n, ex);
    size_t n1 = or_insert(rk, rv, nr, ex, e, ok, ov);
    float e2c[16], w2c[16];
    or_eye_to_clip(cam, e2c);
    or_mat_mul(e2c, world_to_eye, w2c);
    or_update(g, ok, ov, n1, depth, cam->width, cam->height, w2c);
    free(pc);
    free(ex);
    return n1;
}

/* --------------------------------------------------------------- mesher */

#include "mc_table.h"

static inline float voxel_distance(const float* v) { return v[0] / v[1]; } /* Voxel.h:39-44 */

/* Marching-cubes mesher -- Mesher::Generate<bool> (Mesher.cpp:85-229) and
 * Mesher::Mesh (Mesher.cpp:14-45).
 *
 * with_indices = 0: vertices in generation order (voxels from n-2 down to
 * 0, axes x,y,z), no indices (Mesher::Mesh(volume, verts)).
 * with_indices = 1: vertices sorted by id 3*key+axis, indices in
 * generation order mapped to vertex ranks, reproducing the reference's
 * mapping walk (an index whose id has no vertex stops the walk, and every
 * id at or above it keeps its raw id value).
 *
 * The reference's three neighbour pointers start at n-2 and only move down,
 * so a +y/+z/+yz neighbour lookup lands on min(n-2, upper_bound(target)-1);
 * this restatement evaluates that closed form per voxel. */
static size_t upper_bound_u32(const uint32_t* k, size_t n, uint32_t t) {
    size_t lo = 0, hi = n;
    while (lo < hi) {
        size_t mid = (lo + hi) / 2;
        if (k[mid] <= t) lo = mid + 1; else hi = mid;
    }
    return lo;
}

int or_mesh(const or_geom* g, const uint32_t* keys, const float* vals, size_t n, int with_indices,
            float* verts, size_t vcap, uint32_t* idx, size_t icap, size_t* nv_out,
            size_t* ni_out) {
    size_t nv = 0, ni = 0;
    uint32_t* vid = (uint32_t*)malloc((3 * n + 1) * 4);
    uint32_t* iid = with_indices ? (uint32_t*)malloc((15 * n + 1) * 4) : NULL;
    const float zero2[2] = {0.0f, 0.0f};
    const uint32_t dY = pack30(0, 1, 0), dZ = pack30(0, 0, 1), dYZ = pack30(0, 1, 1);
    for (long long ii = (long long)n - 2; ii >= 0; --ii) {
        size_t i = (size_t)ii;
        if (0.0f == vals[2 * i + 1]) continue;
        uint32_t key = keys[i];
        size_t ub;
        ub = upper_bound_u32(keys, n, key + dY);
        size_t iTop = ub - 1 < n - 2 ? ub - 1 : n - 2;
        ub = upper_bound_u32(keys, n, key + dZ);
        size_t iFront = ub - 1 < n - 2 ? ub - 1 : n - 2;
        const float* vx[8];
        vx[0] = vals + 2 * i;
        vx[2] = keys[iTop] == key + dY ? vals + 2 * iTop : zero2;
        vx[4] = keys[iFront] == key + dZ ? vals + 2 * iFront : zero2;
        vx[1] = keys[i + 1] == key + 1 ? vals + 2 * (i + 1) : zero2;
        uint32_t x0 = key & 0x3ffu, y0 = key >> 10 & 0x3ffu, z0 = key >> 20;
        /* Volume::VoxelCenter(int,int,int) -- Volume.cpp:80-88 */
        float c[3] = {(float)(int)x0 * g->vlen + g->center_off,
                      (float)(int)y0 * g->vlen + g->center_off,
                      (float)(int)z0 * g->vlen + g->center_off};
        float dself = voxel_distance(vx[0]);
        const int nb[3] = {1, 2, 4};
        for (int a = 0; a < 3; ++a) {
            const float* o = vx[nb[a]];
            if (o[1] > 0.0f && dself * voxel_distance(o) <= 0.0f) {
                if (nv >= vcap) goto overflow;
                float vert[3] = {c[0], c[1], c[2]};
                vert[a] += fabsf(dself) / (fabsf(dself) + fabsf(voxel_distance(o))) * g->vlen;
                memcpy(verts + 3 * nv, vert, 12);
                vid[nv++] = 3 * key + (uint32_t)a;
            }
        }
        if (!with_indices) continue;
        ub = upper_bound_u32(keys, n, key + dYZ);
        size_t iFT = ub - 1 < n - 2 ? ub - 1 : n - 2;
        vx[6] = keys[iFT] == key + dYZ ? vals + 2 * iFT : zero2;
        vx[3] = keys[iTop + 1] == key + pack30(1, 1, 0) ? vals + 2 * (iTop + 1) : zero2;
        vx[5] = keys[iFront + 1] == key + pack30(1, 0, 1) ? vals + 2 * (iFront + 1) : zero2;
        vx[7] = keys[iFT + 1] == key + pack30(1, 1, 1) ? vals + 2 * (iFT + 1) : zero2;
        int skip = 0;
        for (int q = 1; q < 8; ++q) skip |= (0.0f == vx[q][1]);
        if (skip) continue;
        int lut = (voxel_distance(vx[0]) < 0.0f) << 2 | (voxel_distance(vx[1]) < 0.0f) << 3 |
                  (voxel_distance(vx[2]) < 0.0f) << 6 | (voxel_distance(vx[3]) < 0.0f) << 7 |
                  (voxel_distance(vx[4]) < 0.0f) << 1 | (voxel_distance(vx[5]) < 0.0f) << 0 |
                  (voxel_distance(vx[6]) < 0.0f) << 5 | (voxel_distance(vx[7]) < 0.0f) << 4;
        uint32_t x1 = x0 + 1, y1 = y0 + 1, z1 = z0 + 1;
        uint32_t l2g[12] = {
            pack30(x0, y0, z1) * 3,     pack30(x0, y0, z0) * 3 + 2, pack30(x0, y0, z0) * 3,
            pack30(x1, y0, z0) * 3 + 2, pack30(x0, y1, z1) * 3,     pack30(x0, y1, z0) * 3 + 2,
            pack30(x0, y1, z0) * 3,     pack30(x1, y1, z0) * 3 + 2, pack30(x1, y0, z1) * 3 + 1,
            pack30(x0, y0, z1) * 3 + 1, pack30(x0, y0, z0) * 3 + 1, pack30(x1, y0, z0) * 3 + 1};
        int cnt = kifi_mc_tri_count(lut) * 3;
        for (int t = 0; t < cnt; ++t) {
            if (ni >= icap) goto overflow;
            iid[ni++] = l2g[kifi_mc_tri_edge(lut, t)];
        }
    }
    if (with_indices) {
        /* sort vertices by id (stable radix sort of (id, position)) */
        uint32_t* perm = (uint32_t*)malloc((nv + 1) * 4);
        for (size_t i = 0; i < nv; ++i) perm[i] = (uint32_t)i;
        or_radix_sort_pairs_u32(vid, perm, nv);
        float* sorted = (float*)malloc((3 * nv + 1) * 4);
        for (size_t i = 0; i < nv; ++i) memcpy(sorted + 3 * i, verts + 3 * (size_t)perm[i], 12);
        memcpy(verts, sorted, 12 * nv);
        free(sorted);
        free(perm);
        /* map index ids to vertex ranks -- Mesher.cpp:28-44 */
        uint32_t* pos = (uint32_t*)malloc((ni + 1) * 4);
        for (size_t i = 0; i < ni; ++i) pos[i] = (uint32_t)i;
        or_radix_sort_pairs_u32(iid, pos, ni);
        size_t j = 0;
        for (size_t i = 0; i < nv; ++i)
            while (j < ni && iid[j] == vid[i]) iid[j++] = (uint32_t)i;
        for (size_t i = 0; i < ni; ++i) idx[pos[i]] = iid[i];
        free(pos);
    }
    free(vid);
    free(iid);
    *nv_out = nv;
    *ni_out = ni;
    return 0;
overflow:
    free(vid);
    free(iid);
    *nv_out = nv;
    *ni_out = ni;
    return 1;
}

/* ---------------------------------------------------------------- ICP */

/* float-to-int conversion with x86 CVTTSS2SI semantics (the reference's
 * platform): truncation, and INT_MIN for NaN or out-of-range values. */
static inline int32_t cvt_i32_x86(float f) {
    if (f >= -2147483648.0f && f < 2147483648.0f) return (int32_t)f;
    return INT32_MIN;
}
/* two's-complement int32 subtraction (the reference relies on wraparound) */
static inline int32_t wrap_sub(int32_t a, int32_t b) {
    return (int32_t)(uint32_t)((uint32_t)a - (uint32_t)b);
}

/* kahan_sum<float>::operator+= -- numeric.h:59-68 */
typedef struct { float s, c; } kahan_f;
static inline void kahan_add(kahan_f* k, float x) {
    float y = x - k->c;
    float t = k->s + y;
    k->c = t - k->s - y;
    k->s = t;
}

/* Cyclic Jacobi eigen-decomposition of a symmetric 4x4 matrix in double
 * (Golub & Van Loan, "Matrix Computations", sec. 8.5: classical rotations
 * applied in row-cyclic order until the off-diagonal norm vanishes).
 * a is row-major and is destroyed; v receives eigenvectors in its columns. */
void or_jacobi4(double* a, double* ev, double* v) {
    for (int i = 0; i < 16; ++i) v[i] = (i % 5 == 0) ? 1.0 : 0.0;
    for (int sweep = 0; sweep < 64; ++sweep) {
        double off = 0.0;
        for (int p = 0; p < 4; ++p)
            for (int q = p + 1; q < 4; ++q) off += a[4 * p + q] * a[4 * p + q];
        if (off == 0.0) break;
        for (int p = 0; p < 3; ++p)
            for (int q = p + 1; q < 4; ++q) {
                double apq = a[4 * p + q];
                if (apq == 0.0) continue;
                double theta = (a[4 * q + q] - a[4 * p + p]) / (2.0 * apq);
                double t = (theta >= 0.0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
                double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
                for (int k = 0; k < 4; ++k) { /* A <- A J */
                    double akp = a[4 * k + p], akq = a[4 * k + q];
                    a[4 * k + p] = c * akp - s * akq;
                    a[4 * k + q] = s * akp + c * akq;
                }
                for (int k = 0; k < 4; ++k) { /* A <- J^T A */
                    double apk = a[4 * p + k], aqk = a[4 * q + k];
                    a[4 * p + k] = c * apk - s * aqk;
                    a[4 * q + k] = s * apk + c * aqk;
                }
                for (int k = 0; k < 4; ++k) { /* V <- V J */
                    double vkp = v[4 * k + p], vkq = v[4 * k + q];
                    v[4 * k + p] = c * vkp - s * vkq;
                    v[4 * k + q] = s * vkp + c * vkq;
                }
            }
    }
    for (int i = 0; i < 4; ++i) ev[i] = a[5 * i];
}

typedef struct {
    int n_assoc;          /* associations of the last iteration */
    double sums[15];      /* last iteration: src sum (3), dst sum (3), S (9) */
} or_icp_stats;

/* quaternion (x = scalar part) to rotation -- ICP.cpp:233-254 */
static void or_quat_to_rot(const double* q, double* R) {
    double xy = q[0] * q[1], xz = q[0] * q[2], xw = q[0] * q[3], yy = q[1] * q[1],
           yz = q[1] * q[2], yw = q[1] * q[3], zz = q[2] * q[2], zw = q[2] * q[3], ww = q[3] * q[3];
    R[0] = 1.0 - 2.0 * (zz + ww); R[1] = 2.0 * (yz - xw);       R[2] = 2.0 * (yw + xz);
    R[3] = 2.0 * (yz + xw);       R[4] = 1.0 - 2.0 * (yy + ww); R[5] = 2.0 * (zw - xy);
    R[6] = 2.0 * (yw - xz);       R[7] = 2.0 * (zw + xy);       R[8] = 1.0 - 2.0 * (yy + zz);
}

/* 0: the reference's float Kahan sums and float N (parity mode);
 * 1: every sum, the centred cross-covariance and N in double (the FP64
 *    reference solution the GPU's float-float solve is measured against). */
static int g_icp_fp64 = 0;
void or_icp_set_fp64(int on) { g_icp_fp64 = on; }

/* The association search of one source (ICP.cpp:100-131): the first strict
 * minimum of len^2 < 0.01 over the window at (u, v), clamped to columns
 * [0, 640) and rows [0, 480); returns len^2 (0.01 when none) and the
 * winner's linear target index in *at (-1 when none). */
static float icp_search(const float* synth, size_t nsynth, int sw, int32_t u, int32_t v, const float* wp,
                        int64_t* at_out) {
    float mind = 0.01f;
    int64_t best = -1;
    /* any u >= 640 or v >= 480 leaves the window empty, so the
     * reference's wrapping u + 21 / v + 21 cannot matter */
    int64_t yend = (int64_t)v + 21 < 480 ? (int64_t)v + 21 : 480;
    int64_t xend = (int64_t)u + 21 < 640 ? (int64_t)u + 21 : 640;
    for (int64_t y1 = v; y1 < yend; ++y1)
        for (int64_t x1 = u; x1 < xend; ++x1) {
            size_t at = (size_t)y1 * (size_t)sw + (size_t)x1;
            if (at >= nsynth) continue;
            const float* q = synth + 3 * at;
            if (q[0] == 0.0f && q[1] == 0.0f && q[2] == 0.0f) continue;
            float dx = q[0] - wp[0], dy = q[1] - wp[1], dz = q[2] - wp[2];
            float dw = 1.0f - wp[3];
            float l2 = (dx * dx + dy * dy) + (dz * dz + dw * dw);
            if (l2 < mind) { mind = l2; best = (int64_t)at; }
        }
    *at_out = best;
    return mind;
}

/* One ICP::AlignStep (ICP.cpp:35-265) with the Horn solve in double.
 *
 * Association, Kahan centroid and cross-covariance sums follow the reference
 * in float and in its order (rows, every 4th column).  The symmetric 4x4
 * N matrix is formed in float as the reference does, then solved by the
 * double Jacobi routine above; the rotation, translation and the returned
 * step matrix (T*R, row-major 4x4 in `step` as double) are computed in
 * double.
 *
 * The synthetic buffer is sw x sh float3 world points, (0,0,0) = invalid.
 * As in the reference the search window is clamped to columns [0, 640) and
 * rows [0, 480) (ICP.cpp:108-109) and the buffer is indexed y*sw + x;
 * reads that land past the buffer's end count as invalid points. */
int or_icp_step(const float* depth, const or_camera* cam, const float* e2w_guess,
                const float* synth, int sw, int sh, const float* synth_e2w, double* step,
                or_icp_stats* stats) {
    float dst_w2e[16], e2c[16], m[16];
    or_invert_transform(synth_e2w, dst_w2e);
    or_eye_to_clip(cam, e2c);
    or_mat_mul(e2c, dst_w2e, m);
    float fl[4] = {1.0f / cam->fx, 1.0f / cam->fy, 1.0f, 1.0f};
    float pp[4] = {(0.5f - cam->cx) * fl[0], (cam->cy - 0.5f) * fl[1], 0.0f * fl[2], 0.0f * fl[3]};
    float half_w = (float)sw * 0.5f, half_h = (float)sh * 0.5f;
    kahan_f ssum[4] = {{0}}, dsum[4] = {{0}};
    size_t cap = (size_t)cam->width * cam->height / 4 + 4, na = 0;
    float* assoc = (float*)malloc(cap * 6 * 4);
    const size_t nsynth = (size_t)sw * sh;
    for (int y = 0; y < cam->height; ++y)
        for (int x = 0; x < cam->width; x += 4) {
            float d = depth[(size_t)y * cam->width + x];
            if (0.0f == d) continue;
            float pt[4] = {(float)x, -(float)y, -1.0f, 0.0f};
            for (int l = 0; l < 4; ++l) pt[l] = (pt[l] * fl[l] + pp[l]) * d;
            pt[3] = 1.0f;
            float wp[4], cl[4];
            or_mat_vec(e2w_guess, pt, wp);
            or_mat_vec(m, wp, cl);
            float uvx = cl[0] / cl[3], uvy = cl[1] / cl[3];
            int32_t u = wrap_sub(cvt_i32_x86(uvx * half_w + half_w), 10);
            int32_t v = wrap_sub(wrap_sub((int32_t)sh - 1, cvt_i32_x86(uvy * half_h + half_h)), 10);
            if (u < 0) u = 0;
            if (v < 0) v = 0;
            int64_t at;
            float mind = icp_search(synth, nsynth, sw, u, v, wp, &at), p2[3] = {0, 0, 0};
            if (at >= 0) memcpy(p2, synth + 3 * at, 12);
            if (mind < 0.01f) {
                float* a = assoc + 6 * na++;
                a[0] = wp[0]; a[1] = wp[1]; a[2] = wp[2];
                a[3] = p2[0]; a[4] = p2[1]; a[5] = p2[2];
                for (int l = 0; l < 3; ++l) { kahan_add(&ssum[l], wp[l]); kahan_add(&dsum[l], p2[l]); }
                kahan_add(&ssum[3], wp[3]);
                kahan_add(&dsum[3], 1.0f);
            }
        }
    if (g_icp_fp64) {
        /* FP64 reference solution of the same associations: double sums,
         * two-pass centred cross-covariance, N in double */
        double ms[3] = {0, 0, 0}, md[3] = {0, 0, 0}, Sd[9] = {0};
        for (size_t i = 0; i < na; ++i)
            for (int l = 0; l < 3; ++l) { ms[l] += assoc[6 * i + l]; md[l] += assoc[6 * i + 3 + l]; }
        for (int l = 0; l < 3; ++l) { ms[l] /= (double)na; md[l] /= (double)na; }
        for (size_t i = 0; i < na; ++i)
            for (int r = 0; r < 3; ++r)
                for (int c = 0; c < 3; ++c)
                    Sd[3 * r + c] += ((double)assoc[6 * i + r] - ms[r]) * ((double)assoc[6 * i + 3 + c] - md[c]);
        free(assoc);
        double Xx = Sd[0], Xy = Sd[1], Xz = Sd[2], Yx = Sd[3], Yy = Sd[4], Yz = Sd[5], Zx = Sd[6], Zy = Sd[7], Zz = Sd[8];
        double a[16] = {Xx + Yy + Zz, Yz - Zy, Zx - Xz, Xy - Yx,
                        Yz - Zy, Xx - Yy - Zz, Xy + Yx, Zx + Xz,
                        Zx - Xz, Xy + Yx, Yy - Xx - Zz, Yz + Zy,
                        Xy - Yx, Zx + Xz, Yz + Zy, Zz - Xx - Yy};
        double ev[4], V[16];
        or_jacobi4(a, ev, V);
        int imax = 0;
        for (int i = 1; i < 4; ++i)
            if (ev[i] > ev[imax]) imax = i;
        double q[4] = {V[0 + imax], V[4 + imax], V[8 + imax], V[12 + imax]};
        double ql = sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
        for (int l = 0; l < 4; ++l) q[l] /= ql;
        double R[9];
        or_quat_to_rot(q, R);
        for (int r = 0; r < 4; ++r)
            for (int c = 0; c < 4; ++c) step[4 * r + c] = (r == c) ? 1.0 : 0.0;
        for (int r = 0; r < 3; ++r) {
            double t = md[r];
            for (int c = 0; c < 3; ++c) {
                step[4 * r + c] = R[3 * r + c];
                t -= R[3 * r + c] * ms[c];
            }
            step[4 * r + 3] = t;
        }
        if (stats) stats->n_assoc = (int)na;
        return na > 0 ? 0 : 1;
    }
    float nf = (float)na;
    float sm[4], dm[4];
    for (int l = 0; l < 4; ++l) { sm[l] = ssum[l].s / nf; dm[l] = dsum[l].s / nf; }
    kahan_f S[9] = {{0}};
    for (size_t i = 0; i < na; ++i) {
        const float* a = assoc + 6 * i;
        float s[3] = {a[0] - sm[0], a[1] - sm[1], a[2] - sm[2]};
        float t[3] = {a[3] - dm[0], a[4] - dm[1], a[5] - dm[2]};
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) kahan_add(&S[3 * r + c], s[r] * t[c]);
    }
    free(assoc);
    float Sxx = S[0].s, Sxy = S[1].s, Sxz = S[2].s, Syx = S[3].s, Syy = S[4].s, Syz = S[5].s,
          Szx = S[6].s, Szy = S[7].s, Szz = S[8].s;
    float nm[16] = {Sxx + Syy + Szz, Syz - Szy, Szx - Sxz, Sxy - Syx,
                    0, Sxx - Syy - Szz, Sxy + Syx, Szx + Sxz,
                    0, 0, Syy - Sxx - Szz, Syz + Szy,
                    0, 0, 0, Szz - Sxx - Syy};
    double a[16], ev[4], V[16];
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) a[4 * r + c] = r <= c ? nm[4 * r + c] : nm[4 * c + r];
    or_jacobi4(a, ev, V);
    int imax = 0;
    for (int i = 1; i < 4; ++i)
        if (ev[i] > ev[imax]) imax = i;
    double q[4] = {V[0 + imax], V[4 + imax], V[8 + imax], V[12 + imax]};
    double ql = sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
    for (int l = 0; l < 4; ++l) q[l] /= ql;
    double R[9];
    or_quat_to_rot(q, R);
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) step[4 * r + c] = (r == c) ? 1.0 : 0.0;
    for (int r = 0; r < 3; ++r) {
        double t = (double)dm[r];
        for (int c = 0; c < 3; ++c) {
            step[4 * r + c] = R[3 * r + c];
            t -= R[3 * r + c] * (double)sm[c];
        }
        step[4 * r + 3] = t;
    }
    if (stats) {
        stats->n_assoc = (int)na;
        for (int l = 0; l < 3; ++l) { stats->sums[l] = ssum[l].s; stats->sums[3 + l] = dsum[l].s; }
        for (int l = 0; l < 9; ++l) stats->sums[6 + l] = S[l].s;
    }
    return na > 0 ? 0 : 1;
}

/* ICP::Align (ICP.cpp:9-31) with a caller-chosen iteration count: the pose
 * is accumulated in double as step * pose; the float pose handed to each
 * step is the double pose rounded to float.  Poses are eye-to-world,
 * in/out as kifi float4x4 (column-major); pose_d gets the double result
 * column-major. */
/* The association of one AlignStep under pose e2w, per source in the
 * reference's order (rows, every 4th column; ICP.cpp:66-131): the winner's
 * linear target index (-1 when none, also for pixels without depth) and
 * its len^2 (0.01 when none). */
void or_icp_associate(const float* depth, const or_camera* cam, const float* e2w, const float* synth, int sw,
                      int sh, const float* synth_e2w, int64_t* out_at, float* out_l2) {
    float dst_w2e[16], e2c[16], m[16];
    or_invert_transform(synth_e2w, dst_w2e);
    or_eye_to_clip(cam, e2c);
    or_mat_mul(e2c, dst_w2e, m);
    float fl[4] = {1.0f / cam->fx, 1.0f / cam->fy, 1.0f, 1.0f};
    float pp[4] = {(0.5f - cam->cx) * fl[0], (cam->cy - 0.5f) * fl[1], 0.0f * fl[2], 0.0f * fl[3]};
    float half_w = (float)sw * 0.5f, half_h = (float)sh * 0.5f;
    const size_t nsynth = (size_t)sw * sh;
    size_t k = 0;
    for (int y = 0; y < cam->height; ++y)
        for (int x = 0; x < cam->width; x += 4, ++k) {
            out_at[k] = -1;
            out_l2[k] = 0.01f;
            float d = depth[(size_t)y * cam->width + x];
            if (0.0f == d) continue;
            float pt[4] = {(float)x, -(float)y, -1.0f, 0.0f};
            for (int l = 0; l < 4; ++l) pt[l] = (pt[l] * fl[l] + pp[l]) * d;
            pt[3] = 1.0f;
            float wp[4], cl[4];
            or_mat_vec(e2w, pt, wp);
            or_mat_vec(m, wp, cl);
            float uvx = cl[0] / cl[3], uvy = cl[1] / cl[3];
            int32_t u = wrap_sub(cvt_i32_x86(uvx * half_w + half_w), 10);
            int32_t v = wrap_sub(wrap_sub((int32_t)sh - 1, cvt_i32_x86(uvy * half_h + half_h)), 10);
            if (u < 0) u = 0;
            if (v < 0) v = 0;
            out_l2[k] = icp_search(synth, nsynth, sw, u, v, wp, &out_at[k]);
        }
}

void or_icp_align(const float* depth, const or_camera* cam, const float* e2w_guess,
                  const float* synth, int sw, int sh, const float* synth_e2w, int iters,
                  float* out_pose, double* pose_d, or_icp_stats* stats) {
    double P[16]; /* row-major */
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) P[4 * r + c] = e2w_guess[4 * c + r];
    float pf[16];
    memcpy(pf, e2w_guess, 64);
    for (int it = 0; it < iters; ++it) {
        double S[16], Q[16];
        or_icp_step(depth, cam, pf, synth, sw, sh, synth_e2w, S, stats);
        for (int r = 0; r < 4; ++r)
            for (int c = 0; c < 4; ++c) {
                double acc = 0.0;
                for (int k = 0; k < 4; ++k) acc += S[4 * r + k] * P[4 * k + c];
                Q[4 * r + c] = acc;
            }
        memcpy(P, Q, sizeof P);
        for (int r = 0; r < 4; ++r)
            for (int c = 0; c < 4; ++c) pf[4 * c + r] = (float)P[4 * r + c];
    }
    memcpy(out_pose, pf, 64);
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) pose_d[4 * c + r] = P[4 * r + c];
}

/* ------------------------------------------------------------- renderer */

/* Renderer::Bin -- Renderer.cpp:39-80: z-buffered splat of world points
 * into a w x h float3 buffer; the first point with the smallest clip z
 * wins a pixel; (0,0,0) marks empty pixels. */
void or_bin(const float* pts, size_t n, const float* world_to_clip, float* out, int w, int h) {
    float* zb = (float*)malloc((size_t)w * h * 4);
    for (size_t i = 0; i < (size_t)w * h; ++i) zb[i] = FLT_MAX;
    memset(out, 0, (size_t)w * h * 12);
    float hw = (float)w * 0.5f, hh = (float)h * 0.5f;
    for (size_t i = 0; i < n; ++i) {
        float p[4] = {pts[3 * i], pts[3 * i + 1], pts[3 * i + 2], 1.0f}, c[4];
        or_mat_vec(world_to_clip, p, c);
        float x = c[0] / c[3], y = c[1] / c[3], z = c[2] / c[3];
        int32_t u = cvt_i32_x86(x * hw + hw);
        int32_t v = wrap_sub((int32_t)h - 1, cvt_i32_x86(y * hh + hh));
        if (u >= 0 && u < w && v >= 0 && v < h && z >= -1.0f && z <= 1.0f) {
            size_t at = (size_t)v * w + u;
            if (z < zb[at]) {
                zb[at] = z;
                memcpy(out + 3 * at, pts + 3 * i, 12);
            }
        }
    }
    free(zb);
}

/* World points of a depth frame (0,0,0 where there is no depth), with the
 * back-projection arithmetic of DepthMap2PointCloud (Integrator.cpp:121-144)
 * -- the target buffer for ICP between consecutive frames. */
void or_backproject(const float* depth, const or_camera* cam, const float* eye_to_world,
                    float* out) {
    float fl_inv_x = 1.0f / cam->fx, fl_inv_y = 1.0f / cam->fy;
    float pp_x = (0.5f - cam->cx) * fl_inv_x;
    float pp_y = (cam->cy - 0.5f) * fl_inv_y;
    for (int v = 0; v < cam->height; ++v) {
        float row = 0.0f + -(float)v;
        for (int u = 0; u < cam->width; ++u) {
            size_t i = (size_t)v * cam->width + u;
            float d = depth[i];
            float w[4] = {0.0f, 0.0f, 0.0f, 0.0f};
            if (d > 0.0f) {
                float p[4];
                p[0] = ((float)u * fl_inv_x + pp_x) * d + 0.0f;
                p[1] = (row * fl_inv_y + pp_y) * d + 0.0f;
                p[2] = (-1.0f * 1.0f + 0.0f) * d + 0.0f;
                p[3] = (0.0f * 1.0f + 0.0f) * d + 1.0f;
                or_mat_vec(eye_to_world, p, w);
            }
            out[3 * i] = w[0];
            out[3 * i + 1] = w[1];
            out[3 * i + 2] = w[2];
        }
    }
}

/* kahan_sum<float> over a range -- numeric.h:52-74 */
float or_kahan_sum(const float* x, size_t n) {
    kahan_f k = {0.0f, 0.0f};
    for (size_t i = 0; i < n; ++i) kahan_add(&k, x[i]);
    return k.s;
}
