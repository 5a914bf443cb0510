/*
 * kifi_oracle_k64.c -- the oracle's fusion path with 64-bit voxel keys.
 *
 * TEST INFRASTRUCTURE ONLY (the checker, never linked by the library).
 *
 * The reference keys voxels with util::pack (KinectFission/kifi/util/
 * math.h:442-457): 10 bits per axis, so its volumes stop at 1024 voxels per
 * axis.  The GPU library goes beyond that with keys z<<2b | y<<b | x,
 * b = max(10, log2 res), held in 64 bits.  This file is kifi_oracle.c's
 * splat / sort / unique / expand / insert / update / mesh with that key
 * (same float expressions, same order, same quirks) and b passed in.  With
 * b = 10 a 64-bit key is the number the 30-bit key is, so at up to 1024
 * voxels per axis every function here must agree with its 30-bit
 * counterpart bit for bit; tests/test_oracle_k64.py checks exactly that,
 * which ties this file to the pinned 30-bit oracle.
 */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "kifi_oracle.h"
#include "mc_table.h"

static inline uint64_t pack64(uint64_t x, uint64_t y, uint64_t z, int b) {
    return z << (2 * b) | y << b | x;
}

/* Integrator::DepthMap2PointCloud -- Integrator.cpp:76-183 (as or_splat) */
size_t or64_splat(const or_geom* g, int b, const float* depth, const or_camera* cam,
                  const float* world_to_eye, uint64_t* out) {
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
            if (ix >= 0.0f && ix < max_index && iy >= 0.0f && iy < max_index && iz >= 0.0f &&
                iz < max_index)
                out[n++] = pack64((uint32_t)ix, (uint32_t)iy, (uint32_t)iz, b);
        }
    }
    return n;
}

/* Stable LSD radix sort of 64-bit keys (8-bit digits over all 8 bytes),
 * with optional 32-bit payloads -- util::radix_sort's method
 * (algorithm.h:63-134) widened to 64-bit keys. */
void or64_radix_sort_pairs(uint64_t* keys, uint32_t* vals, size_t n) {
    uint64_t* tk = (uint64_t*)malloc(n * 8 + 8);
    uint32_t* tv = vals ? (uint32_t*)malloc(n * 4 + 4) : NULL;
    uint64_t *sk = keys, *dk = tk;
    uint32_t *sv = vals, *dv = tv;
    for (int shift = 0; shift != 64; shift += 8) {
        size_t cnt[256] = {0};
        for (size_t i = 0; i < n; ++i) ++cnt[(sk[i] >> shift) & 0xff];
        size_t acc = 0;
        for (int d = 0; d < 256; ++d) { size_t t = cnt[d]; cnt[d] = acc; acc += t; }
        for (size_t i = 0; i < n; ++i) {
            size_t d = cnt[(sk[i] >> shift) & 0xff]++;
            dk[d] = sk[i];
            if (vals) dv[d] = sv[i];
        }
        uint64_t* s = sk; sk = dk; dk = s;
        uint32_t* t = sv; sv = dv; dv = t;
    }
    /* eight passes: the result is back in keys / vals */
    free(tk);
    free(tv);
}

void or64_radix_sort(uint64_t* keys, size_t n) { or64_radix_sort_pairs(keys, NULL, n); }

size_t or64_unique(uint64_t* keys, size_t n) {
    if (n == 0) return 0;
    size_t m = 1;
    for (size_t i = 1; i < n; ++i)
        if (keys[i] != keys[m - 1]) keys[m++] = keys[i];
    return m;
}

static size_t set_union_u64(const uint64_t* a, size_t na, const uint64_t* b, size_t nb, uint64_t* out) {
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

/* Integrator::ExpandChunks -- Integrator.cpp:186-250 (as or_expand) */
size_t or64_expand(const uint64_t* keys, size_t n, int b, uint64_t* out) {
    if (n == 0) return 0;
    uint64_t* a = (uint64_t*)malloc(8 * n * 8);
    uint64_t* t2 = (uint64_t*)malloc(8 * n * 8);
    uint64_t* sh = (uint64_t*)malloc(8 * n * 8);
    memcpy(a, keys, n * 8);
    size_t m = n;
    const uint64_t deltas[2] = {pack64(0, 0, 1, b), pack64(0, 1, 0, b)};
    for (int s = 0; s < 2; ++s) {
        for (size_t i = 0; i < m; ++i) sh[i] = a[i] + deltas[s];
        m = set_union_u64(a, m, sh, m, t2);
        uint64_t* t = a; a = t2; t2 = t;
    }
    size_t dst = 0;
    uint64_t prev = a[0];
    for (size_t i = 0; i < m; ++i) {
        uint64_t x = a[i];
        out[dst] = prev;
        dst += (x != prev);
        out[dst++] = x;
        prev = x + 1;
    }
    free(a);
    free(t2);
    free(sh);
    return dst;
}

/* flat_map::insert -- flat_map.h:164-197 (as or_insert) */
size_t or64_insert(const uint64_t* rk, const float* rv, size_t nr, const uint64_t* nk, size_t nn, uint64_t* ok,
                   float* ov) {
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

/* Integrator::UpdateVoxels -- Integrator.cpp:253-358 (as or_update) */
void or64_update(const or_geom* g, int b, const uint64_t* keys, float* vals, size_t n, const float* depth,
                 int width, int height, const float* world_to_clip) {
    const uint64_t mask = ((uint64_t)1 << b) - 1;
    float hw = (float)width * 0.5f, hh = (float)height * 0.5f;
    size_t end = n / 4 * 4;
    for (size_t i = 0; i < end; ++i) {
        uint64_t k = keys[i];
        float p[4] = {(float)(uint32_t)(k & mask), (float)(uint32_t)(k >> b & mask), (float)(uint32_t)(k >> (2 * b)),
                      1.0f};
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
        if (!(u >= 0.0f && u < (float)width && v >= 0.0f && v < (float)height && z >= -1.0f && z < 1.0f &&
              w >= -FLT_MAX && w < FLT_MAX))
            continue;
        size_t px = (uint32_t)u;
        size_t py = (size_t)height - (uint32_t)v - 1;
        float d = depth[py * (size_t)width + px];
        float sd = d - dist;
        if (d > 0.0f && sd >= -g->trunc) {
            float upd = (g->trunc < sd) ? g->trunc : sd;
            vals[2 * i] += upd;
            vals[2 * i + 1] += 1.0f;
        }
    }
}

/* Integrator::Integrate -- Integrator.cpp:26-71 (as or_integrate) */
size_t or64_integrate(const or_geom* g, int b, const float* depth, const or_camera* cam, const float* world_to_eye,
                      const uint64_t* rk, const float* rv, size_t nr, uint64_t* ok, float* ov) {
    size_t P = (size_t)cam->width * cam->height;
    uint64_t* pc = (uint64_t*)malloc(P * 8 + 8);
    uint64_t* ex = (uint64_t*)malloc(8 * P * 8 + 8);
    size_t n = or64_splat(g, b, depth, cam, world_to_eye, pc);
    or64_radix_sort(pc, n);
    n = or64_unique(pc, n);
    size_t e = or64_expand(pc, n, b, ex);
    size_t n1 = or64_insert(rk, rv, nr, ex, e, ok, ov);
    float e2c[16], w2c[16];
    or_eye_to_clip(cam, e2c);
    or_mat_mul(e2c, world_to_eye, w2c);
    or64_update(g, b, ok, ov, n1, depth, cam->width, cam->height, w2c);
    free(pc);
    free(ex);
    return n1;
}

static inline float voxel_distance(const float* v) { return v[0] / v[1]; } /* Voxel.h:39-44 */

static size_t upper_bound_u64(const uint64_t* k, size_t n, uint64_t t) {
    size_t lo = 0, hi = n;
    while (lo < hi) {
        size_t mid = (lo + hi) / 2;
        if (k[mid] <= t) lo = mid + 1; else hi = mid;
    }
    return lo;
}

/* Mesher::Generate / Mesher::Mesh -- Mesher.cpp:14-45, 85-229 (as or_mesh).
 * Edge ids 3*key+axis are 64-bit; an index whose id has no vertex keeps the
 * low 32 bits of its id. */
int or64_mesh(const or_geom* g, int b, const uint64_t* keys, const float* vals, size_t n, int with_indices,
              float* verts, size_t vcap, uint32_t* idx, size_t icap, size_t* nv_out, size_t* ni_out) {
    const uint64_t mask = ((uint64_t)1 << b) - 1;
    size_t nv = 0, ni = 0;
    uint64_t* vid = (uint64_t*)malloc((3 * n + 1) * 8);
    uint64_t* iid = with_indices ? (uint64_t*)malloc((15 * n + 1) * 8) : NULL;
    const float zero2[2] = {0.0f, 0.0f};
    const uint64_t dY = pack64(0, 1, 0, b), dZ = pack64(0, 0, 1, b), dYZ = pack64(0, 1, 1, b);
    for (long long ii = (long long)n - 2; ii >= 0; --ii) {
        size_t i = (size_t)ii;
        if (0.0f == vals[2 * i + 1]) continue;
        uint64_t key = keys[i];
        size_t ub;
        ub = upper_bound_u64(keys, n, key + dY);
        size_t iTop = ub - 1 < n - 2 ? ub - 1 : n - 2;
        ub = upper_bound_u64(keys, n, key + dZ);
        size_t iFront = ub - 1 < n - 2 ? ub - 1 : n - 2;
        const float* vx[8];
        vx[0] = vals + 2 * i;
        vx[2] = keys[iTop] == key + dY ? vals + 2 * iTop : zero2;
        vx[4] = keys[iFront] == key + dZ ? vals + 2 * iFront : zero2;
        vx[1] = keys[i + 1] == key + 1 ? vals + 2 * (i + 1) : zero2;
        uint64_t x0 = key & mask, y0 = key >> b & mask, z0 = key >> (2 * b);
        float c[3] = {(float)(int)x0 * g->vlen + g->center_off, (float)(int)y0 * g->vlen + g->center_off,
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
                vid[nv++] = 3 * key + (uint64_t)a;
            }
        }
        if (!with_indices) continue;
        ub = upper_bound_u64(keys, n, key + dYZ);
        size_t iFT = ub - 1 < n - 2 ? ub - 1 : n - 2;
        vx[6] = keys[iFT] == key + dYZ ? vals + 2 * iFT : zero2;
        vx[3] = keys[iTop + 1] == key + pack64(1, 1, 0, b) ? vals + 2 * (iTop + 1) : zero2;
        vx[5] = keys[iFront + 1] == key + pack64(1, 0, 1, b) ? vals + 2 * (iFront + 1) : zero2;
        vx[7] = keys[iFT + 1] == key + pack64(1, 1, 1, b) ? vals + 2 * (iFT + 1) : zero2;
        int skip = 0;
        for (int q = 1; q < 8; ++q) skip |= (0.0f == vx[q][1]);
        if (skip) continue;
        int lut = (voxel_distance(vx[0]) < 0.0f) << 2 | (voxel_distance(vx[1]) < 0.0f) << 3 |
                  (voxel_distance(vx[2]) < 0.0f) << 6 | (voxel_distance(vx[3]) < 0.0f) << 7 |
                  (voxel_distance(vx[4]) < 0.0f) << 1 | (voxel_distance(vx[5]) < 0.0f) << 0 |
                  (voxel_distance(vx[6]) < 0.0f) << 5 | (voxel_distance(vx[7]) < 0.0f) << 4;
        uint64_t x1 = x0 + 1, y1 = y0 + 1, z1 = z0 + 1;
        uint64_t l2g[12] = {
            pack64(x0, y0, z1, b) * 3,     pack64(x0, y0, z0, b) * 3 + 2, pack64(x0, y0, z0, b) * 3,
            pack64(x1, y0, z0, b) * 3 + 2, pack64(x0, y1, z1, b) * 3,     pack64(x0, y1, z0, b) * 3 + 2,
            pack64(x0, y1, z0, b) * 3,     pack64(x1, y1, z0, b) * 3 + 2, pack64(x1, y0, z1, b) * 3 + 1,
            pack64(x0, y0, z1, b) * 3 + 1, pack64(x0, y0, z0, b) * 3 + 1, pack64(x1, y0, z0, b) * 3 + 1};
        int cnt = kifi_mc_tri_count(lut) * 3;
        for (int t = 0; t < cnt; ++t) {
            if (ni >= icap) goto overflow;
            iid[ni++] = l2g[kifi_mc_tri_edge(lut, t)];
        }
    }
    if (with_indices) {
        uint32_t* perm = (uint32_t*)malloc((nv + 1) * 4);
        for (size_t i = 0; i < nv; ++i) perm[i] = (uint32_t)i;
        or64_radix_sort_pairs(vid, perm, nv);
        float* sorted = (float*)malloc((3 * nv + 1) * 4);
        for (size_t i = 0; i < nv; ++i) memcpy(sorted + 3 * i, verts + 3 * (size_t)perm[i], 12);
        memcpy(verts, sorted, 12 * nv);
        free(sorted);
        free(perm);
        /* map index ids to vertex ranks -- Mesher.cpp:28-44 */
        uint32_t* pos = (uint32_t*)malloc((ni + 1) * 4);
        for (size_t i = 0; i < ni; ++i) pos[i] = (uint32_t)i;
        or64_radix_sort_pairs(iid, pos, ni);
        size_t j = 0;
        for (size_t i = 0; i < nv; ++i)
            while (j < ni && iid[j] == vid[i]) iid[j++] = (uint64_t)i;
        for (size_t i = 0; i < ni; ++i) idx[pos[i]] = (uint32_t)iid[i];
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
