/*
 * kifi_oracle.h -- types and the float4x4 helpers shared by the oracle's
 * translation units (kifi_oracle.c: 30-bit keys and ICP, kifi_oracle_k64.c:
 * 64-bit keys).  Test infrastructure only.
 */
#pragma once

typedef struct {
    int width, height;
    float fx, fy, cx, cy;
    float znear, zfar;
} or_camera;

typedef struct {
    int res;
    float side, trunc;
    float vlen;         /* side / res                     Volume.cpp:28 */
    float center_off;   /* vlen * 0.5 + min               Volume.cpp:29 */
    float vlen_inv;     /* 1 / vlen                       Volume.cpp:34 */
    float index_off;    /* vlen_inv * -min                Volume.cpp:36 */
} or_geom;

void or_mat_vec(const float* m, const float* v, float* out);
void or_mat_mul(const float* a, const float* b, float* out);
void or_invert_transform(const float* in, float* out);
void or_eye_to_clip(const or_camera* c, float* out);
