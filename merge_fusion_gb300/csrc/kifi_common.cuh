// kifi_common.cuh -- shared device/host definitions of the GB300 depth-fusion
// library: IEEE float helpers in the reference's operation order, the voxel
// key codec, camera / volume geometry and the per-volume device control
// block.
//
// Parity rule for every kernel in this library: each float expression that
// the reference (denniskb/merge_fusion, KinectFission/kifi) evaluates is
// written with explicit round-to-nearest intrinsics (__fmul_rn, __fadd_rn,
// __fdiv_rn), so no multiply/add pair is ever contracted into an FMA and every
// division is IEEE-correct, whatever nvcc's -fmad setting.  That reproduces
// the reference's SSE1 arithmetic bit for bit.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/kifi_gpu.h"

#if defined(__CUDACC__)
#define KIFI_HD __host__ __device__ __forceinline__
#else
#define KIFI_HD inline
#endif

namespace kifi {

// ----------------------------------------------------------- float helpers
// On the host these compile to plain float operations; the library's host
// code is built with -ffp-contract=off so they stay unfused there too.
#if defined(__CUDA_ARCH__)
KIFI_HD float fmul(float a, float b) { return __fmul_rn(a, b); }
KIFI_HD float fadd(float a, float b) { return __fadd_rn(a, b); }
KIFI_HD float fsub(float a, float b) { return __fsub_rn(a, b); }
KIFI_HD float fdiv(float a, float b) { return __fdiv_rn(a, b); }
#else
KIFI_HD float fmul(float a, float b) { return a * b; }
KIFI_HD float fadd(float a, float b) { return a + b; }
KIFI_HD float fsub(float a, float b) { return a - b; }
KIFI_HD float fdiv(float a, float b) { return a / b; }
#endif

struct Mat4 {
    float m[16];  // kifi float4x4 memory order: column c at m[4c..4c+3]
};

// float4x4 * float4 = (c0*x + c1*y) + (c2*z + c3*w), lane by lane
// (KinectFission/kifi/util/math.h:362-365 and the SSE form :381-397).
KIFI_HD void mat_vec(const float* m, const float v[4], float out[4]) {
    float r[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        float a = fmul(m[0 + i], v[0]);
        float b = fmul(m[4 + i], v[1]);
        float c = fmul(m[8 + i], v[2]);
        float d = fmul(m[12 + i], v[3]);
        r[i] = fadd(fadd(a, b), fadd(c, d));
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) out[i] = r[i];
}

// float4x4 * float4x4, column by column (math.h:367-377)
KIFI_HD Mat4 mat_mul(const Mat4& a, const Mat4& b) {
    Mat4 r;
    for (int c = 0; c < 4; ++c) mat_vec(a.m, b.m + 4 * c, r.m + 4 * c);
    return r;
}

// util::invert_transform, the rigid inverse (math.h:615-625)
KIFI_HD Mat4 invert_transform(const Mat4& in) {
    Mat4 r = in;
    float t[4] = {-r.m[12], -r.m[13], -r.m[14], 1.0f};
    r.m[12] = 0.0f; r.m[13] = 0.0f; r.m[14] = 0.0f; r.m[15] = 1.0f;
    float s;
    s = r.m[1]; r.m[1] = r.m[4]; r.m[4] = s;
    s = r.m[2]; r.m[2] = r.m[8]; r.m[8] = s;
    s = r.m[6]; r.m[6] = r.m[9]; r.m[9] = s;
    float c3[4];
    mat_vec(r.m, t, c3);
    for (int i = 0; i < 4; ++i) r.m[12 + i] = c3[i];
    return r;
}

// DepthSensorParams::EyeToClipRH (DepthSensorParams.cpp:47-63)
KIFI_HD Mat4 eye_to_clip(const kifi_camera& c) {
    Mat4 r;
    for (int i = 0; i < 16; ++i) r.m[i] = 0.0f;
    r.m[0 + 4 * 0] = fdiv(fmul(2.0f, c.fx), (float)c.width);
    r.m[0 + 4 * 2] = fsub((float)c.width, fmul(2.0f, c.cx));
    r.m[1 + 4 * 1] = fdiv(fmul(2.0f, c.fy), (float)c.height);
    r.m[1 + 4 * 2] = fsub((float)c.height, fmul(2.0f, c.cy));
    // -(far + near) / (far - near)  and  -2 * far * near / (far - near)
    r.m[2 + 4 * 2] = fdiv(-fadd(c.zfar_m, c.znear_m), fsub(c.zfar_m, c.znear_m));
    r.m[2 + 4 * 3] = fdiv(fmul(fmul(-2.0f, c.zfar_m), c.znear_m), fsub(c.zfar_m, c.znear_m));
    r.m[3 + 4 * 2] = -1.0f;
    return r;
}

// ------------------------------------------------------------ key codec
// Linear 30-bit keys, key = z<<20 | y<<10 | x (util::pack / unpack,
// KinectFission/kifi/util/math.h:442-457).  Sorted key order is therefore
// z-major, then y, then x -- the order the mesher's neighbour walk and the
// update's tail rule depend on.
KIFI_HD uint32_t pack30(uint32_t x, uint32_t y, uint32_t z) { return z << 20 | y << 10 | x; }
KIFI_HD uint32_t key_x(uint32_t k) { return k & 0x3ffu; }
KIFI_HD uint32_t key_y(uint32_t k) { return k >> 10 & 0x3ffu; }
KIFI_HD uint32_t key_z(uint32_t k) { return k >> 20; }

// The same linear order for volumes beyond 1024 voxels per axis: 64-bit keys
// z << 2b | y << b | x with b = log2(res) bits per axis.  Codec<uint32_t> is
// util::pack (b = 10, fixed at compile time); Codec<uint64_t> takes b at run
// time.  With b = 10 both encode a voxel to the same number.
template <typename K>
struct Codec;
template <>
struct Codec<uint32_t> {
    static constexpr int b = 10;
    KIFI_HD explicit Codec(int) {}
    KIFI_HD uint32_t pack(uint32_t x, uint32_t y, uint32_t z) const { return pack30(x, y, z); }
    KIFI_HD uint32_t x(uint32_t k) const { return key_x(k); }
    KIFI_HD uint32_t y(uint32_t k) const { return key_y(k); }
    KIFI_HD uint32_t z(uint32_t k) const { return key_z(k); }
    KIFI_HD uint32_t row(uint32_t k) const { return k >> 10; }  // (z, y) row
};
template <>
struct Codec<uint64_t> {
    int b;
    KIFI_HD explicit Codec(int bits) : b(bits) {}
    KIFI_HD uint64_t pack(uint32_t x, uint32_t y, uint32_t z) const {
        return (uint64_t)z << (2 * b) | (uint64_t)y << b | (uint64_t)x;
    }
    KIFI_HD uint32_t x(uint64_t k) const { return (uint32_t)(k & ((1ull << b) - 1)); }
    KIFI_HD uint32_t y(uint64_t k) const { return (uint32_t)((k >> b) & ((1ull << b) - 1)); }
    KIFI_HD uint32_t z(uint64_t k) const { return (uint32_t)(k >> (2 * b)); }
    KIFI_HD uint64_t row(uint64_t k) const { return k >> b; }
};

// ------------------------------------------------------- volume geometry
// Volume's precomputed terms (Volume.cpp:12-37).
struct Geom {
    int res;
    int kb;            // key bits per axis: 10 (30-bit keys) or log2(res) (64-bit keys)
    float side, trunc;
    float vlen;        // side / res
    float center_off;  // vlen * 0.5 + min      (VoxelCenter)
    float vlen_inv;    // 1 / vlen
    float index_off;   // vlen_inv * -min       (VoxelIndex)
};

KIFI_HD Geom make_geom(int res, float side, float trunc) {
    Geom g;
    g.res = res;
    g.kb = 10;
    g.side = side;
    g.trunc = trunc;
    float mn = fmul(-0.5f, side);
    g.vlen = fdiv(side, (float)res);
    g.center_off = fadd(fmul(g.vlen, 0.5f), mn);
    g.vlen_inv = fdiv(1.0f, g.vlen);
    g.index_off = fmul(g.vlen_inv, -mn);
    return g;
}

// Per-frame constants derived from the camera and the world-to-eye pose
// (Integrator.cpp:41-42 and the set-ups of DepthMap2PointCloud :82-99 and
// UpdateVoxels :262-267).
struct FrameConst {
    Mat4 eye_to_world;
    Mat4 world_to_clip;
    float fl_inv_x, fl_inv_y;  // 1/fx, 1/fy
    float pp_x, pp_y;          // (0.5-cx)/fx, (cy-0.5)/fy  (as products with 1/f)
    float half_w, half_h;      // width*0.5, height*0.5
    float max_index;           // res - 1
    int width, height;
    int z_bounded;             // |clip z| <= 1e18 for every voxel centre of the volume
    int fast_uv;               // frame small enough for the reciprocal fast path
    float neg_zero;            // -0.0f, a value the device code cannot see at compile time
};

KIFI_HD FrameConst make_frame_const(const kifi_camera& cam, const Mat4& world_to_eye, int res) {
    FrameConst f;
    f.eye_to_world = invert_transform(world_to_eye);
    f.world_to_clip = mat_mul(eye_to_clip(cam), world_to_eye);
    f.fl_inv_x = fdiv(1.0f, cam.fx);
    f.fl_inv_y = fdiv(1.0f, cam.fy);
    f.pp_x = fmul(fsub(0.5f, cam.cx), f.fl_inv_x);
    f.pp_y = fmul(fsub(cam.cy, 0.5f), f.fl_inv_y);
    f.half_w = fmul((float)cam.width, 0.5f);
    f.half_h = fmul((float)cam.height, 0.5f);
    f.max_index = (float)(res - 1);
    f.width = cam.width;
    f.height = cam.height;
    f.z_bounded = 0;
    f.fast_uv = (cam.width <= 4096 && cam.height <= 4096) ? 1 : 0;
    f.neg_zero = -0.0f;
    return f;
}

// Host-side bound for UpdateVoxels' z lane: voxel centres lie in the cube
// [-side/2, side/2]^3 with w = 1, so |clip z| <= sum_j |m[2][j]| * side/2
// + |m[2][3]| (with slack for the float roundings of the four products).
inline int clip_z_bounded(const Mat4& w2c, float side) {
    double b = 0.0;
    for (int j = 0; j < 3; ++j) b += fabs((double)w2c.m[4 * j + 2]) * (0.5 * side + 1.0);
    b += fabs((double)w2c.m[14]);
    for (int i = 0; i < 16; ++i)
        if (!(fabs((double)w2c.m[i]) < 1e30)) return 0;
    return b * 1.001 <= 1e18 ? 1 : 0;
}

// --------------------------------------------------- device control block
// One per volume, in device memory.  Kernels read sizes from here, so the
// per-frame pipeline needs no host round trip and can be captured in a
// CUDA graph.
struct DeviceCtl {
    unsigned long long n[2];       // voxel count of key/value buffer 0 and 1
    unsigned int cur;              // which buffer holds the resident volume
    unsigned int n_new;            // keys appended by the splat/emit kernel
    unsigned long long excluded_key;  // max splat key + pack(1,1,1), or 0
    unsigned int status;           // KIFI_ERR_* bits raised on the device
    unsigned long long sort_epoch; // generation tag of the sort look-back words
    unsigned int tile_counter[8];  // dynamic tile ids (one per sort pass / merge)
    unsigned long long merge_e;    // settled merge: keys new to the volume,
    unsigned long long merge_n1;   //   resident voxels after it,
    unsigned int merge_ok;         //   and whether they fit the capacity
    unsigned long long frames;     // merges committed (frames integrated + inserts)
    // sizes of the last kFrameLog merges: resident before, new, resident after
    unsigned long long log_n0[64], log_new[64], log_n1[64];
};
constexpr int kFrameLog = 64;

// status bits raised on the device (reported through kifi_volume_sync)
enum : unsigned int {
    KIFI_DEV_ERR_CAPACITY = 1u,
    KIFI_DEV_ERR_TIMEOUT = 2u,
};

}  // namespace kifi
