// C-ABI driver around the reference's own kifi classes, compiled with them
// into oracle/_ref/libkifi_ref.so by oracle/build_ref.py.
//
// Test and baseline infrastructure only: it lets the parity tests and the
// CPU baseline of bench.py call the reference's unmodified algorithms
// (Integrator, Mesher, ICP, Renderer, DepthStream, util::radix_sort,
// util::set_union, util::kahan_sum) through plain pointers.
//
// Matrices are 16 floats in kifi's float4x4 memory order: four columns of
// four floats (KinectFission/kifi/util/math.h:59-61).
#define private public  // reach the private static stages of Integrator / ICP
#include <kifi/DepthSensorParams.h>
#include <kifi/DepthStream.h>
#include <kifi/ICP.h>
#include <kifi/Integrator.h>
#include <kifi/Mesher.h>
#include <kifi/Renderer.h>
#include <kifi/Volume.h>
#include <kifi/Voxel.h>
#include <kifi/util/algorithm.h>
#include <kifi/util/numeric.h>
#undef private

#include <fcntl.h>
#include <unistd.h>

#include <algorithm>
#include <cstring>
#include <vector>

using namespace kifi;

namespace {

util::float4x4 load_mat(const float* m) {
    util::float4x4 r;
    std::memcpy(&r, m, 64);
    return r;
}
void store_mat(const util::float4x4& r, float* m) { std::memcpy(m, &r, 64); }

DepthSensorParams make_cam(int w, int h, float fx, float fy, float cx, float cy, float znear,
                           float zfar) {
    return DepthSensorParams(util::int2(w, h), util::float2(fx, fy), util::float2(cx, cy),
                             util::float2(znear, zfar));
}

// The reference prints per-frame timings and association counts to stdout;
// keep stdout clean for callers that emit machine-readable output.
struct Quiet {
    int saved = -1;
    explicit Quiet(bool on) {
        if (!on) return;
        std::fflush(stdout);
        saved = dup(1);
        int devnull = open("/dev/null", O_WRONLY);
        dup2(devnull, 1);
        close(devnull);
    }
    ~Quiet() {
        if (saved < 0) return;
        std::fflush(stdout);
        dup2(saved, 1);
        close(saved);
    }
};
bool g_quiet = true;

struct RefVolume {
    Volume vol;
    Integrator integ;
    Mesher mesher;
    std::vector<util::float3> verts;
    std::vector<unsigned> idx;
    RefVolume(int res, float side, float trunc) : vol(res, side, trunc) {}
};

}  // namespace

extern "C" {

void kref_set_quiet(int on) { g_quiet = on != 0; }

// Volume( res, side, trunc )  -- Volume.cpp:12-37
void* kref_volume_create(int res, float side, float trunc) { return new RefVolume(res, side, trunc); }
void kref_volume_destroy(void* h) { delete static_cast<RefVolume*>(h); }
size_t kref_volume_size(void* h) { return static_cast<RefVolume*>(h)->vol.Data().size(); }

// Copies keys (u32) and voxels (distance-sum, weight) out of the flat_map.
void kref_volume_export(void* h, unsigned* keys, float* values) {
    auto& d = static_cast<RefVolume*>(h)->vol.Data();
    size_t n = d.size();
    for (size_t i = 0; i < n; ++i) {
        keys[i] = d.keys_cbegin()[i];
        std::memcpy(values + 2 * i, &d.values_cbegin()[i], 8);
    }
}

// flat_map::insert (flat_map.h:164-197): union, existing entries win.
void kref_volume_insert(void* h, const unsigned* keys, const float* values, size_t n) {
    auto& d = static_cast<RefVolume*>(h)->vol.Data();
    std::vector<Voxel> vals(n);
    for (size_t i = 0; i < n; ++i) std::memcpy(&vals[i], values + 2 * i, 8);
    d.insert(keys, keys + n, vals.begin());
}

// Integrator::Integrate -- Integrator.cpp:26-71
void kref_integrate(void* h, const float* depth, int w, int hgt, float fx, float fy, float cx,
                    float cy, float znear, float zfar, const float* world_to_eye) {
    RefVolume* r = static_cast<RefVolume*>(h);
    util::vector2d<float> frame(w, hgt);
    std::memcpy(frame.data(), depth, sizeof(float) * (size_t)w * hgt);
    Quiet q(g_quiet);
    r->integ.Integrate(r->vol, frame, make_cam(w, hgt, fx, fy, cx, cy, znear, zfar),
                       load_mat(world_to_eye));
}

// Integrator::DepthMap2PointCloud -- Integrator.cpp:76-183.  Returns nSplats;
// out must hold w*h keys.
size_t kref_splat(void* h, const float* depth, int w, int hgt, float fx, float fy, float cx,
                  float cy, float znear, float zfar, const float* world_to_eye, unsigned* out) {
    RefVolume* r = static_cast<RefVolume*>(h);
    util::vector2d<float> frame(w, hgt);
    std::memcpy(frame.data(), depth, sizeof(float) * (size_t)w * hgt);
    util::float4x4 eye_to_world = load_mat(world_to_eye);
    util::invert_transform(eye_to_world);
    std::vector<unsigned> pc(frame.size());
    size_t n = Integrator::DepthMap2PointCloud(
        r->vol, frame, make_cam(w, hgt, fx, fy, cx, cy, znear, zfar), eye_to_world, pc);
    std::copy(pc.begin(), pc.begin() + n, out);
    return n;
}

// radix_sort + unique + ExpandChunks exactly as Integrate chains them
// (Integrator.cpp:47-57).  keys is sorted/expanded in place into out;
// returns the final count.  out must hold 8*n entries.
size_t kref_sort_unique_expand(const unsigned* keys, size_t n, unsigned* out) {
    std::vector<unsigned> pc(keys, keys + n), scratch;
    scratch.reserve(n);
    scratch.resize(n);
    util::radix_sort(pc.data(), pc.data() + n, scratch.data());
    pc.resize(std::distance(pc.begin(), std::unique(pc.begin(), pc.end())));
    Integrator::ExpandChunks(pc, scratch);
    std::copy(pc.begin(), pc.end(), out);
    return pc.size();
}

// util::radix_sort, keys only (algorithm.h:63-91)
void kref_radix_sort(unsigned* keys, size_t n) {
    std::vector<unsigned> scratch(n);
    util::radix_sort(keys, keys + n, scratch.data());
}

// util::radix_sort, key/value pairs (algorithm.h:93-134)
void kref_radix_sort_pairs(unsigned* keys, unsigned* values, size_t n) {
    std::vector<unsigned> scratch(2 * n);
    util::radix_sort(keys, keys + n, values, scratch.data());
}

// util::set_union with values (algorithm.h:138-198).  Returns output size.
size_t kref_set_union(const int* k1, const int* v1, size_t n1, const int* k2, const int* v2,
                      size_t n2, int* ko, int* vo) {
    int* end = util::set_union(k1, k1 + n1, k2, k2 + n2, v1, v2, ko, vo);
    return (size_t)(end - ko);
}

// util::kahan_sum<float> over n values (numeric.h:52-74)
float kref_kahan_sum(const float* x, size_t n) {
    util::kahan_sum<float> s;
    for (size_t i = 0; i < n; ++i) s += x[i];
    return s;
}

// util::partial_sum_exclusive (numeric.h:78-108), in place
void kref_partial_sum_exclusive(int* a, size_t n) { util::partial_sum_exclusive(a, a + n, a); }

// Mesher::Mesh -- Mesher.cpp:14-45.  First call computes and caches the mesh
// and returns the counts; kref_mesh_fetch copies it out.
void kref_mesh(void* h, int with_indices, size_t* n_verts, size_t* n_idx) {
    RefVolume* r = static_cast<RefVolume*>(h);
    if (with_indices)
        r->mesher.Mesh(r->vol, r->verts, r->idx);
    else {
        r->mesher.Mesh(r->vol, r->verts);
        r->idx.clear();
    }
    *n_verts = r->verts.size();
    *n_idx = r->idx.size();
}
void kref_mesh_fetch(void* h, float* verts, unsigned* idx) {
    RefVolume* r = static_cast<RefVolume*>(h);
    if (!r->verts.empty()) std::memcpy(verts, r->verts.data(), 12 * r->verts.size());
    if (!r->idx.empty()) std::memcpy(idx, r->idx.data(), 4 * r->idx.size());
}

// ICP::AlignStep applied `iters` times exactly as ICP::Align chains it
// (ICP.cpp:9-31; Align itself fixes iters at 4).  synth is a sw*sh row-major
// float3 buffer of world points, (0,0,0) = invalid.  Poses are eye-to-world.
void kref_icp_align(const float* depth, int w, int hgt, const float* eye_to_world_guess,
                    const float* synth, int sw, int sh, const float* synth_eye_to_world, float fx,
                    float fy, float cx, float cy, float znear, float zfar, int iters,
                    float* out_pose) {
    util::vector2d<float> frame(w, hgt);
    std::memcpy(frame.data(), depth, sizeof(float) * (size_t)w * hgt);
    // The reference's search window is clamped to 640x480 whatever the
    // buffer's size (ICP.cpp:108-109) and indexes y*sw + x, so for buffers
    // smaller than that it reads past the end.  Back the buffer with
    // zero-filled storage that covers every such read and then shrink the
    // logical size: those reads see (0,0,0), i.e. invalid points.
    int alloc_h = std::max(sh, 480 + (640 + sw - 1) / sw);
    util::vector2d<util::float3> buf(sw, alloc_h);
    std::memcpy(buf.data(), synth, 12 * (size_t)sw * sh);
    buf.resize(sw, sh);
    DepthSensorParams cam = make_cam(w, hgt, fx, fy, cx, cy, znear, zfar);
    ICP icp;
    util::float4x4 result = load_mat(eye_to_world_guess);
    util::float4x4 synth_pose = load_mat(synth_eye_to_world);
    Quiet q(g_quiet);
    for (int i = 0; i < iters; ++i)
        result = icp.AlignStep(frame, result, buf, synth_pose, cam) * result;
    store_mat(result, out_pose);
}

// Renderer::Bin -- Renderer.cpp:39-80
void kref_bin(const float* points, size_t n, const float* world_to_clip, float* out, int w,
              int hgt) {
    std::vector<util::float3> pc(n);
    std::memcpy(pc.data(), points, 12 * n);
    util::vector2d<util::float3> buf(w, hgt);
    Renderer r;
    r.Bin(pc, load_mat(world_to_clip), buf);
    std::memcpy(out, buf.data(), 12 * (size_t)w * hgt);
}

// DepthSensorParams::EyeToClipRH -- DepthSensorParams.cpp:47-63
void kref_eye_to_clip(int w, int hgt, float fx, float fy, float cx, float cy, float znear,
                      float zfar, float* out) {
    store_mat(make_cam(w, hgt, fx, fy, cx, cy, znear, zfar).EyeToClipRH(), out);
}

// util::invert_transform -- math.h:615-625
void kref_invert_transform(const float* in, float* out) {
    util::float4x4 m = load_mat(in);
    util::invert_transform(m);
    store_mat(m, out);
}

// DepthStream (DepthStream.cpp:15-102): open, report geometry and frame
// count, read frames.
void* kref_depthstream_open(const char* path) { return new DepthStream(path); }
void kref_depthstream_close(void* h) { delete static_cast<DepthStream*>(h); }
int kref_depthstream_frame_count(void* h) { return static_cast<DepthStream*>(h)->FrameCount(); }
// Mesher::Mesh2Obj (Mesher.cpp:50-78)
void kref_mesh2obj(const float* verts, size_t nv, const unsigned* idx, size_t ni, const char* path) {
    std::vector<util::float3> v(nv);
    std::memcpy(v.data(), verts, 12 * nv);
    std::vector<unsigned> i(idx, idx + ni);
    Mesher::Mesh2Obj(v, i, path);
}

int kref_depthstream_next(void* h, float* depth, int capacity, int* w, int* hgt, float* view) {
    util::vector2d<float> frame;
    util::float4x4 v;
    if (!static_cast<DepthStream*>(h)->NextFrame(frame, v)) return 0;
    *w = (int)frame.width();
    *hgt = (int)frame.height();
    if ((int)frame.size() <= capacity) std::memcpy(depth, frame.data(), 4 * frame.size());
    store_mat(v, view);
    return 1;
}

}  // extern "C"
