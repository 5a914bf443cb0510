// kifi_api_io.cu -- file I/O around the fusion path:
//
//  * kifi::DepthStream (KinectFission/kifi/DepthStream.h:13-45,
//    DepthStream.cpp:15-102): the .depth v1/v2 recording reader.  The host
//    path returns what DepthStream::NextFrame returns (float metres, the
//    view matrix); the device path copies the raw texels -- uint16
//    millimetres or float metres -- to a device buffer through pinned,
//    double-buffered staging, and the fusion kernels convert millimetres
//    with the same `texel * 0.001f` as DepthStream.cpp:89-90.
//  * kifi::Mesher::Mesh2Obj (Mesher.cpp:50-78): Wavefront OBJ text.
//  * Volume checkpoints (no counterpart in the reference): a header, the
//    resident keys in the volume's width, and the voxels, restored by a
//    set-union insert into a fresh volume of the same key width.
//
// .depth layout (poly2depth/README.txt, DepthStream.cpp:23-51): 15 bytes of
// magic (not checked by the reference, not checked here), int version;
// version 2 adds int width, int height, int texel type (0 = 16-bit mm,
// 1 = float m); then int frame count, and per frame 16 floats of view matrix
// followed by width * height texels.  DepthStream turns the 16 floats into a
// float4x4 with a transposing constructor and transposes it back
// (DepthStream.cpp:69-71), so the matrix it returns holds the file's 16
// floats in order; so does this reader.
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

#include "kifi_api_util.h"

using namespace kifi;

struct kifi_depthstream {
    std::FILE* f = nullptr;
    int width = 0, height = 0;
    int texel_u16 = 1;  // 1: 16-bit millimetres, 0: float metres
    int n_frames = 0, i_frame = 0;
    std::vector<unsigned char> raw;  // host path staging
    void* pinned[2] = {nullptr, nullptr};
    cudaEvent_t copied[2] = {nullptr, nullptr};
    int slot = 0, device = -1;
    size_t texel_bytes() const { return (size_t)width * height * (texel_u16 ? 2 : 4); }
};

namespace {

constexpr char kCheckpointMagic[8] = {'K', 'I', 'F', 'I', 'V', 'O', 'L', '1'};

struct CheckpointHeader {
    char magic[8];
    int32_t resolution;
    float side_length_m;
    float truncation_m;
    uint32_t key_bits;  // 0 (files before 64-bit keys) or 32: uint32 keys; 64: uint64 keys
    uint64_t n_voxels;
};

bool read_exact(std::FILE* f, void* dst, size_t bytes) { return std::fread(dst, 1, bytes, f) == bytes; }

// view + texels of the next frame into host memory
kifi_status read_frame(kifi_depthstream* s, void* texels, float view[16]) {
    if (s->i_frame >= s->n_frames) return fail(KIFI_ERR_END_OF_STREAM, "no frames left in the .depth stream");
    float v[16];
    if (!read_exact(s->f, v, sizeof v) || !read_exact(s->f, texels, s->texel_bytes()))
        return fail(KIFI_ERR_FORMAT, ".depth stream truncated inside a frame");
    if (view) std::memcpy(view, v, sizeof v);
    ++s->i_frame;
    return KIFI_OK;
}

}  // namespace

extern "C" {

kifi_status kifi_depthstream_open(const char* path, kifi_depthstream** out) {
    if (!path || !out) return fail(KIFI_ERR_INVALID_ARGUMENT, "null argument");
    *out = nullptr;
    std::FILE* f = std::fopen(path, "rb");
    if (!f) return fail(KIFI_ERR_IO, "cannot open the .depth file");
    kifi_depthstream* s = new (std::nothrow) kifi_depthstream();
    if (!s) {
        std::fclose(f);
        return fail(KIFI_ERR_OUT_OF_MEMORY, "host allocation");
    }
    s->f = f;
    int version = 0;
    bool ok = std::fseek(f, 15, SEEK_SET) == 0 && read_exact(f, &version, 4);
    if (ok && version == 1) {
        s->width = 640;
        s->height = 480;
        s->texel_u16 = 1;
    } else if (ok && version == 2) {
        int texel = -1;
        ok = read_exact(f, &s->width, 4) && read_exact(f, &s->height, 4) && read_exact(f, &texel, 4);
        ok = ok && (texel == 0 || texel == 1);
        s->texel_u16 = texel == 0 ? 1 : 0;
    } else {
        ok = false;
    }
    ok = ok && read_exact(f, &s->n_frames, 4);
    // frame width even: the reference converts texel pairs (DepthStream.cpp:62,84-91)
    ok = ok && s->width > 0 && s->height > 0 && s->width % 2 == 0 && s->n_frames >= 0 &&
         (size_t)s->width * s->height <= ((size_t)1 << 28);
    if (!ok) {
        kifi_depthstream_close(s);
        return fail(KIFI_ERR_FORMAT, "not a .depth v1/v2 stream (header)");
    }
    *out = s;
    return KIFI_OK;
}

kifi_status kifi_depthstream_close(kifi_depthstream* s) {
    if (!s) return KIFI_OK;
    for (int k = 0; k < 2; ++k) {
        if (s->copied[k]) {
            cudaEventSynchronize(s->copied[k]);
            cudaEventDestroy(s->copied[k]);
        }
        if (s->pinned[k]) cudaFreeHost(s->pinned[k]);
    }
    if (s->f) std::fclose(s->f);
    delete s;
    return KIFI_OK;
}

kifi_status kifi_depthstream_info(kifi_depthstream* s, int* width, int* height, int* texel_is_u16,
                                  int* frame_count) {
    if (!s) return fail(KIFI_ERR_INVALID_ARGUMENT, "null stream");
    if (width) *width = s->width;
    if (height) *height = s->height;
    if (texel_is_u16) *texel_is_u16 = s->texel_u16;
    if (frame_count) *frame_count = s->n_frames;
    return KIFI_OK;
}

kifi_status kifi_depthstream_next_frame(kifi_depthstream* s, float* out_depth_m, float out_view[16]) {
    if (!s || !out_depth_m) return fail(KIFI_ERR_INVALID_ARGUMENT, "null argument");
    const size_t n = (size_t)s->width * s->height;
    if (!s->texel_u16) return read_frame(s, out_depth_m, out_view);
    s->raw.resize(n * 2);
    kifi_status st = read_frame(s, s->raw.data(), out_view);
    if (st) return st;
    for (size_t i = 0; i < n; ++i) {
        unsigned short mm;
        std::memcpy(&mm, s->raw.data() + 2 * i, 2);  // little endian, as the reference
        out_depth_m[i] = fmul((float)mm, 0.001f);
    }
    return KIFI_OK;
}

kifi_status kifi_depthstream_next_frame_device(kifi_depthstream* s, void* depth_dev, float out_view[16],
                                               void* stream) {
    if (!s || !depth_dev) return fail(KIFI_ERR_INVALID_ARGUMENT, "null argument");
    int dev = 0;
    KIFI_CUDA(cudaGetDevice(&dev));
    if (s->device != dev) {  // (re)create the staging on the current device
        for (int k = 0; k < 2; ++k) {
            if (s->copied[k]) {
                KIFI_CUDA(cudaEventSynchronize(s->copied[k]));
                cudaEventDestroy(s->copied[k]);
                s->copied[k] = nullptr;
            }
            if (s->pinned[k]) cudaFreeHost(s->pinned[k]);
            s->pinned[k] = nullptr;
        }
        for (int k = 0; k < 2; ++k) {
            KIFI_CUDA(cudaHostAlloc(&s->pinned[k], s->texel_bytes(), cudaHostAllocDefault));
            KIFI_CUDA(cudaEventCreateWithFlags(&s->copied[k], cudaEventDisableTiming));
        }
        s->device = dev;
    }
    const int k = s->slot;
    KIFI_CUDA(cudaEventSynchronize(s->copied[k]));  // the copy out of this slot two frames ago
    kifi_status st = read_frame(s, s->pinned[k], out_view);
    if (st) return st;
    cudaStream_t cs = (cudaStream_t)stream;
    KIFI_CUDA(cudaMemcpyAsync(depth_dev, s->pinned[k], s->texel_bytes(), cudaMemcpyHostToDevice, cs));
    KIFI_CUDA(cudaEventRecord(s->copied[k], cs));
    s->slot = 1 - k;
    return KIFI_OK;
}

kifi_status kifi_mesh_to_obj(const float* verts, size_t n_verts, const uint32_t* indices, size_t n_indices,
                             const char* path) {
    if (!path || (n_verts && !verts) || (n_indices && !indices))
        return fail(KIFI_ERR_INVALID_ARGUMENT, "null argument");
    if (n_indices % 3) return fail(KIFI_ERR_INVALID_ARGUMENT, "index count not a multiple of 3");
    std::FILE* f = std::fopen(path, "w");
    if (!f) return fail(KIFI_ERR_IO, "cannot open the .obj file");
    bool ok = true;
    for (size_t i = 0; i < n_verts && ok; ++i)
        ok = std::fprintf(f, "v %f %f %f\n", verts[3 * i], verts[3 * i + 1], verts[3 * i + 2]) > 0;
    for (size_t i = 0; i < n_indices && ok; i += 3)
        ok = std::fprintf(f, "f %d %d %d\n", (int)(indices[i] + 1), (int)(indices[i + 1] + 1),
                          (int)(indices[i + 2] + 1)) > 0;
    ok = (std::fclose(f) == 0) && ok;
    return ok ? KIFI_OK : fail(KIFI_ERR_IO, "writing the .obj file failed");
}

kifi_status kifi_volume_save(kifi_volume* vol, const char* path) {
    if (!vol || !path) return fail(KIFI_ERR_INVALID_ARGUMENT, "null argument");
    size_t n = 0;
    kifi_status st = kifi_volume_size(vol, &n);
    if (st) return st;
    const int kbytes = vol->vb.key_bytes;
    std::vector<unsigned char> keys((n + 1) * kbytes);
    std::vector<float> values(2 * (n + 1));
    size_t got = 0;
    st = kbytes == 8 ? kifi_volume_export64(vol, (uint64_t*)keys.data(), values.data(), n + 1, &got)
                     : kifi_volume_export(vol, (uint32_t*)keys.data(), values.data(), n + 1, &got);
    if (st) return st;
    CheckpointHeader h{};
    std::memcpy(h.magic, kCheckpointMagic, 8);
    h.resolution = vol->g.res;
    h.side_length_m = vol->g.side;
    h.truncation_m = vol->g.trunc;
    h.key_bits = (uint32_t)(8 * kbytes);
    h.n_voxels = got;
    std::FILE* f = std::fopen(path, "wb");
    if (!f) return fail(KIFI_ERR_IO, "cannot open the checkpoint file");
    bool ok = std::fwrite(&h, sizeof h, 1, f) == 1 && std::fwrite(keys.data(), kbytes, got, f) == got &&
              std::fwrite(values.data(), 8, got, f) == got;
    ok = (std::fclose(f) == 0) && ok;
    return ok ? KIFI_OK : fail(KIFI_ERR_IO, "writing the checkpoint failed");
}

kifi_status kifi_volume_load(const char* path, int device, kifi_volume** out) {
    if (!path || !out) return fail(KIFI_ERR_INVALID_ARGUMENT, "null argument");
    *out = nullptr;
    std::FILE* f = std::fopen(path, "rb");
    if (!f) return fail(KIFI_ERR_IO, "cannot open the checkpoint file");
    CheckpointHeader h{};
    bool ok = read_exact(f, &h, sizeof h) && std::memcmp(h.magic, kCheckpointMagic, 8) == 0 &&
              h.n_voxels <= ((uint64_t)1 << 32) && (h.key_bits == 0 || h.key_bits == 32 || h.key_bits == 64) &&
              h.resolution >= 2 && h.resolution <= 8192 && !(h.resolution & (h.resolution - 1));
    const bool wide = h.key_bits == 64;
    std::vector<uint64_t> keys;
    std::vector<float> values;
    if (ok) {
        keys.resize(h.n_voxels);
        values.resize(2 * h.n_voxels);
        if (wide) {
            ok = read_exact(f, keys.data(), 8 * h.n_voxels);
        } else {
            std::vector<uint32_t> k32(h.n_voxels);
            ok = read_exact(f, k32.data(), 4 * h.n_voxels);
            for (size_t i = 0; ok && i < k32.size(); ++i) keys[i] = k32[i];
        }
        ok = ok && read_exact(f, values.data(), 8 * h.n_voxels);
    }
    std::fclose(f);
    if (!ok) return fail(KIFI_ERR_FORMAT, "not a volume checkpoint, or truncated");
    const uint64_t r = (uint64_t)h.resolution;
    int b = 10;
    if (wide)
        while ((1 << b) < h.resolution) ++b;
    const uint64_t mask = ((uint64_t)1 << b) - 1;
    for (size_t i = 0; ok && i < keys.size(); ++i) {
        const uint64_t k = keys[i];
        ok = (k & mask) < r && (k >> b & mask) < r && (k >> (2 * b)) < r;
        if (i) ok = ok && keys[i - 1] < k;
    }
    if (!ok) return fail(KIFI_ERR_FORMAT, "checkpoint keys not sorted, unique and inside the volume");
    kifi_volume_desc d{};
    d.resolution = h.resolution;
    d.side_length_m = h.side_length_m;
    d.truncation_m = h.truncation_m;
    d.initial_capacity = keys.size() + 1;
    d.device = device;
    d.key_bits = wide ? 64 : 32;
    kifi_volume* v = nullptr;
    kifi_status st = kifi_volume_create(&d, &v);
    if (st) return st;
    if (!keys.empty() && (st = kifi_volume_insert64(v, keys.data(), values.data(), keys.size()))) {
        kifi_volume_destroy(v);
        return st;
    }
    *out = v;
    return KIFI_OK;
}

}  // extern "C"
