// kifi_api.cu -- the C ABI of libkifi_gpu.so (include/kifi_gpu.h): volume
// handles, device memory and stream management, and the host side of
// Integrator::Integrate, flat_map::insert, Mesher::Mesh and
// util::radix_sort.  Host code only; every computation runs in the kernels
// of kifi_integrate.cu, kifi_sort.cu and kifi_mesh.cu.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <string>

#include "kifi_api_util.h"

using namespace kifi;

namespace kifi {
thread_local std::string g_last_error;

kifi_status fail(kifi_status s, const char* what) {
    g_last_error = what;
    return s;
}

kifi_status cuda_fail(cudaError_t e, const char* what) {
    g_last_error = std::string(what) + ": " + cudaGetErrorString(e);
    if (e == cudaErrorMemoryAllocation) return KIFI_ERR_OUT_OF_MEMORY;
    if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return KIFI_ERR_NO_DEVICE;
    return KIFI_ERR_CUDA;
}

void tracking_launch_shape(LaunchShape* ls) {
    ls->splat_ctas = ls->sms * 16;
    ls->sort_ctas = ls->sms * 16;
    ls->merge_ctas = ls->sms * 32;
    ls->beside_tracking = true;
}

kifi_status launch_shape(int device, LaunchShape* ls) {
    int sms = 0;
    KIFI_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    ls->sms = sms;
    ls->sort_ctas = sms * 4;
    ls->merge_ctas = sms * merge_blocks_per_sm();
    ls->splat_ctas = sms * 4;
    ls->beside_tracking = false;
    return KIFI_OK;
}

bool camera_ok(const kifi_camera* c) {
    return c && c->width > 0 && c->height > 0 && c->fx != 0.0f && c->fy != 0.0f &&
           (size_t)c->width * c->height <= (size_t)1 << 26;
}
}  // namespace kifi

namespace {

bool is_pow2(int x) { return x > 0 && !(x & (x - 1)); }

// voxels per axis at most: 13-bit key fields, a 2^39-bit occupancy bitmap
constexpr int kMaxResolution = 8192;

}  // namespace

namespace {

size_t vb_key_bytes(const VolumeBuffers& vb) { return (size_t)vb.key_bytes; }

void free_volume_buffers(VolumeBuffers& vb) {
    for (int i = 0; i < 2; ++i) {
        cudaFree(vb.keys[i]);
        cudaFree(vb.vals[i]);
        vb.keys[i] = nullptr;
        vb.vals[i] = nullptr;
    }
    cudaFree(vb.splits);
    vb.splits = nullptr;
}

size_t split_count(const VolumeBuffers& vb, size_t cap) { return merge_max_tiles(vb, cap) + 2; }

// Reads the device control block (waits for the stream).
kifi_status read_ctl(kifi_volume* v) {
    KIFI_CUDA(cudaMemcpyAsync(v->ctl_host, v->ctl, sizeof(DeviceCtl), cudaMemcpyDeviceToHost,
                              v->stream));
    KIFI_CUDA(cudaStreamSynchronize(v->stream));
    v->n_upper = (size_t)v->ctl_host->n[v->ctl_host->cur];
    return KIFI_OK;
}

// Turns device-raised status bits into a status code and clears them.
kifi_status take_device_status(kifi_volume* v) {
    unsigned int st = v->ctl_host->status;
    if (!st) return KIFI_OK;
    KIFI_CUDA(cudaMemsetAsync(&v->ctl->status, 0, sizeof(unsigned int), v->stream));
    if (st & KIFI_DEV_ERR_TIMEOUT) {
        // the frame was not merged, but its new keys' occupancy bits may have
        // been set: derive the bitmap from the resident keys again
        KIFI_CUDA(bitmap_rebuild_enqueue(v->ctl, v->g, v->vb, v->ls, v->stream));
        KIFI_CUDA(cudaStreamSynchronize(v->stream));
        return fail(KIFI_ERR_TIMEOUT, "a bounded device wait gave up; the frame was not fused");
    }
    KIFI_CUDA(cudaStreamSynchronize(v->stream));
    return fail(KIFI_ERR_CAPACITY, "volume capacity exceeded on the device");
}

kifi_status grow_volume(kifi_volume* v, size_t need) {
    if (need <= v->vb.cap) return KIFI_OK;
    kifi_status s = read_ctl(v);
    if (s) return s;
    size_t cap = v->vb.cap * 2;
    if (cap < need) cap = need;
    const unsigned int cur = v->ctl_host->cur;
    const size_t n = (size_t)v->ctl_host->n[cur];
    VolumeBuffers nb = v->vb;
    for (int i = 0; i < 2; ++i) {
        nb.keys[i] = nullptr;
        nb.vals[i] = nullptr;
    }
    nb.splits = nullptr;
    for (int i = 0; i < 2; ++i) {
        cudaError_t e1 = cudaMalloc(&nb.keys[i], (cap + kPad) * vb_key_bytes(v->vb));
        cudaError_t e2 = e1 ? e1 : cudaMalloc(&nb.vals[i], (cap + kPad) * sizeof(float2));
        if (e1 || e2) {
            free_volume_buffers(nb);
            return cuda_fail(e1 ? e1 : e2, "growing the volume");
        }
    }
    cudaError_t es = cudaMalloc(&nb.splits, split_count(v->vb, cap) * sizeof(unsigned long long));
    if (es) {
        free_volume_buffers(nb);
        return cuda_fail(es, "growing the volume");
    }
    KIFI_CUDA(cudaMemcpyAsync(nb.keys[cur], v->vb.keys[cur], n * vb_key_bytes(v->vb),
                              cudaMemcpyDeviceToDevice, v->stream));
    KIFI_CUDA(cudaMemcpyAsync(nb.vals[cur], v->vb.vals[cur], n * sizeof(float2),
                              cudaMemcpyDeviceToDevice, v->stream));
    KIFI_CUDA(cudaStreamSynchronize(v->stream));
    free_volume_buffers(v->vb);
    v->vb.keys[0] = nb.keys[0];
    v->vb.keys[1] = nb.keys[1];
    v->vb.vals[0] = nb.vals[0];
    v->vb.vals[1] = nb.vals[1];
    v->vb.splits = nb.splits;
    v->vb.cap = cap;
    return KIFI_OK;
}

// Room for `n_new` keys new to the volume per call (8 per pixel for frames).
kifi_status reserve_new(kifi_volume* v, size_t n_new) {
    if (n_new <= v->vb.new_cap) return KIFI_OK;
    KIFI_CUDA(cudaStreamSynchronize(v->stream));
    cudaFree(v->vb.new_keys);
    cudaFree(v->vb.new_idx);
    v->vb.new_keys = v->vb.new_idx = nullptr;
    v->vb.new_cap = 0;
    sort_scratch_free(&v->ss);
    KIFI_CUDA(cudaMalloc(&v->vb.new_keys, (n_new + kPad) * vb_key_bytes(v->vb)));
    KIFI_CUDA(cudaMalloc(&v->vb.new_idx, (n_new + kPad) * sizeof(uint32_t)));
    KIFI_CUDA(sort_scratch_alloc(&v->ss, n_new, v->stream));
    v->vb.new_cap = n_new;
    return KIFI_OK;
}

kifi_status reserve_depth(kifi_volume* v, size_t bytes) {
    if (bytes > v->depth_dev_bytes) {
        KIFI_CUDA(cudaStreamSynchronize(v->stream));
        cudaFree(v->depth_dev);
        v->depth_dev = nullptr;
        v->depth_dev_bytes = 0;
        KIFI_CUDA(cudaMalloc(&v->depth_dev, bytes));
        v->depth_dev_bytes = bytes;
    }
    return KIFI_OK;
}

kifi_status frame_prologue(kifi_volume* v, const kifi_camera* cam) {
    const size_t P = (size_t)cam->width * cam->height;
    kifi_status s = reserve_new(v, 8 * P);
    if (s) return s;
    if (v->n_upper + 8 * P > v->vb.cap) {
        if ((s = read_ctl(v))) return s;
        if (v->n_upper + 8 * P > v->vb.cap && (s = grow_volume(v, v->n_upper + 8 * P))) return s;
    }
    return KIFI_OK;
}

}  // namespace

kifi_status kifi_volume_prepare_frame(kifi_volume* v, const kifi_camera* cam) { return frame_prologue(v, cam); }

namespace {

// Host frame -> device: straight from page-locked memory, else staged
// through the volume's pinned buffer.
kifi_status upload_depth(kifi_volume* v, const void* src, size_t bytes) {
    kifi_status s = reserve_depth(v, bytes);
    if (s) return s;
    cudaPointerAttributes attr;
    bool pinned = cudaPointerGetAttributes(&attr, src) == cudaSuccess &&
                  (attr.type == cudaMemoryTypeHost);
    cudaGetLastError();
    if (!pinned) {
        if (bytes > v->depth_pinned_bytes) {
            KIFI_CUDA(cudaStreamSynchronize(v->stream));
            cudaFreeHost(v->depth_pinned);
            v->depth_pinned = nullptr;
            v->depth_pinned_bytes = 0;
            KIFI_CUDA(cudaMallocHost(&v->depth_pinned, bytes));
            v->depth_pinned_bytes = bytes;
        } else {
            // the previous frame's copy out of the staging buffer must be done
            KIFI_CUDA(cudaStreamSynchronize(v->stream));
        }
        std::memcpy(v->depth_pinned, src, bytes);
        src = v->depth_pinned;
    }
    KIFI_CUDA(cudaMemcpyAsync(v->depth_dev, src, bytes, cudaMemcpyHostToDevice, v->stream));
    return KIFI_OK;
}

kifi_status integrate_sync(kifi_volume* v, const void* host_depth, bool u16,
                           const kifi_camera* cam, const float* w2e) {
    if (!v || !host_depth || !camera_ok(cam) || !w2e)
        return fail(KIFI_ERR_INVALID_ARGUMENT, "integrate: bad argument");
    KIFI_CUDA(cudaSetDevice(v->device));
    kifi_status s = frame_prologue(v, cam);
    if (s) return s;
    const size_t bytes = (size_t)cam->width * cam->height * (u16 ? 2 : 4);
    if ((s = upload_depth(v, host_depth, bytes))) return s;
    if ((s = kifi_volume_enqueue_frame(v, v->depth_dev, u16, cam, w2e))) return s;
    if ((s = read_ctl(v))) return s;
    return take_device_status(v);
}

}  // namespace

kifi_status kifi_volume_enqueue_frame(kifi_volume* v, const void* depth_dev, bool u16,
                                      const kifi_camera* cam, const float* w2e) {
    cudaEvent_t* ev = nullptr;
    std::array<cudaEvent_t, kStageEvents> evs{};
    if (v->profiling) {
        for (int k = 0; k < kStageEvents; ++k) {
            if (v->event_pool.empty()) {
                cudaEvent_t e;
                KIFI_CUDA(cudaEventCreate(&e));
                v->event_pool.push_back(e);
            }
            evs[k] = v->event_pool.back();
            v->event_pool.pop_back();
        }
        ev = evs.data();
    }
    cudaError_t e = integrate_enqueue(v->ctl, v->g, v->vb, v->ss, depth_dev, u16, *cam,
                                      load_mat(w2e), v->ls, v->stream, ev);
    if (ev) v->pending.push_back(evs);
    if (e != cudaSuccess) return cuda_fail(e, "integrate");
    v->n_upper += 8 * (size_t)cam->width * cam->height;
    return KIFI_OK;
}

extern "C" {

const char* kifi_status_string(kifi_status s) {
    switch (s) {
        case KIFI_OK: return "ok";
        case KIFI_ERR_INVALID_ARGUMENT: return "invalid argument";
        case KIFI_ERR_OUT_OF_MEMORY: return "out of memory";
        case KIFI_ERR_CUDA: return "CUDA error";
        case KIFI_ERR_CAPACITY: return "capacity exceeded";
        case KIFI_ERR_TIMEOUT: return "device wait timed out";
        case KIFI_ERR_UNSUPPORTED: return "unsupported";
        case KIFI_ERR_NO_DEVICE: return "no CUDA device";
        case KIFI_ERR_IO: return "I/O error";
        case KIFI_ERR_FORMAT: return "bad file format";
        case KIFI_ERR_END_OF_STREAM: return "end of stream";
    }
    return "unknown status";
}

const char* kifi_last_error(void) { return g_last_error.c_str(); }

kifi_status kifi_device_count(int* count) {
    if (!count) return fail(KIFI_ERR_INVALID_ARGUMENT, "null count");
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess) {
        cudaGetLastError();
        n = 0;
    }
    *count = n;
    return KIFI_OK;
}

kifi_status kifi_volume_create(const kifi_volume_desc* d, kifi_volume** out) {
    if (!d || !out) return fail(KIFI_ERR_INVALID_ARGUMENT, "null argument");
    *out = nullptr;
    // Volume.cpp:22-26 (a power of two up to 1024 there: 30-bit keys); beyond
    // 1024 voxels per axis the volume keys voxels with 64 bits
    if (!(d->resolution >= 2 && d->resolution <= kMaxResolution && is_pow2(d->resolution)))
        return fail(KIFI_ERR_INVALID_ARGUMENT, "resolution must be a power of two in [2, 8192]");
    if (d->key_bits != 0 && d->key_bits != 32 && d->key_bits != 64)
        return fail(KIFI_ERR_INVALID_ARGUMENT, "key_bits must be 0, 32 or 64");
    if (d->key_bits == 32 && d->resolution > 1024)
        return fail(KIFI_ERR_INVALID_ARGUMENT, "32-bit keys hold at most 1024 voxels per axis");
    if (!(d->side_length_m > 0.0f) || !(d->truncation_m > 0.0f))
        return fail(KIFI_ERR_INVALID_ARGUMENT, "side length and truncation must be > 0");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return fail(KIFI_ERR_NO_DEVICE, "no CUDA device");
    }
    if (d->device < 0 || d->device >= ndev) return fail(KIFI_ERR_INVALID_ARGUMENT, "bad device");
    kifi_volume* v = new (std::nothrow) kifi_volume();
    if (!v) return fail(KIFI_ERR_OUT_OF_MEMORY, "host allocation");
    v->device = d->device;
    kifi_status s = KIFI_OK;
    auto bail = [&](kifi_status st) {
        kifi_volume_destroy(v);
        return st;
    };
    if (cudaSetDevice(v->device) != cudaSuccess) return bail(cuda_fail(cudaGetLastError(), "cudaSetDevice"));
    if (d->stream) {
        v->stream = (cudaStream_t)d->stream;
    } else {
        cudaError_t e = cudaStreamCreateWithFlags(&v->stream, cudaStreamNonBlocking);
        if (e) return bail(cuda_fail(e, "cudaStreamCreate"));
        v->own_stream = true;
    }
    v->g = make_geom(d->resolution, d->side_length_m, d->truncation_m);
    if (d->key_bits == 64 || d->resolution > 1024) {
        // b = max(10, log2 res): below 1024 voxels per axis the 64-bit key of a
        // voxel is the number the 30-bit key would be
        int b = 10;
        while ((1 << b) < d->resolution) ++b;
        v->g.kb = b;
        v->vb.key_bytes = 8;
    }
    if ((s = launch_shape(v->device, &v->ls))) return bail(s);
    cudaError_t e;
    if ((e = cudaMalloc(&v->ctl, sizeof(DeviceCtl)))) return bail(cuda_fail(e, "control block"));
    // zeroing on the volume's stream: the library's streams are non-blocking and would not wait
    // for a memset on the legacy default stream
    if ((e = cudaMemsetAsync(v->ctl, 0, sizeof(DeviceCtl), v->stream))) return bail(cuda_fail(e, "control block"));
    if ((e = cudaMallocHost(&v->ctl_host, sizeof(DeviceCtl)))) return bail(cuda_fail(e, "pinned"));
    std::memset(v->ctl_host, 0, sizeof(DeviceCtl));
    // the bitmap's 4x4x4 bricks need at least 4 voxels per axis
    const size_t r = d->resolution < 4 ? 4 : (size_t)d->resolution;
    v->vb.bitmap_words = (r * r * r + 31) / 32;
    if ((e = cudaMalloc(&v->vb.bitmap, v->vb.bitmap_words * 4))) return bail(cuda_fail(e, "bitmap"));
    if ((e = cudaMemsetAsync(v->vb.bitmap, 0, v->vb.bitmap_words * 4, v->stream))) return bail(cuda_fail(e, "bitmap"));
    size_t cap = d->initial_capacity;
    if (cap == 0) cap = r * r * r < ((size_t)1 << 22) ? r * r * r : ((size_t)1 << 22);
    for (int i = 0; i < 2; ++i) {
        if ((e = cudaMalloc(&v->vb.keys[i], (cap + kPad) * vb_key_bytes(v->vb))))
            return bail(cuda_fail(e, "volume keys"));
        if ((e = cudaMalloc(&v->vb.vals[i], (cap + kPad) * sizeof(float2))))
            return bail(cuda_fail(e, "volume values"));
    }
    if ((e = cudaMalloc(&v->vb.splits, split_count(v->vb, cap) * sizeof(unsigned long long))))
        return bail(cuda_fail(e, "merge splits"));
    v->vb.cap = cap;
    if ((s = reserve_new(v, 8 * 640 * 480))) return bail(s);
    *out = v;
    return KIFI_OK;
}

kifi_status kifi_volume_destroy(kifi_volume* v) {
    if (!v) return KIFI_OK;
    cudaSetDevice(v->device);
    if (v->stream) cudaStreamSynchronize(v->stream);
    free_volume_buffers(v->vb);
    cudaFree(v->vb.bitmap);
    cudaFree(v->vb.new_keys);
    cudaFree(v->vb.new_idx);
    sort_scratch_free(&v->ss);
    mesh_scratch_free(&v->ms);
    cudaFree(v->ctl);
    cudaFreeHost(v->ctl_host);
    cudaFree(v->depth_dev);
    cudaFreeHost(v->depth_pinned);
    cudaFree(v->mesh_verts);
    cudaFree(v->mesh_idx);
    for (auto e : v->event_pool) cudaEventDestroy(e);
    for (auto& ev : v->pending)
        for (auto e : ev) cudaEventDestroy(e);
    for (auto& ev : v->mesh_pending)
        for (auto e : ev) cudaEventDestroy(e);
    if (v->own_stream && v->stream) cudaStreamDestroy(v->stream);
    delete v;
    return KIFI_OK;
}

kifi_status kifi_volume_sync(kifi_volume* v) {
    if (!v) return fail(KIFI_ERR_INVALID_ARGUMENT, "null volume");
    KIFI_CUDA(cudaSetDevice(v->device));
    kifi_status s = read_ctl(v);
    if (s) return s;
    return take_device_status(v);
}

void* kifi_volume_stream(kifi_volume* v) { return v ? (void*)v->stream : nullptr; }

kifi_status kifi_volume_size(kifi_volume* v, size_t* n) {
    if (!v || !n) return fail(KIFI_ERR_INVALID_ARGUMENT, "null argument");
    kifi_status s = kifi_volume_sync(v);
    *n = v->n_upper;
    return s;
}

// Copies the resident keys to the host as `out_bytes`-wide numbers: a copy
// when the widths agree, a narrowing through a host buffer when a 64-bit
// volume's keys (b = 10) are read as 30-bit keys, a widening otherwise.
static kifi_status export_keys(kifi_volume* v, void* keys, int out_bytes, float* values, size_t capacity,
                               size_t* n) {
    if (!v || !n) return fail(KIFI_ERR_INVALID_ARGUMENT, "null argument");
    if (out_bytes == 4 && v->vb.key_bytes == 8 && v->g.kb != 10)
        return fail(KIFI_ERR_UNSUPPORTED, "keys of this volume need 64 bits (kifi_volume_export64)");
    kifi_status s = kifi_volume_sync(v);
    if (s) return s;
    const size_t cnt = v->n_upper;
    *n = cnt;
    if (cnt > capacity) return fail(KIFI_ERR_CAPACITY, "export buffer too small");
    if (cnt == 0) return KIFI_OK;
    const unsigned int cur = v->ctl_host->cur;
    std::vector<uint64_t> wide;
    std::vector<uint32_t> narrow;
    if (keys) {
        if (out_bytes == v->vb.key_bytes) {
            KIFI_CUDA(cudaMemcpyAsync(keys, v->vb.keys[cur], cnt * out_bytes, cudaMemcpyDeviceToHost, v->stream));
        } else if (out_bytes == 4) {
            wide.resize(cnt);
            KIFI_CUDA(cudaMemcpyAsync(wide.data(), v->vb.keys[cur], cnt * 8, cudaMemcpyDeviceToHost, v->stream));
        } else {
            narrow.resize(cnt);
            KIFI_CUDA(cudaMemcpyAsync(narrow.data(), v->vb.keys[cur], cnt * 4, cudaMemcpyDeviceToHost, v->stream));
        }
    }
    if (values)
        KIFI_CUDA(cudaMemcpyAsync(values, v->vb.vals[cur], cnt * 8, cudaMemcpyDeviceToHost, v->stream));
    KIFI_CUDA(cudaStreamSynchronize(v->stream));
    for (size_t i = 0; i < wide.size(); ++i) ((uint32_t*)keys)[i] = (uint32_t)wide[i];
    for (size_t i = 0; i < narrow.size(); ++i) ((uint64_t*)keys)[i] = narrow[i];
    return KIFI_OK;
}

kifi_status kifi_volume_export(kifi_volume* v, uint32_t* keys, float* values, size_t capacity, size_t* n) {
    return export_keys(v, keys, 4, values, capacity, n);
}

kifi_status kifi_volume_export64(kifi_volume* v, uint64_t* keys, float* values, size_t capacity, size_t* n) {
    return export_keys(v, keys, 8, values, capacity, n);
}

kifi_status kifi_volume_key_bits(kifi_volume* v, int* key_bits, int* bits_per_axis) {
    if (!v) return fail(KIFI_ERR_INVALID_ARGUMENT, "null volume");
    if (key_bits) *key_bits = v->vb.key_bytes * 8;
    if (bits_per_axis) *bits_per_axis = v->g.kb;
    return KIFI_OK;
}

kifi_status kifi_volume_clear(kifi_volume* v) {
    if (!v) return fail(KIFI_ERR_INVALID_ARGUMENT, "null volume");
    KIFI_CUDA(cudaSetDevice(v->device));
    KIFI_CUDA(cudaMemsetAsync(v->vb.bitmap, 0, v->vb.bitmap_words * 4, v->stream));
    KIFI_CUDA(cudaMemsetAsync(v->ctl, 0, sizeof(DeviceCtl), v->stream));
    KIFI_CUDA(cudaStreamSynchronize(v->stream));
    v->n_upper = 0;
    return KIFI_OK;
}

kifi_status kifi_volume_reserve(kifi_volume* v, size_t capacity) {
    if (!v) return fail(KIFI_ERR_INVALID_ARGUMENT, "null volume");
    KIFI_CUDA(cudaSetDevice(v->device));
    return grow_volume(v, capacity);
}

// flat_map::insert of n sorted unique keys given `in_bytes` wide.
static kifi_status insert_keys(kifi_volume* v, const void* keys_in, int in_bytes, const float* values, size_t n) {
    if (!v || (n && !keys_in)) return fail(KIFI_ERR_INVALID_ARGUMENT, "null argument");
    if (n == 0) return KIFI_OK;
    if (n >= ((size_t)1 << 30)) return fail(KIFI_ERR_INVALID_ARGUMENT, "too many keys");
    const uint32_t res = (uint32_t)v->g.res;
    const int b = in_bytes == 4 ? 10 : v->g.kb;
    const uint64_t mask = ((uint64_t)1 << b) - 1;
    // keys in the volume's width (the 64-bit key of a 30-bit key is the same number when b = 10)
    std::vector<unsigned char> conv;
    const void* src = keys_in;
    if (in_bytes != v->vb.key_bytes) {
        if (v->g.kb != 10) return fail(KIFI_ERR_UNSUPPORTED, "keys of this volume need 64 bits (kifi_volume_insert64)");
        conv.resize(n * v->vb.key_bytes);
        for (size_t i = 0; i < n; ++i) {
            if (in_bytes == 4) ((uint64_t*)conv.data())[i] = ((const uint32_t*)keys_in)[i];
            else ((uint32_t*)conv.data())[i] = (uint32_t)((const uint64_t*)keys_in)[i];
        }
        src = conv.data();
    }
    for (size_t i = 0; i < n; ++i) {
        const uint64_t k = in_bytes == 4 ? (uint64_t)((const uint32_t*)keys_in)[i] : ((const uint64_t*)keys_in)[i];
        const uint64_t prev =
            i ? (in_bytes == 4 ? (uint64_t)((const uint32_t*)keys_in)[i - 1] : ((const uint64_t*)keys_in)[i - 1]) : 0;
        if (k >> (3 * b) || (k & mask) >= res || (k >> b & mask) >= res || (k >> (2 * b)) >= res)
            return fail(KIFI_ERR_INVALID_ARGUMENT, "key outside the volume");
        if (i && prev >= k) return fail(KIFI_ERR_INVALID_ARGUMENT, "keys not sorted/unique");
    }
    KIFI_CUDA(cudaSetDevice(v->device));
    kifi_status s = reserve_new(v, n);
    if (s) return s;
    if ((s = read_ctl(v))) return s;
    if ((s = grow_volume(v, v->n_upper + n))) return s;
    const size_t kbytes = (size_t)v->vb.key_bytes;
    void* dk = nullptr;
    float2* dv = nullptr;
    unsigned int* dn = nullptr;
    auto cleanup = [&]() {
        cudaFree(dk);
        cudaFree(dv);
        cudaFree(dn);
    };
    cudaError_t e = cudaMalloc(&dk, n * kbytes);
    if (!e && values) e = cudaMalloc(&dv, n * 8);
    if (!e) e = cudaMalloc(&dn, 4);
    if (e) {
        cleanup();
        return cuda_fail(e, "insert staging");
    }
    const unsigned int n32 = (unsigned int)n;
    e = cudaMemcpyAsync(dk, src, n * kbytes, cudaMemcpyHostToDevice, v->stream);
    if (!e && values) e = cudaMemcpyAsync(dv, values, n * 8, cudaMemcpyHostToDevice, v->stream);
    if (!e) e = cudaMemcpyAsync(dn, &n32, 4, cudaMemcpyHostToDevice, v->stream);
    if (!e) e = insert_filter_enqueue(v->ctl, v->g, v->vb, dk, dn, v->ls, v->stream);
    if (!e) e = sort_keys(v->vb.new_keys, v->vb.key_bytes, 3 * v->g.kb, v->vb.new_idx, &v->ctl->n_new, v->ss,
                          &v->ctl->status, v->ls.sort_ctas, v->stream);
    if (!e) e = insert_merge_enqueue(v->ctl, v->g, v->vb, dv, v->ls, v->stream);
    if (!e) e = cudaStreamSynchronize(v->stream);
    cleanup();
    if (e) return cuda_fail(e, "insert");
    if ((s = read_ctl(v))) return s;
    return take_device_status(v);
}

kifi_status kifi_volume_insert(kifi_volume* v, const uint32_t* keys, const float* values, size_t n) {
    return insert_keys(v, keys, 4, values, n);
}

kifi_status kifi_volume_insert64(kifi_volume* v, const uint64_t* keys, const float* values, size_t n) {
    return insert_keys(v, keys, 8, values, n);
}

kifi_status kifi_integrate_f32(kifi_volume* v, const float* depth_m, const kifi_camera* cam,
                               const float world_to_eye[16]) {
    return integrate_sync(v, depth_m, false, cam, world_to_eye);
}

kifi_status kifi_integrate_u16(kifi_volume* v, const uint16_t* depth_mm, const kifi_camera* cam,
                               const float world_to_eye[16]) {
    return integrate_sync(v, depth_mm, true, cam, world_to_eye);
}

kifi_status kifi_integrate_device(kifi_volume* v, const void* depth_dev, int depth_is_u16,
                                  const kifi_camera* cam, const float world_to_eye[16]) {
    if (!v || !depth_dev || !camera_ok(cam) || !world_to_eye)
        return fail(KIFI_ERR_INVALID_ARGUMENT, "integrate: bad argument");
    KIFI_CUDA(cudaSetDevice(v->device));
    kifi_status s = frame_prologue(v, cam);
    if (s) return s;
    return kifi_volume_enqueue_frame(v, depth_dev, depth_is_u16 != 0, cam, world_to_eye);
}

kifi_status kifi_volume_set_launch_mode(kifi_volume* v, int beside_tracking) {
    if (!v) return fail(KIFI_ERR_INVALID_ARGUMENT, "null volume");
    KIFI_CUDA(cudaSetDevice(v->device));
    kifi_status s = launch_shape(v->device, &v->ls);
    if (s) return s;
    if (beside_tracking) tracking_launch_shape(&v->ls);
    return KIFI_OK;
}

kifi_status kifi_volume_set_profiling(kifi_volume* v, int on) {
    if (!v) return fail(KIFI_ERR_INVALID_ARGUMENT, "null volume");
    v->profiling = on != 0;
    return KIFI_OK;
}

kifi_status kifi_volume_stage_times(kifi_volume* v, double out_ms[4], int* frames) {
    if (!v || !out_ms) return fail(KIFI_ERR_INVALID_ARGUMENT, "null argument");
    KIFI_CUDA(cudaSetDevice(v->device));
    for (int k = 0; k < kStageEvents - 1; ++k) out_ms[k] = 0.0;
    const int n = (int)v->pending.size();
    for (auto& ev : v->pending) {
        KIFI_CUDA(cudaEventSynchronize(ev[kStageEvents - 1]));
        for (int k = 0; k < kStageEvents - 1; ++k) {
            float ms = 0.0f;
            KIFI_CUDA(cudaEventElapsedTime(&ms, ev[k], ev[k + 1]));
            out_ms[k] += ms;
        }
        for (int k = 0; k < kStageEvents; ++k) v->event_pool.push_back(ev[k]);
    }
    v->pending.clear();
    if (frames) *frames = n;
    return KIFI_OK;
}

kifi_status kifi_volume_frame_log(kifi_volume* v, uint64_t* n_before, uint64_t* n_new,
                                  uint64_t* n_after, int capacity, int* count) {
    if (!v || !count) return fail(KIFI_ERR_INVALID_ARGUMENT, "null argument");
    kifi_status s = kifi_volume_sync(v);
    if (s) return s;
    const DeviceCtl* h = v->ctl_host;
    const unsigned long long total = h->frames;
    int n = (int)(total < (unsigned long long)kFrameLog ? total : kFrameLog);
    if (n > capacity) n = capacity;
    for (int i = 0; i < n; ++i) {
        const unsigned int slot = (unsigned int)((total - n + i) % kFrameLog);
        if (n_before) n_before[i] = h->log_n0[slot];
        if (n_new) n_new[i] = h->log_new[slot];
        if (n_after) n_after[i] = h->log_n1[slot];
    }
    *count = n;
    return KIFI_OK;
}

// Meshes into the volume's device buffers; returns the counts.  The
// counting passes and the emission run back to back (the emission reads the
// counts on the device); when the buffers turn out too small, they are grown
// to the counts and the emission runs again.
static kifi_status mesh_to_device(kifi_volume* v, int with_indices, size_t* n_verts,
                                  size_t* n_indices) {
    *n_verts = *n_indices = 0;
    kifi_status s = kifi_volume_sync(v);
    if (s) return s;
    const size_t n = v->n_upper;
    if (n < 2) return KIFI_OK;  // the reference's loop starts at size-2
    if (n >= ((size_t)1 << 28)) return fail(KIFI_ERR_UNSUPPORTED, "mesh of more than 2^28 voxels");
    const unsigned int cur = v->ctl_host->cur;
    KIFI_CUDA(mesh_scratch_reserve(&v->ms, n, v->g.kb));
    const unsigned int n32 = (unsigned int)n;
    KIFI_CUDA(cudaMemcpyAsync(v->ms.n_dev, &n32, sizeof n32, cudaMemcpyHostToDevice, v->stream));
    std::array<cudaEvent_t, 5> ev{};
    if (v->profiling) {
        for (int k = 0; k < 5; ++k) {
            if (v->event_pool.empty()) {
                cudaEvent_t e;
                KIFI_CUDA(cudaEventCreate(&e));
                v->event_pool.push_back(e);
            }
            ev[k] = v->event_pool.back();
            v->event_pool.pop_back();
        }
        KIFI_CUDA(cudaEventRecord(ev[0], v->stream));
    }
    KIFI_CUDA(mesh_count_enqueue(v->vb.keys[cur], v->vb.key_bytes, v->vb.vals[cur], n, v->g.kb,
                                 with_indices ? 1 : 0, v->ms, v->ls.sms, v->stream, ev[0] ? &ev[1] : nullptr));
    if (ev[0]) KIFI_CUDA(cudaEventRecord(ev[3], v->stream));
    MeshCounts* mc = &v->ctl_host_mesh;
    for (int attempt = 0; attempt < 2; ++attempt) {
        KIFI_CUDA(mesh_emit_enqueue(v->g, v->vb.keys[cur], v->vb.key_bytes, v->vb.vals[cur], n,
                                    with_indices ? 1 : 0, v->ms, v->mesh_verts_cap, v->mesh_idx_cap, v->mesh_verts,
                                    v->mesh_idx, v->ls.sms, v->stream));
        if (attempt == 0 && ev[0]) {
            KIFI_CUDA(cudaEventRecord(ev[4], v->stream));
            v->mesh_pending.push_back(ev);
        }
        KIFI_CUDA(cudaMemcpyAsync(mc, v->ms.counts, sizeof(MeshCounts), cudaMemcpyDeviceToHost, v->stream));
        KIFI_CUDA(cudaStreamSynchronize(v->stream));
        if (mc->error) return fail(KIFI_ERR_TIMEOUT, "mesh classification: a bounded wait gave up");
        if (!mc->overflow) break;
        if (attempt == 1) return fail(KIFI_ERR_CUDA, "mesh emission overflowed buffers sized to its counts");
        const size_t nv = (size_t)mc->n_verts, ni = with_indices ? (size_t)mc->n_idx : 0;
        if (nv > v->mesh_verts_cap) {
            cudaFree(v->mesh_verts);
            v->mesh_verts = nullptr;
            v->mesh_verts_cap = 0;
            KIFI_CUDA(cudaMalloc(&v->mesh_verts, (nv + kPad) * 12));
            v->mesh_verts_cap = nv;
        }
        if (ni > v->mesh_idx_cap) {
            cudaFree(v->mesh_idx);
            v->mesh_idx = nullptr;
            v->mesh_idx_cap = 0;
            KIFI_CUDA(cudaMalloc(&v->mesh_idx, (ni + kPad) * 4));
            v->mesh_idx_cap = ni;
        }
    }
    *n_verts = (size_t)mc->n_verts;
    *n_indices = with_indices ? (size_t)mc->n_idx : 0;
    v->mesh_counts_valid = true;
    return KIFI_OK;
}

kifi_status kifi_volume_mesh_stage_times(kifi_volume* v, double out_ms[5], int* meshes) {
    if (!v || !out_ms) return fail(KIFI_ERR_INVALID_ARGUMENT, "null argument");
    KIFI_CUDA(cudaSetDevice(v->device));
    double sum[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    const int n = (int)v->mesh_pending.size();
    for (auto& ev : v->mesh_pending) {
        KIFI_CUDA(cudaEventSynchronize(ev[4]));
        for (int k = 0; k < 4; ++k) {
            float ms = 0.0f;
            KIFI_CUDA(cudaEventElapsedTime(&ms, ev[k], ev[k + 1]));
            sum[k] += ms;
            sum[4] += ms;
        }
        for (int k = 0; k < 5; ++k) v->event_pool.push_back(ev[k]);
    }
    v->mesh_pending.clear();
    for (int k = 0; k < 5; ++k) out_ms[k] = n ? sum[k] / n : 0.0;
    if (meshes) *meshes = n;
    return KIFI_OK;
}

kifi_status kifi_volume_mesh_times(kifi_volume* v, double* out_ms, int* meshes) {
    if (!v || !out_ms) return fail(KIFI_ERR_INVALID_ARGUMENT, "null argument");
    double st[5];
    kifi_status s = kifi_volume_mesh_stage_times(v, st, meshes);
    *out_ms = st[4];
    return s;
}

kifi_status kifi_mesh(kifi_volume* v, int with_indices, float* verts, size_t vert_capacity,
                      uint32_t* indices, size_t index_capacity, size_t* n_verts,
                      size_t* n_indices) {
    if (!v || !n_verts || !n_indices) return fail(KIFI_ERR_INVALID_ARGUMENT, "null argument");
    KIFI_CUDA(cudaSetDevice(v->device));
    size_t nv = 0, ni = 0;
    kifi_status s = mesh_to_device(v, with_indices, &nv, &ni);
    *n_verts = nv;
    *n_indices = ni;
    if (s) return s;
    if (nv > vert_capacity || ni > index_capacity || (nv && !verts) || (ni && !indices))
        return fail(KIFI_ERR_CAPACITY, "mesh output buffers too small");
    if (nv)
        KIFI_CUDA(cudaMemcpyAsync(verts, v->mesh_verts, nv * 12, cudaMemcpyDeviceToHost, v->stream));
    if (ni)
        KIFI_CUDA(cudaMemcpyAsync(indices, v->mesh_idx, ni * 4, cudaMemcpyDeviceToHost, v->stream));
    KIFI_CUDA(cudaStreamSynchronize(v->stream));
    return KIFI_OK;
}

kifi_status kifi_mesh_device(kifi_volume* v, int with_indices, size_t* n_verts, size_t* n_indices,
                             const float** verts_dev, const uint32_t** indices_dev) {
    if (!v || !n_verts || !n_indices) return fail(KIFI_ERR_INVALID_ARGUMENT, "null argument");
    KIFI_CUDA(cudaSetDevice(v->device));
    kifi_status s = mesh_to_device(v, with_indices, n_verts, n_indices);
    if (s) return s;
    if (verts_dev) *verts_dev = v->mesh_verts;
    if (indices_dev) *indices_dev = v->mesh_idx;
    return KIFI_OK;
}

// keys of key_bytes (4 or 8) bytes, all bits significant
static kifi_status radix_sort_host(void* keys, int key_bytes, uint32_t* values, size_t n) {
    if (n == 0) return KIFI_OK;
    if (!keys) return fail(KIFI_ERR_INVALID_ARGUMENT, "null keys");
    if (n >= ((size_t)1 << 30)) return fail(KIFI_ERR_UNSUPPORTED, "sort of 2^30 or more keys");
    int dev = 0;
    KIFI_CUDA(cudaGetDevice(&dev));
    LaunchShape ls;
    kifi_status s = launch_shape(dev, &ls);
    if (s) return s;
    cudaStream_t st;
    KIFI_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    SortScratch ss;
    void* dk = nullptr;
    uint32_t* dv = nullptr;
    unsigned int *dn = nullptr, *dstatus = nullptr;
    const unsigned int n32 = (unsigned int)n;
    const size_t kb = (size_t)key_bytes;
    unsigned int status = 0;
    cudaError_t e = sort_scratch_alloc(&ss, n, st);
    if (!e) e = cudaMalloc(&dk, (n + kPad) * kb);
    if (!e && values) e = cudaMalloc(&dv, (n + kPad) * 4);
    if (!e) e = cudaMalloc(&dn, 4);
    if (!e) e = cudaMalloc(&dstatus, 4);
    if (!e) e = cudaMemsetAsync(dstatus, 0, 4, st);
    if (!e) e = cudaMemcpyAsync(dk, keys, n * kb, cudaMemcpyHostToDevice, st);
    if (!e && values) e = cudaMemcpyAsync(dv, values, n * 4, cudaMemcpyHostToDevice, st);
    if (!e) e = cudaMemcpyAsync(dn, &n32, 4, cudaMemcpyHostToDevice, st);
    if (!e) e = sort_keys(dk, key_bytes, 8 * key_bytes, dv, dn, ss, dstatus, ls.sort_ctas, st);
    if (!e) e = cudaMemcpyAsync(keys, dk, n * kb, cudaMemcpyDeviceToHost, st);
    if (!e && values) e = cudaMemcpyAsync(values, dv, n * 4, cudaMemcpyDeviceToHost, st);
    if (!e) e = cudaMemcpyAsync(&status, dstatus, 4, cudaMemcpyDeviceToHost, st);
    if (!e) e = cudaStreamSynchronize(st);
    sort_scratch_free(&ss);
    cudaFree(dk);
    cudaFree(dv);
    cudaFree(dn);
    cudaFree(dstatus);
    cudaStreamDestroy(st);
    if (e) return cuda_fail(e, "radix sort");
    if (status) return fail(KIFI_ERR_TIMEOUT, "radix sort look-back gave up");
    return KIFI_OK;
}

kifi_status kifi_radix_sort_u32(uint32_t* keys, size_t n) { return radix_sort_host(keys, 4, nullptr, n); }

kifi_status kifi_radix_sort_pairs_u32(uint32_t* keys, uint32_t* values, size_t n) {
    if (n && !values) return fail(KIFI_ERR_INVALID_ARGUMENT, "null values");
    return radix_sort_host(keys, 4, values, n);
}

kifi_status kifi_radix_sort_u64(uint64_t* keys, size_t n) { return radix_sort_host(keys, 8, nullptr, n); }

kifi_status kifi_radix_sort_pairs_u64(uint64_t* keys, uint32_t* values, size_t n) {
    if (n && !values) return fail(KIFI_ERR_INVALID_ARGUMENT, "null values");
    return radix_sort_host(keys, 8, values, n);
}

}  // extern "C"
