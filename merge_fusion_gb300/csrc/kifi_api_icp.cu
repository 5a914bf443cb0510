// kifi_api_icp.cu -- C ABI of the ICP context and of Renderer::Bin
// (include/kifi_gpu.h).  Host code; the kernels live in kifi_icp.cu.
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstring>
#include <new>

#include "kifi_api_util.h"

using namespace kifi;

struct kifi_icp {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    LaunchShape ls{};
    IcpState* st = nullptr;
    void* depth_dev = nullptr;
    size_t depth_bytes = 0;
    float4* synth = nullptr;  // target in the association's float4 layout
    size_t synth_cap = 0;     // bytes
    void* staging = nullptr;  // host float3 targets on their way in
    size_t staging_cap = 0;
    int sw = 0, sh = 0;
    Mat4 synth_e2w{};
    bool have_target = false;
    int last_iters = 0;
    IcpState* head = nullptr;        // pinned host copy of the state's head (poses, statistics)
    bool record = false;             // keep the last iteration's association
    long long* pairs = nullptr;      // per source: target index, or -1
    float* pairs_len2 = nullptr;     // per source: len^2
    size_t pairs_cap = 0, pairs_n = 0;
    void* zbuf = nullptr;            // Bin's z-buffer (8 bytes per target pixel)
    size_t zbuf_cap = 0;
    IcpPoseMail* mail = nullptr;     // page-locked, mapped: the last step's pose ...
    IcpPoseMail* mail_dev = nullptr; // ... its device address
    unsigned long long mail_seq = 0; // ... and the number of the latest alignment
    bool publish = false;            // alignments publish their pose (icp_publish_pose)
};

namespace {

int icp_ctas(const kifi_icp* c, size_t n_src) {
    size_t b = (n_src + 7) / 8;  // association: one warp per source, 8 warps per CTA
    size_t cap = (size_t)c->ls.sms * 8;
    if (cap > (size_t)kIcpMaxCtas) cap = kIcpMaxCtas;
    return (int)(b < 1 ? 1 : (b > cap ? cap : b));
}

kifi_status reserve_bytes(void** p, size_t* cap, size_t bytes, cudaStream_t st) {
    if (bytes <= *cap) return KIFI_OK;
    KIFI_CUDA(cudaStreamSynchronize(st));
    cudaFree(*p);
    *p = nullptr;
    *cap = 0;
    KIFI_CUDA(cudaMalloc(p, bytes));
    *cap = bytes;
    return KIFI_OK;
}

kifi_status reserve_target(kifi_icp* c, int w, int h) {
    return reserve_bytes((void**)&c->synth, &c->synth_cap, (size_t)w * h * sizeof(float4), c->stream);
}

kifi_status enqueue_align(kifi_icp* c, const void* depth_dev, bool u16, const kifi_camera* cam,
                          const float* guess, int iterations) {
    if (!c->have_target) return fail(KIFI_ERR_INVALID_ARGUMENT, "ICP target not set");
    if (iterations < 0 || iterations > kIcpMaxStats)
        return fail(KIFI_ERR_INVALID_ARGUMENT, "iterations must be in [0, 64]");
    const size_t n_src = (size_t)((cam->width + 3) / 4) * cam->height;
    IcpArgs a{};
    a.depth = depth_dev;
    a.depth_u16 = u16 ? 1 : 0;
    a.width = cam->width;
    a.height = cam->height;
    // ICP.cpp:48-57: flInv, ppOverFl, and EyeToClipRH * inverse(synth pose)
    a.fl_inv_x = fdiv(1.0f, cam->fx);
    a.fl_inv_y = fdiv(1.0f, cam->fy);
    a.pp_x = fmul(fsub(0.5f, cam->cx), a.fl_inv_x);
    a.pp_y = fmul(fsub(cam->cy, 0.5f), a.fl_inv_y);
    Mat4 proj = mat_mul(eye_to_clip(*cam), invert_transform(c->synth_e2w));
    std::memcpy(a.proj, proj.m, 64);
    a.synth = c->synth;
    a.synth_w = c->sw;
    a.synth_h = c->sh;
    a.neg_zero = -0.0f;
    if (c->record) {
        if (n_src > c->pairs_cap) {
            KIFI_CUDA(cudaStreamSynchronize(c->stream));
            cudaFree(c->pairs);
            cudaFree(c->pairs_len2);
            c->pairs = nullptr;
            c->pairs_len2 = nullptr;
            c->pairs_cap = 0;
            KIFI_CUDA(cudaMalloc(&c->pairs, n_src * sizeof(long long)));
            KIFI_CUDA(cudaMalloc(&c->pairs_len2, n_src * sizeof(float)));
            c->pairs_cap = n_src;
        }
        a.pairs = c->pairs;
        a.pairs_len2 = c->pairs_len2;
        c->pairs_n = n_src;
    }
    if (c->publish) ++c->mail_seq;
    KIFI_CUDA(icp_align_enqueue(a, c->st, load_mat(guess), iterations, icp_ctas(c, n_src),
                                c->stream, c->publish ? c->mail_dev : nullptr, c->mail_seq));
    c->last_iters = iterations;
    return KIFI_OK;
}

}  // namespace

// The arguments of one frame pair's alignment for a batched launch (the
// single-pair path's IcpArgs, without association recording).
kifi_status kifi_icp_batch_args(kifi_icp* c, const void* depth_dev, const kifi_camera* cam, IcpArgs* a,
                                IcpState** st, int iterations) {
    if (!c->have_target) return fail(KIFI_ERR_INVALID_ARGUMENT, "ICP target not set");
    *a = IcpArgs{};
    a->depth = depth_dev;
    a->depth_u16 = 1;
    a->width = cam->width;
    a->height = cam->height;
    a->fl_inv_x = fdiv(1.0f, cam->fx);
    a->fl_inv_y = fdiv(1.0f, cam->fy);
    a->pp_x = fmul(fsub(0.5f, cam->cx), a->fl_inv_x);
    a->pp_y = fmul(fsub(cam->cy, 0.5f), a->fl_inv_y);
    const Mat4 proj = mat_mul(eye_to_clip(*cam), invert_transform(c->synth_e2w));
    std::memcpy(a->proj, proj.m, 64);
    a->synth = c->synth;
    a->synth_w = c->sw;
    a->synth_h = c->sh;
    a->neg_zero = -0.0f;
    *st = c->st;
    c->last_iters = iterations;
    return KIFI_OK;
}

// Room for a target of the camera's size; records that the next target is
// this frame's back-projection (written by a batched launch) and returns
// where it goes.
kifi_status kifi_icp_batch_target(kifi_icp* c, const kifi_camera* cam, const float* eye_to_world, float4** out) {
    kifi_status s = reserve_target(c, cam->width, cam->height);
    if (s) return s;
    c->sw = cam->width;
    c->sh = cam->height;
    c->synth_e2w = load_mat(eye_to_world);
    c->have_target = true;
    *out = c->synth;
    return KIFI_OK;
}

// Everything an alignment against a target of the camera's size may need to
// allocate, done ahead (outside any stream capture).
kifi_status kifi_icp_prepare_frame(kifi_icp* c, const kifi_camera* cam) {
    return reserve_target(c, cam->width, cam->height);
}

extern "C" {

kifi_status kifi_icp_create(int device, void* stream, kifi_icp** out) {
    if (!out) return fail(KIFI_ERR_INVALID_ARGUMENT, "null argument");
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return fail(KIFI_ERR_NO_DEVICE, "no CUDA device");
    }
    if (device < 0 || device >= ndev) return fail(KIFI_ERR_INVALID_ARGUMENT, "bad device");
    kifi_icp* c = new (std::nothrow) kifi_icp();
    if (!c) return fail(KIFI_ERR_OUT_OF_MEMORY, "host allocation");
    c->device = device;
    kifi_status s;
    cudaError_t e = cudaSetDevice(device);
    if (!e) {
        if (stream) c->stream = (cudaStream_t)stream;
        else {
            // the highest priority: tracking is the pipeline's critical path,
            // and its CTAs are placed ahead of pending fusion CTAs
            int lowest = 0, greatest = 0;
            e = cudaDeviceGetStreamPriorityRange(&lowest, &greatest);
            if (!e) e = cudaStreamCreateWithPriority(&c->stream, cudaStreamNonBlocking, greatest);
            c->own_stream = !e;
        }
    }
    if (!e) e = cudaMalloc(&c->st, sizeof(IcpState));
    if (!e) e = cudaMallocHost(&c->head, offsetof(IcpState, part));
    if (!e) e = cudaHostAlloc((void**)&c->mail, sizeof(IcpPoseMail), cudaHostAllocMapped);
    if (!e) {
        c->mail->seq = 0;
        e = cudaHostGetDevicePointer((void**)&c->mail_dev, c->mail, 0);
    }
    if (!e) e = cudaMemsetAsync(c->st, 0, sizeof(IcpState), c->stream);  // ordered before the context's work
    if (e) {
        kifi_icp_destroy(c);
        return cuda_fail(e, "ICP context");
    }
    if ((s = launch_shape(device, &c->ls))) {
        kifi_icp_destroy(c);
        return s;
    }
    if ((e = icp_init_device())) {
        kifi_icp_destroy(c);
        return cuda_fail(e, "ICP kernel attributes");
    }
    *out = c;
    return KIFI_OK;
}

kifi_status kifi_icp_destroy(kifi_icp* c) {
    if (!c) return KIFI_OK;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    cudaFree(c->st);
    cudaFreeHost(c->head);
    cudaFreeHost(c->mail);
    cudaFree(c->depth_dev);
    cudaFree(c->synth);
    cudaFree(c->pairs);
    cudaFree(c->pairs_len2);
    cudaFree(c->staging);
    cudaFree(c->zbuf);
    if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return KIFI_OK;
}

void* kifi_icp_stream(kifi_icp* c) { return c ? (void*)c->stream : nullptr; }

kifi_status kifi_icp_record_associations(kifi_icp* c, int on) {
    if (!c) return fail(KIFI_ERR_INVALID_ARGUMENT, "null ICP");
    c->record = on != 0;
    return KIFI_OK;
}

kifi_status kifi_icp_associations(kifi_icp* c, int64_t* target_index, float* len2, size_t capacity, size_t* n) {
    if (!c || !n) return fail(KIFI_ERR_INVALID_ARGUMENT, "null argument");
    KIFI_CUDA(cudaSetDevice(c->device));
    *n = c->pairs_n;
    if (c->pairs_n > capacity) return fail(KIFI_ERR_CAPACITY, "association buffers too small");
    if (c->pairs_n) {
        if (target_index)
            KIFI_CUDA(cudaMemcpyAsync(target_index, c->pairs, c->pairs_n * 8, cudaMemcpyDeviceToHost, c->stream));
        if (len2) KIFI_CUDA(cudaMemcpyAsync(len2, c->pairs_len2, c->pairs_n * 4, cudaMemcpyDeviceToHost, c->stream));
    }
    KIFI_CUDA(cudaStreamSynchronize(c->stream));
    return KIFI_OK;
}

kifi_status kifi_icp_set_target(kifi_icp* c, const float* points, int width, int height,
                                const float synth_eye_to_world[16]) {
    if (!c || !points || width <= 0 || height <= 0 || !synth_eye_to_world)
        return fail(KIFI_ERR_INVALID_ARGUMENT, "bad argument");
    KIFI_CUDA(cudaSetDevice(c->device));
    kifi_status s = reserve_target(c, width, height);
    if (s) return s;
    const size_t bytes = (size_t)width * height * 12;
    if ((s = reserve_bytes(&c->staging, &c->staging_cap, bytes, c->stream))) return s;
    KIFI_CUDA(cudaMemcpyAsync(c->staging, points, bytes, cudaMemcpyHostToDevice, c->stream));
    KIFI_CUDA(expand_target_enqueue((const float*)c->staging, width * height, c->synth,
                                    c->ls.sms * 4, c->stream));
    KIFI_CUDA(cudaStreamSynchronize(c->stream));
    c->sw = width;
    c->sh = height;
    c->synth_e2w = load_mat(synth_eye_to_world);
    c->have_target = true;
    return KIFI_OK;
}

kifi_status kifi_icp_set_target_from_depth(kifi_icp* c, const void* depth, int on_device,
                                           int depth_is_u16, const kifi_camera* cam,
                                           const float eye_to_world[16]) {
    if (!c || !depth || !camera_ok(cam) || !eye_to_world)
        return fail(KIFI_ERR_INVALID_ARGUMENT, "bad argument");
    KIFI_CUDA(cudaSetDevice(c->device));
    kifi_status s = reserve_target(c, cam->width, cam->height);
    if (s) return s;
    const void* src = depth;
    if (!on_device) {
        const size_t bytes = (size_t)cam->width * cam->height * (depth_is_u16 ? 2 : 4);
        if ((s = reserve_bytes(&c->depth_dev, &c->depth_bytes, bytes, c->stream))) return s;
        KIFI_CUDA(cudaMemcpyAsync(c->depth_dev, depth, bytes, cudaMemcpyHostToDevice, c->stream));
        src = c->depth_dev;
    }
    const Mat4 e2w = load_mat(eye_to_world);
    KIFI_CUDA(backproject_enqueue(src, depth_is_u16 != 0, *cam, e2w, c->synth, c->ls.sms * 4,
                                  c->stream));
    if (!on_device) KIFI_CUDA(cudaStreamSynchronize(c->stream));
    c->sw = cam->width;
    c->sh = cam->height;
    c->synth_e2w = e2w;
    c->have_target = true;
    return KIFI_OK;
}

kifi_status kifi_icp_set_target_bin_device(kifi_icp* c, const float* points_dev, size_t n,
                                           const float world_to_clip[16], int width, int height,
                                           const float synth_eye_to_world[16]) {
    if (!c || (n && !points_dev) || !world_to_clip || width <= 0 || height <= 0 || !synth_eye_to_world)
        return fail(KIFI_ERR_INVALID_ARGUMENT, "bad argument");
    if (n >= ((size_t)1 << 32)) return fail(KIFI_ERR_UNSUPPORTED, "more than 2^32 points");
    KIFI_CUDA(cudaSetDevice(c->device));
    kifi_status s = reserve_target(c, width, height);
    if (s) return s;
    if ((s = reserve_bytes(&c->zbuf, &c->zbuf_cap, (size_t)width * height * 8, c->stream))) return s;
    KIFI_CUDA(bin_target_enqueue(points_dev, (unsigned int)n, load_mat(world_to_clip), width, height,
                                 (unsigned long long*)c->zbuf, c->synth, c->ls.sms * 4, c->stream));
    c->sw = width;
    c->sh = height;
    c->synth_e2w = load_mat(synth_eye_to_world);
    c->have_target = true;
    return KIFI_OK;
}

kifi_status kifi_icp_align(kifi_icp* c, const float* depth_m, const kifi_camera* cam,
                           const float eye_to_world_guess[16], int iterations,
                           float out_eye_to_world[16]) {
    if (!c || !depth_m || !camera_ok(cam) || !eye_to_world_guess || !out_eye_to_world)
        return fail(KIFI_ERR_INVALID_ARGUMENT, "bad argument");
    KIFI_CUDA(cudaSetDevice(c->device));
    const size_t bytes = (size_t)cam->width * cam->height * 4;
    kifi_status s = reserve_bytes(&c->depth_dev, &c->depth_bytes, bytes, c->stream);
    if (s) return s;
    KIFI_CUDA(cudaMemcpyAsync(c->depth_dev, depth_m, bytes, cudaMemcpyHostToDevice, c->stream));
    if ((s = enqueue_align(c, c->depth_dev, false, cam, eye_to_world_guess, iterations))) return s;
    return kifi_icp_result(c, out_eye_to_world, nullptr, nullptr, nullptr, 0, nullptr);
}

kifi_status kifi_icp_align_device(kifi_icp* c, const void* depth_dev, int depth_is_u16,
                                  const kifi_camera* cam, const float eye_to_world_guess[16],
                                  int iterations) {
    if (!c || !depth_dev || !camera_ok(cam) || !eye_to_world_guess)
        return fail(KIFI_ERR_INVALID_ARGUMENT, "bad argument");
    KIFI_CUDA(cudaSetDevice(c->device));
    return enqueue_align(c, depth_dev, depth_is_u16 != 0, cam, eye_to_world_guess, iterations);
}

kifi_status kifi_icp_result(kifi_icp* c, float out_eye_to_world[16], double out_eye_to_world_d[16],
                            int* n_assoc, double* rms, int capacity, int* iterations) {
    if (!c) return fail(KIFI_ERR_INVALID_ARGUMENT, "null context");
    KIFI_CUDA(cudaSetDevice(c->device));
    // read the head of the state: poses and per-iteration statistics (pinned)
    IcpState* h = c->head;
    cudaError_t e = cudaMemcpyAsync(h, c->st, offsetof(IcpState, part), cudaMemcpyDeviceToHost, c->stream);
    if (!e) e = cudaStreamSynchronize(c->stream);
    if (e) return cuda_fail(e, "ICP result");
    if (out_eye_to_world) std::memcpy(out_eye_to_world, h->pose_f, 64);
    if (out_eye_to_world_d)
        for (int i = 0; i < 16; ++i) out_eye_to_world_d[i] = (double)h->pose_f[i] + (double)h->pose_lo[i];
    const int it = h->iter < kIcpMaxStats ? h->iter : kIcpMaxStats;
    if (iterations) *iterations = h->iter;
    for (int i = 0; i < it && i < capacity; ++i) {
        if (n_assoc) n_assoc[i] = h->stats[i].n_assoc;
        // sqrt(sum / n) in float, as the device formed it before
        const int n = h->stats[i].n_assoc;
        if (rms) rms[i] = n > 0 ? (double)std::sqrt(h->stats[i].sum_l2 / (float)n) : 0.0;
    }
    return KIFI_OK;
}

}  // extern "C"

// The pose of the latest alignment as its last step publishes it (see
// IcpPoseMail), polled without synchronising the stream: the caller gets
// it as soon as the final finisher has written it, not after the work
// queued behind it.  Polls for at most two seconds, then takes the
// synchronising path, which also reports device errors.
void icp_publish_pose(kifi_icp* c, bool on) { c->publish = on; }

kifi_status icp_wait_pose(kifi_icp* c, float out_eye_to_world[16]) {
    if (c->last_iters > 0 && c->publish && c->mail) {
        const unsigned long long want = c->mail_seq;
        const volatile unsigned long long* seq = &c->mail->seq;
        const auto t0 = std::chrono::steady_clock::now();
        for (unsigned long long spins = 0;; ++spins) {
            if (*seq == want) {
                std::atomic_thread_fence(std::memory_order_acquire);
                const volatile float* pose = c->mail->pose;
                for (int i = 0; i < 16; ++i) out_eye_to_world[i] = pose[i];
                return KIFI_OK;
            }
            if ((spins & 1023) == 1023 && std::chrono::steady_clock::now() - t0 > std::chrono::seconds(2)) break;
        }
    }
    return kifi_icp_result(c, out_eye_to_world, nullptr, nullptr, nullptr, 0, nullptr);
}

extern "C" {

kifi_status kifi_icp_iteration_times(kifi_icp* c, float* body_us, float* tail_us, int capacity,
                                     int* iterations) {
    if (!c) return fail(KIFI_ERR_INVALID_ARGUMENT, "null context");
    KIFI_CUDA(cudaSetDevice(c->device));
    IcpState* h = c->head;
    cudaError_t e = cudaMemcpyAsync(h, c->st, offsetof(IcpState, part), cudaMemcpyDeviceToHost, c->stream);
    if (!e) e = cudaStreamSynchronize(c->stream);
    if (e) return cuda_fail(e, "ICP timings");
    const int it = h->iter < kIcpMaxStats ? h->iter : kIcpMaxStats;
    if (iterations) *iterations = h->iter;
    for (int i = 0; i < it && i < capacity; ++i) {
        if (body_us) body_us[i] = h->stats[i].body_us;
        if (tail_us) tail_us[i] = h->stats[i].tail_us;
    }
    return KIFI_OK;
}

kifi_status kifi_bin(const float* points, size_t n, const float world_to_clip[16], float* out,
                     int width, int height) {
    if ((n && !points) || !world_to_clip || !out || width <= 0 || height <= 0)
        return fail(KIFI_ERR_INVALID_ARGUMENT, "bad argument");
    if (n >= ((size_t)1 << 32)) return fail(KIFI_ERR_UNSUPPORTED, "more than 2^32 points");
    int dev = 0;
    KIFI_CUDA(cudaGetDevice(&dev));
    LaunchShape ls;
    kifi_status s = launch_shape(dev, &ls);
    if (s) return s;
    cudaStream_t st;
    KIFI_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    float *dp = nullptr, *dout = nullptr;
    unsigned long long* zb = nullptr;
    const size_t pix = (size_t)width * height;
    cudaError_t e = cudaMalloc(&dp, n * 12 + 16);
    if (!e) e = cudaMalloc(&dout, pix * 12);
    if (!e) e = cudaMalloc(&zb, pix * 8);
    if (!e && n) e = cudaMemcpyAsync(dp, points, n * 12, cudaMemcpyHostToDevice, st);
    if (!e) e = bin_enqueue(dp, (unsigned int)n, load_mat(world_to_clip), width, height, zb, dout,
                            ls.sms * 4, st);
    if (!e) e = cudaMemcpyAsync(out, dout, pix * 12, cudaMemcpyDeviceToHost, st);
    if (!e) e = cudaStreamSynchronize(st);
    cudaFree(dp);
    cudaFree(dout);
    cudaFree(zb);
    cudaStreamDestroy(st);
    if (e) return cuda_fail(e, "bin");
    return KIFI_OK;
}

}  // extern "C"
