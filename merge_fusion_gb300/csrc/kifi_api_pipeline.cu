// kifi_api_pipeline.cu -- kifi::Pipeline on the GPU (KinectFission/kifi/
// Pipeline.h:16-56, Pipeline.cpp:26-56): per frame, fuse the depth frame with
// its given pose (the live path, Pipeline.cpp:32-35) and track it with ICP
// against the previous frame (the tracking path the reference keeps under
// #else, :36-55), and extract the mesh every N frames.
//
// Fusion runs on the volume's stream and tracking on the ICP context's
// stream, so the HBM-bound merge/update and the L1-bound ICP window search
// overlap on the GPU.  Events order the shared inputs: a frame slot is only
// overwritten after the tracking stream has finished reading it.
#include <cstring>
#include <new>

#include "kifi_api_util.h"

using namespace kifi;

struct kifi_pipeline {
    kifi_pipeline_desc desc{};
    kifi_volume* vol = nullptr;
    kifi_icp* icp = nullptr;
    cudaStream_t vs = nullptr, is = nullptr;
    void* slot[2] = {nullptr, nullptr};  // host-fed frames (uint16 or float)
    size_t slot_bytes = 0;
    cudaEvent_t uploaded[2] = {nullptr, nullptr};   // frame in slot k is on the device
    cudaEvent_t released[2] = {nullptr, nullptr};   // tracking no longer reads slot k
    cudaEvent_t fused = nullptr;
    long long frame = 0;
    float prev_e2w[16];
    bool have_prev = false;
    size_t mesh_verts = 0, mesh_indices = 0;
};

namespace {

kifi_status track_and_fuse(kifi_pipeline* p, const void* depth_dev, bool u16, int k,
                           const float* world_to_eye) {
    const kifi_camera& cam = p->desc.camera;
    kifi_status s;
    // fusion on the volume's stream
    if ((s = kifi_integrate_device(p->vol, depth_dev, u16 ? 1 : 0, &cam, world_to_eye))) return s;
    // tracking on the ICP stream, once the frame is on the device
    const Mat4 e2w = invert_transform(load_mat(world_to_eye));
    if (p->desc.icp_iterations > 0) {
        if (k >= 0) KIFI_CUDA(cudaStreamWaitEvent(p->is, p->uploaded[k], 0));
        if (p->have_prev &&
            (s = kifi_icp_align_device(p->icp, depth_dev, u16 ? 1 : 0, &cam, p->prev_e2w,
                                       p->desc.icp_iterations)))
            return s;
        // this frame becomes the next frame's target
        if ((s = kifi_icp_set_target_from_depth(p->icp, depth_dev, 1, u16 ? 1 : 0, &cam, e2w.m)))
            return s;
        if (k >= 0) KIFI_CUDA(cudaEventRecord(p->released[k], p->is));
    }
    std::memcpy(p->prev_e2w, e2w.m, 64);
    p->have_prev = true;
    ++p->frame;
    if (p->desc.mesh_every > 0 && p->frame % p->desc.mesh_every == 0) {
        if ((s = kifi_mesh_device(p->vol, p->desc.mesh_with_indices, &p->mesh_verts,
                                  &p->mesh_indices, nullptr, nullptr)))
            return s;
    }
    return KIFI_OK;
}

}  // namespace

extern "C" {

kifi_status kifi_pipeline_create(const kifi_pipeline_desc* d, kifi_pipeline** out) {
    if (!d || !out || !camera_ok(&d->camera)) return fail(KIFI_ERR_INVALID_ARGUMENT, "bad argument");
    *out = nullptr;
    if (d->icp_iterations < 0 || d->icp_iterations > kIcpMaxStats || d->mesh_every < 0)
        return fail(KIFI_ERR_INVALID_ARGUMENT, "bad iteration count or mesh period");
    kifi_pipeline* p = new (std::nothrow) kifi_pipeline();
    if (!p) return fail(KIFI_ERR_OUT_OF_MEMORY, "host allocation");
    p->desc = *d;
    kifi_volume_desc vd{};
    vd.resolution = d->resolution;
    vd.side_length_m = d->side_length_m;
    vd.truncation_m = d->truncation_m;
    vd.initial_capacity = d->initial_capacity;
    vd.device = d->device;
    kifi_status s = kifi_volume_create(&vd, &p->vol);
    if (!s) s = kifi_icp_create(d->device, nullptr, &p->icp);
    if (s) {
        kifi_pipeline_destroy(p);
        return s;
    }
    p->vs = (cudaStream_t)kifi_volume_stream(p->vol);
    p->is = (cudaStream_t)kifi_icp_stream(p->icp);
    cudaError_t e = cudaSuccess;
    for (int k = 0; k < 2 && !e; ++k) {
        e = cudaEventCreateWithFlags(&p->uploaded[k], cudaEventDisableTiming);
        if (!e) e = cudaEventCreateWithFlags(&p->released[k], cudaEventDisableTiming);
        if (!e) e = cudaEventRecord(p->released[k], p->is);
    }
    if (!e) e = cudaEventCreateWithFlags(&p->fused, cudaEventDisableTiming);
    if (e) {
        kifi_pipeline_destroy(p);
        return cuda_fail(e, "pipeline events");
    }
    *out = p;
    return KIFI_OK;
}

kifi_status kifi_pipeline_destroy(kifi_pipeline* p) {
    if (!p) return KIFI_OK;
    if (p->vs) cudaStreamSynchronize(p->vs);
    if (p->is) cudaStreamSynchronize(p->is);
    for (int k = 0; k < 2; ++k) {
        cudaFree(p->slot[k]);
        if (p->uploaded[k]) cudaEventDestroy(p->uploaded[k]);
        if (p->released[k]) cudaEventDestroy(p->released[k]);
    }
    if (p->fused) cudaEventDestroy(p->fused);
    kifi_icp_destroy(p->icp);
    kifi_volume_destroy(p->vol);
    delete p;
    return KIFI_OK;
}

kifi_volume* kifi_pipeline_volume(kifi_pipeline* p) { return p ? p->vol : nullptr; }
kifi_icp* kifi_pipeline_icp(kifi_pipeline* p) { return p ? p->icp : nullptr; }

kifi_status kifi_pipeline_integrate_device(kifi_pipeline* p, const void* depth_dev, int depth_is_u16,
                                           const float world_to_eye[16]) {
    if (!p || !depth_dev || !world_to_eye) return fail(KIFI_ERR_INVALID_ARGUMENT, "bad argument");
    KIFI_CUDA(cudaSetDevice(p->desc.device));
    return track_and_fuse(p, depth_dev, depth_is_u16 != 0, -1, world_to_eye);
}

kifi_status kifi_pipeline_integrate(kifi_pipeline* p, const void* depth_host, int depth_is_u16,
                                    const float world_to_eye[16], float out_eye_to_world[16]) {
    if (!p || !depth_host || !world_to_eye) return fail(KIFI_ERR_INVALID_ARGUMENT, "bad argument");
    KIFI_CUDA(cudaSetDevice(p->desc.device));
    const kifi_camera& cam = p->desc.camera;
    const size_t bytes = (size_t)cam.width * cam.height * (depth_is_u16 ? 2 : 4);
    if (bytes > p->slot_bytes) {
        KIFI_CUDA(cudaStreamSynchronize(p->vs));
        KIFI_CUDA(cudaStreamSynchronize(p->is));
        for (int k = 0; k < 2; ++k) {
            cudaFree(p->slot[k]);
            p->slot[k] = nullptr;
        }
        p->slot_bytes = 0;
        for (int k = 0; k < 2; ++k) KIFI_CUDA(cudaMalloc(&p->slot[k], bytes));
        p->slot_bytes = bytes;
    }
    const int k = (int)(p->frame & 1);
    KIFI_CUDA(cudaStreamWaitEvent(p->vs, p->released[k], 0));
    KIFI_CUDA(cudaMemcpyAsync(p->slot[k], depth_host, bytes, cudaMemcpyHostToDevice, p->vs));
    KIFI_CUDA(cudaEventRecord(p->uploaded[k], p->vs));
    kifi_status s = track_and_fuse(p, p->slot[k], depth_is_u16 != 0, k, world_to_eye);
    if (s) return s;
    return kifi_pipeline_sync(p, out_eye_to_world);
}

kifi_status kifi_pipeline_sync(kifi_pipeline* p, float out_eye_to_world[16]) {
    if (!p) return fail(KIFI_ERR_INVALID_ARGUMENT, "null pipeline");
    KIFI_CUDA(cudaSetDevice(p->desc.device));
    kifi_status s = kifi_volume_sync(p->vol);
    if (s) return s;
    if (out_eye_to_world) {
        if (p->desc.icp_iterations > 0 && p->frame > 1)
            return kifi_icp_result(p->icp, out_eye_to_world, nullptr, nullptr, nullptr, 0, nullptr);
        std::memcpy(out_eye_to_world, p->prev_e2w, 64);
    }
    KIFI_CUDA(cudaStreamSynchronize(p->is));
    return KIFI_OK;
}

kifi_status kifi_pipeline_mesh_counts(kifi_pipeline* p, size_t* n_verts, size_t* n_indices) {
    if (!p || !n_verts || !n_indices) return fail(KIFI_ERR_INVALID_ARGUMENT, "null argument");
    *n_verts = p->mesh_verts;
    *n_indices = p->mesh_indices;
    return KIFI_OK;
}

}  // extern "C"
