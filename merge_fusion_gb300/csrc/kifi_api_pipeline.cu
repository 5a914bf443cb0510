// kifi_api_pipeline.cu -- kifi::Pipeline on the GPU (KinectFission/kifi/
// Pipeline.h:16-56, Pipeline.cpp:26-56): per frame, fuse the depth frame with
// its given pose (the live path, Pipeline.cpp:32-35) and track it with ICP
// against the previous frame (the tracking path the reference keeps under
// #else, :36-55), and extract the mesh every N frames.
//
// Fusion runs on the volume's stream and tracking on the ICP context's
// stream, so the HBM-bound merge/update and the shared-memory-bound ICP
// window search overlap on the GPU.  Events order the shared inputs: a frame
// slot is only overwritten after the tracking stream has finished reading it.
//
// With graphs on (kifi_pipeline_set_graphs), a frame -- the upload of a host
// frame, the fusion launches and the tracking launches on both streams -- is
// captured into one CUDA graph.  Every host-side check that could allocate
// or wait (volume capacity, ICP buffers) runs before the capture, so the
// capture holds launches and copies only.  The first frame instantiates the
// graph; later frames apply their parameters (poses, frame pointers) to the
// instantiated graph with cudaGraphExecUpdate, and it is launched as one
// unit.  A frame whose captured topology differs (the first tracked frame,
// a grown volume) instantiates anew.  Meshing stays outside the graph.
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
    bool graphs = false;
    cudaGraphExec_t exec = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr, after = nullptr;
    long long graph_builds = 0, graph_updates = 0;
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

// One frame as a CUDA graph (see the file comment).  host_src: a page-locked
// host frame to upload into depth_dev inside the graph, or null.
kifi_status frame_graph(kifi_pipeline* p, const void* host_src, size_t bytes, const void* depth_dev, bool u16,
                        const float* world_to_eye) {
    const kifi_camera& cam = p->desc.camera;
    const bool track = p->desc.icp_iterations > 0;
    kifi_status s = kifi_volume_prepare_frame(p->vol, &cam);
    if (s) return s;
    if (track && (s = kifi_icp_prepare_frame(p->icp, &cam))) return s;
    const Mat4 e2w = invert_transform(load_mat(world_to_eye));
    // stage timer events cannot be waited on once captured: none in the graph
    const bool profiling = p->vol->profiling;
    p->vol->profiling = false;
    KIFI_CUDA(cudaStreamBeginCapture(p->vs, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = cudaSuccess;
    if (host_src) e = cudaMemcpyAsync((void*)depth_dev, host_src, bytes, cudaMemcpyHostToDevice, p->vs);
    if (!e) s = kifi_volume_enqueue_frame(p->vol, depth_dev, u16, &cam, world_to_eye);
    if (!e && !s && track) {
        e = cudaEventRecord(p->fork, p->vs);
        if (!e) e = cudaStreamWaitEvent(p->is, p->fork, 0);
        if (!e && p->have_prev)
            s = kifi_icp_align_device(p->icp, depth_dev, u16 ? 1 : 0, &cam, p->prev_e2w, p->desc.icp_iterations);
        if (!e && !s) s = kifi_icp_set_target_from_depth(p->icp, depth_dev, 1, u16 ? 1 : 0, &cam, e2w.m);
        if (!e) e = cudaEventRecord(p->join, p->is);
        if (!e) e = cudaStreamWaitEvent(p->vs, p->join, 0);
    }
    cudaGraph_t g = nullptr;
    const cudaError_t ee = cudaStreamEndCapture(p->vs, &g);
    p->vol->profiling = profiling;
    if (!e) e = ee;
    if (e || s) {
        if (g) cudaGraphDestroy(g);
        return s ? s : cuda_fail(e, "frame capture");
    }
    if (p->exec) {
        cudaGraphExecUpdateResultInfo info;
        if (cudaGraphExecUpdate(p->exec, g, &info) == cudaSuccess) {
            ++p->graph_updates;
        } else {
            cudaGetLastError();
            cudaGraphExecDestroy(p->exec);
            p->exec = nullptr;
        }
    }
    if (!p->exec) {
        e = cudaGraphInstantiate(&p->exec, g, 0);
        if (e) p->exec = nullptr;
        else ++p->graph_builds;
    }
    cudaGraphDestroy(g);
    if (e) return cuda_fail(e, "frame graph instantiation");
    KIFI_CUDA(cudaGraphLaunch(p->exec, p->vs));
    if (track) {  // later work on the tracking stream (results, the next frame) follows the graph
        KIFI_CUDA(cudaEventRecord(p->after, p->vs));
        KIFI_CUDA(cudaStreamWaitEvent(p->is, p->after, 0));
    }
    std::memcpy(p->prev_e2w, e2w.m, 64);
    p->have_prev = true;
    ++p->frame;
    if (p->desc.mesh_every > 0 && p->frame % p->desc.mesh_every == 0) {
        if ((s = kifi_mesh_device(p->vol, p->desc.mesh_with_indices, &p->mesh_verts, &p->mesh_indices,
                                  nullptr, nullptr)))
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
    if (!e) e = cudaEventCreateWithFlags(&p->fork, cudaEventDisableTiming);
    if (!e) e = cudaEventCreateWithFlags(&p->join, cudaEventDisableTiming);
    if (!e) e = cudaEventCreateWithFlags(&p->after, cudaEventDisableTiming);
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
    if (p->fork) cudaEventDestroy(p->fork);
    if (p->join) cudaEventDestroy(p->join);
    if (p->after) cudaEventDestroy(p->after);
    if (p->exec) cudaGraphExecDestroy(p->exec);
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
    if (p->graphs) return frame_graph(p, nullptr, 0, depth_dev, depth_is_u16 != 0, world_to_eye);
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
    if (p->graphs) {
        cudaPointerAttributes attr;
        const bool pinned = cudaPointerGetAttributes(&attr, depth_host) == cudaSuccess &&
                            attr.type == cudaMemoryTypeHost;
        cudaGetLastError();
        if (pinned) {  // the upload is part of the frame's graph
            kifi_status s = frame_graph(p, depth_host, bytes, p->slot[k], depth_is_u16 != 0, world_to_eye);
            if (s) return s;
            KIFI_CUDA(cudaEventRecord(p->released[k], p->vs));
            return kifi_pipeline_sync(p, out_eye_to_world);
        }
    }
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

kifi_status kifi_pipeline_set_graphs(kifi_pipeline* p, int on) {
    if (!p) return fail(KIFI_ERR_INVALID_ARGUMENT, "null pipeline");
    p->graphs = on != 0;
    return KIFI_OK;
}

kifi_status kifi_pipeline_graph_stats(kifi_pipeline* p, long long* instantiated, long long* updated) {
    if (!p) return fail(KIFI_ERR_INVALID_ARGUMENT, "null pipeline");
    if (instantiated) *instantiated = p->graph_builds;
    if (updated) *updated = p->graph_updates;
    return KIFI_OK;
}

kifi_status kifi_pipeline_mesh_counts(kifi_pipeline* p, size_t* n_verts, size_t* n_indices) {
    if (!p || !n_verts || !n_indices) return fail(KIFI_ERR_INVALID_ARGUMENT, "null argument");
    *n_verts = p->mesh_verts;
    *n_indices = p->mesh_indices;
    return KIFI_OK;
}

}  // extern "C"
