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
//
// Meshing every N frames never blocks the host: on a mesh frame a third
// stream waits for that frame's fusion, copies the resident voxels into a
// snapshot (count and buffer read on the device) and runs the counting
// passes; the volume stream only waits for the copy before fusing the next
// frame.  Later pipeline calls poll the counts without blocking and, once
// they are in, size the outputs (stream-ordered allocation) and enqueue the
// vertex/index emission on the mesh stream.  kifi_pipeline_mesh_counts waits
// for the latest mesh.
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
    // asynchronous meshing
    cudaStream_t ms = nullptr;
    MeshScratch mscr{};
    void* snap_keys = nullptr;  // the volume's key width
    float2* snap_vals = nullptr;
    size_t snap_cap = 0, snap_n = 0;
    float* mverts = nullptr;
    uint32_t* midx = nullptr;
    size_t mverts_cap = 0, midx_cap = 0;
    MeshCounts* counts_host = nullptr;  // page-locked
    cudaEvent_t frame_done = nullptr, snap_done = nullptr, counts_ready = nullptr;
    bool counting = false;
    cudaGraphExec_t exec = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr, after = nullptr;
    long long graph_builds = 0, graph_updates = 0;
};

namespace {

// counts of the snapshot in: size the outputs and enqueue the emission
kifi_status mesh_emit(kifi_pipeline* p) {
    const MeshCounts& c = *p->counts_host;
    const size_t nv = (size_t)c.n_verts, ni = p->desc.mesh_with_indices ? (size_t)c.n_idx : 0;
    if (nv + kPad > p->mverts_cap) {
        if (p->mverts) KIFI_CUDA(cudaFreeAsync(p->mverts, p->ms));
        p->mverts_cap = (nv + kPad) + (nv + kPad) / 4;
        KIFI_CUDA(cudaMallocAsync((void**)&p->mverts, p->mverts_cap * 12, p->ms));
    }
    if (ni + kPad > p->midx_cap) {
        if (p->midx) KIFI_CUDA(cudaFreeAsync(p->midx, p->ms));
        p->midx_cap = (ni + kPad) + (ni + kPad) / 4;
        KIFI_CUDA(cudaMallocAsync((void**)&p->midx, p->midx_cap * 4, p->ms));
    }
    KIFI_CUDA(mesh_emit_enqueue(p->vol->g, p->snap_keys, p->vol->vb.key_bytes, p->snap_vals, p->snap_n,
                                p->desc.mesh_with_indices, p->mscr, nv, ni, p->mverts, p->midx, p->vol->ls.sms,
                                p->ms));
    p->mesh_verts = nv;
    p->mesh_indices = ni;
    p->counting = false;
    return KIFI_OK;
}

// a mesh whose counts are in gets its emission; with `wait`, wait for them
kifi_status mesh_poll(kifi_pipeline* p, bool wait) {
    if (!p->counting) return KIFI_OK;
    if (wait) {
        KIFI_CUDA(cudaEventSynchronize(p->counts_ready));
    } else {
        const cudaError_t q = cudaEventQuery(p->counts_ready);
        if (q == cudaErrorNotReady) return KIFI_OK;
        if (q != cudaSuccess) return cuda_fail(q, "mesh counts");
    }
    return mesh_emit(p);
}

// snapshot + counting passes of the volume as of the frame just enqueued
kifi_status mesh_begin(kifi_pipeline* p) {
    kifi_status s = mesh_poll(p, true);  // one mesh at a time
    if (s) return s;
    kifi_volume* v = p->vol;
    if (p->snap_cap < v->vb.cap) {
        KIFI_CUDA(cudaStreamSynchronize(p->ms));
        cudaFree(p->snap_keys);
        cudaFree(p->snap_vals);
        p->snap_keys = nullptr;
        p->snap_vals = nullptr;
        p->snap_cap = 0;
        KIFI_CUDA(cudaMalloc(&p->snap_keys, (v->vb.cap + kPad) * v->vb.key_bytes));
        KIFI_CUDA(cudaMalloc(&p->snap_vals, (v->vb.cap + kPad) * 8));
        p->snap_cap = v->vb.cap;
    }
    // the passes' grids cover the host's upper bound of the voxel count
    p->snap_n = v->n_upper < p->snap_cap ? v->n_upper : p->snap_cap;
    if (p->mscr.cap < p->snap_n) {  // with headroom: freeing scratch waits for the device
        const size_t want = p->snap_n + p->snap_n / 4;
        KIFI_CUDA(mesh_scratch_reserve(&p->mscr, want < p->snap_cap ? want : p->snap_cap, v->g.kb));
    }
    KIFI_CUDA(cudaEventRecord(p->frame_done, p->vs));
    KIFI_CUDA(cudaStreamWaitEvent(p->ms, p->frame_done, 0));
    KIFI_CUDA(mesh_snapshot_enqueue(v->ctl, v->vb, p->snap_keys, p->snap_vals, p->snap_n, p->mscr.n_dev, v->ls.sms,
                                    p->ms));
    KIFI_CUDA(cudaEventRecord(p->snap_done, p->ms));
    KIFI_CUDA(cudaStreamWaitEvent(p->vs, p->snap_done, 0));  // fusion may overwrite the buffers after the copy
    KIFI_CUDA(mesh_count_enqueue(p->snap_keys, v->vb.key_bytes, p->snap_vals, p->snap_n, v->g.kb,
                                 p->desc.mesh_with_indices, p->mscr, v->ls.sms, p->ms));
    KIFI_CUDA(cudaMemcpyAsync(p->counts_host, p->mscr.counts, sizeof(MeshCounts), cudaMemcpyDeviceToHost, p->ms));
    KIFI_CUDA(cudaEventRecord(p->counts_ready, p->ms));
    p->counting = true;
    return KIFI_OK;
}

kifi_status track_and_fuse(kifi_pipeline* p, const void* depth_dev, bool u16, int k,
                           const float* world_to_eye) {
    const kifi_camera& cam = p->desc.camera;
    kifi_status s = mesh_poll(p, false);
    if (s) return s;
    // tracking on the ICP stream, once the frame is on the device; enqueued
    // first, as it is the frame's critical path
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
    // fusion on the volume's stream
    if ((s = kifi_integrate_device(p->vol, depth_dev, u16 ? 1 : 0, &cam, world_to_eye))) return s;
    std::memcpy(p->prev_e2w, e2w.m, 64);
    p->have_prev = true;
    ++p->frame;
    if (p->desc.mesh_every > 0 && p->frame % p->desc.mesh_every == 0 && (s = mesh_begin(p))) return s;
    return KIFI_OK;
}

// One frame as a CUDA graph (see the file comment).  host_src: a page-locked
// host frame to upload into depth_dev inside the graph, or null.
kifi_status frame_graph(kifi_pipeline* p, const void* host_src, size_t bytes, const void* depth_dev, bool u16,
                        const float* world_to_eye) {
    const kifi_camera& cam = p->desc.camera;
    const bool track = p->desc.icp_iterations > 0;
    kifi_status s = mesh_poll(p, false);
    if (s) return s;
    if ((s = kifi_volume_prepare_frame(p->vol, &cam))) return s;
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
    if (p->desc.mesh_every > 0 && p->frame % p->desc.mesh_every == 0 && (s = mesh_begin(p))) return s;
    return KIFI_OK;
}

// The caller's result of a host frame: the tracked pose.  Tracking waits for
// the frame's upload, so once its result is in the host frame is free; the
// frame's fusion may still run (every call that reads the volume waits for it
// and reports its device errors, as after kifi_pipeline_integrate_device).
kifi_status frame_result(kifi_pipeline* p, int k, float out_eye_to_world[16]) {
    if (p->desc.icp_iterations > 0) {
        if (p->frame > 1)
            return kifi_icp_result(p->icp, out_eye_to_world, nullptr, nullptr, nullptr, 0, nullptr);
        KIFI_CUDA(cudaStreamSynchronize(p->is));  // the first frame only sets the target
    } else {
        KIFI_CUDA(cudaEventSynchronize(p->uploaded[k]));
    }
    if (out_eye_to_world) std::memcpy(out_eye_to_world, p->prev_e2w, 64);
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
    vd.key_bits = d->key_bits;
    kifi_status s = kifi_volume_create(&vd, &p->vol);
    if (!s && d->icp_iterations > 0) {
        p->vol->tracking_grids = true;
        tracking_launch_shape(&p->vol->ls);
    }
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
    if (!e) e = cudaStreamCreateWithFlags(&p->ms, cudaStreamNonBlocking);
    if (!e) e = cudaEventCreateWithFlags(&p->frame_done, cudaEventDisableTiming);
    if (!e) e = cudaEventCreateWithFlags(&p->snap_done, cudaEventDisableTiming);
    if (!e) e = cudaEventCreateWithFlags(&p->counts_ready, cudaEventDisableTiming);
    if (!e) e = cudaHostAlloc((void**)&p->counts_host, sizeof(MeshCounts), cudaHostAllocDefault);
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
    if (p->ms) {
        cudaStreamSynchronize(p->ms);
        if (p->mverts) cudaFreeAsync(p->mverts, p->ms);
        if (p->midx) cudaFreeAsync(p->midx, p->ms);
        cudaStreamSynchronize(p->ms);
        cudaStreamDestroy(p->ms);
    }
    mesh_scratch_free(&p->mscr);
    cudaFree(p->snap_keys);
    cudaFree(p->snap_vals);
    if (p->counts_host) cudaFreeHost(p->counts_host);
    if (p->frame_done) cudaEventDestroy(p->frame_done);
    if (p->snap_done) cudaEventDestroy(p->snap_done);
    if (p->counts_ready) cudaEventDestroy(p->counts_ready);
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
    return frame_result(p, k, out_eye_to_world);
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
    KIFI_CUDA(cudaSetDevice(p->desc.device));
    kifi_status s = mesh_poll(p, true);
    if (s) return s;
    KIFI_CUDA(cudaStreamSynchronize(p->ms));
    *n_verts = p->mesh_verts;
    *n_indices = p->mesh_indices;
    return KIFI_OK;
}

}  // extern "C"
