// kifi_api_pipeline.cu -- kifi::Pipeline on the GPU (KinectFission/kifi/
// Pipeline.h:16-56, Pipeline.cpp:26-56), in one of two modes:
//
//  open loop (default): per frame, fuse the depth frame with its given pose
//    (the live path, Pipeline.cpp:32-35) and track it with ICP against the
//    previous frame's back-projection, with the previous given pose as the
//    guess; the tracked pose is reported, fusion does not use it.
//  closed loop (kifi_pipeline_desc::closed_loop): the reference's tracking
//    path (:36-55).  Per frame after the first, ICP aligns the frame
//    against the Bin of the model's mesh, starting from the previous tracked
//    pose; the frame is fused with the tracked pose; then the volume is
//    meshed (vertices only, Mesher::Mesh(verts)) and the vertices are binned
//    through EyeToClipRH * worldToEye into a 1024 x 768 target for the next
//    frame.  Each stage needs the one before, so nothing overlaps across
//    frames; the host reads the tracked pose back before it enqueues the
//    fusion.
//
// The mesh every N frames (both modes) is the caller's output mesh.
//
// Fusion runs on the volume's stream and tracking on the ICP context's
// stream, so the HBM-bound merge/update and the shared-memory-bound ICP
// window search overlap on the GPU.  Host frames are uploaded on a third
// stream into kFrameSlots device slots; events order the shared inputs: both
// streams wait for a frame's upload, and a slot is only overwritten after
// tracking and fusion have finished reading it.  With four slots a frame's
// upload waits for the fusion of the frame four back, so fusion may lag
// tracking by up to three frames before it holds tracking up.
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
// snapshot (count and buffer read on the device), runs the counting passes
// and the vertex/index emission, which reads the counts on the device; the
// volume stream only waits for the copy before fusing the next frame.  The
// emission writes into buffers sized by earlier meshes; when a mesh needs
// more, it writes nothing and flags it, and the next pipeline call that sees
// the counts grows the buffers (stream-ordered allocation) and emits again.
// kifi_pipeline_mesh_counts, kifi_pipeline_sync and kifi_pipeline_join cover
// the mesh stream.
#include <algorithm>
#include <array>
#include <cstring>
#include <new>
#include <vector>

#include "kifi_api_util.h"

using namespace kifi;

namespace {
// the synthetic target the reference's tracking pipeline bins into (Pipeline.cpp:50)
constexpr int kClosedLoopTargetW = 1024, kClosedLoopTargetH = 768;

// A host frame in page-locked memory the device can address, read over the
// host link into a frame slot: one 16-byte load per thread, all in flight
// at once (a copy-engine transfer of a 600 KB frame takes several times as
// long to start and finish); the bytes past the last full vector by CTA 0.
__global__ void k_upload(const uint4* __restrict__ src, uint4* __restrict__ dst, size_t n16,
                         const unsigned char* __restrict__ src_b, unsigned char* __restrict__ dst_b,
                         size_t n_bytes) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n16; i += (size_t)gridDim.x * blockDim.x)
        dst[i] = src[i];
    if (blockIdx.x == 0)
        for (size_t j = n16 * 16 + threadIdx.x; j < n_bytes; j += blockDim.x) dst_b[j] = src_b[j];
}
}  // namespace

constexpr int kFrameSlots = 4;  // device slots of host-fed frames

struct kifi_pipeline {
    kifi_pipeline_desc desc{};
    kifi_volume* vol = nullptr;
    kifi_icp* icp = nullptr;
    cudaStream_t vs = nullptr, is = nullptr;
    cudaStream_t us = nullptr;  // uploads of host-fed frames
    cudaStream_t fs = nullptr;  // the volume's (fusion) stream, when the pipeline made it
    void* slot[kFrameSlots] = {};  // host-fed frames (uint16 or float)
    size_t slot_bytes = 0;
    cudaEvent_t uploaded[kFrameSlots] = {};    // frame in slot k is on the device
    cudaEvent_t released[kFrameSlots] = {};    // tracking no longer reads slot k
    cudaEvent_t slot_fused[kFrameSlots] = {};  // fusion no longer reads slot k
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
    long long meshes = 0, mesh_reemits = 0;
    bool closed = false;
    cudaEvent_t vol_done = nullptr;     // closed loop: the frame's mesh is on the device
    cudaEvent_t join_ev[3] = {nullptr, nullptr, nullptr};
    // stage timers while the volume's profiling is on: ICP alignment spans
    // on the tracking stream, mesh spans (counting + emission) on the mesh stream
    std::vector<cudaEvent_t> ev_pool;
    std::vector<std::array<cudaEvent_t, 2>> track_pending, mesh_pending;
    double track_ms = 0.0, mesh_ms = 0.0;
    int track_n = 0, mesh_n = 0;
};

namespace {

kifi_status take_event(kifi_pipeline* p, cudaEvent_t* e) {
    if (p->ev_pool.empty()) {
        cudaEvent_t x;
        KIFI_CUDA(cudaEventCreate(&x));
        p->ev_pool.push_back(x);
    }
    *e = p->ev_pool.back();
    p->ev_pool.pop_back();
    return KIFI_OK;
}

// both events of a timed span, or none when profiling is off
kifi_status span_begin(kifi_pipeline* p, std::array<cudaEvent_t, 2>& ev, cudaStream_t st) {
    ev = {nullptr, nullptr};
    if (!p->vol->profiling) return KIFI_OK;
    kifi_status s = take_event(p, &ev[0]);
    if (!s) s = take_event(p, &ev[1]);
    if (s) return s;
    KIFI_CUDA(cudaEventRecord(ev[0], st));
    return KIFI_OK;
}

kifi_status span_end(std::vector<std::array<cudaEvent_t, 2>>& pending, std::array<cudaEvent_t, 2>& ev,
                     cudaStream_t st) {
    if (!ev[0]) return KIFI_OK;
    KIFI_CUDA(cudaEventRecord(ev[1], st));
    pending.push_back(ev);
    return KIFI_OK;
}

// emission of the snapshot into the current buffers, then its counts to the host
kifi_status mesh_emit(kifi_pipeline* p, std::array<cudaEvent_t, 2>* ev) {
    KIFI_CUDA(mesh_emit_enqueue(p->vol->g, p->snap_keys, p->vol->vb.key_bytes, p->snap_vals, p->snap_n,
                                p->desc.mesh_with_indices, p->mscr, p->mverts_cap, p->midx_cap, p->mverts, p->midx,
                                p->vol->ls.sms, p->ms));
    if (ev) {
        kifi_status s = span_end(p->mesh_pending, *ev, p->ms);
        if (s) return s;
    }
    KIFI_CUDA(cudaMemcpyAsync(p->counts_host, p->mscr.counts, sizeof(MeshCounts), cudaMemcpyDeviceToHost, p->ms));
    KIFI_CUDA(cudaEventRecord(p->counts_ready, p->ms));
    p->counting = true;
    return KIFI_OK;
}

// A mesh whose emission has run: take its counts, or -- when its buffers
// were too small -- grow them and emit again.  With `wait`, until it is done.
kifi_status mesh_poll(kifi_pipeline* p, bool wait) {
    for (int emitted = 0; p->counting; ++emitted) {
        // buffers grown to the counts hold the mesh: a second overflow is an internal error
        if (emitted > 1) return fail(KIFI_ERR_CUDA, "mesh emission overflowed buffers sized to its counts");
        if (wait) {
            KIFI_CUDA(cudaEventSynchronize(p->counts_ready));
        } else {
            const cudaError_t q = cudaEventQuery(p->counts_ready);
            if (q == cudaErrorNotReady) return KIFI_OK;
            if (q != cudaSuccess) return cuda_fail(q, "mesh counts");
        }
        const MeshCounts& c = *p->counts_host;
        if (c.error) {  // the classification gave up on a bounded wait: no mesh
            p->counting = false;
            return fail(KIFI_ERR_TIMEOUT, "mesh classification: a bounded wait gave up");
        }
        const size_t nv = (size_t)c.n_verts, ni = p->desc.mesh_with_indices ? (size_t)c.n_idx : 0;
        if (!c.overflow) {
            p->mesh_verts = nv;
            p->mesh_indices = ni;
            p->counting = false;
            ++p->meshes;
            return KIFI_OK;
        }
        // half again as much: a growing volume's next meshes still fit
        if (nv > p->mverts_cap) {
            if (p->mverts) KIFI_CUDA(cudaFreeAsync(p->mverts, p->ms));
            p->mverts = nullptr;
            p->mverts_cap = nv + nv / 2;
            KIFI_CUDA(cudaMallocAsync((void**)&p->mverts, (p->mverts_cap + kPad) * 12, p->ms));
        }
        if (ni > p->midx_cap) {
            if (p->midx) KIFI_CUDA(cudaFreeAsync(p->midx, p->ms));
            p->midx = nullptr;
            p->midx_cap = ni + ni / 2;
            KIFI_CUDA(cudaMallocAsync((void**)&p->midx, (p->midx_cap + kPad) * 4, p->ms));
        }
        ++p->mesh_reemits;
        kifi_status s = mesh_emit(p, nullptr);
        if (s) return s;
    }
    return KIFI_OK;
}

// snapshot, counting passes and emission of the volume as of the frame just enqueued
kifi_status mesh_begin(kifi_pipeline* p) {
    kifi_status s = mesh_poll(p, true);  // one mesh at a time: the snapshot and buffers are shared
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
    std::array<cudaEvent_t, 2> ev;
    if ((s = span_begin(p, ev, p->ms))) return s;
    KIFI_CUDA(mesh_count_enqueue(p->snap_keys, v->vb.key_bytes, p->snap_vals, p->snap_n, v->g.kb,
                                 p->desc.mesh_with_indices, p->mscr, v->ls.sms, p->ms));
    return mesh_emit(p, &ev);
}

// ICP alignment of a device frame, timed when profiling
kifi_status align(kifi_pipeline* p, const void* depth_dev, bool u16, const float* guess) {
    std::array<cudaEvent_t, 2> ev;
    kifi_status s = span_begin(p, ev, p->is);
    if (!s) s = kifi_icp_align_device(p->icp, depth_dev, u16 ? 1 : 0, &p->desc.camera, guess,
                                      p->desc.icp_iterations);
    if (!s) s = span_end(p->track_pending, ev, p->is);
    return s;
}

// One frame of the reference's tracking pipeline (Pipeline.cpp:36-55; see
// the file comment).  k: the upload slot of a host frame, or -1.
kifi_status closed_loop_frame(kifi_pipeline* p, const void* depth_dev, bool u16, int k,
                              const float* world_to_eye) {
    const kifi_camera& cam = p->desc.camera;
    kifi_status s = mesh_poll(p, false);
    if (s) return s;
    Mat4 e2w;
    if (p->frame == 0 || p->desc.icp_iterations == 0) {
        // the first pose is the caller's (the reference starts from the
        // identity moved 2 m along z, Pipeline.cpp:20-21)
        e2w = invert_transform(load_mat(world_to_eye));
        if (k >= 0) KIFI_CUDA(cudaEventRecord(p->released[k], p->is));
    } else {
        // m_eyeToWorld = m_icp.Align(rawDepthMap, m_eyeToWorld, synth, m_eyeToWorld, cam) (:37-38)
        if (k >= 0) KIFI_CUDA(cudaStreamWaitEvent(p->is, p->uploaded[k], 0));
        if ((s = align(p, depth_dev, u16, p->prev_e2w))) return s;
        if (k >= 0) KIFI_CUDA(cudaEventRecord(p->released[k], p->is));
        float pose[16];
        if ((s = kifi_icp_result(p->icp, pose, nullptr, nullptr, nullptr, 0, nullptr))) return s;
        e2w = load_mat(pose);
    }
    // tmp = m_eyeToWorld; invert_transform(tmp); Integrate(volume, frame, cam, tmp) (:40-44)
    const Mat4 w2e = invert_transform(e2w);
    if (k >= 0) KIFI_CUDA(cudaStreamWaitEvent(p->vs, p->uploaded[k], 0));
    if ((s = kifi_integrate_device(p->vol, depth_dev, u16 ? 1 : 0, &cam, w2e.m))) return s;
    if (k >= 0) KIFI_CUDA(cudaEventRecord(p->slot_fused[k], p->vs));
    if (p->desc.icp_iterations > 0) {
        // m_mesher.Mesh(m_volume, m_tmpSynthPointCloud) (:46): vertices only
        size_t nv = 0, ni = 0;
        const float* verts = nullptr;
        if ((s = kifi_mesh_device(p->vol, 0, &nv, &ni, &verts, nullptr))) return s;
        // m_renderer.Bin(cloud, EyeToClipRH() * tmp, synth 1024 x 768) (:48-52)
        KIFI_CUDA(cudaEventRecord(p->vol_done, p->vs));
        KIFI_CUDA(cudaStreamWaitEvent(p->is, p->vol_done, 0));
        const Mat4 w2c = mat_mul(eye_to_clip(cam), w2e);
        if ((s = kifi_icp_set_target_bin_device(p->icp, verts, nv, w2c.m, kClosedLoopTargetW, kClosedLoopTargetH,
                                                e2w.m)))
            return s;
    }
    std::memcpy(p->prev_e2w, e2w.m, 64);
    p->have_prev = true;
    ++p->frame;
    if (p->desc.mesh_every > 0 && p->frame % p->desc.mesh_every == 0 && (s = mesh_begin(p))) return s;
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
        // a host-fed frame's caller waits for the pose: published by the last step
        icp_publish_pose(p->icp, k >= 0);
        if (p->have_prev && (s = align(p, depth_dev, u16, p->prev_e2w))) return s;
        // this frame becomes the next frame's target
        if ((s = kifi_icp_set_target_from_depth(p->icp, depth_dev, 1, u16 ? 1 : 0, &cam, e2w.m)))
            return s;
        if (k >= 0) KIFI_CUDA(cudaEventRecord(p->released[k], p->is));
    }
    // fusion on the volume's stream, once the frame is on the device
    if (k >= 0) KIFI_CUDA(cudaStreamWaitEvent(p->vs, p->uploaded[k], 0));
    if ((s = kifi_integrate_device(p->vol, depth_dev, u16 ? 1 : 0, &cam, world_to_eye))) return s;
    if (k >= 0) KIFI_CUDA(cudaEventRecord(p->slot_fused[k], p->vs));
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
    if (p->closed) {  // the pose was read back before the frame's fusion
        if (out_eye_to_world) std::memcpy(out_eye_to_world, p->prev_e2w, 64);
        return KIFI_OK;
    }
    if (p->desc.icp_iterations > 0) {
        if (p->frame > 1) {
            float pose[16];
            kifi_status s = icp_wait_pose(p->icp, pose);
            if (!s && out_eye_to_world) std::memcpy(out_eye_to_world, pose, 64);
            return s;
        }
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
    if (d->closed_loop != 0 && d->closed_loop != 1) return fail(KIFI_ERR_INVALID_ARGUMENT, "closed_loop must be 0 or 1");
    kifi_pipeline* p = new (std::nothrow) kifi_pipeline();
    if (!p) return fail(KIFI_ERR_OUT_OF_MEMORY, "host allocation");
    p->desc = *d;
    p->closed = d->closed_loop == 1;
    kifi_volume_desc vd{};
    vd.resolution = d->resolution;
    vd.side_length_m = d->side_length_m;
    vd.truncation_m = d->truncation_m;
    vd.initial_capacity = d->initial_capacity;
    vd.device = d->device;
    vd.key_bits = d->key_bits;
    {
        // fusion one priority step above the mesh stream (both below tracking), so
        // a frame's fusion CTAs are scheduled ahead of a running mesh's (measured
        // neutral to +0.4%: the mesh is background work)
        int lowest = 0, greatest = 0;
        if (cudaSetDevice(d->device) == cudaSuccess &&
            cudaDeviceGetStreamPriorityRange(&lowest, &greatest) == cudaSuccess && greatest < lowest &&
            cudaStreamCreateWithPriority(&p->fs, cudaStreamNonBlocking, lowest - 1) == cudaSuccess)
            vd.stream = p->fs;
        cudaGetLastError();
    }
    kifi_status s = kifi_volume_create(&vd, &p->vol);
    if (!s && d->icp_iterations > 0 && !p->closed) {  // closed loop: fusion never runs beside tracking
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
    for (int k = 0; k < kFrameSlots && !e; ++k) {
        e = cudaEventCreateWithFlags(&p->uploaded[k], cudaEventDisableTiming);
        if (!e) e = cudaEventCreateWithFlags(&p->released[k], cudaEventDisableTiming);
        if (!e) e = cudaEventRecord(p->released[k], p->is);
        if (!e) e = cudaEventCreateWithFlags(&p->slot_fused[k], cudaEventDisableTiming);
    }
    if (!e) {  // uploads run at the tracking stream's priority: they start each frame's critical path
        int lowest = 0, greatest = 0;
        e = cudaDeviceGetStreamPriorityRange(&lowest, &greatest);
        if (!e) e = cudaStreamCreateWithPriority(&p->us, cudaStreamNonBlocking, greatest);
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
    if (!e) e = cudaEventCreateWithFlags(&p->vol_done, cudaEventDisableTiming);
    for (int i = 0; i < 3 && !e; ++i) e = cudaEventCreateWithFlags(&p->join_ev[i], cudaEventDisableTiming);
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
    if (p->us) cudaStreamSynchronize(p->us);
    for (int k = 0; k < kFrameSlots; ++k) {
        cudaFree(p->slot[k]);
        if (p->uploaded[k]) cudaEventDestroy(p->uploaded[k]);
        if (p->released[k]) cudaEventDestroy(p->released[k]);
        if (p->slot_fused[k]) cudaEventDestroy(p->slot_fused[k]);
    }
    if (p->us) cudaStreamDestroy(p->us);
    if (p->fused) cudaEventDestroy(p->fused);
    if (p->fork) cudaEventDestroy(p->fork);
    if (p->join) cudaEventDestroy(p->join);
    if (p->after) cudaEventDestroy(p->after);
    if (p->vol_done) cudaEventDestroy(p->vol_done);
    for (int i = 0; i < 3; ++i)
        if (p->join_ev[i]) cudaEventDestroy(p->join_ev[i]);
    for (auto& a : p->track_pending) p->ev_pool.insert(p->ev_pool.end(), a.begin(), a.end());
    for (auto& a : p->mesh_pending) p->ev_pool.insert(p->ev_pool.end(), a.begin(), a.end());
    for (cudaEvent_t x : p->ev_pool) cudaEventDestroy(x);
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
    kifi_volume_destroy(p->vol);  // synchronises the fusion stream first
    if (p->fs) cudaStreamDestroy(p->fs);
    delete p;
    return KIFI_OK;
}

kifi_volume* kifi_pipeline_volume(kifi_pipeline* p) { return p ? p->vol : nullptr; }
kifi_icp* kifi_pipeline_icp(kifi_pipeline* p) { return p ? p->icp : nullptr; }

kifi_status kifi_pipeline_integrate_device(kifi_pipeline* p, const void* depth_dev, int depth_is_u16,
                                           const float world_to_eye[16]) {
    if (!p || !depth_dev || !world_to_eye) return fail(KIFI_ERR_INVALID_ARGUMENT, "bad argument");
    KIFI_CUDA(cudaSetDevice(p->desc.device));
    if (p->closed) return closed_loop_frame(p, depth_dev, depth_is_u16 != 0, -1, world_to_eye);
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
        for (int k = 0; k < kFrameSlots; ++k) {
            cudaFree(p->slot[k]);
            p->slot[k] = nullptr;
        }
        p->slot_bytes = 0;
        for (int k = 0; k < kFrameSlots; ++k) KIFI_CUDA(cudaMalloc(&p->slot[k], bytes));
        p->slot_bytes = bytes;
    }
    const int k = (int)(p->frame % kFrameSlots);
    if (p->graphs) {
        KIFI_CUDA(cudaStreamWaitEvent(p->vs, p->released[k], 0));
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
    // the upload stream: slot k is free once the frame kFrameSlots back is no
    // longer read by tracking or fusion; it does not queue behind the recent
    // frames' fusion, so tracking starts as soon as the frame is on the device
    KIFI_CUDA(cudaStreamWaitEvent(p->us, p->released[k], 0));
    KIFI_CUDA(cudaStreamWaitEvent(p->us, p->slot_fused[k], 0));
    cudaPointerAttributes attr;
    const void* src_dev = nullptr;
    if (cudaPointerGetAttributes(&attr, depth_host) == cudaSuccess && attr.type == cudaMemoryTypeHost &&
        attr.devicePointer && ((uintptr_t)attr.devicePointer & 15u) == 0)
        src_dev = attr.devicePointer;
    cudaGetLastError();  // a pageable pointer is not an error here
    if (src_dev) {
        const size_t n16 = bytes / 16;
        const int threads = 256;
        const int blocks = (int)std::max<size_t>(1, std::min<size_t>((n16 + threads - 1) / threads, 4096));
        k_upload<<<blocks, threads, 0, p->us>>>((const uint4*)src_dev, (uint4*)p->slot[k], n16,
                                                (const unsigned char*)src_dev, (unsigned char*)p->slot[k], bytes);
        KIFI_CUDA(cudaGetLastError());
    } else {
        KIFI_CUDA(cudaMemcpyAsync(p->slot[k], depth_host, bytes, cudaMemcpyHostToDevice, p->us));
    }
    KIFI_CUDA(cudaEventRecord(p->uploaded[k], p->us));
    kifi_status s = p->closed ? closed_loop_frame(p, p->slot[k], depth_is_u16 != 0, k, world_to_eye)
                              : track_and_fuse(p, p->slot[k], depth_is_u16 != 0, k, world_to_eye);
    if (s) return s;
    return frame_result(p, k, out_eye_to_world);
}

kifi_status kifi_pipeline_sync(kifi_pipeline* p, float out_eye_to_world[16]) {
    if (!p) return fail(KIFI_ERR_INVALID_ARGUMENT, "null pipeline");
    KIFI_CUDA(cudaSetDevice(p->desc.device));
    kifi_status s = kifi_volume_sync(p->vol);
    if (s) return s;
    if ((s = mesh_poll(p, true))) return s;
    KIFI_CUDA(cudaStreamSynchronize(p->ms));
    if (out_eye_to_world) {
        if (!p->closed && p->desc.icp_iterations > 0 && p->frame > 1)
            return kifi_icp_result(p->icp, out_eye_to_world, nullptr, nullptr, nullptr, 0, nullptr);
        std::memcpy(out_eye_to_world, p->prev_e2w, 64);
    }
    KIFI_CUDA(cudaStreamSynchronize(p->is));
    return KIFI_OK;
}

kifi_status kifi_pipeline_join(kifi_pipeline* p, void* stream) {
    if (!p) return fail(KIFI_ERR_INVALID_ARGUMENT, "null pipeline");
    KIFI_CUDA(cudaSetDevice(p->desc.device));
    const cudaStream_t own[3] = {p->vs, p->is, p->ms};
    for (int i = 0; i < 3; ++i) {
        KIFI_CUDA(cudaEventRecord(p->join_ev[i], own[i]));
        KIFI_CUDA(cudaStreamWaitEvent((cudaStream_t)stream, p->join_ev[i], 0));
    }
    return KIFI_OK;
}

kifi_status kifi_pipeline_stage_times(kifi_pipeline* p, double out_ms[2], int out_counts[2]) {
    if (!p) return fail(KIFI_ERR_INVALID_ARGUMENT, "null pipeline");
    KIFI_CUDA(cudaSetDevice(p->desc.device));
    kifi_status s = mesh_poll(p, true);
    if (s) return s;
    std::vector<std::array<cudaEvent_t, 2>>* lists[2] = {&p->track_pending, &p->mesh_pending};
    double* acc[2] = {&p->track_ms, &p->mesh_ms};
    int* cnt[2] = {&p->track_n, &p->mesh_n};
    for (int i = 0; i < 2; ++i) {
        for (auto& a : *lists[i]) {
            float ms = 0.0f;
            KIFI_CUDA(cudaEventSynchronize(a[1]));
            KIFI_CUDA(cudaEventElapsedTime(&ms, a[0], a[1]));
            *acc[i] += ms;
            ++*cnt[i];
            p->ev_pool.push_back(a[0]);
            p->ev_pool.push_back(a[1]);
        }
        lists[i]->clear();
        if (out_ms) out_ms[i] = *cnt[i] ? *acc[i] / *cnt[i] : 0.0;
        if (out_counts) out_counts[i] = *cnt[i];
        *acc[i] = 0.0;
        *cnt[i] = 0;
    }
    return KIFI_OK;
}

kifi_status kifi_pipeline_set_graphs(kifi_pipeline* p, int on) {
    if (!p) return fail(KIFI_ERR_INVALID_ARGUMENT, "null pipeline");
    if (on && p->closed) return fail(KIFI_ERR_UNSUPPORTED, "graphs are not offered in closed-loop mode");
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

kifi_status kifi_pipeline_mesh_stats(kifi_pipeline* p, long long* meshes, long long* reemitted) {
    if (!p) return fail(KIFI_ERR_INVALID_ARGUMENT, "null pipeline");
    if (meshes) *meshes = p->meshes;
    if (reemitted) *reemitted = p->mesh_reemits;
    return KIFI_OK;
}

}  // extern "C"
