// kifi_api_batch.cu -- many independent depth sequences fused and tracked
// together (include/kifi_gpu.h, kifi_batch_*; no counterpart in the
// reference, which runs one kifi::Pipeline at a time).
//
// A batch holds one volume and one ICP context per scene.  A step takes one
// frame for every scene that still has frames and enqueues each stage once
// for all of them: frame set-up, splat + dilation + emission, the sort
// (prepare, histogram, digit passes), the merge partition and the fused
// merge + TSDF update on the fusion stream; the ICP begin, one launch per
// AlignStep and the next targets' back-projection on the tracking stream.
// Each launch shares its CTAs out among the scenes (a block map per stage,
// sized by the scene's frame or volume); a scene's CTAs run the
// single-volume kernel body on that scene's arguments, read from a device
// table uploaded once per step.  Scenes with 32-bit and 64-bit keys are two
// groups, one fusion launch sequence each.  With kifi_batch_set_persistent a
// group's fusion is instead one persistent launch whose CTAs walk a device
// work queue of (stage, scene, chunk) items (k_fuse_queue, kifi_integrate.cu).
// Results equal the scenes run one by one (the same kernel bodies on the
// same inputs).
//
// Tracking is the open-loop pipeline's: each frame against the previous
// frame's back-projection, from the previous given pose.
#include <algorithm>
#include <cstring>
#include <new>
#include <vector>

#include "kifi_api_util.h"

using namespace kifi;

namespace {

constexpr size_t kAlign = 256;
size_t up(size_t x) { return (x + kAlign - 1) / kAlign * kAlign; }
unsigned int cdiv(size_t a, size_t b) { return (unsigned int)((a + b - 1) / b); }

// the digit passes of a volume's sort (kifi_sort.cu's rule for key_bits = 3 kb)
int sort_passes(int key_bytes, int kb) {
    int p = (3 * kb + 7) / 8;
    p += p & 1;
    if (p < 2) p = 2;
    const int cap = key_bytes == 8 ? kSortMaxPasses : 4;
    return p > cap ? cap : p;
}

}  // namespace

struct kifi_batch {
    int device = 0;
    int n = 0;
    std::vector<kifi_pipeline_desc> desc;
    std::vector<kifi_volume*> vol;
    std::vector<kifi_icp*> icp;
    std::vector<float> prev_e2w;  // 16 per scene
    std::vector<char> have_prev;
    cudaStream_t fs = nullptr, ts = nullptr;  // fusion, tracking
    // per-step argument tables, two slots used by alternate steps
    void* host[2] = {nullptr, nullptr};
    void* dev[2] = {nullptr, nullptr};
    size_t bytes[2] = {0, 0};
    cudaEvent_t uploaded[2] = {nullptr, nullptr};  // the slot's host table has been copied
    cudaEvent_t tracked[2] = {nullptr, nullptr};   // the slot's step no longer reads its device table
    long long steps = 0;
    // fusion as one persistent launch over a device work queue
    // (kifi_batch_set_persistent), with this many CTAs per SM
    bool persistent = false;
    int queue_ctas_per_sm = 1;
    // step timers
    bool profiling = false;
    std::vector<cudaEvent_t> ev_pool;
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> pending;
    std::vector<float> step_ms;
};

namespace {

kifi_status take_event(kifi_batch* b, cudaEvent_t* e) {
    if (b->ev_pool.empty()) {
        cudaEvent_t x;
        KIFI_CUDA(cudaEventCreate(&x));
        b->ev_pool.push_back(x);
    }
    *e = b->ev_pool.back();
    b->ev_pool.pop_back();
    return KIFI_OK;
}

// a group of scenes that share a key width: their jobs and block maps
struct Group {
    std::vector<int> scenes;
    std::vector<FuseJob> jobs;
    std::vector<unsigned int> splat, hist, pass, part, merge;  // first[] of each map
    int key_bytes = 4, passes = 0;
};

void add_share(std::vector<unsigned int>& first, unsigned int blocks) {
    if (first.empty()) first.push_back(0u);
    first.push_back(first.back() + (blocks ? blocks : 1u));
}

}  // namespace

extern "C" {

kifi_status kifi_batch_create(const kifi_pipeline_desc* descs, int n, kifi_batch** out) {
    if (!descs || n <= 0 || !out) return fail(KIFI_ERR_INVALID_ARGUMENT, "bad argument");
    *out = nullptr;
    for (int i = 0; i < n; ++i) {
        const kifi_pipeline_desc& d = descs[i];
        if (!camera_ok(&d.camera) || d.icp_iterations < 0 || d.icp_iterations > kIcpMaxStats)
            return fail(KIFI_ERR_INVALID_ARGUMENT, "bad scene description");
        if (d.mesh_every != 0 || d.closed_loop != 0)
            return fail(KIFI_ERR_UNSUPPORTED, "a batch neither meshes nor tracks closed loop");
        if (d.device != descs[0].device) return fail(KIFI_ERR_INVALID_ARGUMENT, "a batch lives on one device");
    }
    kifi_batch* b = new (std::nothrow) kifi_batch();
    if (!b) return fail(KIFI_ERR_OUT_OF_MEMORY, "host allocation");
    b->device = descs[0].device;
    b->n = n;
    b->desc.assign(descs, descs + n);
    b->prev_e2w.assign((size_t)n * 16, 0.0f);
    b->have_prev.assign(n, 0);
    cudaError_t e = cudaSetDevice(b->device);
    int lowest = 0, greatest = 0;
    if (!e) e = cudaDeviceGetStreamPriorityRange(&lowest, &greatest);
    if (!e) e = cudaStreamCreateWithFlags(&b->fs, cudaStreamNonBlocking);
    if (!e) e = cudaStreamCreateWithPriority(&b->ts, cudaStreamNonBlocking, greatest);
    for (int k = 0; k < 2 && !e; ++k) {
        e = cudaEventCreateWithFlags(&b->uploaded[k], cudaEventDisableTiming);
        if (!e) e = cudaEventCreateWithFlags(&b->tracked[k], cudaEventDisableTiming);
    }
    if (e) {
        kifi_batch_destroy(b);
        return cuda_fail(e, "batch streams");
    }
    b->vol.assign(n, nullptr);
    b->icp.assign(n, nullptr);
    for (int i = 0; i < n; ++i) {
        kifi_volume_desc vd{};
        vd.resolution = descs[i].resolution;
        vd.side_length_m = descs[i].side_length_m;
        vd.truncation_m = descs[i].truncation_m;
        vd.initial_capacity = descs[i].initial_capacity;
        vd.device = b->device;
        vd.stream = b->fs;  // every volume's own work (growth, exports) is ordered with the batch's fusion
        vd.key_bits = descs[i].key_bits;
        kifi_status s = kifi_volume_create(&vd, &b->vol[i]);
        if (!s) s = kifi_icp_create(b->device, b->ts, &b->icp[i]);
        if (s) {
            kifi_batch_destroy(b);
            return s;
        }
    }
    *out = b;
    return KIFI_OK;
}

kifi_status kifi_batch_destroy(kifi_batch* b) {
    if (!b) return KIFI_OK;
    cudaSetDevice(b->device);
    if (b->fs) cudaStreamSynchronize(b->fs);
    if (b->ts) cudaStreamSynchronize(b->ts);
    for (kifi_icp* c : b->icp) kifi_icp_destroy(c);
    for (kifi_volume* v : b->vol) kifi_volume_destroy(v);
    for (int k = 0; k < 2; ++k) {
        cudaFreeHost(b->host[k]);
        cudaFree(b->dev[k]);
        if (b->uploaded[k]) cudaEventDestroy(b->uploaded[k]);
        if (b->tracked[k]) cudaEventDestroy(b->tracked[k]);
    }
    for (auto& p : b->pending) {
        cudaEventDestroy(p.first);
        cudaEventDestroy(p.second);
    }
    for (cudaEvent_t x : b->ev_pool) cudaEventDestroy(x);
    if (b->fs) cudaStreamDestroy(b->fs);
    if (b->ts) cudaStreamDestroy(b->ts);
    delete b;
    return KIFI_OK;
}

kifi_volume* kifi_batch_volume(kifi_batch* b, int scene) {
    return b && scene >= 0 && scene < b->n ? b->vol[scene] : nullptr;
}

void* kifi_batch_stream(kifi_batch* b) { return b ? (void*)b->fs : nullptr; }

kifi_status kifi_batch_step_device(kifi_batch* b, const void* const* depth_dev, const float* world_to_eye) {
    if (!b || !depth_dev || !world_to_eye) return fail(KIFI_ERR_INVALID_ARGUMENT, "bad argument");
    KIFI_CUDA(cudaSetDevice(b->device));
    const int k = (int)(b->steps & 1);
    // the host table of this slot may be rewritten once its last upload is done
    KIFI_CUDA(cudaEventSynchronize(b->uploaded[k]));
    Group grp[2];  // 32-bit keys, 64-bit keys
    grp[1].key_bytes = 8;
    std::vector<IcpJob> ijobs;
    std::vector<unsigned int> imap;
    std::vector<BackprojectJob> bjobs;
    std::vector<unsigned int> bmap;
    std::vector<int> tracked_scenes;
    for (int i = 0; i < b->n; ++i) {
        if (!depth_dev[i]) continue;
        kifi_volume* v = b->vol[i];
        const kifi_pipeline_desc& d = b->desc[i];
        const kifi_camera& cam = d.camera;
        const size_t P = (size_t)cam.width * cam.height;
        kifi_status s = kifi_volume_prepare_frame(v, &cam);
        if (s) return s;
        Group& g = grp[v->vb.key_bytes == 8 ? 1 : 0];
        const Mat4 w2e = load_mat(world_to_eye + 16 * i);
        FuseJob j{};
        j.ctl = v->ctl;
        j.g = v->g;
        j.vb = v->vb;
        j.ss = v->ss;
        j.ss.status = &v->ctl->status;
        sort_limits(&j.ss);
        j.depth = depth_dev[i];
        j.fc = make_frame_const(cam, w2e, v->g.res);
        j.fc.z_bounded = clip_z_bounded(j.fc.world_to_clip, v->g.side);
        j.max_tiles = (unsigned int)merge_max_tiles(v->vb, v->vb.cap);
        g.scenes.push_back(i);
        g.jobs.push_back(j);
        g.passes = std::max(g.passes, sort_passes(v->vb.key_bytes, v->g.kb));
        add_share(g.splat, cdiv(P, 1024));
        add_share(g.hist, cdiv(P, 4096));
        add_share(g.pass, cdiv(P, 2048));
        add_share(g.part, cdiv(j.max_tiles + 1, 256));
        // the merge's CTAs: about four 2048-voxel tiles each, of the resident bound
        add_share(g.merge, cdiv(std::min(v->n_upper + 8 * P, v->vb.cap), 8192));
        v->n_upper += 8 * P;
        // tracking against the previous frame's back-projection
        if (d.icp_iterations > 0) {
            if (b->have_prev[i]) {
                IcpJob ij{};
                if ((s = kifi_icp_batch_args(b->icp[i], depth_dev[i], &cam, &ij.a, &ij.st, d.icp_iterations)))
                    return s;
                std::memcpy(ij.guess.m, &b->prev_e2w[16 * i], 64);
                ijobs.push_back(ij);
                add_share(imap, (unsigned int)icp_tiles(cam.width, cam.height));
                tracked_scenes.push_back(i);
            }
            const Mat4 e2w = invert_transform(w2e);
            BackprojectJob bj{};
            bj.depth = depth_dev[i];
            bj.width = cam.width;
            bj.height = cam.height;
            bj.fl_inv_x = fdiv(1.0f, cam.fx);
            bj.fl_inv_y = fdiv(1.0f, cam.fy);
            bj.pp_x = fmul(fsub(0.5f, cam.cx), bj.fl_inv_x);
            bj.pp_y = fmul(fsub(cam.cy, 0.5f), bj.fl_inv_y);
            bj.e2w = e2w;
            if ((s = kifi_icp_batch_target(b->icp[i], &cam, e2w.m, &bj.out))) return s;
            bjobs.push_back(bj);
            add_share(bmap, cdiv(P, 256 * 8));
        }
    }
    // every batch uses the same iteration count for its tracked scenes
    int iters = 0;
    for (int i : tracked_scenes) iters = std::max(iters, b->desc[i].icp_iterations);
    for (int i : tracked_scenes)
        if (b->desc[i].icp_iterations != iters)
            return fail(KIFI_ERR_UNSUPPORTED, "the scenes of a batch track with one iteration count");

    // one table: both groups' jobs and maps (and, for the persistent fusion,
    // the queue counter and per-scene stage counts, zero), the ICP jobs and
    // map, the back-projections and map
    size_t off = 0;
    size_t o_jobs[2], o_maps[2][5], o_queue[2] = {0, 0}, queue_words[2] = {0, 0}, o_ij = 0, o_im = 0, o_bj = 0,
                                                         o_bm = 0;
    for (int gi = 0; gi < 2; ++gi) {
        o_jobs[gi] = off;
        off = up(off + grp[gi].jobs.size() * sizeof(FuseJob));
        for (int m = 0; m < 5; ++m) {
            o_maps[gi][m] = off;
            off = up(off + (grp[gi].jobs.size() + 1) * sizeof(unsigned int));
        }
        if (b->persistent && !grp[gi].jobs.empty()) {
            o_queue[gi] = off;
            queue_words[gi] = 1 + grp[gi].jobs.size() * (size_t)(5 + grp[gi].passes);
            off = up(off + queue_words[gi] * sizeof(unsigned int));
        }
    }
    o_ij = off;
    off = up(off + ijobs.size() * sizeof(IcpJob));
    o_im = off;
    off = up(off + (ijobs.size() + 1) * sizeof(unsigned int));
    o_bj = off;
    off = up(off + bjobs.size() * sizeof(BackprojectJob));
    o_bm = off;
    off = up(off + (bjobs.size() + 1) * sizeof(unsigned int));
    if (off > b->bytes[k]) {
        // the slot's device table may still be read by the step two back
        KIFI_CUDA(cudaStreamSynchronize(b->fs));
        KIFI_CUDA(cudaStreamSynchronize(b->ts));
        cudaFreeHost(b->host[k]);
        cudaFree(b->dev[k]);
        b->host[k] = b->dev[k] = nullptr;
        b->bytes[k] = 0;
        const size_t want = off + off / 2;
        KIFI_CUDA(cudaMallocHost(&b->host[k], want));
        KIFI_CUDA(cudaMalloc(&b->dev[k], want));
        b->bytes[k] = want;
    }
    unsigned char* h = (unsigned char*)b->host[k];
    unsigned char* dv = (unsigned char*)b->dev[k];
    for (int gi = 0; gi < 2; ++gi) {
        Group& g = grp[gi];
        if (g.jobs.empty()) continue;
        std::memcpy(h + o_jobs[gi], g.jobs.data(), g.jobs.size() * sizeof(FuseJob));
        std::vector<unsigned int>* maps[5] = {&g.splat, &g.hist, &g.pass, &g.part, &g.merge};
        for (int m = 0; m < 5; ++m) std::memcpy(h + o_maps[gi][m], maps[m]->data(), maps[m]->size() * 4);
        if (queue_words[gi]) std::memset(h + o_queue[gi], 0, queue_words[gi] * sizeof(unsigned int));
    }
    if (!ijobs.empty()) {
        std::memcpy(h + o_ij, ijobs.data(), ijobs.size() * sizeof(IcpJob));
        std::memcpy(h + o_im, imap.data(), imap.size() * 4);
    }
    if (!bjobs.empty()) {
        std::memcpy(h + o_bj, bjobs.data(), bjobs.size() * sizeof(BackprojectJob));
        std::memcpy(h + o_bm, bmap.data(), bmap.size() * 4);
    }
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (b->profiling) {
        kifi_status s = take_event(b, &e0);
        if (!s) s = take_event(b, &e1);
        if (s) return s;
        KIFI_CUDA(cudaEventRecord(e0, b->fs));
    }
    // the step two back (same slot) must be done reading the device table
    KIFI_CUDA(cudaStreamWaitEvent(b->fs, b->tracked[k], 0));
    KIFI_CUDA(cudaMemcpyAsync(dv, h, off, cudaMemcpyHostToDevice, b->fs));
    KIFI_CUDA(cudaEventRecord(b->uploaded[k], b->fs));
    KIFI_CUDA(cudaStreamWaitEvent(b->ts, b->uploaded[k], 0));
    // tracking first: the step's critical path, on the higher-priority stream
    if (!ijobs.empty()) {
        BlockMap im{(const unsigned int*)(dv + o_im), (int)ijobs.size(), imap.back()};
        KIFI_CUDA(icp_align_batch_enqueue((const IcpJob*)(dv + o_ij), (int)ijobs.size(), im, iters, b->ts));
    }
    if (!bjobs.empty()) {
        BlockMap bm{(const unsigned int*)(dv + o_bm), (int)bjobs.size(), bmap.back()};
        KIFI_CUDA(backproject_batch_enqueue((const BackprojectJob*)(dv + o_bj), (int)bjobs.size(), bm, b->ts));
    }
    for (int gi = 0; gi < 2; ++gi) {
        Group& g = grp[gi];
        if (g.jobs.empty()) continue;
        const int n = (int)g.jobs.size();
        auto map = [&](int m, const std::vector<unsigned int>& f) {
            return BlockMap{(const unsigned int*)(dv + o_maps[gi][m]), n, f.back()};
        };
        FuseMaps fm{map(0, g.splat), map(1, g.hist), map(2, g.pass), map(3, g.part), map(4, g.merge)};
        if (b->persistent) {
            FuseQueuePlan q;
            q.n = n;
            q.passes = g.passes;
            q.stages = 5 + g.passes;
            const BlockMap* bm[5] = {&fm.splat, &fm.hist, &fm.pass, &fm.partition, &fm.merge};
            for (int m = 0; m < 5; ++m) q.maps[m] = *bm[m];
            q.first[0] = 0u;
            for (int k = 0; k < q.stages; ++k)
                q.first[k + 1] = q.first[k] + (k == 0 ? (unsigned int)n : q.maps[fuse_stage_map(k, q.passes)].grid);
            unsigned int* qw = (unsigned int*)(dv + o_queue[gi]);
            const int ctas = b->vol[g.scenes[0]]->ls.sms * b->queue_ctas_per_sm;
            KIFI_CUDA(integrate_queue_enqueue((const FuseJob*)(dv + o_jobs[gi]), g.key_bytes, q, qw, qw + 1, ctas,
                                              b->fs));
        } else {
            KIFI_CUDA(
                integrate_batch_enqueue((const FuseJob*)(dv + o_jobs[gi]), n, g.key_bytes, g.passes, fm, b->fs));
        }
    }
    KIFI_CUDA(cudaEventRecord(b->tracked[k], b->ts));
    if (e0) {
        KIFI_CUDA(cudaStreamWaitEvent(b->fs, b->tracked[k], 0));
        KIFI_CUDA(cudaEventRecord(e1, b->fs));
        b->pending.emplace_back(e0, e1);
    }
    for (int i = 0; i < b->n; ++i) {
        if (!depth_dev[i]) continue;
        const Mat4 e2w = invert_transform(load_mat(world_to_eye + 16 * i));
        std::memcpy(&b->prev_e2w[16 * i], e2w.m, 64);
        b->have_prev[i] = 1;
    }
    ++b->steps;
    return KIFI_OK;
}

kifi_status kifi_batch_sync(kifi_batch* b) {
    if (!b) return fail(KIFI_ERR_INVALID_ARGUMENT, "null batch");
    KIFI_CUDA(cudaSetDevice(b->device));
    KIFI_CUDA(cudaStreamSynchronize(b->ts));
    for (kifi_volume* v : b->vol) {
        kifi_status s = kifi_volume_sync(v);  // the fusion stream; reports device errors
        if (s) return s;
    }
    return KIFI_OK;
}

kifi_status kifi_batch_pose(kifi_batch* b, int scene, float out_eye_to_world[16]) {
    if (!b || scene < 0 || scene >= b->n || !out_eye_to_world) return fail(KIFI_ERR_INVALID_ARGUMENT, "bad argument");
    KIFI_CUDA(cudaSetDevice(b->device));
    if (!b->have_prev[scene]) return fail(KIFI_ERR_INVALID_ARGUMENT, "the scene has no frame yet");
    // the tracked pose once the scene has been aligned; before that the given one
    if (b->desc[scene].icp_iterations > 0) {
        int iters = 0;
        kifi_status s = kifi_icp_result(b->icp[scene], out_eye_to_world, nullptr, nullptr, nullptr, 0, &iters);
        if (s) return s;
        if (iters > 0) return KIFI_OK;
    }
    std::memcpy(out_eye_to_world, &b->prev_e2w[16 * scene], 64);
    return KIFI_OK;
}

kifi_status kifi_batch_set_persistent(kifi_batch* b, int on, int ctas_per_sm) {
    if (!b || ctas_per_sm < 0 || ctas_per_sm > 32) return fail(KIFI_ERR_INVALID_ARGUMENT, "bad argument");
    b->persistent = on != 0;
    b->queue_ctas_per_sm = ctas_per_sm > 0 ? ctas_per_sm : 1;
    return KIFI_OK;
}

kifi_status kifi_batch_set_profiling(kifi_batch* b, int on) {
    if (!b) return fail(KIFI_ERR_INVALID_ARGUMENT, "null batch");
    b->profiling = on != 0;
    return KIFI_OK;
}

kifi_status kifi_batch_step_times(kifi_batch* b, float* out_ms, int capacity, int* steps) {
    if (!b || !steps) return fail(KIFI_ERR_INVALID_ARGUMENT, "bad argument");
    KIFI_CUDA(cudaSetDevice(b->device));
    for (auto& p : b->pending) {
        float ms = 0.0f;
        KIFI_CUDA(cudaEventSynchronize(p.second));
        KIFI_CUDA(cudaEventElapsedTime(&ms, p.first, p.second));
        b->step_ms.push_back(ms);
        b->ev_pool.push_back(p.first);
        b->ev_pool.push_back(p.second);
    }
    b->pending.clear();
    *steps = (int)b->step_ms.size();
    for (int i = 0; i < *steps && i < capacity && out_ms; ++i) out_ms[i] = b->step_ms[i];
    b->step_ms.clear();
    return KIFI_OK;
}

}  // extern "C"
