// kifi_api_util.h -- error plumbing shared by the host-side ABI translation
// units (kifi_api.cu, kifi_api_icp.cu).
#pragma once

#include <array>
#include <string>
#include <vector>

#include "kifi_internal.h"

namespace kifi {

extern thread_local std::string g_last_error;

// records `what` as the thread's last error and returns s
kifi_status fail(kifi_status s, const char* what);
// maps a CUDA error to a status and records it
kifi_status cuda_fail(cudaError_t e, const char* what);
kifi_status launch_shape(int device, LaunchShape* ls);
// Fusion launch shape for a volume whose frames are also tracked on a
// higher-priority stream: many CTAs per SM that each finish quickly, so the
// tracking kernels reclaim SMs between CTAs instead of waiting for
// persistent fusion CTAs to drain.
void tracking_launch_shape(LaunchShape* ls);

bool camera_ok(const kifi_camera* c);

constexpr size_t kPad = 64;  // slack elements behind every device array

inline Mat4 load_mat(const float* m) {
    Mat4 r;
    for (int i = 0; i < 16; ++i) r.m[i] = m[i];
    return r;
}

}  // namespace kifi

// A volume handle (include/kifi_gpu.h): device state of one kifi::Volume.
// stage timer events per frame: start, after splat+emit, after the sort,
// after the merge partition, after the merge+update
constexpr int kStageEvents = 5;

struct kifi_volume {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    kifi::Geom g{};
    kifi::DeviceCtl* ctl = nullptr;       // device
    kifi::DeviceCtl* ctl_host = nullptr;  // pinned mirror for read-backs
    kifi::VolumeBuffers vb{};
    kifi::SortScratch ss{};
    kifi::MeshScratch ms{};
    // ls.beside_tracking: fusion beside a tracking stream, grids of
    // short-lived CTAs (see tracking_launch_shape), also the only shapes the
    // autotuner tries
    kifi::LaunchShape ls{};
    void* depth_dev = nullptr;
    size_t depth_dev_bytes = 0;
    void* depth_pinned = nullptr;
    size_t depth_pinned_bytes = 0;
    size_t n_upper = 0;  // upper bound of the resident count of queued work
    float* mesh_verts = nullptr;
    size_t mesh_verts_cap = 0;
    uint32_t* mesh_idx = nullptr;
    size_t mesh_idx_cap = 0;
    kifi::MeshCounts ctl_host_mesh{};
    bool mesh_counts_valid = false;
    // stage timers (kifi_volume_set_profiling): per integrated frame four
    // events around splat+emit, sort and merge+update
    bool profiling = false;
    std::vector<cudaEvent_t> event_pool;
    std::vector<std::array<cudaEvent_t, kStageEvents>> pending;
    // kifi_mesh* timers: before the row directory, after it, after the
    // classification, after the scan, after the emission
    std::vector<std::array<cudaEvent_t, 5>> mesh_pending;
};

// integrate entry shared by the ABI translation units: enqueues one frame
// (device depth) on the volume's stream, growing buffers first when needed.
// Host-side capacity checks (and growth) a frame of `cam` may need, done
// ahead of enqueueing it -- nothing in kifi_volume_enqueue_frame then waits.
kifi_status kifi_volume_prepare_frame(kifi_volume* v, const kifi_camera* cam);
kifi_status kifi_icp_prepare_frame(kifi_icp* c, const kifi_camera* cam);
// whether the context's alignments publish their final pose to its mailbox,
// and that pose of the latest alignment, polled (kifi_api_icp.cu)
void icp_publish_pose(kifi_icp* c, bool on);
kifi_status icp_wait_pose(kifi_icp* c, float out_eye_to_world[16]);
// batched alignment (kifi_api_batch.cu): one pair's arguments, and the next target's slot
kifi_status kifi_icp_batch_args(kifi_icp* c, const void* depth_dev, const kifi_camera* cam, kifi::IcpArgs* a,
                                kifi::IcpState** st, int iterations);
kifi_status kifi_icp_batch_target(kifi_icp* c, const kifi_camera* cam, const float* eye_to_world, float4** out);
kifi_status kifi_volume_enqueue_frame(kifi_volume* v, const void* depth_dev, bool u16,
                                      const kifi_camera* cam, const float* world_to_eye);

#define KIFI_CUDA(call)                                                 \
    do {                                                                \
        cudaError_t kifi_e_ = (call);                                   \
        if (kifi_e_ != cudaSuccess) return ::kifi::cuda_fail(kifi_e_, #call); \
    } while (0)
