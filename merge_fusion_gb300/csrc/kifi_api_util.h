// kifi_api_util.h -- error plumbing shared by the host-side ABI translation
// units (kifi_api.cu, kifi_api_icp.cu).
#pragma once

#include <string>

#include "kifi_internal.h"

namespace kifi {

extern thread_local std::string g_last_error;

// records `what` as the thread's last error and returns s
kifi_status fail(kifi_status s, const char* what);
// maps a CUDA error to a status and records it
kifi_status cuda_fail(cudaError_t e, const char* what);
kifi_status launch_shape(int device, LaunchShape* ls);
bool camera_ok(const kifi_camera* c);

constexpr size_t kPad = 64;  // slack elements behind every device array

inline Mat4 load_mat(const float* m) {
    Mat4 r;
    for (int i = 0; i < 16; ++i) r.m[i] = m[i];
    return r;
}

}  // namespace kifi

#define KIFI_CUDA(call)                                                 \
    do {                                                                \
        cudaError_t kifi_e_ = (call);                                   \
        if (kifi_e_ != cudaSuccess) return ::kifi::cuda_fail(kifi_e_, #call); \
    } while (0)
