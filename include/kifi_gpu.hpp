// kifi_gpu.hpp -- header-only C++ classes with the signatures of the
// reference's fusion-path classes, implemented over the C ABI of
// kifi_gpu.h.  They replace
//
//   kifi::Volume      KinectFission/kifi/Volume.h:12-51
//   kifi::Integrator  KinectFission/kifi/Integrator.h:13-50 (Integrate)
//   kifi::Mesher      KinectFission/kifi/Mesher.h:14-18     (both Mesh overloads)
//   kifi::ICP         KinectFission/kifi/ICP.h:15-27        (Align)
//   kifi::Renderer    KinectFission/kifi/Renderer.h:23-29   (Bin)
//
// and keep using the reference's own value types (util::vector2d,
// util::float3, util::float4x4, kifi::Voxel, kifi::DepthSensorParams).  A
// translation unit includes this header instead of the reference's
// Volume.h / Integrator.h / Mesher.h / ICP.h / Renderer.h, with the
// reference's source tree on the include path for the util headers.
//
// Differences a caller can see:
//  * the volume lives in GPU memory; Volume::Data() returns a host copy,
//    refreshed on every call (keys and voxels exactly as the reference's
//    flat_map holds them);
//  * errors throw kifi::gpu_error (the reference asserts);
//  * ICP::Align runs `iterations` AlignSteps (the reference fixes 4).
#pragma once

#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include <kifi/DepthSensorParams.h>
#include <kifi/Voxel.h>
#include <kifi/util/flat_map.h>
#include <kifi/util/math.h>
#include <kifi/util/vector2d.h>

#include "kifi_gpu.h"

namespace kifi {

struct gpu_error : std::runtime_error {
    kifi_status status;
    gpu_error(kifi_status s, const char* what)
        : std::runtime_error(std::string(what) + ": " + kifi_status_string(s) + " (" + kifi_last_error() + ")"),
          status(s) {}
};

namespace gpu_detail {
inline void check(kifi_status s, const char* what) {
    if (s != KIFI_OK) throw gpu_error(s, what);
}
// float4x4 is four float4 columns (util/math.h:59-61): kifi's column order
inline void to_array(util::float4x4 const& m, float out[16]) { std::memcpy(out, &m, 64); }
inline util::float4x4 from_array(const float in[16]) {
    util::float4x4 m;
    std::memcpy(&m, in, 64);
    return m;
}
inline kifi_camera camera(DepthSensorParams const& p) {
    kifi_camera c;
    c.width = p.ResolutionPixels().x;
    c.height = p.ResolutionPixels().y;
    c.fx = p.FocalLengthPixels().x;
    c.fy = p.FocalLengthPixels().y;
    c.cx = p.PrincipalPointPixels().x;
    c.cy = p.PrincipalPointPixels().y;
    c.znear_m = p.SensibleRangeMeters().x;
    c.zfar_m = p.SensibleRangeMeters().y;
    return c;
}
}  // namespace gpu_detail

class Volume {
public:
    Volume(int resolution, float sideLength, float truncationMargin, int device = 0)
        : m_res(resolution), m_sideLen(sideLength), m_truncMargin(truncationMargin) {
        kifi_volume_desc d;
        std::memset(&d, 0, sizeof d);
        d.resolution = resolution;
        d.side_length_m = sideLength;
        d.truncation_m = truncationMargin;
        d.device = device;
        gpu_detail::check(kifi_volume_create(&d, &m_vol), "Volume");
    }
    ~Volume() { kifi_volume_destroy(m_vol); }
    Volume(Volume const&) = delete;
    Volume& operator=(Volume const&) = delete;

    int Resolution() const { return m_res; }
    float VoxelLength() const { return m_sideLen / m_res; }
    float SideLength() const { return m_sideLen; }
    float TruncationMargin() const { return m_truncMargin; }
    util::float4 Minimum() const {
        const float m = -0.5f * m_sideLen;
        return util::float4(m, m, m, 1.0f);
    }
    util::float4 Maximum() const {
        const float m = 0.5f * m_sideLen;
        return util::float4(m, m, m, 1.0f);
    }

    // Volume::Data (Volume.h:29-30): a host copy of the resident voxels
    util::flat_map<unsigned, Voxel>& Data() {
        size_t n = 0;
        gpu_detail::check(kifi_volume_size(m_vol, &n), "Volume::Data");
        std::vector<unsigned> keys(n + 1);
        std::vector<Voxel> voxels(n + 1);
        size_t got = 0;
        gpu_detail::check(kifi_volume_export(m_vol, keys.data(), reinterpret_cast<float*>(voxels.data()),
                                             n + 1, &got),
                          "Volume::Data");
        m_host.clear();
        m_host.insert(keys.begin(), keys.begin() + got, voxels.begin());
        return m_host;
    }

    kifi_volume* handle() const { return m_vol; }

private:
    kifi_volume* m_vol = nullptr;
    int m_res;
    float m_sideLen, m_truncMargin;
    util::flat_map<unsigned, Voxel> m_host;
};

class Integrator {
public:
    // Integrator::Integrate (Integrator.h:19-26)
    void Integrate(Volume& volume, util::vector2d<float> const& frame, DepthSensorParams const& cameraParams,
                   util::float4x4 const& worldToEye) {
        const kifi_camera cam = gpu_detail::camera(cameraParams);
        if (frame.width() != (size_t)cam.width || frame.height() != (size_t)cam.height)
            throw gpu_error(KIFI_ERR_INVALID_ARGUMENT, "Integrator::Integrate: frame size");
        float w2e[16];
        gpu_detail::to_array(worldToEye, w2e);
        gpu_detail::check(kifi_integrate_f32(volume.handle(), frame.data(), &cam, w2e), "Integrator::Integrate");
    }
};

class Mesher {
public:
    // Mesher::Mesh (Mesher.h:17)
    void Mesh(Volume const& volume, std::vector<util::float3>& outVertices) {
        std::vector<unsigned> none;
        run(volume, 0, outVertices, none);
    }
    // Mesher::Mesh (Mesher.h:18)
    void Mesh(Volume const& volume, std::vector<util::float3>& outVertices, std::vector<unsigned>& outIndices) {
        run(volume, 1, outVertices, outIndices);
    }

private:
    static void run(Volume const& volume, int with_indices, std::vector<util::float3>& v,
                    std::vector<unsigned>& idx) {
        size_t nv = 0, ni = 0;
        kifi_status s = kifi_mesh(volume.handle(), with_indices, nullptr, 0, nullptr, 0, &nv, &ni);
        if (s != KIFI_OK && s != KIFI_ERR_CAPACITY) gpu_detail::check(s, "Mesher::Mesh");
        v.resize(nv);
        idx.resize(with_indices ? ni : 0);
        gpu_detail::check(kifi_mesh(volume.handle(), with_indices, reinterpret_cast<float*>(v.data()), nv,
                                    with_indices ? idx.data() : nullptr, with_indices ? ni : 0, &nv, &ni),
                          "Mesher::Mesh");
    }
};

class ICP {
public:
    explicit ICP(int device = 0, int iterations = 4) : m_iterations(iterations) {
        gpu_detail::check(kifi_icp_create(device, nullptr, &m_icp), "ICP");
    }
    ~ICP() { kifi_icp_destroy(m_icp); }
    ICP(ICP const&) = delete;
    ICP& operator=(ICP const&) = delete;

    // ICP::Align (ICP.h:18-27): eye-to-world poses, as ICP.cpp:9-31 uses them
    util::float4x4 Align(util::vector2d<float> const& rawDepthMap, util::float4x4 const& rawDepthMapEyeToWorldGuess,
                         util::vector2d<util::float3> const& synthDepthBuffer,
                         util::float4x4 const& synthDepthBufferEyeToWorld, DepthSensorParams const& cameraParams) {
        const kifi_camera cam = gpu_detail::camera(cameraParams);
        float guess[16], synth[16], out[16];
        gpu_detail::to_array(rawDepthMapEyeToWorldGuess, guess);
        gpu_detail::to_array(synthDepthBufferEyeToWorld, synth);
        gpu_detail::check(kifi_icp_set_target(m_icp, reinterpret_cast<const float*>(synthDepthBuffer.data()),
                                              (int)synthDepthBuffer.width(), (int)synthDepthBuffer.height(), synth),
                          "ICP::Align");
        gpu_detail::check(kifi_icp_align(m_icp, rawDepthMap.data(), &cam, guess, m_iterations, out), "ICP::Align");
        return gpu_detail::from_array(out);
    }

private:
    kifi_icp* m_icp = nullptr;
    int m_iterations;
};

class Renderer {
public:
    // Renderer::Bin (Renderer.h:23-29)
    void Bin(std::vector<util::float3> const& pointCloud, util::float4x4 const& worldToClip,
             util::vector2d<util::float3>& outPointBuffer) {
        float w2c[16];
        gpu_detail::to_array(worldToClip, w2c);
        gpu_detail::check(kifi_bin(reinterpret_cast<const float*>(pointCloud.data()), pointCloud.size(), w2c,
                                   reinterpret_cast<float*>(outPointBuffer.data()), (int)outPointBuffer.width(),
                                   (int)outPointBuffer.height()),
                          "Renderer::Bin");
    }
};

}  // namespace kifi
