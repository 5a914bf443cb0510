// The reference's Integrator / Mesher unit-test case (KinectFission/
// UnitTests/Integrator.cpp:19-53, UnitTests/Mesher.cpp:21-50) written against
// include/kifi_gpu.hpp: Volume(256, 2.0, 0.02), KinectParams(640x480, Far),
// one frame.  Reads the frame (640*480 float metres) and its world-to-eye
// pose (16 floats, kifi column order) from the file named by argv[1] and
// prints "voxels verts_only verts indices".
#include <cstdio>
#include <vector>

#include "kifi_gpu.hpp"

using namespace kifi;

int main(int argc, char** argv) {
    if (argc < 2) return 2;
    std::FILE* f = std::fopen(argv[1], "rb");
    if (!f) return 3;
    util::vector2d<float> frame(640, 480);
    float view[16];
    const bool ok = std::fread(frame.data(), 4, 640 * 480, f) == 640 * 480 && std::fread(view, 4, 16, f) == 16;
    std::fclose(f);
    if (!ok) return 4;
    util::float4x4 worldToEye;
    std::memcpy(&worldToEye, view, 64);
    try {
        Volume volume(256, 2.0f, 0.02f);
        Integrator integrator;
        integrator.Integrate(volume, frame,
                             DepthSensorParams::KinectParams(KinectDepthSensorResolution640x480, KinectDepthSensorModeFar),
                             worldToEye);
        Mesher mesher;
        std::vector<util::float3> v0, v1;
        std::vector<unsigned> idx;
        mesher.Mesh(volume, v0);
        mesher.Mesh(volume, v1, idx);
        std::printf("%zu %zu %zu %zu\n", volume.Data().size(), v0.size(), v1.size(), idx.size());
    } catch (gpu_error const& e) {
        std::fprintf(stderr, "%s\n", e.what());
        return 1;
    }
    return 0;
}
