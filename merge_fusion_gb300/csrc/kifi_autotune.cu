// kifi_autotune.cu -- picks the persistent CTA counts of a volume's fusion
// kernels (splat+emit, the sort passes, the merge/update) by measurement.
// No counterpart in the reference.
//
// The kernels' results do not depend on these counts (the emit appends new
// keys in any order and the sort orders them; the merge is partitioned by
// merge path, independent of the grid), so any choice is safe.  The tuner
// snapshots the volume's device state -- control block, the resident key /
// voxel buffer and the occupancy bitmap -- and integrates the same frame
// once per candidate, restoring the snapshot before each run and timing the
// stages with CUDA events.  Stages are varied one at a time around the
// current shape (grids of 1, 2, 4, 8 x the SM count for the splat and the
// sort; 1 or 2 x the occupancy-derived count for the merge), each run
// repeated, the fastest kept per stage.  The volume is restored at the end,
// untouched.  Choices are cached per (device name, resolution, frame size)
// for the process and, when KIFI_AUTOTUNE_CACHE names a file, in that file
// (one line per entry).
#include <algorithm>
#include <array>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "kifi_api_util.h"

using namespace kifi;

namespace {

std::mutex g_mu;
std::map<std::string, LaunchShape> g_cache;
bool g_loaded = false;

std::string cache_key(int device, int res, int key_bits, bool tracking, int w, int h) {
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) {
        cudaGetLastError();
        std::strcpy(prop.name, "unknown");
        prop.multiProcessorCount = 0;
    }
    char buf[512];
    // 30-bit keys of a stand-alone volume keep the key format of earlier caches
    std::snprintf(buf, sizeof buf, "%s|%d|%d|%s%s%dx%d", prop.name, prop.multiProcessorCount, res,
                  key_bits == 64 ? "k64|" : "", tracking ? "trk|" : "", w, h);
    for (char* c = buf; *c; ++c)
        if (*c == ' ') *c = '_';
    return buf;
}

void load_file() {
    if (g_loaded) return;
    g_loaded = true;
    const char* path = std::getenv("KIFI_AUTOTUNE_CACHE");
    if (!path) return;
    std::FILE* f = std::fopen(path, "r");
    if (!f) return;
    char key[400];
    LaunchShape s{};
    while (std::fscanf(f, "%399s %d %d %d %d", key, &s.sms, &s.splat_ctas, &s.sort_ctas, &s.merge_ctas) == 5)
        g_cache[key] = s;
    std::fclose(f);
}

void save_file() {
    const char* path = std::getenv("KIFI_AUTOTUNE_CACHE");
    if (!path) return;
    std::FILE* f = std::fopen(path, "w");
    if (!f) return;
    for (auto& kv : g_cache)
        std::fprintf(f, "%s %d %d %d %d\n", kv.first.c_str(), kv.second.sms, kv.second.splat_ctas,
                     kv.second.sort_ctas, kv.second.merge_ctas);
    std::fclose(f);
}

struct Snapshot {
    void* ctl = nullptr;
    void* keys = nullptr;
    void* vals = nullptr;
    void* bitmap = nullptr;
    ~Snapshot() {
        cudaFree(ctl);
        cudaFree(keys);
        cudaFree(vals);
        cudaFree(bitmap);
    }
};

}  // namespace

extern "C" kifi_status kifi_volume_autotune(kifi_volume* v, const void* depth_dev, int depth_is_u16,
                                            const kifi_camera* cam, const float world_to_eye[16], int force,
                                            int out_ctas[3]) {
    if (!v || !depth_dev || !camera_ok(cam) || !world_to_eye)
        return fail(KIFI_ERR_INVALID_ARGUMENT, "autotune: bad argument");
    KIFI_CUDA(cudaSetDevice(v->device));
    const std::string key =
        cache_key(v->device, v->g.res, 8 * v->vb.key_bytes, v->ls.beside_tracking, cam->width, cam->height);
    {
        std::lock_guard<std::mutex> lock(g_mu);
        load_file();
        auto it = g_cache.find(key);
        if (!force && it != g_cache.end() && it->second.sms == v->ls.sms) {
            const bool beside = v->ls.beside_tracking;  // part of the key, not of the cached counts
            v->ls = it->second;
            v->ls.beside_tracking = beside;
            if (out_ctas) {
                out_ctas[0] = v->ls.splat_ctas;
                out_ctas[1] = v->ls.sort_ctas;
                out_ctas[2] = v->ls.merge_ctas;
            }
            return KIFI_OK;
        }
    }
    kifi_status s = kifi_volume_prepare_frame(v, cam);
    if (s) return s;
    if ((s = kifi_volume_sync(v))) return s;
    const unsigned int cur = v->ctl_host->cur;
    const size_t n = (size_t)v->ctl_host->n[cur];
    Snapshot snap;
    KIFI_CUDA(cudaMalloc(&snap.ctl, sizeof(DeviceCtl)));
    KIFI_CUDA(cudaMalloc(&snap.keys, (n + kPad) * v->vb.key_bytes));
    KIFI_CUDA(cudaMalloc(&snap.vals, (n + kPad) * 8));
    KIFI_CUDA(cudaMalloc(&snap.bitmap, v->vb.bitmap_words * 4));
    cudaStream_t st = v->stream;
    KIFI_CUDA(cudaMemcpyAsync(snap.ctl, v->ctl, sizeof(DeviceCtl), cudaMemcpyDeviceToDevice, st));
    KIFI_CUDA(cudaMemcpyAsync(snap.keys, v->vb.keys[cur], n * v->vb.key_bytes, cudaMemcpyDeviceToDevice, st));
    KIFI_CUDA(cudaMemcpyAsync(snap.vals, v->vb.vals[cur], n * 8, cudaMemcpyDeviceToDevice, st));
    KIFI_CUDA(cudaMemcpyAsync(snap.bitmap, v->vb.bitmap, v->vb.bitmap_words * 4, cudaMemcpyDeviceToDevice, st));
    auto restore = [&]() -> kifi_status {
        KIFI_CUDA(cudaMemcpyAsync(v->ctl, snap.ctl, sizeof(DeviceCtl), cudaMemcpyDeviceToDevice, st));
        KIFI_CUDA(cudaMemcpyAsync(v->vb.keys[cur], snap.keys, n * v->vb.key_bytes, cudaMemcpyDeviceToDevice, st));
        KIFI_CUDA(cudaMemcpyAsync(v->vb.vals[cur], snap.vals, n * 8, cudaMemcpyDeviceToDevice, st));
        KIFI_CUDA(cudaMemcpyAsync(v->vb.bitmap, snap.bitmap, v->vb.bitmap_words * 4, cudaMemcpyDeviceToDevice, st));
        return KIFI_OK;
    };
    const size_t n_upper0 = v->n_upper;
    const bool profiling0 = v->profiling;
    std::vector<std::array<cudaEvent_t, kStageEvents>> pending0;
    pending0.swap(v->pending);
    v->profiling = true;
    // stage times of one frame integrated with shape `ls` (median of 3)
    auto run = [&](const LaunchShape& ls, double out[4]) -> kifi_status {
        std::vector<double> t[4];
        for (int r = 0; r < 3; ++r) {
            kifi_status rs = restore();
            if (rs) return rs;
            v->ls = ls;
            v->n_upper = n_upper0;
            if ((rs = kifi_volume_enqueue_frame(v, depth_dev, depth_is_u16 != 0, cam, world_to_eye))) return rs;
            double ms[4];
            int frames = 0;
            if ((rs = kifi_volume_stage_times(v, ms, &frames))) return rs;
            for (int k = 0; k < 4; ++k) t[k].push_back(ms[k]);
        }
        for (int k = 0; k < 4; ++k) {
            std::sort(t[k].begin(), t[k].end());
            out[k] = t[k][1];
        }
        return KIFI_OK;
    };
    const LaunchShape base = v->ls;
    LaunchShape best = base;
    double bt[4];
    if ((s = run(base, bt))) goto done;
    {
        const int sms = base.sms;
        // Beside a tracking stream only short-lived grids, at least as many CTAs
        // as tracking_launch_shape: the tuner times fusion alone, where fewer,
        // longer-lived CTAs win, but in the pipeline such CTAs hold SMs the
        // higher-priority tracking steps wait for (measured: 1846 against
        // 1948 frames/s with 8/2/16 x the SM count for splat/sort/merge).
        const bool tr = v->ls.beside_tracking;
        const std::vector<int> splat_m = tr ? std::vector<int>{16, 32} : std::vector<int>{1, 2, 4, 8};
        // a sort pass's CTAs leave as soon as the tiles run out, so small grids are candidates too
        const std::vector<int> sort_m = tr ? std::vector<int>{16, 32} : std::vector<int>{1, 2, 4, 8};
        const std::vector<int> merge_m = tr ? std::vector<int>{32, 64} : std::vector<int>{1, 2, 8};
        for (int m : splat_m) {  // splat + emit (stage 0)
            LaunchShape c = best;
            c.splat_ctas = m * sms;
            double t[4];
            if ((s = run(c, t))) goto done;
            if (t[0] < bt[0]) {
                best.splat_ctas = c.splat_ctas;
                bt[0] = t[0];
            }
        }
        for (int m : sort_m) {  // sort passes (stage 1)
            LaunchShape c = best;
            c.sort_ctas = m * sms;
            double t[4];
            if ((s = run(c, t))) goto done;
            if (t[1] < bt[1]) {
                best.sort_ctas = c.sort_ctas;
                bt[1] = t[1];
            }
        }
        for (int m : merge_m) {  // merge + update (stage 3)
            LaunchShape c = best;
            c.merge_ctas = tr ? m * sms : m * base.merge_ctas;
            double t[4];
            if ((s = run(c, t))) goto done;
            if (t[3] < bt[3]) {
                best.merge_ctas = c.merge_ctas;
                bt[3] = t[3];
            }
        }
    }
done:
    {
        const kifi_status rs = restore();
        v->ls = s ? base : best;
        v->n_upper = n_upper0;
        v->profiling = profiling0;
        v->pending.swap(pending0);
        for (auto& ev : pending0)
            for (int k = 0; k < kStageEvents; ++k) v->event_pool.push_back(ev[k]);
        KIFI_CUDA(cudaStreamSynchronize(st));
        if (s) return s;
        if (rs) return rs;
    }
    {
        std::lock_guard<std::mutex> lock(g_mu);
        g_cache[key] = best;
        save_file();
    }
    if (out_ctas) {
        out_ctas[0] = best.splat_ctas;
        out_ctas[1] = best.sort_ctas;
        out_ctas[2] = best.merge_ctas;
    }
    return KIFI_OK;
}
