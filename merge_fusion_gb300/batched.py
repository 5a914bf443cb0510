"""Many independent scenes fused at once: seeded rooms with uneven frame
sizes, voxel sizes and trajectory lengths.  Two ways to run them:

  * batch (default): one kifi_batch -- every step is one launch per stage of
    the path for all scenes, each launch sharing its CTAs out among the
    scenes (kifi_batch_step_device);
  * queue: the same batch with each step's fusion as one persistent launch
    whose CTAs walk a device work queue (kifi_batch_set_persistent);
  * streams: each scene a kifi_pipeline (its own volume, ICP context and
    CUDA streams); every step enqueues the next frame of every scene, so the
    GPU runs the scenes' kernels concurrently.

    python -m merge_fusion_gb300.batched [--scenes 64] [--seed 7] [--mode batch|queue|streams]

Scene i draws its frame size from {320x240, 512x424, 640x480, 1024x848},
its voxel size from {2, 4, 8} mm (truncation 5 voxels; a 4.096 m cube of
2048, 1024 or 512 voxels per axis, so 2 mm scenes use 64-bit keys) and its
trajectory length from [50, 300] frames.  To bound the rendering time a
scene renders at most `unique` frames of its trajectory and plays them
forward and back.  Reported: frames
per second over all scenes and the per-scene step latency (p50, p99), from
CUDA events on each scene's volume and ICP streams."""
import argparse
import ctypes as C
import json
import time

import numpy as np

from . import _lib, scenes
from ._lib import Camera, PipelineDesc, check

SIZES = [(320, 240, 292.5), (512, 424, 365.0), (640, 480, 585.0), (1024, 848, 730.0)]
VOXELS_MM = [2, 4, 8]


def scene_specs(n, seed):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        w, h, f = SIZES[int(rng.integers(len(SIZES)))]
        vox = VOXELS_MM[int(rng.integers(len(VOXELS_MM)))]
        res = {2: 2048, 4: 1024, 8: 512}[vox]
        out.append({"seed": seed * 1000 + i, "width": w, "height": h, "f": f, "voxel_mm": vox, "res": res,
                    "scale": 1.0, "frames": int(rng.integers(50, 301))})
    return out


def frame_order(n_unique, n_frames):
    """Indices 0..n_unique-1 played forward and back until n_frames."""
    cyc = list(range(n_unique)) + list(range(n_unique - 2, 0, -1))
    return [cyc[i % len(cyc)] for i in range(n_frames)]


class Scene:
    def __init__(self, spec, unique, icp_iters, mesh_every, device="cuda"):
        lib = _lib.load()
        self.spec = spec
        w, h, f = spec["width"], spec["height"], spec["f"]
        n_unique = min(unique, spec["frames"])
        self.frames, poses = scenes.render_room_torch(n_unique, seed=spec["seed"], width=w, height=h, f=f,
                                                      scale=spec.get("scale", 1.0), device=device)
        self.w2e = [scenes.kifi_matrix(np.linalg.inv(p)) for p in poses]
        self.order = frame_order(n_unique, spec["frames"])
        d = PipelineDesc()
        d.camera = Camera(w, h, f, f, w / 2.0, h / 2.0, 0.4, 4.0)
        vox = spec["voxel_mm"] * 1e-3
        d.resolution, d.side_length_m, d.truncation_m = spec["res"], spec["res"] * vox, 5 * vox
        d.icp_iterations, d.mesh_every, d.mesh_with_indices = icp_iters, mesh_every, 1
        d.device = 0
        self.pipe = C.c_void_p()
        check(lib.kifi_pipeline_create(C.byref(d), C.byref(self.pipe)), "pipeline")
        self.vs = lib.kifi_volume_stream(lib.kifi_pipeline_volume(self.pipe))
        self.ist = lib.kifi_icp_stream(lib.kifi_pipeline_icp(self.pipe))
        self.next = 0
        self.events = []

    def done(self):
        return self.next >= len(self.order)

    def step(self, lib, torch, timed):
        j = self.order[self.next]
        if timed:
            e0 = torch.cuda.Event(enable_timing=True)
            e0.record(torch.cuda.ExternalStream(self.vs))
        m = self.w2e[j]
        check(lib.kifi_pipeline_integrate_device(self.pipe, C.c_void_p(self.frames[j].data_ptr()), 1,
                                                 m.ctypes.data_as(C.c_void_p)), "frame")
        if timed:
            e1 = torch.cuda.Event(enable_timing=True)
            e2 = torch.cuda.Event(enable_timing=True)
            e1.record(torch.cuda.ExternalStream(self.vs))
            e2.record(torch.cuda.ExternalStream(self.ist))
            self.events.append((e0, e1, e2))
        self.next += 1

    def latencies_ms(self):
        return [max(a.elapsed_time(b), a.elapsed_time(c)) for a, b, c in self.events]

    def close(self, lib):
        lib.kifi_pipeline_destroy(self.pipe)


def _desc(spec, icp_iters, mesh_every):
    d = PipelineDesc()
    w, h, f = spec["width"], spec["height"], spec["f"]
    d.camera = Camera(w, h, f, f, w / 2.0, h / 2.0, 0.4, 4.0)
    vox = spec["voxel_mm"] * 1e-3
    d.resolution, d.side_length_m, d.truncation_m = spec["res"], spec["res"] * vox, 5 * vox
    d.icp_iterations, d.mesh_every, d.mesh_with_indices = icp_iters, mesh_every, 1
    d.device = 0
    return d


def render_batch(specs, unique=40):
    """Each scene's unique frames on the device, its poses and its playback
    order; and the seconds it took."""
    import torch
    t0 = time.perf_counter()
    data = []
    for spec in specs:
        n_unique = min(unique, spec["frames"])
        fr, poses = scenes.render_room_torch(n_unique, seed=spec["seed"], width=spec["width"],
                                             height=spec["height"], f=spec["f"], scale=spec.get("scale", 1.0),
                                             device="cuda", noise="device")
        data.append((fr, np.stack([scenes.kifi_matrix(np.linalg.inv(p)) for p in poses]),
                     frame_order(n_unique, spec["frames"])))
    torch.cuda.synchronize()
    return data, time.perf_counter() - t0


def run_batch(specs, unique=40, icp_iters=15, warmup_steps=3, persistent=False, queue_ctas_per_sm=1,
              rendered=None):
    """All scenes through one kifi_batch: a step is one launch per stage for
    every scene that still has frames, or with `persistent` one persistent
    fusion launch over a device work queue (kifi_batch_set_persistent) plus
    the tracking launches.  `rendered`: render_batch's result, to reuse.
    Returns the same summary as run()."""
    import torch
    lib = _lib.load()
    data, t_render = rendered if rendered is not None else render_batch(specs, unique)
    n = len(specs)
    descs = (PipelineDesc * n)(*[_desc(s, icp_iters, 0) for s in specs])
    for d, s in zip(descs, specs):
        # room for the scene's volume plus a frame's worth of new voxels, so
        # the steps need no host-side capacity checks that wait for the device
        d.initial_capacity = {2: 64 << 20, 4: 16 << 20, 8: 6 << 20}[s["voxel_mm"]] + 8 * s["width"] * s["height"]
    b = C.c_void_p()
    check(lib.kifi_batch_create(descs, n, C.byref(b)), "batch")
    try:
        check(lib.kifi_batch_set_persistent(b, 1 if persistent else 0, queue_ctas_per_sm), "persistent")
        steps = max(s["frames"] for s in specs)
        ptrs = (C.c_void_p * n)()
        poses = np.zeros((n, 16), np.float32)

        def step(t):
            active = 0
            for i, (fr, w2e, order) in enumerate(data):
                if t < len(order):
                    ptrs[i] = fr[order[t]].data_ptr()
                    poses[i] = w2e[order[t]]
                    active += 1
                else:
                    ptrs[i] = None
            check(lib.kifi_batch_step_device(b, ptrs, poses.ctypes.data_as(C.c_void_p)), "step %d" % t)
            return active

        for t in range(warmup_steps):
            step(t)
        check(lib.kifi_batch_sync(b), "sync")
        check(lib.kifi_batch_set_profiling(b, 1))
        stream = torch.cuda.ExternalStream(lib.kifi_batch_stream(b))
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        frames = 0
        for t in range(warmup_steps, steps):
            frames += step(t)
        e1.record(stream)
        check(lib.kifi_batch_sync(b), "sync")
        e1.synchronize()
        elapsed = e0.elapsed_time(e1) / 1e3
        lat = np.zeros(steps, np.float32)
        nl = C.c_int()
        check(lib.kifi_batch_step_times(b, lat.ctypes.data_as(C.c_void_p), steps, C.byref(nl)))
        lat = lat[:nl.value]
        total = 0
        for i in range(n):
            nv = C.c_size_t()
            check(lib.kifi_volume_size(lib.kifi_batch_volume(b, i), C.byref(nv)))
            total += nv.value
    finally:
        lib.kifi_batch_destroy(b)
    return {"mode": "batch, persistent fusion queue (%d CTAs per SM)" % queue_ctas_per_sm if persistent
            else "batch, one launch per stage", "scenes": n, "frames": int(frames), "seconds": elapsed,
            "frames_per_s": frames / elapsed, "steps": int(nl.value),
            "step_latency_ms_p50": float(np.percentile(lat, 50)), "step_latency_ms_p99": float(np.percentile(lat, 99)),
            "resident_voxels_total": int(total), "render_seconds": t_render, "icp_iterations": icp_iters,
            "unique_frames_per_scene": unique,
            "latency_note": "a step runs every active scene's frame together, so each scene's step latency is "
                            "the step's (device span from the argument upload to the end of fusion and tracking)"}


def run(specs, unique=40, icp_iters=15, mesh_every=0, warmup_steps=3):
    import torch
    lib = _lib.load()
    t0 = time.perf_counter()
    sc = [Scene(s, unique, icp_iters, mesh_every) for s in specs]
    torch.cuda.synchronize()
    t_render = time.perf_counter() - t0
    for _ in range(warmup_steps):
        for s in sc:
            if not s.done():
                s.step(lib, torch, False)
    torch.cuda.synchronize()
    n0 = sum(s.next for s in sc)
    t1 = time.perf_counter()
    while True:
        active = [s for s in sc if not s.done()]
        if not active:
            break
        for s in active:
            s.step(lib, torch, True)
    for s in sc:
        check(lib.kifi_pipeline_sync(s.pipe, None), "sync")
    torch.cuda.synchronize()
    elapsed = time.perf_counter() - t1
    frames = sum(s.next for s in sc) - n0
    lat = np.concatenate([np.asarray(s.latencies_ms()) for s in sc])
    per_scene_p50 = [float(np.median(s.latencies_ms())) for s in sc]
    sizes = {}
    for s in sc:
        n = C.c_size_t()
        check(lib.kifi_volume_size(lib.kifi_pipeline_volume(s.pipe), C.byref(n)))
        sizes[s.spec["seed"]] = n.value
    for s in sc:
        s.close(lib)
    return {"mode": "streams", "scenes": len(specs), "frames": int(frames), "seconds": elapsed,
            "frames_per_s": frames / elapsed,
            "step_latency_ms_p50": float(np.percentile(lat, 50)), "step_latency_ms_p99": float(np.percentile(lat, 99)),
            "per_scene_p50_ms": {"min": min(per_scene_p50), "max": max(per_scene_p50)},
            "resident_voxels_total": int(sum(sizes.values())), "render_seconds": t_render,
            "icp_iterations": icp_iters, "unique_frames_per_scene": unique}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--scenes", type=int, default=64)
    ap.add_argument("--seed", type=int, default=7)
    ap.add_argument("--unique", type=int, default=40)
    ap.add_argument("--icp-iterations", type=int, default=15)
    ap.add_argument("--mode", default="batch", choices=["batch", "queue", "streams"])
    ap.add_argument("--queue-ctas", type=int, default=1, help="persistent fusion CTAs per SM (--mode queue)")
    args = ap.parse_args()
    import torch
    torch.cuda.set_device(0)
    specs = scene_specs(args.scenes, args.seed)
    if args.mode in ("batch", "queue"):
        res = run_batch(specs, unique=args.unique, icp_iters=args.icp_iterations, persistent=args.mode == "queue",
                        queue_ctas_per_sm=args.queue_ctas)
    else:
        res = run(specs, unique=args.unique, icp_iters=args.icp_iterations)
    res["mix"] = {"sizes": {"%dx%d" % (w, h): sum(1 for s in specs if s["width"] == w) for w, h, _ in SIZES},
                  "voxels_mm": {str(v): sum(1 for s in specs if s["voxel_mm"] == v) for v in VOXELS_MM},
                  "trajectory_frames": [min(s["frames"] for s in specs), max(s["frames"] for s in specs)]}
    print(json.dumps(res), flush=True)


if __name__ == "__main__":
    main()
