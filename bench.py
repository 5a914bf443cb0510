"""Benchmark: fused frames/s at 640x480 and 4 mm voxels (the kifi fusion
path of denniskb/merge_fusion on one GB300).

Workload (one step = one frame): a seeded synthetic room (4 x 3 x 4 m, 40 boxes,
20 spheres) ray-cast to 640x480 uint16 millimetre depth (f = 585, 2% dropout,
depth noise 0.0012 + 0.0019 (z-0.4)^2 m) along a smooth trajectory; volume
res 1024 x 4 mm (4.096 m cube), truncation 2 cm.  Every frame is fused with
its given pose (splat + sort + merge/TSDF update) and tracked by 15 ICP
iterations against the previous frame; the mesh (vertices + indices) is
extracted every 10 frames.  Before the warm-up, `--prefill` frames build
the resident volume so that the timed frames run at a realistic size.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Prints one JSON line.  `value` times K frames with the frames already in
device memory; `e2e` times K further frames through the public C ABI
(kifi_pipeline_integrate) from pinned host memory, each call uploading its
frame and reading its tracked pose back.  `--impl reference` times the
reference's own CPU code (oracle/_ref, else the C restatement in oracle/)
on the same workload on the host cores.
"""
import argparse
import atexit
import ctypes as C
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "fused frames/sec at 640x480 & 4mm voxels; ICP iters/frame learned vs plain"
UNIT = "frames/s"
W, H, F_PX = 640, 480, 585.0
RES, SIDE, TRUNC = 1024, 4.096, 0.02
ICP_ITERS, MESH_EVERY = 15, 10
SEED = 0
CAM = (W, H, F_PX, F_PX, W / 2.0, H / 2.0, 0.4, 4.0)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=95)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--prefill", type=int, default=100)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=15.0,
                    help="bounded CPU-baseline sample (seconds of CPU work)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-learned", action="store_true", help="skip the learned-vs-plain ICP measurement")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default launch shape")
    ap.add_argument("--graphs", action="store_true",
                    help="one CUDA graph per frame (kifi_pipeline_set_graphs) instead of plain launches")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(x, world, device="cuda"):
    """The largest x over the ranks of the process group (x itself alone)."""
    if world <= 1:
        return float(x)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(world, steps, seconds):
    """Whole-job frames/s: every rank fuses `steps` frames of its own scene,
    timed by the slowest rank."""
    return world * steps / seconds


def rank_seed(rank):
    """Each rank fuses its own seeded scene (replicas, weak scaling)."""
    return SEED + rank


def measured_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_traffic_per_voxel():
    """DRAM bytes per (N0 + N1) voxel of the merge+update kernel from the
    committed ncu summary, or None."""
    p = os.path.join(ROOT, "profiles", "merge_update_traffic.json")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        return json.load(f)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during a timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []  # (host time, csv line)
        self.windows = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "20"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            atexit.register(self.__exit__, None, None, None)  # also when a timed region raises
            # the timed regions are tens of milliseconds: start them only
            # once nvidia-smi is producing samples
            t_end = time.perf_counter() + 5.0
            while not self.lines and time.perf_counter() < t_end and self.proc.poll() is None:
                time.sleep(0.005)
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.perf_counter(), line.strip()))

    def window(self):
        """Context manager marking one timed region on the host clock."""
        sampler = self

        class _W:
            def __enter__(self):
                self.t0 = time.perf_counter()

            def __exit__(self, *a):
                sampler.windows.append((self.t0, time.perf_counter()))
        return _W()

    def __exit__(self, *a):
        if self.proc and self.proc.poll() is None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        """Median SM clock and the active throttle reasons over the samples
        taken inside the marked windows (all samples when none was marked;
        a window shorter than the sampling period keeps the sample nearest
        to it)."""
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        picked = self.lines
        if self.windows:
            picked = []
            for a, b in self.windows:
                inside = [x for x in self.lines if a <= x[0] <= b]
                if not inside and self.lines:
                    inside = [min(self.lines, key=lambda x: min(abs(x[0] - a), abs(x[0] - b)))]
                picked += [x for x in inside if x not in picked]
        for _, ln in picked:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": smax, "reasons": [], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm), "regions_ms": [round((b - a) * 1e3, 1) for a, b in self.windows]}


# ------------------------------------------------------------- CPU baseline

def cpu_baseline(frames_u16, poses, start, n_max, seconds, resident=None):
    """The reference's CPU path (oracle/_ref, else the oracle port) on the
    same frames: integrate + 15 ICP iterations against the previous frame,
    plus one mesh per 10 frames.  Runs until `seconds` of work or n_max
    frames.  Returns (frames/s, kind, frames timed, mesh seconds)."""
    from oracle import build_ref
    kind = "reference"
    try:
        from oracle import ref as impl
        if not impl.available():
            build_ref.build()
        if not impl.available():
            raise OSError("reference CPU build unavailable")
    except Exception:
        kind = "port"
        impl = None
    from oracle import cpu
    if impl is not None:
        vol = impl.Volume(RES, SIDE, TRUNC)
        if resident is not None and resident[0].size:
            vol.insert(resident[0], resident[1])
        icp = lambda d, g, t, tp: impl.icp_align(d, CAM, g, t, tp, ICP_ITERS)  # noqa: E731
        mesh = lambda: vol.mesh(True)  # noqa: E731
        integ = lambda d, m: vol.integrate(d, CAM, m)  # noqa: E731
    else:
        vol = cpu.Volume(RES, SIDE, TRUNC)
        if resident is not None:
            vol.keys, vol.values = resident[0].copy(), resident[1].copy()
        icp = lambda d, g, t, tp: cpu.icp_align(d, CAM, g, t, tp, ICP_ITERS)  # noqa: E731
        mesh = lambda: vol.mesh(True)  # noqa: E731
        integ = lambda d, m: vol.integrate(d, CAM, m)  # noqa: E731
    from merge_fusion_gb300.scenes import kifi_matrix
    t_total, n = 0.0, 0
    target = None
    t_mesh = None
    while n < n_max and t_total < seconds:
        i = start + n
        depth = frames_u16[i].astype(np.float32) * np.float32(0.001)  # DepthStream conversion
        w2e = kifi_matrix(np.linalg.inv(poses[i]))
        e2w_prev = kifi_matrix(poses[i - 1])
        t0 = time.perf_counter()
        integ(depth, w2e)
        if target is None:
            prev = frames_u16[i - 1].astype(np.float32) * np.float32(0.001)
            target = cpu.backproject(prev, CAM, e2w_prev)
        icp(depth, e2w_prev, target, e2w_prev)
        target = cpu.backproject(depth, CAM, kifi_matrix(poses[i]))
        t_total += time.perf_counter() - t0
        n += 1
    t0 = time.perf_counter()
    mesh()
    t_mesh = time.perf_counter() - t0
    per_frame = t_total / max(n, 1) + t_mesh / MESH_EVERY
    return 1.0 / per_frame, kind, n, t_mesh


# ------------------------------------------------------------------ GPU arm

def run_gpu(args, rank, world, local):
    import torch
    import torch.distributed as dist
    from merge_fusion_gb300 import _lib, scenes
    from merge_fusion_gb300._lib import Camera, PipelineDesc, check
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl")
    lib = _lib.load()
    K, Wu, Fp = args.steps, args.warmup, args.prefill
    n_frames = Fp + Wu + 2 * K + 1
    # independent scene per rank (replicas; weak scaling)
    seed = rank_seed(rank)
    frames, poses = scenes.render_room_torch(n_frames, seed=seed, device="cuda")
    torch.cuda.synchronize()
    frames_host = frames.cpu().numpy().view(np.uint16)
    pinned = torch.empty((2 * K + 1, H, W), dtype=torch.int16).pin_memory()
    pinned.copy_(frames[Fp + Wu:Fp + Wu + 2 * K + 1].cpu())
    w2e = [scenes.kifi_matrix(np.linalg.inv(p)) for p in poses]

    cam = Camera(W, H, F_PX, F_PX, W / 2.0, H / 2.0, 0.4, 4.0)
    d = PipelineDesc()
    d.camera = cam
    d.resolution, d.side_length_m, d.truncation_m = RES, SIDE, TRUNC
    d.icp_iterations, d.mesh_every, d.mesh_with_indices = ICP_ITERS, MESH_EVERY, 1
    d.initial_capacity = 48 << 20
    d.device = local
    pipe = C.c_void_p()
    check(lib.kifi_pipeline_create(C.byref(d), C.byref(pipe)), "pipeline")
    check(lib.kifi_pipeline_set_graphs(pipe, 1 if args.graphs else 0))
    vol = lib.kifi_pipeline_volume(pipe)
    vs = torch.cuda.ExternalStream(lib.kifi_volume_stream(vol))
    ist = torch.cuda.ExternalStream(lib.kifi_icp_stream(lib.kifi_pipeline_icp(pipe)))

    def ptr(a):
        return a.ctypes.data_as(C.c_void_p)

    def step_device(i):
        check(lib.kifi_pipeline_integrate_device(pipe, C.c_void_p(frames[i].data_ptr()), 1,
                                                 ptr(w2e[i])), "frame %d" % i)

    for i in range(Fp + Wu):
        step_device(i)
    check(lib.kifi_pipeline_sync(pipe, None))
    # launch shape of the fusion kernels, measured on the next frame (the volume is left unchanged)
    tuned = np.zeros(3, np.int32)
    if not args.no_autotune:
        check(lib.kifi_volume_autotune(vol, C.c_void_p(frames[Fp + Wu].data_ptr()), 1, C.byref(cam),
                                       ptr(w2e[Fp + Wu]), 1, ptr(tuned)), "autotune")
    n_resident = C.c_size_t()
    check(lib.kifi_volume_size(vol, C.byref(n_resident)))
    n_start = int(n_resident.value)  # resident voxels when the timed frames begin

    # bounded CPU baseline starts from the same resident volume
    resident = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        nvox = n_resident.value
        rk = np.zeros(nvox + 1, np.uint32)
        rv = np.zeros((nvox + 1, 2), np.float32)
        got = C.c_size_t()
        check(lib.kifi_volume_export(vol, ptr(rk), ptr(rv), nvox + 1, C.byref(got)))
        resident = (rk[:got.value], rv[:got.value])

    # ---- device-resident timed region
    check(lib.kifi_volume_set_profiling(vol, 1))
    t0 = Fp + Wu
    ms_stage = np.zeros(4)
    nst = C.c_int()
    check(lib.kifi_volume_stage_times(vol, ptr(ms_stage), C.byref(nst)))  # reset
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    # one sampler over both timed regions (device-resident, then end to end)
    clocks = ClockSampler(local).__enter__()
    with clocks.window():
        start.record(vs)
        ist.wait_event(start)
        for i in range(t0, t0 + K):
            step_device(i)
        fin = torch.cuda.Event()
        fin.record(ist)
        vs.wait_event(fin)
        end.record(vs)
        end.synchronize()
    ms = start.elapsed_time(end)
    check(lib.kifi_volume_stage_times(vol, ptr(ms_stage), C.byref(nst)))
    check(lib.kifi_volume_set_profiling(vol, 0))
    n0 = np.zeros(64, np.uint64)
    ne = np.zeros(64, np.uint64)
    n1 = np.zeros(64, np.uint64)
    cnt = C.c_int()
    check(lib.kifi_volume_frame_log(vol, ptr(n0), ptr(ne), ptr(n1), 64, C.byref(cnt)))
    m = min(cnt.value, K)
    n0, ne, n1 = n0[cnt.value - m:cnt.value], ne[cnt.value - m:cnt.value], n1[cnt.value - m:cnt.value]
    ms = max_over_ranks(ms, world)

    # ---- end to end through the public ABI from pinned host memory
    out_pose = np.zeros(16, np.float32)
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    with clocks.window():
        te0 = time.perf_counter()
        for j in range(K):
            i = t0 + K + j
            check(lib.kifi_pipeline_integrate(pipe, C.c_void_p(pinned[K + j].data_ptr()), 1,
                                              ptr(w2e[i]), ptr(out_pose)), "e2e frame %d" % i)
        # each call returns with its tracked pose; the last frames' fusion finishes inside the timing
        check(lib.kifi_pipeline_sync(pipe, None), "e2e sync")
        e2e_s = time.perf_counter() - te0
    clocks.__exit__(None, None, None)
    e2e_s = max_over_ranks(e2e_s, world)

    # the merge kernel with tracking idle: a few fusion-only frames after the
    # timed regions (the last rendered frame again, on the pipeline's volume)
    ISO = 5
    iso_stage = np.zeros(4)
    iso_n = C.c_int()
    check(lib.kifi_volume_set_profiling(vol, 1))
    check(lib.kifi_volume_stage_times(vol, ptr(iso_stage), C.byref(iso_n)))  # reset
    for _ in range(ISO):
        check(lib.kifi_integrate_device(vol, C.c_void_p(frames[n_frames - 1].data_ptr()), 1, C.byref(cam),
                                        ptr(w2e[n_frames - 1])), "isolated frame")
    check(lib.kifi_volume_stage_times(vol, ptr(iso_stage), C.byref(iso_n)))
    check(lib.kifi_volume_set_profiling(vol, 0))
    i0, ie, i1 = np.zeros(64, np.uint64), np.zeros(64, np.uint64), np.zeros(64, np.uint64)
    iso_cnt = C.c_int()
    check(lib.kifi_volume_frame_log(vol, ptr(i0), ptr(ie), ptr(i1), 64, C.byref(iso_cnt)))
    lo, hi = iso_cnt.value - ISO, iso_cnt.value
    iso_bytes = float((12.0 * i0[lo:hi].astype(np.float64) + 4.0 * ie[lo:hi] + 12.0 * i1[lo:hi] +
                       2.0 * W * H).mean())
    iso_ms = iso_stage[3] / max(iso_n.value, 1)

    nv, ni = C.c_size_t(), C.c_size_t()
    check(lib.kifi_pipeline_mesh_counts(pipe, C.byref(nv), C.byref(ni)))
    gb, gu = C.c_longlong(), C.c_longlong()
    check(lib.kifi_pipeline_graph_stats(pipe, C.byref(gb), C.byref(gu)))
    check(lib.kifi_volume_size(vol, C.byref(n_resident)))

    if rank != 0:
        lib.kifi_pipeline_destroy(pipe)
        if world > 1:
            dist.destroy_process_group()
        return

    value = job_throughput(world, K, ms / 1e3)
    P = W * H
    algo_bytes = (12.0 * n0.astype(np.float64) + 4.0 * ne + 12.0 * n1 + 2.0 * P)
    merge_ms = ms_stage[3] / max(nst.value, 1)
    achieved = float(algo_bytes.mean()) / (merge_ms / 1e3) / 1e9
    peak, peak_kind = measured_peak()
    traffic = None
    tr = ncu_traffic_per_voxel()
    if tr:
        traffic = float(tr["bytes_per_voxel"] * float((n0 + n1).mean()) + tr.get("bytes_fixed", 0.0))
    # per frame: frame set-up, splat+emit, sort (prepare, histogram, 4 passes),
    # merge partition, merge+update; ICP: begin, one step per iteration, the
    # next target's back-projection; a mesh is 7 launches (snapshot, row
    # directory, classification, two scan kernels, two emission passes)
    launches_per_frame = 10 + (ICP_ITERS + 2)
    gpu_launches = K * launches_per_frame + (K // MESH_EVERY) * 7
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K,
        "warmup": Wu, "ms_per_step": ms / K, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+u32", "data": "synthetic",
        "config": {"workload": "room 4x3x4 m, 40 boxes + 20 spheres, 640x480 uint16 depth, "
                               "res 1024 x 4 mm, trunc 2 cm, ICP 15 it/frame, mesh every 10",
                   "prefill_frames": Fp, "resident_voxels_start": n_start,
                   "resident_voxels_end": int(n1[-1]) if m else None,
                   "roofline_frames": "the last %d timed frames (the device frame log's length)" % m,
                   "l2": "volume (>240 MB) larger than L2; every frame is a new depth image",
                   "parallelism": "replicas" if world > 1 else "single"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "kernel": "k_merge_update (fused merge-path union + TSDF update)",
                     "peak_source": peak_kind,
                     "bytes_per_launch": float(algo_bytes.mean()),
                     "ms_per_launch": merge_ms,
                     "isolated": {"ms_per_launch": iso_ms, "achieved": iso_bytes / (iso_ms * 1e-3) / 1e9,
                                  "frac": iso_bytes / (iso_ms * 1e-3) / 1e9 / peak, "bytes_per_launch": iso_bytes,
                                  "frames": ISO,
                                  "note": "fusion-only frames after the timed regions, tracking idle; inside the "
                                          "pipeline the merge yields SMs to the higher-priority tracking steps"}},
        "stage_ms_per_frame": {"splat_emit": ms_stage[0] / max(nst.value, 1),
                               "sort": ms_stage[1] / max(nst.value, 1),
                               "merge_partition": ms_stage[2] / max(nst.value, 1),
                               "merge_update": merge_ms},
        "e2e": {"value": job_throughput(world, K, e2e_s), "unit": UNIT, "h2d_bytes_per_step": 2 * P + 64,
                "d2h_bytes_per_step": 64 + 1024},
        "gpu_launches": gpu_launches,
        "graphs": {"on": bool(args.graphs), "instantiated": int(gb.value), "updated": int(gu.value)},
        "autotune": None if args.no_autotune else {"splat_ctas": int(tuned[0]), "sort_ctas": int(tuned[1]),
                                                   "merge_ctas": int(tuned[2])},
        "mesh": {"vertices": nv.value, "indices": ni.value},
    }
    line["clocks"] = clocks.summary()
    if resident is not None:
        v, kind, nfr, tmesh = cpu_baseline(frames_host, poses, t0, K, args.cpu_seconds, resident)
        line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": 1, "kind": kind,
                                "sample": "%d frames (integrate + 15 ICP iterations each) from the "
                                          "same resident volume, plus one mesh (%.2f s) amortised "
                                          "over 10 frames; single-threaded, as the reference is"
                                          % (nfr, tmesh)}
    lib.kifi_pipeline_destroy(pipe)
    if not args.no_learned:
        line["icp_iterations"] = learned_vs_plain()
    print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


# ------------------------------------------------------------ reference arm

REF_MAX_TIMED_FRAMES = 12  # about 16 s of the reference's single-threaded CPU work


def learned_vs_plain():
    """ICP iterations to converge (RMS change < 1e-4 m) with the learned warm
    start vs plain identity-initialised ICP, on held-out room trajectories
    (seeds the training never saw), with the trained weights in the repo."""
    from merge_fusion_gb300 import proposer as mp
    path = os.path.join(ROOT, "merge_fusion_gb300", "weights", "proposer_room.npz")
    if not os.path.exists(path):
        return None
    net = mp.PoseProposer(max_batch=8)
    params, mean, std = mp.load(path)
    net.set_params(params)
    seeds = [SEED + 21000, SEED + 21001]
    res = mp.evaluate(net, mean, std, seeds, 40, max_pairs=96)
    net.close()
    return {"plain": res["plain_iterations"], "learned": res["learned_iterations"], "ratio": res["ratio"],
            "pairs": res["pairs"], "fallbacks": res["fallbacks"], "criterion": "RMS change < 1e-4 m",
            "held_out": "room trajectories %d-%d, pairs (a, a+k), k = 1..3" % (seeds[0], seeds[-1]),
            "median_pose_diff": res["median_pose_diff"], "plain_spread_median": res["plain_spread_median"]}


def run_reference(args, rank, world):
    if rank != 0:
        return
    from merge_fusion_gb300 import scenes
    # a bounded sample of the same workload: the first frames of the timed range
    K, Wu, Fp = min(args.steps, REF_MAX_TIMED_FRAMES), min(args.warmup, 3), args.prefill
    n_frames = Fp + Wu + K + 1
    frames, poses = scenes.render_room_torch(n_frames, seed=SEED, device="cpu")
    frames = frames.numpy().view(np.uint16)
    from oracle import build_ref
    kind = "reference"
    try:
        from oracle import ref as impl
        if not impl.available():
            build_ref.build()
        if not impl.available():
            raise OSError("no reference build")
        vol = impl.Volume(RES, SIDE, TRUNC)
    except Exception:
        from oracle import cpu as impl
        kind = "port"
        vol = impl.Volume(RES, SIDE, TRUNC)
    from oracle import cpu
    w2e = [scenes.kifi_matrix(np.linalg.inv(p)) for p in poses]
    e2w = [scenes.kifi_matrix(p) for p in poses]
    depth = lambda i: frames[i].astype(np.float32) * np.float32(0.001)  # noqa: E731
    for i in range(Fp):  # build the resident volume (fusion only)
        vol.integrate(depth(i), CAM, w2e[i])
    target = cpu.backproject(depth(Fp - 1), CAM, e2w[Fp - 1])
    times = []
    for s in range(Wu + K):
        i = Fp + s
        t0 = time.perf_counter()
        d = depth(i)
        vol.integrate(d, CAM, w2e[i])
        impl.icp_align(d, CAM, e2w[i - 1], target, e2w[i - 1], ICP_ITERS)
        target = cpu.backproject(d, CAM, e2w[i])
        if (s + 1) % MESH_EVERY == 0:
            vol.mesh(True)
        times.append(time.perf_counter() - t0)
    tt = sum(times[Wu:])
    value = K / tt
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": K, "warmup": Wu, "ms_per_step": 1e3 * tt / K, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+u32", "data": "synthetic",
            "config": {"workload": "room 4x3x4 m, 40 boxes + 20 spheres, 640x480 uint16 depth, "
                                   "res 1024 x 4 mm, trunc 2 cm, ICP 15 it/frame, mesh every 10",
                       "prefill_frames": Fp},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": 1, "kind": kind,
                             "sample": "%d timed frames (of the %d requested) after %d warm-up "
                                       "frames and %d fusion-only prefill frames; single-threaded "
                                       "like the reference" % (K, args.steps, Wu, Fp)},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    rank, world, local = dist_env()
    # in-tree build (no-op when up to date); the GPU arm fails loudly without it
    from merge_fusion_gb300 import build
    build.build()
    if args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_gpu(args, rank, world, local)


if __name__ == "__main__":
    main()
