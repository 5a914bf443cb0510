"""Benchmark: fused frames/s at 640x480 and 4 mm voxels (the kifi fusion
path of denniskb/merge_fusion on one GB300).

Workload: a seeded synthetic room (4 x 3 x 4 m, 40 boxes, 20 spheres)
ray-cast to 640x480 uint16 millimetre depth (f = 585, 2% dropout, depth
noise 0.0012 + 0.0019 (z-0.4)^2 m) along a smooth trajectory; volume res
1024 x 4 mm (4.096 m cube), truncation 2 cm.  Every frame is fused with its
given pose (splat + sort + merge/TSDF update) and tracked by 15 ICP
iterations against the previous frame; the mesh (vertices + indices) is
extracted every 10 frames.  One step is one mesh period: ten frames and the
mesh that ends it.  The sequence has 300 frames; a run that needs more
plays it forward, then back (consecutive frames stay adjacent for ICP).
Before the warm-up, `--prefill` frames build the resident volume so that the
timed frames run at a realistic size.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Prints one JSON line.  `value` times K steps with the frames already in
device memory: CUDA events on the volume stream, with the tracking and
meshing streams joined before the end event.  `e2e` times K further steps
through the public C ABI (kifi_pipeline_integrate) from pinned host memory,
each call uploading its frame and reading its tracked pose back, ending
with kifi_pipeline_sync (fusion, tracking and meshing done).
`--impl reference` times the reference's own CPU code (oracle/_ref, else the
C restatement in oracle/) on a bounded sample of the same workload.
"""
import argparse
import atexit
import ctypes as C
import datetime
import json
import os
import platform
import subprocess
import sys
import tempfile
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
FRAMES_PER_STEP = MESH_EVERY  # a step is one mesh period
SEQ_FRAMES = 300  # the sequence's length; longer runs play it forward, then back


def playback(t):
    """Sequence frame of the t-th frame fused: 0, 1, .., 299, 298, .., 1, 0, 1, .."""
    period = 2 * SEQ_FRAMES - 2
    r = t % period
    return r if r < SEQ_FRAMES else period - r
SEED = 0
CAM = (W, H, F_PX, F_PX, W / 2.0, H / 2.0, 0.4, 4.0)
WORKLOAD = ("room 4x3x4 m, 40 boxes + 20 spheres, 640x480 uint16 depth, res 1024 x 4 mm, trunc 2 cm, "
            "ICP 15 it/frame, mesh every 10")
# kernels launched per frame: frame set-up (with the sort's set-up), splat+emit
# (with the digit counts), three digit passes, merge partition, merge+update;
# tracking: ICP begin, one step per iteration, the next target's
# back-projection; per mesh: snapshot, row directory, tile ranges, status
# bytes, classification, tile-sum scan, two emission passes
LAUNCHES_FUSION, LAUNCHES_TRACKING, LAUNCHES_MESH = 7, ICP_ITERS + 2, 8
# bytes the host reads back per tracked frame: the head of the ICP state
# (float and float-float pose, counters, 64 iteration records of 20 bytes)
ICP_HEAD_BYTES = 192 + 64 * 20
MESH_COUNTS_BYTES = 32
FP32_LANES_PER_SM = 128  # FP32 FMA lanes of a Blackwell SM: 2 flop per lane per clock


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20, help="timed steps (one mesh period of 10 frames each)")
    ap.add_argument("--warmup", type=int, default=5, help="untimed steps before the timed ones")
    ap.add_argument("--prefill", type=int, default=100, help="frames fused before the warm-up")
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=15.0,
                    help="bounded CPU-baseline sample (seconds of CPU work)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-learned", action="store_true", help="skip the learned-vs-plain ICP measurement")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default launch shape")
    ap.add_argument("--no-batched", action="store_true",
                    help="skip the 64-scene batched run (uneven frame sizes, voxel sizes and lengths)")
    ap.add_argument("--graphs", action="store_true",
                    help="one CUDA graph per frame (kifi_pipeline_set_graphs) instead of plain launches")
    ap.add_argument("--capacity-mvox", type=int, default=48,
                    help="volume capacity preset, millions of voxels (small cases for profiling use less)")
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


def job_throughput(world, frames, seconds):
    """Whole-job frames/s: every rank fuses `frames` frames of its own scene,
    timed by the slowest rank."""
    return world * frames / seconds


def rank_seed(rank):
    """Each rank fuses its own seeded scene (replicas, weak scaling)."""
    return SEED + rank


def workload_config(prefill, frames_per_step):
    return {"workload": WORKLOAD, "prefill_frames": prefill, "frames_per_step": frames_per_step,
            "l2": "volume (>240 MB) larger than L2; every frame is a new depth image"}


def measured_peaks():
    """(HBM GB/s, SM max MHz, source) from MEASURED_PEAKS.json, else the fallback."""
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), float(d.get("sm_max_mhz", 2070.0)), "measured"
    return 6800.0, 2070.0, "fallback"


def ncu_traffic(name):
    """DRAM bytes per unit of a kernel from a committed ncu summary, or None."""
    p = os.path.join(ROOT, "profiles", name)
    if not os.path.exists(p):
        return None
    with open(p) as f:
        return json.load(f)


def host_cpu():
    """CPU model and logical core count of this host."""
    model = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.startswith("Model name:"):
                model = ln.split(":", 1)[1].strip()
                break
    except (OSError, subprocess.SubprocessError):
        pass
    if not model:
        try:
            with open("/proc/cpuinfo") as f:
                for ln in f:
                    if ln.lower().startswith("model name"):
                        model = ln.split(":", 1)[1].strip()
                        break
        except OSError:
            pass
    try:
        usable = len(os.sched_getaffinity(0))  # the cores this process may run on
    except (AttributeError, OSError):
        usable = os.cpu_count()
    return {"cpu_model": model or platform.processor() or platform.machine(), "nproc": usable,
            "cpu_count": os.cpu_count(), "machine": platform.machine()}


def _smi_time(stamp):
    """nvidia-smi's sample timestamp ("YYYY/MM/DD HH:MM:SS.mmm", local time)
    as seconds since the epoch, or None."""
    try:
        return datetime.datetime.strptime(stamp.strip(), "%Y/%m/%d %H:%M:%S.%f").timestamp()
    except ValueError:
        return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during a timed region.
    Samples are placed by nvidia-smi's own timestamp, not by when their line
    reached this process (output may arrive in batches)."""

    FIELDS = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []  # (sample time, csv line without the timestamp)
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
            # start the timed regions only once nvidia-smi is producing samples
            t_end = time.time() + 5.0
            while not self.lines and time.time() < t_end and self.proc.poll() is None:
                time.sleep(0.005)
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.add(line, time.time())

    def add(self, line, arrival):
        stamp, _, rest = line.strip().partition(",")
        t = _smi_time(stamp)
        self.lines.append((arrival if t is None else t, rest.strip()))

    def window(self):
        """Context manager marking one timed region on the host's wall clock."""
        sampler = self

        class _W:
            def __enter__(self):
                self.t0 = time.time()

            def __exit__(self, *a):
                sampler.windows.append((self.t0, time.time()))
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

def _cpu_impl(resident):
    """The reference's CPU code (oracle/_ref) with a volume holding `resident`,
    else the oracle's C restatement.  Returns (kind, integrate, icp, mesh)."""
    from oracle import build_ref, cpu
    try:
        from oracle import ref as impl
        if not impl.available():
            build_ref.build()
        if not impl.available():
            raise OSError("reference CPU build unavailable")
        vol = impl.Volume(RES, SIDE, TRUNC)
        if resident is not None and resident[0].size:
            vol.insert(resident[0], resident[1])
        kind = "reference"
        icp = impl.icp_align
    except Exception:
        vol = cpu.Volume(RES, SIDE, TRUNC)
        if resident is not None:
            vol.keys, vol.values = resident[0].copy(), resident[1].copy()
        kind = "port"
        icp = cpu.icp_align
    return (kind, lambda d, m: vol.integrate(d, CAM, m),
            lambda d, g, t, tp: icp(d, CAM, g, t, tp, ICP_ITERS), lambda: vol.mesh(True))


def cpu_frames(frames_u16, poses, start, n_max, seconds, resident, with_mesh=True):
    """The reference's CPU path on the same frames: integrate + 15 ICP
    iterations against the previous frame, plus one mesh per 10 frames.
    Runs until `seconds` of work or n_max frames.  Returns (frames/s, kind,
    frames timed, mesh seconds)."""
    from oracle import cpu
    from merge_fusion_gb300.scenes import kifi_matrix
    kind, integ, icp, mesh = _cpu_impl(resident)
    t_total, n = 0.0, 0
    target = None
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
    t_mesh = 0.0
    if with_mesh:
        t0 = time.perf_counter()
        mesh()
        t_mesh = time.perf_counter() - t0
    per_frame = t_total / max(n, 1) + t_mesh / MESH_EVERY
    return 1.0 / per_frame, kind, n, t_mesh


def _cpu_worker(path, seconds):
    """One process of the multi-core aggregate: the same bounded sample from
    the same resident volume (inputs in the npz file at `path`)."""
    d = np.load(path)
    poses = list(d["poses"])
    fps, kind, n, tm = cpu_frames(d["frames"], poses, 1, d["frames"].shape[0] - 1, seconds,
                                  (d["keys"], d["values"]))
    return fps, kind, n, tm


def cpu_aggregate(frames_u16, poses, start, n_max, seconds, resident, procs):
    """One scene per core: `procs` processes each run the single-core sample
    at once; the aggregate is the sum of their frames/s."""
    import multiprocessing as mp
    fd, path = tempfile.mkstemp(suffix=".npz", prefix="kifi_cpu_")
    os.close(fd)
    try:
        np.savez(path, frames=frames_u16[start - 1:start + n_max], poses=np.asarray(poses[start - 1:start + n_max]),
                 keys=resident[0], values=resident[1])
        with mp.get_context("spawn").Pool(procs) as pool:
            res = pool.starmap(_cpu_worker, [(path, seconds)] * procs)
    finally:
        os.unlink(path)
    return sum(r[0] for r in res), res


# ------------------------------------------------------------------ GPU arm

def roofline_entry(bound, achieved, peak, unit, per_launch, ms, peak_source, extra=None):
    e = {"bound": bound, "achieved": achieved, "peak": peak, "unit": unit, "frac": achieved / peak,
         "ms_per_launch": ms, "peak_source": peak_source}
    e.update(per_launch)
    if extra:
        e.update(extra)
    return e


def run_gpu(args, rank, world, local):
    import torch
    import torch.distributed as dist
    from merge_fusion_gb300 import _lib, scenes
    from merge_fusion_gb300._lib import Camera, PipelineDesc, check
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl")
    lib = _lib.load()
    K, Wu, Fp, FS = args.steps, args.warmup, args.prefill, FRAMES_PER_STEP
    KF = K * FS
    n_frames = Fp + (Wu + 2 * K) * FS + 1  # frames fused, in playback order
    # independent scene per rank (replicas; weak scaling)
    seed = rank_seed(rank)
    seq_frames, seq_poses = scenes.render_room_torch(SEQ_FRAMES, seed=seed, device="cuda")
    torch.cuda.synchronize()
    order = [playback(t) for t in range(n_frames)]
    frames = [seq_frames[j] for j in order]  # device views, in the order they are fused
    poses = [seq_poses[j] for j in order]
    seq_host = seq_frames.cpu().numpy().view(np.uint16)
    t0 = Fp + Wu * FS
    pinned = torch.empty((KF, H, W), dtype=torch.int16).pin_memory()
    for j in range(KF):
        pinned[j].copy_(frames[t0 + KF + j].cpu())
    w2e = [scenes.kifi_matrix(np.linalg.inv(p)) for p in poses]
    sms = torch.cuda.get_device_properties(local).multi_processor_count

    cam = Camera(W, H, F_PX, F_PX, W / 2.0, H / 2.0, 0.4, 4.0)
    d = PipelineDesc()
    d.camera = cam
    d.resolution, d.side_length_m, d.truncation_m = RES, SIDE, TRUNC
    d.icp_iterations, d.mesh_every, d.mesh_with_indices = ICP_ITERS, MESH_EVERY, 1
    d.initial_capacity = args.capacity_mvox << 20
    d.device = local
    pipe = C.c_void_p()
    check(lib.kifi_pipeline_create(C.byref(d), C.byref(pipe)), "pipeline")
    check(lib.kifi_pipeline_set_graphs(pipe, 1 if args.graphs else 0))
    vol = lib.kifi_pipeline_volume(pipe)
    icp = lib.kifi_pipeline_icp(pipe)
    vs_handle = lib.kifi_volume_stream(vol)
    vs = torch.cuda.ExternalStream(vs_handle)
    ist = torch.cuda.ExternalStream(lib.kifi_icp_stream(icp))

    def ptr(a):
        return a.ctypes.data_as(C.c_void_p)

    def step_device(i):
        check(lib.kifi_pipeline_integrate_device(pipe, C.c_void_p(frames[i].data_ptr()), 1,
                                                 ptr(w2e[i])), "frame %d" % i)

    def mesh_stats():
        m, r = C.c_longlong(), C.c_longlong()
        check(lib.kifi_pipeline_mesh_stats(pipe, C.byref(m), C.byref(r)))
        return m.value, r.value

    def mesh_counts():
        nv, ni = C.c_size_t(), C.c_size_t()
        check(lib.kifi_pipeline_mesh_counts(pipe, C.byref(nv), C.byref(ni)))
        return nv.value, ni.value

    for i in range(t0):  # prefill, then the warm-up steps
        step_device(i)
    check(lib.kifi_pipeline_sync(pipe, None))
    # launch shape of the fusion kernels, measured on the next frame (the volume is left unchanged)
    tuned = np.zeros(3, np.int32)
    if not args.no_autotune:
        check(lib.kifi_volume_autotune(vol, C.c_void_p(frames[t0].data_ptr()), 1, C.byref(cam),
                                       ptr(w2e[t0]), 1, ptr(tuned)), "autotune")
    n_resident = C.c_size_t()
    check(lib.kifi_volume_size(vol, C.byref(n_resident)))
    n_start = int(n_resident.value)  # resident voxels when the timed frames begin

    # the CPU baseline starts from the same resident volume
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
    ms_stage = np.zeros(4)
    pipe_ms = np.zeros(2)
    pipe_n = np.zeros(2, np.int32)
    nst = C.c_int()
    check(lib.kifi_volume_stage_times(vol, ptr(ms_stage), C.byref(nst)))  # reset
    check(lib.kifi_pipeline_stage_times(pipe, ptr(pipe_ms), ptr(pipe_n)))  # reset
    meshes0, reemit0 = mesh_stats()
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    # one sampler over both timed regions (device-resident, then end to end)
    clocks = ClockSampler(local).__enter__()
    with clocks.window():
        start.record(vs)
        ist.wait_event(start)
        for i in range(t0, t0 + KF):
            step_device(i)
        # the end event follows every stream of the pipeline: fusion, tracking, meshing
        check(lib.kifi_pipeline_join(pipe, C.c_void_p(vs_handle)))
        end.record(vs)
        end.synchronize()
    ms = start.elapsed_time(end)
    region_mesh = mesh_counts()  # the last mesh of the region, complete at the end event
    check(lib.kifi_volume_stage_times(vol, ptr(ms_stage), C.byref(nst)))
    check(lib.kifi_pipeline_stage_times(pipe, ptr(pipe_ms), ptr(pipe_n)))
    check(lib.kifi_volume_set_profiling(vol, 0))
    check(lib.kifi_pipeline_sync(pipe, None))
    synced_mesh = mesh_counts()
    meshes1, reemit1 = mesh_stats()
    n0 = np.zeros(64, np.uint64)
    ne = np.zeros(64, np.uint64)
    n1 = np.zeros(64, np.uint64)
    cnt = C.c_int()
    check(lib.kifi_volume_frame_log(vol, ptr(n0), ptr(ne), ptr(n1), 64, C.byref(cnt)))
    m = min(cnt.value, KF)
    n0, ne, n1 = (a[cnt.value - m:cnt.value].astype(np.float64) for a in (n0, ne, n1))
    ms = max_over_ranks(ms, world)

    # ---- end to end through the public ABI from pinned host memory
    out_pose = np.zeros(16, np.float32)
    # the call's arguments as ctypes objects, made before the timed region
    e2e_args = [(C.c_void_p(pinned[j].data_ptr()), ptr(w2e[t0 + KF + j])) for j in range(KF)]
    out_ptr = ptr(out_pose)
    integrate = lib.kifi_pipeline_integrate
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    with clocks.window():
        te0 = time.perf_counter()
        for j in range(KF):
            rc = integrate(pipe, e2e_args[j][0], 1, e2e_args[j][1], out_ptr)
            if rc:
                check(rc, "e2e frame %d" % (t0 + KF + j))
        # each call returns with its tracked pose; the last frames' fusion and mesh finish inside the timing
        check(lib.kifi_pipeline_sync(pipe, None), "e2e sync")
        e2e_s = time.perf_counter() - te0
    clocks.__exit__(None, None, None)
    e2e_s = max_over_ranks(e2e_s, world)

    # ---- isolated kernels, after the timed regions
    # fusion-only frames (the last rendered frame again, on the pipeline's volume), tracking idle, with
    # the volume's launch shape for fusion alone (persistent grids, the merge build with 4 CTAs per SM);
    # one untimed frame first loads that shape's kernels
    ISO = 5
    iso_stage = np.zeros(4)
    iso_n = C.c_int()
    check(lib.kifi_volume_set_launch_mode(vol, 0))
    check(lib.kifi_volume_set_profiling(vol, 1))
    for k in range(ISO + 1):
        if k == 1:
            check(lib.kifi_volume_stage_times(vol, ptr(iso_stage), C.byref(iso_n)))  # reset
        check(lib.kifi_integrate_device(vol, C.c_void_p(frames[n_frames - 1].data_ptr()), 1, C.byref(cam),
                                        ptr(w2e[n_frames - 1])), "isolated frame")
    check(lib.kifi_volume_stage_times(vol, ptr(iso_stage), C.byref(iso_n)))
    check(lib.kifi_volume_set_launch_mode(vol, 1))
    # a mesh of the whole volume alone (the first call sizes the volume's mesh buffers)
    iso_mesh = np.zeros(5)
    iso_meshes = C.c_int()
    nvi, nii = C.c_size_t(), C.c_size_t()
    for k in range(3):
        if k == 1:
            check(lib.kifi_volume_mesh_stage_times(vol, ptr(iso_mesh), C.byref(iso_meshes)))  # reset
        check(lib.kifi_mesh_device(vol, 1, C.byref(nvi), C.byref(nii), None, None), "isolated mesh")
    check(lib.kifi_volume_mesh_stage_times(vol, ptr(iso_mesh), C.byref(iso_meshes)))
    iso_mesh_ms = C.c_double(iso_mesh[4])
    check(lib.kifi_volume_set_profiling(vol, 0))
    i0, ie, i1 = np.zeros(64, np.uint64), np.zeros(64, np.uint64), np.zeros(64, np.uint64)
    iso_cnt = C.c_int()
    check(lib.kifi_volume_frame_log(vol, ptr(i0), ptr(ie), ptr(i1), 64, C.byref(iso_cnt)))
    lo, hi = iso_cnt.value - ISO, iso_cnt.value
    i0, ie, i1 = (a[lo:hi].astype(np.float64) for a in (i0, ie, i1))
    n_mesh_vox = C.c_size_t()
    check(lib.kifi_volume_size(vol, C.byref(n_mesh_vox)))
    # one ICP alignment alone (the pipeline's last target), after a first one that keeps the GPU busy
    ia0, ia1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    last = n_frames - 1
    guess = scenes.kifi_matrix(poses[last - 1])
    check(lib.kifi_icp_align_device(icp, C.c_void_p(frames[last].data_ptr()), 1, C.byref(cam), ptr(guess),
                                    ICP_ITERS))
    ia0.record(ist)
    check(lib.kifi_icp_align_device(icp, C.c_void_p(frames[last].data_ptr()), 1, C.byref(cam), ptr(guess),
                                    ICP_ITERS))
    ia1.record(ist)
    ia1.synchronize()
    iso_icp_ms = ia0.elapsed_time(ia1)
    body = np.zeros(64, np.float32)
    tail = np.zeros(64, np.float32)
    nit = C.c_int()
    check(lib.kifi_icp_iteration_times(icp, ptr(body), ptr(tail), 64, C.byref(nit)))

    gb, gu = C.c_longlong(), C.c_longlong()
    check(lib.kifi_pipeline_graph_stats(pipe, C.byref(gb), C.byref(gu)))

    if rank != 0:
        lib.kifi_pipeline_destroy(pipe)
        if world > 1:
            dist.destroy_process_group()
        return

    P = W * H
    peak, sm_mhz_max, peak_kind = measured_peaks()
    fp32_peak = sms * FP32_LANES_PER_SM * 2 * sm_mhz_max * 1e6 / 1e12  # TFLOP/s
    fp32_src = "computed: %d SMs x %d FP32 lanes x 2 flop x %.0f MHz" % (sms, FP32_LANES_PER_SM, sm_mhz_max)
    per = max(nst.value, 1)

    def gbs(nbytes, ms_):
        return nbytes / (ms_ * 1e-3) / 1e9 if ms_ > 0 else 0.0

    # algorithmic bytes per launch (each input read once, each output written once)
    merge_bytes = float((12.0 * n0 + 4.0 * ne + 12.0 * n1 + 2.0 * P).mean())
    splat_bytes = float((2.0 * P + 4.0 * ne).mean())
    sort_bytes = float((8.0 * ne).mean())
    merge_ms = ms_stage[3] / per
    iso_per = max(iso_n.value, 1)
    iso_merge_bytes = float((12.0 * i0 + 4.0 * ie + 12.0 * i1 + 2.0 * P).mean())
    iso_splat_bytes = float((2.0 * P + 4.0 * ie).mean())
    iso_sort_bytes = float((8.0 * ie).mean())
    mv, mi = region_mesh
    mesh_bytes = 12.0 * float(n1[-1]) + 12.0 * mv + 4.0 * mi  # keys+values, vertices, triangles (12 B each)
    iso_mesh_bytes = 12.0 * n_mesh_vox.value + 12.0 * nvi.value + 4.0 * nii.value
    icp_flops = (P / 4.0) * 441.0 * 10.0  # per iteration: P/4 sources x 441 candidates x 10 flop
    track_step_ms = pipe_ms[0] / ICP_ITERS
    iso_step_ms = iso_icp_ms / ICP_ITERS
    tr_merge = ncu_traffic("merge_update_traffic.json")
    traffic = None
    if tr_merge:
        traffic = float(tr_merge["bytes_per_voxel"] * float((n0 + n1).mean()) + tr_merge.get("bytes_fixed", 0.0))

    kernels = {
        "k_splat_emit": roofline_entry(
            "hbm", gbs(splat_bytes, ms_stage[0] / per), peak, "GB/s",
            {"bytes_per_launch": splat_bytes, "bytes_rule": "2 B per pixel + 4 B per new key"},
            ms_stage[0] / per, peak_kind,
            {"isolated": {"ms_per_launch": iso_stage[0] / iso_per,
                          "frac": gbs(iso_splat_bytes, iso_stage[0] / iso_per) / peak}}),
        "sort (three 10-bit digit passes; set-up and digit counts ride on the set-up and splat kernels)": roofline_entry(
            "hbm", gbs(sort_bytes, ms_stage[1] / per), peak, "GB/s",
            {"bytes_per_launch": sort_bytes, "bytes_rule": "8 B per new key"}, ms_stage[1] / per, peak_kind,
            {"isolated": {"ms_per_launch": iso_stage[1] / iso_per,
                          "frac": gbs(iso_sort_bytes, iso_stage[1] / iso_per) / peak}}),
        "k_merge_update": roofline_entry(
            "hbm", gbs(merge_bytes, merge_ms), peak, "GB/s",
            {"bytes_per_launch": merge_bytes, "bytes_rule": "12 B per resident voxel in and out + 4 B per new key "
                                                            "+ 2 B per pixel"}, merge_ms, peak_kind,
            {"traffic": traffic,
             "isolated": {"ms_per_launch": iso_stage[3] / iso_per,
                          "frac": gbs(iso_merge_bytes, iso_stage[3] / iso_per) / peak}}),
        "mesher (row directory, classify, scan, emit)": roofline_entry(
            "hbm", gbs(mesh_bytes, pipe_ms[1]), peak, "GB/s",
            {"bytes_per_launch": mesh_bytes, "bytes_rule": "12 B per voxel + 12 B per vertex + 12 B per triangle",
             "per": "mesh"}, pipe_ms[1], peak_kind,
            {"meshes": int(pipe_n[1]),
             "isolated": {"ms_per_launch": iso_mesh_ms.value, "voxels": n_mesh_vox.value,
                          "frac": gbs(iso_mesh_bytes, iso_mesh_ms.value) / peak,
                          "stage_ms": {"row_directory": iso_mesh[0], "classification": iso_mesh[1],
                                       "scan": iso_mesh[2], "emission": iso_mesh[3]}}}),
        "k_icp_step": roofline_entry(
            "fp32", icp_flops / (track_step_ms * 1e-3) / 1e12 if track_step_ms > 0 else 0.0, fp32_peak, "TFLOP/s",
            {"flop_per_launch": icp_flops, "flop_rule": "P/4 sources x 441 window candidates x 10 flop"},
            track_step_ms, fp32_src,
            {"isolated": {"ms_per_launch": iso_step_ms,
                          "frac": icp_flops / (iso_step_ms * 1e-3) / 1e12 / fp32_peak if iso_step_ms > 0 else 0.0,
                          "association_us_median": float(np.median(body[:min(nit.value, 64)])),
                          "finisher_us_median": float(np.median(tail[:min(nit.value, 64)]))}}),
    }
    value = job_throughput(world, KF, ms / 1e3)
    steps_launches = K * (FS * (LAUNCHES_FUSION + LAUNCHES_TRACKING) + LAUNCHES_MESH)
    # `config` names the workload (the reference arm prints the same dict); `run` describes this run
    cfg = workload_config(Fp, FS)
    run = {"resident_voxels_start": n_start, "resident_voxels_end": int(n1[-1]) if m else None,
           "roofline_frames": "the last %d timed frames (the device frame log's length)" % m,
           "sequence_frames": SEQ_FRAMES, "frames_fused": n_frames,
           "playback": "frames 0-299 forward, then back (%d frames fused in all)" % n_frames,
           "parallelism": "replicas" if world > 1 else "single"}
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K,
        "warmup": Wu, "ms_per_step": ms / K, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+u32", "data": "synthetic",
        "config": cfg, "run": run,
        "roofline": dict(kernels["k_merge_update"], kernel="k_merge_update (fused merge-path union + TSDF update)",
                         kernels=kernels),
        "stage_ms_per_frame": {"splat_emit": ms_stage[0] / per, "sort": ms_stage[1] / per,
                               "merge_partition": ms_stage[2] / per, "merge_update": merge_ms,
                               "icp_alignment": pipe_ms[0], "mesh_per_10_frames": pipe_ms[1]},
        "e2e": {"value": job_throughput(world, KF, e2e_s), "unit": UNIT,
                "h2d_bytes_per_step": FS * (2 * P + 64),
                "d2h_bytes_per_step": FS * ICP_HEAD_BYTES + MESH_COUNTS_BYTES},
        "gpu_launches": steps_launches,
        "mesh": {"meshes_in_region": meshes1 - meshes0, "reemitted_in_region": reemit1 - reemit0,
                 "vertices": region_mesh[0], "indices": region_mesh[1],
                 "same_after_sync": region_mesh == synced_mesh,
                 "joined": "the device region's end event follows the mesh stream (kifi_pipeline_join)"},
        "graphs": {"on": bool(args.graphs), "instantiated": int(gb.value), "updated": int(gu.value)},
        "autotune": None if args.no_autotune else {"splat_ctas": int(tuned[0]), "sort_ctas": int(tuned[1]),
                                                   "merge_ctas": int(tuned[2])},
    }
    line["clocks"] = clocks.summary()
    if resident is not None:
        frames_host = seq_host[order[:t0 + KF + 1]]  # the playback order, up to the timed frames
        v, kind, nfr, tmesh = cpu_frames(frames_host, poses, t0, KF, args.cpu_seconds, resident)
        hc = host_cpu()
        cb = {"value": v, "unit": UNIT, "cores": 1, "kind": kind,
              "sample": "%d frames (integrate + 15 ICP iterations each) from the same resident volume, plus one "
                        "mesh (%.2f s) amortised over 10 frames; single-threaded, as the reference is"
                        % (nfr, tmesh)}
        cb.update(hc)
        procs = max(1, int(hc["nproc"] or 1))
        try:
            agg, res = cpu_aggregate(frames_host, poses, t0, KF, args.cpu_seconds, resident, procs)
            cb["aggregate"] = {"value": agg, "unit": UNIT, "processes": procs,
                               "sample": "one scene per core: %d processes each run the same bounded sample "
                                         "at once (%d-%d frames each); frames/s summed" %
                                         (procs, min(r[2] for r in res), max(r[2] for r in res))}
        except Exception as e:  # the aggregate is context, not the baseline
            cb["aggregate"] = {"unavailable": str(e)[:200]}
        line["cpu_baseline"] = cb
    lib.kifi_pipeline_destroy(pipe)
    if not args.no_learned:
        line["icp_iterations"] = learned_vs_plain()
    if not args.no_batched:
        line["batched"] = batched_scenes()
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
    out = {"plain": res["plain_iterations"], "learned": res["learned_iterations"], "ratio": res["ratio"],
           "pairs": res["pairs"], "fallbacks": res["fallbacks"], "criterion": "RMS change < 1e-4 m",
           "held_out": "room trajectories %d-%d, pairs (a, a+k), k = 1..3" % (seeds[0], seeds[-1]),
           "median_pose_diff": res["median_pose_diff"], "plain_spread_median": res["plain_spread_median"]}
    for k in ("plain_error_median", "learned_error_median", "same_pose_1e-5"):
        if k in res:
            out[k] = res[k]
    return out


def batched_scenes():
    """64 seeded scenes with uneven frame sizes ({320x240, 512x424, 640x480,
    1024x848}), voxel sizes ({2, 4, 8} mm, truncation 5 voxels) and
    trajectory lengths (50-300 frames) through one kifi_batch: each step is
    one launch per stage for every scene that still has frames.  The same
    frames again with the fusion as one persistent launch over a device work
    queue (`persistent_queue`)."""
    from merge_fusion_gb300 import batched as bt
    specs = bt.scene_specs(64, 7)
    rendered = bt.render_batch(specs, unique=40)
    res = bt.run_batch(specs, unique=40, icp_iters=ICP_ITERS, rendered=rendered)
    q = bt.run_batch(specs, unique=40, icp_iters=ICP_ITERS, persistent=True, queue_ctas_per_sm=1, rendered=rendered)
    res["persistent_queue"] = {k: q[k] for k in ("mode", "frames", "seconds", "frames_per_s", "step_latency_ms_p50",
                                                 "step_latency_ms_p99")}
    res["mix"] = {"sizes": {"%dx%d" % (w, h): sum(1 for s in specs if s["width"] == w) for w, h, _ in bt.SIZES},
                  "voxels_mm": {str(v): sum(1 for s in specs if s["voxel_mm"] == v) for v in bt.VOXELS_MM},
                  "trajectory_frames": [min(s["frames"] for s in specs), max(s["frames"] for s in specs)]}
    return res


def run_reference(args, rank, world):
    if rank != 0:
        return
    from merge_fusion_gb300 import scenes
    # a bounded sample of the same workload: the first frames of the timed range
    K = min(args.steps * FRAMES_PER_STEP, REF_MAX_TIMED_FRAMES)
    Wu, Fp = min(args.warmup, 3), args.prefill
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
    hc = host_cpu()
    cb = {"value": value, "unit": UNIT, "cores": 1, "kind": kind,
          "sample": "%d timed frames (of the %d requested) after %d warm-up frames and %d fusion-only prefill "
                    "frames; single-threaded: the reference fuses one scene on one thread"
                    % (K, args.steps * FRAMES_PER_STEP, Wu, Fp)}
    cb.update(hc)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tt / K * FRAMES_PER_STEP,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+u32",
            "data": "synthetic", "config": workload_config(Fp, FRAMES_PER_STEP),
            "cpu_baseline": cb,
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
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
