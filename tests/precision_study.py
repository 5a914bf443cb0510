"""Precision study on a large volume with 64-bit keys (a test-side driver:
it runs the GPU library and checks it against the oracle).

    python -m tests.precision_study [--frames 200] [--tsdf-frames 10]
                                    [--chain-frames 200] [--workers 15]

Workload: frames of 512x424 uint16 depth (fx = fy = 365, cx = 256,
cy = 212) of the seeded room generator stretched to 8 x 3 x 8 m, fused into
a 4096^3 volume of 2 mm voxels (8.192 m cube, truncation 1 cm), which needs
64-bit keys (12 bits per axis).  Reported:

* fusion: resident voxels as the frames go in and the GPU's fusion rate
  (frames already on the device, ground-truth poses);
* TSDF error: the GPU volume after the first `tsdf_frames` frames against
  the oracle's 64-bit path (keys equal, values compared bit for bit and by
  absolute error);
* per-frame pose error: each frame-to-frame ICP (15 iterations) of the GPU
  -- float per-point work, compensated float reductions, float-float Horn
  solve and pose -- against the oracle's FP64 run on the same inputs
  (double sums, double Horn matrix and Jacobi eigen-solve, double pose);
  also the GPU's float pose against the reference's own float arithmetic;
* accumulated drift: the GPU's frame-to-frame tracking chain against an
  FP64 oracle chain from the same first pose, and both against the ground
  truth (translation in metres, rotation in degrees).

The oracle runs in a spawn process pool (single-threaded C per call); the
FP64 chain is sequential and dominates the wall time (about 2 s a frame).
"""
import argparse
import json
import time

import numpy as np

RES, SIDE, TRUNC = 4096, 8.192, 0.01
W, H, F = 512, 424, 365.0
CAM = (W, H, F, F, W / 2.0, H / 2.0, 0.4, 4.0)


def _mat(m16):
    """kifi (16,) column-major -> 4x4 float64."""
    return np.asarray(m16, np.float64).reshape(4, 4).T


def _rotation(m):
    """Nearest rotation to the 3x3 block (polar factor): accumulated poses
    drift slightly off orthonormal, which an angle read off the trace would
    mistake for a rotation."""
    u, _, vt = np.linalg.svd(m[:3, :3])
    return u @ vt


def pose_diff(a16, b16):
    """(translation difference in metres, rotation difference in degrees);
    the angle is 2 asin(|Qa - Qb|_F / sqrt 8), stable for small angles."""
    a, b = _mat(a16), _mat(b16)
    dt = float(np.linalg.norm(a[:3, 3] - b[:3, 3]))
    d = np.linalg.norm(_rotation(a) - _rotation(b)) / np.sqrt(8.0)
    return dt, float(np.degrees(2.0 * np.arcsin(min(1.0, d))))


def orthonormality_defect(m16):
    r = _mat(m16)[:3, :3]
    return float(np.abs(r.T @ r - np.eye(3)).max())


def _depth_m(frame_u16):
    return frame_u16.astype(np.float32) * np.float32(0.001)


def _oracle_step(args):
    """FP64 and reference-float ICP of one frame on the GPU chain's inputs."""
    from oracle import cpu
    depth, prev_depth, guess, iters = args
    tgt = cpu.backproject(_depth_m(prev_depth), CAM, guess)
    _, od, _ = cpu.icp_align(_depth_m(depth), CAM, guess, tgt, guess, iters, fp64=True)
    of, _, _ = cpu.icp_align(_depth_m(depth), CAM, guess, tgt, guess, iters, fp64=False)
    return od, of


def _oracle_chain(args):
    """The FP64 oracle's own frame-to-frame tracking chain."""
    from oracle import cpu
    frames, first_pose, iters = args
    poses = [np.asarray(first_pose, np.float64)]
    for i in range(1, len(frames)):
        guess = poses[-1].astype(np.float32)
        tgt = cpu.backproject(_depth_m(frames[i - 1]), CAM, guess)
        _, od, _ = cpu.icp_align(_depth_m(frames[i]), CAM, guess, tgt, guess, iters, fp64=True)
        poses.append(od)
    return poses


def _oracle_tsdf(args):
    from oracle import cpu
    frames, w2e = args
    v = cpu.Volume64(RES, SIDE, TRUNC)
    for f, m in zip(frames, w2e):
        v.integrate(_depth_m(f), CAM, m)
    return v.keys, v.values


def run(frames=200, tsdf_frames=10, chain_frames=None, workers=4, seed=0, icp_iters=15):
    import ctypes as C
    import multiprocessing as mp
    chain_frames = frames if chain_frames is None else min(chain_frames, frames)
    tsdf_frames = min(tsdf_frames, frames)
    # the pool starts before the first GPU call
    pool = mp.get_context("spawn").Pool(workers)
    try:
        import torch
        from merge_fusion_gb300 import _lib, kifi, scenes
        from merge_fusion_gb300._lib import Camera, check
        from tests.helpers import canon_bits, cam_params
        lib = _lib.load()
        t0 = time.perf_counter()
        dev, poses = scenes.render_room_torch(frames, seed=seed, width=W, height=H, f=F, scale=2.0)
        host = dev.cpu().numpy().view(np.uint16)
        e2w = [scenes.kifi_matrix(p) for p in poses]
        w2e = [scenes.kifi_matrix(np.linalg.inv(p)) for p in poses]
        t_render = time.perf_counter() - t0
        # the oracle's work goes out first so that it overlaps the GPU's
        tsdf_job = pool.apply_async(_oracle_tsdf, ((host[:tsdf_frames], w2e[:tsdf_frames]),))
        chain_job = pool.apply_async(_oracle_chain, ((host[:chain_frames], e2w[0], icp_iters),))

        # fusion with ground-truth poses, frames resident on the device
        vol = kifi.Volume(RES, SIDE, TRUNC)
        assert (vol.key_bits, vol.bits_per_axis) == (64, 12)
        cam = Camera(*CAM)
        st = torch.cuda.ExternalStream(vol.stream())
        counts, gpu_tsdf = {}, None
        fuse_s = 0.0
        for i in range(frames):
            torch.cuda.synchronize()
            t = time.perf_counter()
            check(lib.kifi_integrate_device(vol.handle, C.c_void_p(dev[i].data_ptr()), 1, C.byref(cam),
                                            w2e[i].ctypes.data_as(C.c_void_p)), "integrate")
            vol.sync()
            st.synchronize()
            fuse_s += time.perf_counter() - t
            if i + 1 in (1, 10, 50, 100, 150, 200) or i + 1 == frames:
                counts[i + 1] = vol.size()
            if i + 1 == tsdf_frames:
                gpu_tsdf = vol.export()
        n_final = vol.size()
        vol.close()

        # GPU tracking chain: frame i aligned to frame i-1 at the chain's pose
        icp = kifi.ICP()
        cp = cam_params(CAM)
        chain_f, chain_d, n_assoc = [e2w[0]], [e2w[0].astype(np.float64)], []
        steps = []
        t = time.perf_counter()
        for i in range(1, frames):
            prev = chain_f[-1]
            icp.SetTargetFromDepth(host[i - 1], cp, prev)
            icp.AlignToTarget(_depth_m(host[i]), prev, cp, iterations=icp_iters)
            pf, pd, na, _ = icp.Result()
            chain_f.append(pf.copy())
            chain_d.append(pd.copy())
            n_assoc.append(int(na[-1]) if na.size else 0)
            steps.append((host[i], host[i - 1], prev, icp_iters))
        icp_s = time.perf_counter() - t
        per = pool.map(_oracle_step, steps, chunksize=4)

        err_elem = [float(np.abs(chain_d[i + 1] - od).max()) for i, (od, _) in enumerate(per)]
        err_pose = [pose_diff(chain_d[i + 1], od) for i, (od, _) in enumerate(per)]
        err_float = [float(np.abs(chain_f[i + 1] - of).max()) for i, (_, of) in enumerate(per)]
        err_ref_float = [float(np.abs(of - od).max()) for od, of in per]
        err_gpu_float = [float(np.abs(chain_f[i + 1] - od).max()) for i, (od, _) in enumerate(per)]

        ok, ov = tsdf_job.get()
        gk, gv = gpu_tsdf
        keys_equal = bool(gk.size == ok.size and np.array_equal(gk, ok))
        tsdf = {"frames": tsdf_frames, "voxels_gpu": int(gk.size), "voxels_oracle": int(ok.size),
                "keys_equal": keys_equal}
        if keys_equal:
            bit_diff = int((canon_bits(gv) != canon_bits(ov)).any(1).sum())
            fin = np.isfinite(gv) & np.isfinite(ov)
            tsdf.update(values_bit_different=bit_diff,
                        max_abs_error_distance_sum=float(np.abs(gv[:, 0] - ov[:, 0])[fin[:, 0]].max(initial=0)),
                        max_abs_error_weight=float(np.abs(gv[:, 1] - ov[:, 1])[fin[:, 1]].max(initial=0)))

        chain64 = chain_job.get()
        marks = sorted({m for m in (10, 50, 100, 150, chain_frames) if m <= chain_frames})
        drift = []
        for m in marks:
            j = m - 1
            g_vs_64 = pose_diff(chain_d[j], chain64[j])
            g_vs_gt = pose_diff(chain_d[j], e2w[j])
            o_vs_gt = pose_diff(chain64[j], e2w[j])
            drift.append({"frame": m, "gpu_vs_fp64_m": g_vs_64[0], "gpu_vs_fp64_deg": g_vs_64[1],
                          "gpu_vs_fp64_max_abs": float(np.abs(chain_d[j] - chain64[j]).max()),
                          "orthonormality_defect_gpu": orthonormality_defect(chain_d[j]),
                          "gpu_vs_truth_m": g_vs_gt[0], "gpu_vs_truth_deg": g_vs_gt[1],
                          "fp64_vs_truth_m": o_vs_gt[0], "fp64_vs_truth_deg": o_vs_gt[1]})
        return {
            "workload": "room 8x3x8 m, %d frames of %dx%d uint16, 2 mm voxels (4096^3, 64-bit keys), "
                        "truncation 1 cm, ICP %d iterations frame-to-frame" % (frames, W, H, icp_iters),
            "render_s": t_render,
            "fusion": {"voxels_after_frames": {str(k): int(v) for k, v in counts.items()},
                       "voxels_final": int(n_final), "frames_per_s": frames / fuse_s},
            "tsdf_vs_oracle64": tsdf,
            "icp_per_frame_vs_fp64": {
                "frames": len(per), "max_abs_pose_element": max(err_elem),
                "median_abs_pose_element": float(np.median(err_elem)),
                "max_translation_m": max(e[0] for e in err_pose), "max_rotation_deg": max(e[1] for e in err_pose),
                "float_pose_vs_reference_float_max_abs": max(err_float),
                "gpu_float_pose_vs_fp64_max_abs": max(err_gpu_float),
                "reference_float_pose_vs_fp64_max_abs": max(err_ref_float),
                "mean_associations": float(np.mean(n_assoc)), "gpu_icp_frames_per_s": len(per) / icp_s},
            "drift": drift,
        }
    finally:
        pool.close()
        pool.join()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--frames", type=int, default=200)
    ap.add_argument("--tsdf-frames", type=int, default=10)
    ap.add_argument("--chain-frames", type=int, default=None)
    ap.add_argument("--workers", type=int, default=15)
    ap.add_argument("--seed", type=int, default=0)
    args = ap.parse_args()
    t = time.perf_counter()
    res = run(args.frames, args.tsdf_frames, args.chain_frames, args.workers, args.seed)
    res["wall_s"] = time.perf_counter() - t
    print(json.dumps(res), flush=True)


if __name__ == "__main__":
    main()
