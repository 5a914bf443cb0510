"""Learned ICP warm start: data generation, training and evaluation around
the pose proposer network of libkifi_gpu (kifi_proposer_*).

A training pair is two depth frames (a, b) of a seeded synthetic room
trajectory.  Its label is the pose of frame b relative to frame a, taken from
plain ICP run to convergence from the identity guess (frame a's pose), as
the 6-vector (rotation vector, translation) in frame a's camera frame.  At
inference the predicted relative pose composes onto the guess and ICP starts
from there; when the warm-started ICP ends with an RMS residual above 1.5x
the plain ICP's, the plain result is kept (the fallback)."""
import ctypes as C
import math

import numpy as np

from . import _lib, scenes
from ._lib import Camera, check

IN_H, IN_W = 60, 80
CAMERA = (640, 480, 585.0, 585.0, 320.0, 240.0, 0.4, 4.0)


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


# ------------------------------------------------------------- pose maths

def rotvec_to_matrix(w):
    w = np.asarray(w, np.float64)
    th = np.linalg.norm(w)
    if th < 1e-12:
        return np.eye(3)
    k = w / th
    K = np.array([[0, -k[2], k[1]], [k[2], 0, -k[0]], [-k[1], k[0], 0]])
    return np.eye(3) + math.sin(th) * K + (1 - math.cos(th)) * K @ K


def matrix_to_rotvec(R):
    c = max(-1.0, min(1.0, (np.trace(R) - 1.0) / 2.0))
    th = math.acos(c)
    if th < 1e-9:
        return np.array([R[2, 1] - R[1, 2], R[0, 2] - R[2, 0], R[1, 0] - R[0, 1]]) / 2.0
    v = np.array([R[2, 1] - R[1, 2], R[0, 2] - R[2, 0], R[1, 0] - R[0, 1]])
    return v * th / (2.0 * math.sin(th))


def pose_to_vec(T):
    return np.concatenate([matrix_to_rotvec(T[:3, :3]), T[:3, 3]])


def vec_to_pose(v):
    T = np.eye(4)
    T[:3, :3] = rotvec_to_matrix(v[:3])
    T[:3, 3] = v[3:]
    return T


def kifi_to_mat(m16):
    return np.asarray(m16, np.float64).reshape(4, 4).T


# ---------------------------------------------------------------- network

def init_params(seed=0):
    """He-normal weights, a small output layer, zero biases and padding, in
    the library's parameter layout (float32 vector)."""
    rng = np.random.default_rng(seed)
    convs = [(2, 32, 32), (32, 64, 288), (64, 64, 576), (64, 128, 576)]
    parts = []
    for cin, cout, kp in convs:
        w = np.zeros((cout, kp))
        w[:, :9 * cin] = rng.normal(0.0, np.sqrt(2.0 / (9 * cin)), (cout, 9 * cin))
        parts += [w, np.zeros(cout)]
    parts += [rng.normal(0.0, np.sqrt(2.0 / 128), (64, 128)), np.zeros(64)]
    w2 = np.zeros((16, 64))
    w2[:6] = rng.normal(0.0, 0.01, (6, 64))
    parts += [w2, np.zeros(16)]
    out = []
    for t in parts:
        v = np.asarray(t, np.float32).reshape(-1)
        out += [v, np.zeros((-v.size) % 8, np.float32)]
    return np.concatenate(out)


class PoseProposer:
    """The network (kifi_proposer_*): inputs live in a device FP16 tensor
    [batch, 60, 80, 2]; predictions and losses come back to the host."""

    def __init__(self, device=0, max_batch=256):
        self._h = None
        h = C.c_void_p()
        check(_lib.load().kifi_proposer_create(int(device), int(max_batch), C.byref(h)), "proposer")
        self._h = h
        self.max_batch = int(max_batch)
        n = C.c_size_t()
        check(_lib.load().kifi_proposer_param_count(h, C.byref(n)))
        self.n_params = n.value

    def __del__(self):
        self.close()

    def close(self):
        if self._h is not None:
            _lib.load().kifi_proposer_destroy(self._h)
            self._h = None

    def set_params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        check(_lib.load().kifi_proposer_set_params(self._h, _ptr(p), p.size), "set_params")

    def get_params(self):
        p = np.zeros(self.n_params, np.float32)
        check(_lib.load().kifi_proposer_get_params(self._h, _ptr(p), p.size), "get_params")
        return p

    def make_input(self, depth_a_ptr, depth_b_ptr, u16, width, height, out_ptr):
        check(_lib.load().kifi_proposer_make_input(self._h, C.c_void_p(depth_a_ptr), C.c_void_p(depth_b_ptr),
                                                   1 if u16 else 0, int(width), int(height),
                                                   C.c_void_p(out_ptr)), "make_input")

    def set_inputs(self, x):
        check(_lib.load().kifi_proposer_set_inputs(self._h, C.c_void_p(x.data_ptr()), int(x.shape[0])),
              "set_inputs")

    def predict(self, x):
        self.set_inputs(x)
        out = np.zeros((x.shape[0], 6), np.float32)
        check(_lib.load().kifi_proposer_predict(self._h, int(x.shape[0]), _ptr(out)), "predict")
        return out

    def gradients(self, x, targets):
        self.set_inputs(x)
        loss = np.zeros(1, np.float32)
        g = np.zeros(self.n_params, np.float32)
        check(_lib.load().kifi_proposer_gradients(self._h, C.c_void_p(targets.data_ptr()), int(x.shape[0]),
                                                  _ptr(loss), _ptr(g)), "gradients")
        return float(loss[0]), g

    def train_step(self, x, targets, lr):
        self.set_inputs(x)
        loss = np.zeros(1, np.float32)
        check(_lib.load().kifi_proposer_train_step(self._h, C.c_void_p(targets.data_ptr()), int(x.shape[0]),
                                                   C.c_float(lr), _ptr(loss)), "train_step")
        return float(loss[0])


# ------------------------------------------------------------------ data

class _Icp:
    def __init__(self):
        self.lib = _lib.load()
        self.h = C.c_void_p()
        check(self.lib.kifi_icp_create(0, None, C.byref(self.h)), "icp")
        self.cam = Camera(*CAMERA)

    def close(self):
        self.lib.kifi_icp_destroy(self.h)

    def set_target(self, depth_dev, e2w16):
        check(self.lib.kifi_icp_set_target_from_depth(self.h, C.c_void_p(depth_dev), 1, 1, C.byref(self.cam),
                                                      _ptr(e2w16)), "target")

    def align(self, depth_dev, guess16, iterations):
        """(final pose 4x4 float64, per-iteration RMS)"""
        check(self.lib.kifi_icp_align_device(self.h, C.c_void_p(depth_dev), 1, C.byref(self.cam),
                                             _ptr(guess16), int(iterations)), "align")
        pf = np.zeros(16, np.float32)
        pd = np.zeros(16, np.float64)
        na = np.zeros(64, np.int32)
        rms = np.zeros(64, np.float64)
        it = C.c_int()
        check(self.lib.kifi_icp_result(self.h, _ptr(pf), _ptr(pd), _ptr(na), _ptr(rms), 64, C.byref(it)),
              "result")
        return pd.reshape(4, 4).T.copy(), pf, rms[:it.value].copy()


def pose_error(T, truth):
    """(translation error in metres, rotation error in radians) of an
    eye-to-world pose against the ground truth."""
    T, truth = np.asarray(T, np.float64), np.asarray(truth, np.float64)
    dR = T[:3, :3].T @ truth[:3, :3]
    c = max(-1.0, min(1.0, (np.trace(dR) - 1.0) / 2.0))
    return float(np.linalg.norm(T[:3, 3] - truth[:3, 3])), math.acos(c)


def iterations_to_converge(rms, tol=1e-4):
    """First iteration whose RMS residual changed by less than tol (metres)
    from the previous one; len(rms) when none did."""
    for k in range(1, len(rms)):
        if abs(rms[k] - rms[k - 1]) < tol:
            return k
    return len(rms)


def make_pairs(proposer, seeds, frames_per_traj, steps=(1, 2, 3), icp_iters=40, device="cuda"):
    """Inputs [N, 60, 80, 2] FP16 on the device, labels [N, 6] (relative pose
    vectors from converged plain ICP) and per-pair (seed, a, b, pose a)."""
    import torch
    icp = _Icp()
    xs, ys, meta = [], [], []
    try:
        for seed in seeds:
            frames, poses = scenes.render_room_torch(frames_per_traj, seed=seed, device=device, noise="device")
            e2w = [scenes.kifi_matrix(p) for p in poses]
            n = frames_per_traj - max(steps)
            x = torch.zeros((n * len(steps), IN_H, IN_W, 2), dtype=torch.float16, device=device)
            j = 0
            for a in range(n):
                icp.set_target(frames[a].data_ptr(), e2w[a])
                for k in steps:
                    b = a + k
                    T, _, _ = icp.align(frames[b].data_ptr(), e2w[a], icp_iters)
                    rel = np.linalg.inv(kifi_to_mat(e2w[a])) @ T
                    ys.append(pose_to_vec(rel))
                    proposer.make_input(frames[a].data_ptr(), frames[b].data_ptr(), True, 640, 480,
                                        x[j].data_ptr())
                    meta.append((seed, a, b))
                    j += 1
            xs.append(x)
            del frames
    finally:
        icp.close()
    return torch.cat(xs), np.asarray(ys, np.float64), meta


def train(proposer, x, y, steps=3000, batch=256, lr=1e-3, seed=0, log_every=250):
    """Adam on the standardised labels; returns (mean, std, loss history)."""
    import torch
    mean, std = y.mean(axis=0), y.std(axis=0) + 1e-12
    yt = torch.from_numpy(((y - mean) / std).astype(np.float32)).to(x.device)
    g = torch.Generator(device="cpu").manual_seed(seed)
    hist = []
    for s in range(steps):
        idx = torch.randint(0, x.shape[0], (batch,), generator=g).to(x.device)
        rate = lr * 0.5 * (1.0 + math.cos(math.pi * s / steps))
        loss = proposer.train_step(x[idx].contiguous(), yt[idx].contiguous(), rate)
        if s % log_every == 0 or s == steps - 1:
            hist.append((s, loss))
    return mean, std, hist


def evaluate(proposer, mean, std, seeds, frames_per_traj, steps=(1, 2, 3), icp_iters=60, max_pairs=1000,
             device="cuda"):
    """Plain vs learned-warm-started ICP on held-out trajectories: iterations
    to converge (RMS change < 1e-4 m), the final pose difference, the final
    pose error against the generator's ground truth (translation in metres,
    rotation in radians) of either start, fallbacks."""
    import torch
    icp = _Icp()
    it_plain, it_learned, diffs, spread, fallbacks, n = [], [], [], [], 0, 0
    err_plain, err_learned = [], []
    rng = np.random.default_rng(12345)
    try:
        for seed in seeds:
            frames, poses = scenes.render_room_torch(frames_per_traj, seed=seed, device=device, noise="device")
            e2w = [scenes.kifi_matrix(p) for p in poses]
            na = frames_per_traj - max(steps)
            x = torch.zeros((8, IN_H, IN_W, 2), dtype=torch.float16, device=device)
            for a in range(na):
                for k in steps:
                    if n >= max_pairs:
                        break
                    b = a + k
                    proposer.make_input(frames[a].data_ptr(), frames[b].data_ptr(), True, 640, 480,
                                        x[0].data_ptr())
                    pred = proposer.predict(x)[0].astype(np.float64) * std + mean
                    guess = kifi_to_mat(e2w[a])
                    warm = scenes.kifi_matrix(guess @ vec_to_pose(pred))
                    icp.set_target(frames[a].data_ptr(), e2w[a])
                    Tp, _, rp = icp.align(frames[b].data_ptr(), e2w[a], icp_iters)
                    Tl, _, rl = icp.align(frames[b].data_ptr(), warm, icp_iters)
                    # the method's own spread: plain ICP from a start moved by 1 mm / 0.05 deg
                    jig = vec_to_pose(np.concatenate([rng.normal(size=3) * (8.7e-4 / math.sqrt(3)),
                                                      rng.normal(size=3) * (1e-3 / math.sqrt(3))]))
                    Tj, _, _ = icp.align(frames[b].data_ptr(), scenes.kifi_matrix(guess @ jig), icp_iters)
                    spread.append(float(np.abs(Tj - Tp).max()))
                    kp, kl = iterations_to_converge(rp), iterations_to_converge(rl)
                    if rl[-1] > 1.5 * rp[-1]:  # fallback to the plain result
                        fallbacks += 1
                        kl, Tl = kp, Tp
                    it_plain.append(kp)
                    it_learned.append(kl)
                    diffs.append(float(np.abs(Tl - Tp).max()))
                    err_plain.append(pose_error(Tp, poses[b]))
                    err_learned.append(pose_error(Tl, poses[b]))
                    n += 1
            del frames
            if n >= max_pairs:
                break
    finally:
        icp.close()
    diffs = np.asarray(diffs)
    ep, el = np.asarray(err_plain), np.asarray(err_learned)
    return {"pairs": n, "plain_iterations": float(np.mean(it_plain)),
            "plain_error_median": {"m": float(np.median(ep[:, 0])), "rad": float(np.median(ep[:, 1]))},
            "learned_error_median": {"m": float(np.median(el[:, 0])), "rad": float(np.median(el[:, 1]))},
            "plain_error_p90": {"m": float(np.percentile(ep[:, 0], 90)), "rad": float(np.percentile(ep[:, 1], 90))},
            "learned_error_p90": {"m": float(np.percentile(el[:, 0], 90)),
                                  "rad": float(np.percentile(el[:, 1], 90))},
            "learned_iterations": float(np.mean(it_learned)),
            "ratio": float(np.mean(it_learned) / max(np.mean(it_plain), 1e-12)),
            "fallbacks": fallbacks, "max_pose_diff": float(diffs.max()),
            "median_pose_diff": float(np.median(diffs)),
            "same_pose_1e-5": float((diffs <= 1e-5).mean()),
            "plain_spread_median": float(np.median(spread)), "plain_spread_max": float(np.max(spread)),
            "icp_iterations_run": icp_iters}


def save(path, params, mean, std, info):
    np.savez(path, params=params, mean=mean, std=std, **{k: np.asarray(v) for k, v in info.items()})


def load(path):
    d = np.load(path)
    return d["params"], d["mean"], d["std"]
