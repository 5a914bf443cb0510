"""Seeded synthetic depth sequences for the fusion path (host-side, numpy).

Stand-ins for recorded Kinect streams: analytic scenes are ray-cast into
planar depth images (depth = distance along the camera's viewing axis, the
convention of the reference's .depth generator, poly2depth/Depth.fx:33),
stored as uint16 millimetres like kifi's .depth files, with the depth-noise
model sigma(z) = 0.0012 + 0.0019 (z - 0.4)^2 m and optional pixel dropout.

Camera convention (kifi, KinectFission/kifi/Integrator.cpp:121-139): eye space
is right-handed with the camera looking down -z and y up; pixel (u, v) with v
growing downwards back-projects to ((u+0.5-cx)/fx d, (cy-0.5-v)/fy d, -d).
Poses are 4x4 float64 matrices (element [row, col]); ``world_to_eye`` is
what Integrator::Integrate takes.

Scenes:
* ``sphere_scene``: a 0.5 m sphere at (0, 0, 2) resting on the plane
  y = -0.5, 320x240, f = 292.5, a 5 cm-per-frame arc with 1 deg yaw per frame.
* ``room_scene``: a 4 x 3 x 4 m room centred at the origin holding 40 random
  axis-aligned boxes and 20 spheres (radius 0.1-0.6 m), 640x480, f = 585,
  range 0.4-4.0 m, a smooth trajectory with <= 2 cm and <= 1.5 deg per frame,
  2% dropout.  The scale argument stretches the room (8 x 3 x 8 m at 2).
"""
import math

import numpy as np


class Sequence:
    """A camera, a list of uint16 millimetre frames and their poses."""

    def __init__(self, width, height, fx, fy, cx, cy, znear, zfar, frames, eye_to_world):
        self.width, self.height = width, height
        self.fx, self.fy, self.cx, self.cy = fx, fy, cx, cy
        self.znear, self.zfar = znear, zfar
        self.frames = frames              # list of (h, w) uint16
        self.eye_to_world = eye_to_world  # list of 4x4 float64

    @property
    def camera(self):
        return (self.width, self.height, self.fx, self.fy, self.cx, self.cy, self.znear, self.zfar)

    def world_to_eye(self, i):
        return np.linalg.inv(self.eye_to_world[i])

    def world_to_eye_f32(self, i):
        """The pose as kifi's float4x4 memory (16 floats, column-major)."""
        return np.ascontiguousarray(self.world_to_eye(i).astype(np.float32).T).reshape(16)

    def eye_to_world_f32(self, i):
        return np.ascontiguousarray(self.eye_to_world[i].astype(np.float32).T).reshape(16)

    def depth_m(self, i):
        """Frame i as float metres exactly as kifi::DepthStream converts it."""
        return self.frames[i].astype(np.float32) * np.float32(0.001)


def _rot_y(a):
    c, s = math.cos(a), math.sin(a)
    return np.array([[c, 0, s], [0, 1, 0], [-s, 0, c]])


def _rot_x(a):
    c, s = math.cos(a), math.sin(a)
    return np.array([[1, 0, 0], [0, c, -s], [0, s, c]])


def _pose(R, t):
    m = np.eye(4)
    m[:3, :3] = R
    m[:3, 3] = t
    return m


def _rays(width, height, fx, fy, cx, cy):
    u = np.arange(width, dtype=np.float64)
    v = np.arange(height, dtype=np.float64)
    uu, vv = np.meshgrid(u, v)
    return np.stack([(uu + 0.5 - cx) / fx, (cy - 0.5 - vv) / fy, -np.ones_like(uu)], -1)


def _hit_spheres(o, d, centers, radii, t):
    for c, r in zip(centers, radii):
        oc = o - c
        b = d @ oc
        cc = oc @ oc - r * r
        a = np.einsum("ij,ij->i", d, d)
        disc = b * b - a * cc
        ok = disc >= 0
        sq = np.sqrt(np.where(ok, disc, 0))
        t0 = (-b - sq) / a
        t1 = (-b + sq) / a
        th = np.where(t0 > 1e-6, t0, t1)
        hit = ok & (th > 1e-6) & (th < t)
        t = np.where(hit, th, t)
    return t


def _hit_boxes(o, d, lo, hi, t):
    inv = 1.0 / np.where(d == 0, 1e-30, d)
    for a, b in zip(lo, hi):
        t1 = (a - o) * inv
        t2 = (b - o) * inv
        tn = np.minimum(t1, t2).max(1)
        tf = np.maximum(t1, t2).min(1)
        th = np.where(tn > 1e-6, tn, tf)
        hit = (tn <= tf) & (tf > 1e-6) & (th < t)
        t = np.where(hit, th, t)
    return t


def _room_inside(o, d, half):
    """Distance to the walls of the box [-half, half] from inside."""
    with np.errstate(divide="ignore"):
        tpos = np.where(d > 0, (half - o) / d, np.inf)
        tneg = np.where(d < 0, (-half - o) / d, np.inf)
    return np.minimum(tpos, tneg).min(1)


def _render(ray_eye, pose, scene, rng, znear, zfar, dropout):
    h, w, _ = ray_eye.shape
    R, o = pose[:3, :3], pose[:3, 3]
    d = ray_eye.reshape(-1, 3) @ R.T
    t = np.full(d.shape[0], np.inf)
    if "half" in scene:
        t = _room_inside(o, d, scene["half"])
    if "plane_y" in scene:
        with np.errstate(divide="ignore", invalid="ignore"):
            tp = (scene["plane_y"] - o[1]) / d[:, 1]
        t = np.where((tp > 1e-6) & (tp < t), tp, t)
    if "box_lo" in scene:
        t = _hit_boxes(o, d, scene["box_lo"], scene["box_hi"], t)
    if "sph_c" in scene:
        t = _hit_spheres(o, d, scene["sph_c"], scene["sph_r"], t)
    z = t.reshape(h, w)  # the eye-space ray has z = -1: t is the planar depth
    hit = np.isfinite(z)
    z = np.where(hit, z, 0.0)
    sigma = 0.0012 + 0.0019 * (z - 0.4) ** 2
    z = z + sigma * rng.standard_normal(z.shape)
    mm = np.rint(z * 1000.0)
    valid = hit & (z >= znear) & (z <= zfar)
    if dropout > 0:
        valid &= rng.random(z.shape) >= dropout
    out = np.where(valid, np.clip(mm, 0, 65535), 0).astype(np.uint16)
    return out


def sphere_scene(n_frames=10, seed=0, width=320, height=240):
    """The small sphere-on-a-plane scene: 320x240, f=292.5."""
    rng = np.random.default_rng(seed)
    fx = fy = 292.5 * width / 320.0
    cx, cy = width / 2.0, height / 2.0
    scene = {"plane_y": -0.5, "sph_c": [np.array([0.0, 0.0, 2.0])], "sph_r": [0.5]}
    rays = _rays(width, height, fx, fy, cx, cy)
    frames, poses = [], []
    center = np.array([0.0, 0.0, 2.0])
    radius = 2.0
    for i in range(n_frames):
        a = i * 0.05 / radius  # 5 cm of arc per frame
        pos = center + radius * np.array([math.sin(a), 0.0, -math.cos(a)])
        yaw = math.pi + math.radians(1.0) * i  # looking toward +z, 1 deg/frame
        pose = _pose(_rot_y(yaw), pos)
        poses.append(pose)
        frames.append(_render(rays, pose, scene, rng, 0.4, 4.0, 0.0))
    return Sequence(width, height, fx, fy, cx, cy, 0.4, 4.0, frames, poses)


def room_layout(seed=0, scale=1.0):
    rng = np.random.default_rng(seed + 1000)
    half = np.array([2.0 * scale, 1.5, 2.0 * scale])
    lo, hi, sc, sr = [], [], [], []
    clear = 1.3 * scale  # keep the camera's central region free
    while len(lo) < 40:
        size = rng.uniform(0.1, 0.8, 3)
        c = np.array([rng.uniform(-half[0] + size[0] / 2, half[0] - size[0] / 2),
                      -half[1] + size[1] / 2 + (rng.uniform(0, 1.2) if rng.random() < 0.3 else 0),
                      rng.uniform(-half[2] + size[2] / 2, half[2] - size[2] / 2)])
        if math.hypot(c[0], c[2]) < clear:
            continue
        lo.append(c - size / 2)
        hi.append(c + size / 2)
    while len(sc) < 20:
        r = rng.uniform(0.1, 0.6)
        c = np.array([rng.uniform(-half[0] + r, half[0] - r), rng.uniform(-half[1] + r, half[1] - r),
                      rng.uniform(-half[2] + r, half[2] - r)])
        if math.hypot(c[0], c[2]) < clear + r:
            continue
        sc.append(c)
        sr.append(r)
    return {"half": half, "box_lo": lo, "box_hi": hi, "sph_c": sc, "sph_r": sr}


def room_trajectory(n_frames, seed=0, scale=1.0):
    """Smooth camera path: <= 2 cm and <= 1.5 deg per frame."""
    rng = np.random.default_rng(seed + 2000)
    ph = rng.uniform(0, 2 * math.pi, 4)
    poses = []
    for i in range(n_frames):
        s = i * 0.012 / (0.6 * scale)  # ~1.2 cm per frame along a 0.6 m circle
        pos = np.array([0.6 * scale * math.cos(s + ph[0]), 0.15 * math.sin(0.7 * s + ph[1]),
                        0.6 * scale * math.sin(s + ph[0])])
        yaw = ph[2] + math.radians(1.0) * i
        pitch = math.radians(8.0) * math.sin(0.01 * i + ph[3])
        poses.append(_pose(_rot_y(yaw) @ _rot_x(pitch), pos))
    return poses


def room_scene(n_frames=300, seed=0, width=640, height=480, f=585.0, scale=1.0, dropout=0.02,
               first_frame=0):
    """The 640x480 room workload (and, with scale=2 and 512x424, the large-volume
    room of the 4096^3 study): the seeded room
    rendered on the CPU by the same renderer the benchmark runs on the GPU
    (render_room_torch; both devices give identical frames)."""
    frames, poses = render_room_torch(n_frames, seed, width, height, f, scale, dropout, first_frame,
                                      device="cpu")
    frames = [fr for fr in frames.numpy().view(np.uint16)]
    return Sequence(width, height, f, f, width / 2.0, height / 2.0, 0.4, 4.0, frames, poses)


# ------------------------------------------------------------ torch renderer
# The room scenes are ray-cast with torch, on the GPU (benchmarks, long
# sequences) or on the CPU, and the two give the same frames bit for bit:
# every floating-point step is one IEEE-rounded elementwise operation (add,
# subtract, multiply, divide, square root, min/max, compare, round) applied
# the same way on either device -- no matrix products or floating-point
# sums, whose order and fusion differ between backends.  The Gaussian depth
# noise and the dropout draw come from a counter-based integer hash of
# (seed, frame, pixel), and the Box-Muller transform runs on the host in
# float64, so no device's log or cos enters the frame.

def _hash32(x):
    """lowbias32 integer hash of uint64 arrays holding 32-bit values."""
    x = x & 0xFFFFFFFF
    x = x ^ (x >> 16)
    x = (x * 0x7FEB352D) & 0xFFFFFFFF
    x = x ^ (x >> 15)
    x = (x * 0x846CA68B) & 0xFFFFFFFF
    x = x ^ (x >> 16)
    return x


def _uniform(seed, frame, n, stream):
    """n uniforms in (0, 1] (float64) of one (seed, frame, stream)."""
    salt = _hash32(np.uint64((seed * 7919 + frame * 104729 + stream * 31337) & 0xFFFFFFFF))
    key = _hash32(np.arange(n, dtype=np.uint64) + salt)
    return (key.astype(np.float64) + 0.5) * (1.0 / 4294967296.0)


def room_noise(seed, frame, n):
    """Per pixel a standard normal draw and a dropout uniform (float32)."""
    u1, u2, u3 = (_uniform(seed, frame, n, k) for k in (1, 2, 3))
    gauss = np.sqrt(-2.0 * np.log(u1)) * np.cos(6.283185307179586 * u2)
    return gauss.astype(np.float32), u3.astype(np.float32)


def _device_noise(torch, seed, frame, n, dev):
    """room_noise's draws computed on `dev` with its own log and cos: fast,
    but not bit-identical between devices (training data only)."""
    def mul32(a, m):
        lo, hi = a & 0xFFFF, a >> 16
        return (lo * m + (((hi * m) & 0xFFFF) << 16)) & 0xFFFFFFFF

    def h32(x):
        x = x & 0xFFFFFFFF
        x = x ^ (x >> 16)
        x = mul32(x, 0x7FEB352D)
        x = x ^ (x >> 15)
        x = mul32(x, 0x846CA68B)
        return x ^ (x >> 16)

    pix = torch.arange(n, device=dev, dtype=torch.int64)
    u = []
    for k in (1, 2, 3):
        salt = int(_hash32(np.uint64((seed * 7919 + frame * 104729 + k * 31337) & 0xFFFFFFFF)))
        u.append((h32(pix + salt).to(torch.float64) + 0.5) * (1.0 / 4294967296.0))
    g = torch.sqrt(-2.0 * torch.log(u[0])) * torch.cos(6.283185307179586 * u[1])
    return g.to(torch.float32), u[2].to(torch.float32)


def render_room_torch(n_frames, seed=0, width=640, height=480, f=585.0, scale=1.0, dropout=0.02,
                      first_frame=0, device="cuda", chunk=1 << 16, noise="host"):
    """Frames first_frame .. first_frame+n_frames-1 of the seeded room as a
    uint16 bit pattern in an int16 tensor (n, h, w) on `device`, and their
    eye-to-world poses (float64 4x4).  noise="host" (the default) draws the
    depth noise on the host so every device renders identical frames;
    noise="device" draws it on `device` (faster, for large training sets)."""
    import torch
    layout = room_layout(seed, scale)
    poses = room_trajectory(first_frame + n_frames, seed, scale)[first_frame:]
    fx = fy = f
    cx, cy = width / 2.0, height / 2.0
    dev = torch.device(device)
    f32 = torch.float32

    def t32(a):
        return torch.tensor(np.asarray(a, np.float32), device=dev, dtype=f32)

    # eye-space rays (u + 0.5 - cx) / fx, (cy - 0.5 - v) / fy, -1 from float64 on the host
    u = np.arange(width, dtype=np.float64)
    v = np.arange(height, dtype=np.float64)
    uu, vv = np.meshgrid(u, v)
    rx = t32(((uu + 0.5 - cx) / fx).reshape(-1))
    ry = t32(((cy - 0.5 - vv) / fy).reshape(-1))
    half = t32(layout["half"])
    blo = t32(np.array(layout["box_lo"]))  # (B, 3)
    bhi = t32(np.array(layout["box_hi"]))
    sc = t32(np.array(layout["sph_c"]))    # (S, 3)
    sr = t32(np.array(layout["sph_r"]))
    sr2 = sr * sr
    inf = torch.tensor(float("inf"), device=dev, dtype=f32)
    tiny = torch.tensor(1e-30, device=dev, dtype=f32)
    eps = torch.tensor(1e-6, device=dev, dtype=f32)
    c_s0, c_s1, c_z0 = t32(0.0012), t32(0.0019), t32(0.4)
    c_mm, zn, zf, c_drop = t32(1000.0), t32(0.4), t32(4.0), t32(dropout)
    P = width * height
    out = torch.zeros((n_frames, height, width), dtype=torch.int16, device=dev)
    # host noise for the next frames is drawn on worker threads while the device ray-casts
    from concurrent.futures import ThreadPoolExecutor
    pool = ThreadPoolExecutor(max_workers=4)
    ahead = 8 if noise == "host" else 0
    pending = [pool.submit(room_noise, seed, first_frame + i, P) for i in range(min(ahead, n_frames))]
    for i, pose in enumerate(poses):
        R = np.asarray(pose[:3, :3], np.float32)
        o = t32(pose[:3, 3])
        z = torch.empty(P, device=dev, dtype=f32)
        for s0 in range(0, P, chunk):
            x, y = rx[s0:s0 + chunk], ry[s0:s0 + chunk]
            # world ray d = R (x, y, -1), one rounded multiply and add at a time
            d = torch.stack([x * float(R[k, 0]) + y * float(R[k, 1]) - float(R[k, 2]) for k in range(3)], 1)
            # room walls from inside
            tpos = torch.where(d > 0, (half - o) / d, inf)
            tneg = torch.where(d < 0, (-half - o) / d, inf)
            t = torch.minimum(tpos, tneg).amin(1)
            # boxes (slabs)
            inv = 1.0 / torch.where(d == 0, tiny, d)
            t1 = (blo[None] - o) * inv[:, None]
            t2 = (bhi[None] - o) * inv[:, None]
            tn = torch.minimum(t1, t2).amax(2)
            tf = torch.maximum(t1, t2).amin(2)
            th = torch.where(tn > eps, tn, tf)
            hit = (tn <= tf) & (tf > eps)
            t = torch.minimum(t, torch.where(hit, th, inf).amin(1))
            # spheres: b = d.(o - c), cc = |o - c|^2 - r^2, a = |d|^2
            oc = o[None] - sc
            b = d[:, 0:1] * oc[None, :, 0] + d[:, 1:2] * oc[None, :, 1] + d[:, 2:3] * oc[None, :, 2]
            cc = (oc[:, 0] * oc[:, 0] + oc[:, 1] * oc[:, 1] + oc[:, 2] * oc[:, 2]) - sr2
            a = (d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1] + d[:, 2] * d[:, 2])[:, None]
            disc = b * b - a * cc[None]
            sq = torch.sqrt(torch.clamp(disc, min=0))
            t0 = (-b - sq) / a
            t1s = (-b + sq) / a
            ts = torch.where(t0 > eps, t0, t1s)
            ok = (disc >= 0) & (ts > eps)
            t = torch.minimum(t, torch.where(ok, ts, inf).amin(1))
            z[s0:s0 + chunk] = t  # the eye-space ray has z = -1: t is the planar depth
        if noise == "host":
            gauss, u3 = pending[i].result()
            pending[i] = None
            if i + ahead < n_frames:
                pending.append(pool.submit(room_noise, seed, first_frame + i + ahead, P))
            gauss = torch.from_numpy(gauss).to(dev)
            u3 = torch.from_numpy(u3).to(dev)
        else:
            gauss, u3 = _device_noise(torch, seed, first_frame + i, P, dev)
        hitm = torch.isfinite(z)
        zz = torch.where(hitm, z, torch.zeros_like(z))
        dz = zz - c_z0
        sigma = c_s0 + c_s1 * (dz * dz)
        zz = zz + sigma * gauss
        mm = torch.round(zz * c_mm)
        valid = hitm & (zz >= zn) & (zz <= zf) & (u3 >= c_drop)
        mm = torch.where(valid, torch.clamp(mm, 0, 65535), torch.zeros_like(mm))
        out[i] = mm.to(torch.int32).to(torch.int16).reshape(height, width)  # bit pattern of uint16
    pool.shutdown()
    return out, poses


def kifi_matrix(m):
    """4x4 matrix -> (16,) float32 in kifi float4x4 memory order."""
    return np.ascontiguousarray(np.asarray(m, np.float32).T).reshape(16)
