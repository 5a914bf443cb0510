"""The synthetic room the benchmark and the parity tests fuse.

The benchmark's GPU arm renders its frames with torch on the GPU, its
reference arm on the CPU; both must see the same frames.  The renderer is
built from IEEE-rounded elementwise operations only, so a float32 numpy
restatement of the same operations must give the same frames bit for bit,
and (on a GPU) so must the CUDA device."""
import numpy as np
import pytest


def numpy_room(seed, frame, width, height, f, scale=1.0, dropout=0.02):
    """One frame of the room, restated with numpy float32 operations."""
    from merge_fusion_gb300 import scenes
    layout = scenes.room_layout(seed, scale)
    pose = scenes.room_trajectory(frame + 1, seed, scale)[frame]
    cx, cy = width / 2.0, height / 2.0
    uu, vv = np.meshgrid(np.arange(width, dtype=np.float64), np.arange(height, dtype=np.float64))
    x = ((uu + 0.5 - cx) / f).astype(np.float32).reshape(-1)
    y = ((cy - 0.5 - vv) / f).astype(np.float32).reshape(-1)
    R = np.asarray(pose[:3, :3], np.float32)
    o = np.asarray(pose[:3, 3], np.float32)
    d = np.stack([x * float(R[k, 0]) + y * float(R[k, 1]) - float(R[k, 2]) for k in range(3)], 1)
    half = np.asarray(layout["half"], np.float32)
    inf = np.float32(np.inf)
    eps = np.float32(1e-6)
    with np.errstate(divide="ignore", invalid="ignore"):
        t = np.minimum(np.where(d > 0, (half - o) / d, inf), np.where(d < 0, (-half - o) / d, inf)).min(1)
        inv = np.float32(1.0) / np.where(d == 0, np.float32(1e-30), d)
    blo = np.asarray(layout["box_lo"], np.float32)
    bhi = np.asarray(layout["box_hi"], np.float32)
    t1 = (blo[None] - o) * inv[:, None]
    t2 = (bhi[None] - o) * inv[:, None]
    tn = np.minimum(t1, t2).max(2)
    tf = np.maximum(t1, t2).min(2)
    th = np.where(tn > eps, tn, tf)
    t = np.minimum(t, np.where((tn <= tf) & (tf > eps), th, inf).min(1))
    sc = np.asarray(layout["sph_c"], np.float32)
    sr = np.asarray(layout["sph_r"], np.float32)
    oc = o[None] - sc
    b = d[:, 0:1] * oc[None, :, 0] + d[:, 1:2] * oc[None, :, 1] + d[:, 2:3] * oc[None, :, 2]
    cc = (oc[:, 0] * oc[:, 0] + oc[:, 1] * oc[:, 1] + oc[:, 2] * oc[:, 2]) - sr * sr
    a = (d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1] + d[:, 2] * d[:, 2])[:, None]
    disc = b * b - a * cc[None]
    sq = np.sqrt(np.maximum(disc, np.float32(0)))
    t0 = (-b - sq) / a
    t1s = (-b + sq) / a
    ts = np.where(t0 > eps, t0, t1s)
    t = np.minimum(t, np.where((disc >= 0) & (ts > eps), ts, inf).min(1))
    gauss, u3 = scenes.room_noise(seed, frame, width * height)
    hit = np.isfinite(t)
    zz = np.where(hit, t, np.float32(0))
    dz = zz - np.float32(0.4)
    zz = zz + (np.float32(0.0012) + np.float32(0.0019) * (dz * dz)) * gauss
    mm = np.round(zz * np.float32(1000.0))
    valid = hit & (zz >= np.float32(0.4)) & (zz <= np.float32(4.0)) & (u3 >= np.float32(dropout))
    mm = np.where(valid, np.clip(mm, 0, 65535), np.float32(0))
    return mm.astype(np.int32).astype(np.uint16).reshape(height, width)


@pytest.mark.parametrize("frame,width,height,f,scale", [(0, 160, 120, 146.25, 1.0), (37, 128, 106, 91.25, 2.0)])
def test_torch_renderer_equals_numpy_restatement(frame, width, height, f, scale):
    from merge_fusion_gb300 import scenes
    frames, _ = scenes.render_room_torch(1, seed=3, width=width, height=height, f=f, scale=scale,
                                         first_frame=frame, device="cpu")
    got = frames.numpy().view(np.uint16)[0]
    want = numpy_room(3, frame, width, height, f, scale)
    assert (got > 0).mean() > 0.3
    assert np.array_equal(got, want), int((got != want).sum())


def test_noise_statistics():
    from merge_fusion_gb300 import scenes
    g, u = scenes.room_noise(0, 5, 1 << 18)
    assert abs(float(g.mean())) < 0.01 and abs(float(g.std()) - 1.0) < 0.01
    assert 0.0 < u.min() and u.max() <= 1.0 and abs(float((u < 0.02).mean()) - 0.02) < 0.002
    g2, _ = scenes.room_noise(0, 6, 1 << 18)
    assert not np.array_equal(g, g2)


def test_room_scene_is_the_benchmark_renderer():
    from merge_fusion_gb300 import scenes
    seq = scenes.room_scene(n_frames=2, seed=9, width=160, height=120, f=146.25)
    frames, poses = scenes.render_room_torch(2, seed=9, width=160, height=120, f=146.25, device="cpu")
    assert np.array_equal(np.stack(seq.frames), frames.numpy().view(np.uint16))
    assert np.array_equal(seq.eye_to_world[1], poses[1])


@pytest.mark.gpu
def test_gpu_and_cpu_render_identical_frames(gpu):
    """The benchmark's configuration (seed 0, 640x480, f = 585) at frames of
    its prefill, timed and reference ranges, and the large-volume room."""
    from merge_fusion_gb300 import scenes
    for first, n, kw in ((0, 2, {}), (150, 2, {}), (400, 1, {}),
                         (10, 1, dict(width=512, height=424, f=365.0, scale=2.0))):
        a, _ = scenes.render_room_torch(n, seed=0, first_frame=first, device="cuda", **kw)
        b, _ = scenes.render_room_torch(n, seed=0, first_frame=first, device="cpu", **kw)
        a = a.cpu().numpy().view(np.uint16)
        b = b.numpy().view(np.uint16)
        assert np.array_equal(a, b), (first, int((a != b).sum()))
