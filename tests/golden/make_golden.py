"""Regenerates the golden fixtures of tests/golden/ from the reference.

Run in a checkout that has the reference sources (the development container):

    python tests/golden/make_golden.py

It needs oracle/_ref/libkifi_ref.so (built by oracle/build_ref.py from the
reference's own Integrator / Mesher / ICP code) and the reference's fixture
KinectFission/content/imrod_v2.depth.  It writes

* imrod_v2_frame0.npz -- the fixture's single 640x480 frame (float metres)
  and its pose, read through the reference's DepthStream, so tests can use
  it where the reference checkout is absent;
* golden.json -- what the reference computes on it: voxel counts, SHA-256
  digests of the key and (distance-sum, weight) arrays, mesh counts and
  digests (both Mesh overloads), and ICP poses.

The cases mirror KinectFission/UnitTests/Integrator.cpp:19-53 and
UnitTests/Mesher.cpp:21-50 (Volume(256, 2.0, 0.02), KinectParams(640x480,
Far), one frame), extended with re-integrations under fixed pose offsets.
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import build_ref, ref  # noqa: E402

CAM = (640, 480, 571.26, 571.26, 320.0, 240.0, 0.8, 4.0)  # KinectParams(640x480, Far)
# translation offsets (m) applied to the fixture's world-to-eye pose for the
# extra frames of the multi-frame cases
OFFSETS = [(0.0, 0.0, 0.0), (0.003, -0.002, 0.001), (-0.002, 0.004, -0.003)]
VOLUMES = [(256, 2.0, 0.02), (512, 4.0, 0.02), (1024, 4.096, 0.02)]


def digest(a):
    """SHA-256 of the array bytes; float32 NaNs are canonicalised to
    0x7FC00000 first because NaN payloads differ between platforms."""
    a = np.ascontiguousarray(a)
    if a.dtype == np.float32:
        b = a.view(np.uint32).copy()
        b[np.isnan(a)] = 0x7FC00000
        a = b
    return hashlib.sha256(a.tobytes()).hexdigest()


def posed(view, off):
    v = view.copy()
    v[12:15] += np.asarray(off, np.float32)
    return v


def backproject(depth, view, cam):
    """World points of each pixel (0 = none) -- an ICP target buffer."""
    from oracle import cpu
    e2w = cpu.invert_transform(view).reshape(4, 4).T.astype(np.float64)
    h, w = depth.shape
    ys, xs = np.mgrid[0:h, 0:w]
    d = depth.astype(np.float64)
    p = np.stack([((xs + 0.5 - cam[4]) / cam[2]) * d, ((cam[5] - 0.5 - ys) / cam[3]) * d, -d,
                  np.ones_like(d)], -1)
    wp = (p.reshape(-1, 4) @ e2w.T)[:, :3].reshape(h, w, 3).astype(np.float32)
    wp[depth == 0] = 0
    return wp


def main():
    build_ref.build()
    path = os.path.join(build_ref.REF_ROOT, "KinectFission", "content", "imrod_v2.depth")
    frames = ref.read_depthstream(path)
    depth, view = frames[0]
    np.savez_compressed(os.path.join(HERE, "imrod_v2_frame0.npz"), depth=depth, view=view)
    out = {"camera": CAM, "offsets": OFFSETS, "cases": []}
    for res, side, trunc in VOLUMES:
        vol = ref.Volume(res, side, trunc)
        for nf in range(1, len(OFFSETS) + 1):
            vol.integrate(depth, CAM, posed(view, OFFSETS[nf - 1]))
            keys, vals = vol.export()
            case = {"volume": [res, side, trunc], "frames": nf, "voxels": int(keys.size),
                    "keys_sha256": digest(keys), "values_sha256": digest(vals)}
            if nf in (1, len(OFFSETS)):
                v0, _ = vol.mesh(False)
                v1, i1 = vol.mesh(True)
                case.update({"mesh_verts_only": int(v0.shape[0]),
                             "mesh_verts_only_sha256": digest(v0),
                             "mesh_verts": int(v1.shape[0]), "mesh_indices": int(i1.size),
                             "mesh_verts_sha256": digest(v1), "mesh_indices_sha256": digest(i1)})
            out["cases"].append(case)
    # ICP: the frame against its own back-projection from a displaced guess
    from oracle import cpu
    e2w = cpu.invert_transform(view)
    synth = backproject(depth, view, CAM)
    icp = []
    for off, iters in (((0.01, -0.005, 0.0), 4), ((-0.006, 0.004, 0.008), 8)):
        guess = e2w.copy()
        guess[12:15] += np.asarray(off, np.float32)
        pose = ref.icp_align(depth, CAM, guess, synth, e2w, iters)
        icp.append({"guess_offset": off, "iterations": iters, "pose": [float(x) for x in pose]})
    out["icp"] = icp
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", len(out["cases"]), "integration cases")


if __name__ == "__main__":
    main()
