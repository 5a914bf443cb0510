"""ctypes wrapper of the C restatement (oracle/kifi_oracle.c).

Test infrastructure only.  Matrices are numpy float32 arrays of shape (16,)
in kifi float4x4 memory order (column-major); ``cam`` is a tuple
(width, height, fx, fy, cx, cy, znear, zfar).
"""
import ctypes as C
import os

import numpy as np

from . import ORACLE_LIB, build_oracle

_lib = None


class _Cam(C.Structure):
    _fields_ = [("width", C.c_int), ("height", C.c_int), ("fx", C.c_float), ("fy", C.c_float),
                ("cx", C.c_float), ("cy", C.c_float), ("znear", C.c_float), ("zfar", C.c_float)]


class _Geom(C.Structure):
    _fields_ = [("res", C.c_int), ("side", C.c_float), ("trunc", C.c_float), ("vlen", C.c_float),
                ("center_off", C.c_float), ("vlen_inv", C.c_float), ("index_off", C.c_float)]


class _IcpStats(C.Structure):
    _fields_ = [("n_assoc", C.c_int), ("sums", C.c_double * 15)]


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_LIB):
            build_oracle()
        _lib = C.CDLL(ORACLE_LIB)
        _lib.or_splat.restype = C.c_size_t
        _lib.or_expand.restype = C.c_size_t
        _lib.or_unique_u32.restype = C.c_size_t
        _lib.or_integrate.restype = C.c_size_t
        _lib.or_set_union_i32.restype = C.c_size_t
        _lib.or_insert.restype = C.c_size_t
        _lib.or_kahan_sum.restype = C.c_float
        for f in ("or64_splat", "or64_unique", "or64_expand", "or64_insert", "or64_integrate"):
            getattr(_lib, f).restype = C.c_size_t
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def cam_struct(cam):
    return _Cam(*cam)


def geom(res, side, trunc):
    g = _Geom()
    lib().or_geom_init(C.byref(g), C.c_int(res), C.c_float(side), C.c_float(trunc))
    return g


def f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def eye_to_clip(cam):
    out = np.zeros(16, np.float32)
    lib().or_eye_to_clip(C.byref(cam_struct(cam)), _p(out))
    return out


def mat_mul(a, b):
    a, b = f32(a), f32(b)
    out = np.zeros(16, np.float32)
    lib().or_mat_mul(_p(a), _p(b), _p(out))
    return out


def invert_transform(m):
    m = f32(m)
    out = np.zeros(16, np.float32)
    lib().or_invert_transform(_p(m), _p(out))
    return out


def splat(res, side, trunc, depth, cam, world_to_eye):
    depth, w2e = f32(depth), f32(world_to_eye)
    out = np.zeros(cam[0] * cam[1] + 1, np.uint32)
    g = geom(res, side, trunc)
    n = lib().or_splat(C.byref(g), _p(depth), C.byref(cam_struct(cam)), _p(w2e), _p(out))
    return out[:n].copy()


def radix_sort(keys):
    k = np.ascontiguousarray(keys, dtype=np.uint32).copy()
    lib().or_radix_sort_u32(_p(k), C.c_size_t(k.size))
    return k


def radix_sort_pairs(keys, vals):
    k = np.ascontiguousarray(keys, dtype=np.uint32).copy()
    v = np.ascontiguousarray(vals, dtype=np.uint32).copy()
    lib().or_radix_sort_pairs_u32(_p(k), _p(v), C.c_size_t(k.size))
    return k, v


def unique(sorted_keys):
    k = np.ascontiguousarray(sorted_keys, dtype=np.uint32).copy()
    n = lib().or_unique_u32(_p(k), C.c_size_t(k.size))
    return k[:n].copy()


def expand(sorted_unique_keys):
    k = np.ascontiguousarray(sorted_unique_keys, dtype=np.uint32)
    out = np.zeros(8 * k.size + 1, np.uint32)
    n = lib().or_expand(_p(k), C.c_size_t(k.size), _p(out))
    return out[:n].copy()


def set_union(k1, v1, k2, v2):
    k1, v1, k2, v2 = (np.ascontiguousarray(x, dtype=np.int32) for x in (k1, v1, k2, v2))
    ko = np.full(k1.size + k2.size + 1, -1, np.int32)
    vo = np.full(k1.size + k2.size + 1, -1, np.int32)
    n = lib().or_set_union_i32(_p(k1), _p(v1), C.c_size_t(k1.size), _p(k2), _p(v2),
                               C.c_size_t(k2.size), _p(ko), _p(vo))
    return ko[:n].copy(), vo[:n].copy()


def kahan_sum(x):
    x = f32(x)
    return float(lib().or_kahan_sum(_p(x), C.c_size_t(x.size)))


class Volume:
    """Resident sparse TSDF volume held as sorted keys + (dsum, weight)."""

    def __init__(self, res, side, trunc):
        self.res, self.side, self.trunc = res, side, trunc
        self.g = geom(res, side, trunc)
        self.keys = np.zeros(0, np.uint32)
        self.values = np.zeros((0, 2), np.float32)

    def integrate(self, depth, cam, world_to_eye):
        depth, w2e = f32(depth), f32(world_to_eye)
        n0 = self.keys.size
        cap = n0 + 8 * cam[0] * cam[1] + 1
        ok = np.zeros(cap, np.uint32)
        ov = np.zeros((cap, 2), np.float32)
        rk = np.ascontiguousarray(self.keys)
        rv = np.ascontiguousarray(self.values)
        n1 = lib().or_integrate(C.byref(self.g), _p(depth), C.byref(cam_struct(cam)), _p(w2e),
                                _p(rk), _p(rv), C.c_size_t(n0), _p(ok), _p(ov))
        self.keys = ok[:n1].copy()
        self.values = ov[:n1].copy()

    def mesh(self, with_indices=True):
        n = self.keys.size
        vcap, icap = 3 * n + 1, 15 * n + 1
        verts = np.zeros((vcap, 3), np.float32)
        idx = np.zeros(icap, np.uint32)
        nv, ni = C.c_size_t(), C.c_size_t()
        rc = lib().or_mesh(C.byref(self.g), _p(self.keys), _p(self.values), C.c_size_t(n),
                           C.c_int(1 if with_indices else 0), _p(verts), C.c_size_t(vcap), _p(idx),
                           C.c_size_t(icap), C.byref(nv), C.byref(ni))
        assert rc == 0
        return verts[:nv.value].copy(), idx[:ni.value].copy()


def key_bits_per_axis(res):
    """b of the 64-bit keys z<<2b | y<<b | x: max(10, log2 res)."""
    b = 10
    while (1 << b) < res:
        b += 1
    return b


def splat64(res, side, trunc, depth, cam, world_to_eye):
    depth, w2e = f32(depth), f32(world_to_eye)
    out = np.zeros(cam[0] * cam[1] + 1, np.uint64)
    g = geom(res, side, trunc)
    n = lib().or64_splat(C.byref(g), C.c_int(key_bits_per_axis(res)), _p(depth), C.byref(cam_struct(cam)),
                         _p(w2e), _p(out))
    return out[:n].copy()


def radix_sort64(keys):
    k = np.ascontiguousarray(keys, dtype=np.uint64).copy()
    lib().or64_radix_sort(_p(k), C.c_size_t(k.size))
    return k


def expand64(sorted_unique_keys, b):
    k = np.ascontiguousarray(sorted_unique_keys, dtype=np.uint64)
    out = np.zeros(8 * k.size + 1, np.uint64)
    n = lib().or64_expand(_p(k), C.c_size_t(k.size), C.c_int(b), _p(out))
    return out[:n].copy()


class Volume64(Volume):
    """The same volume keyed by 64-bit keys z<<2b | y<<b | x."""

    def __init__(self, res, side, trunc):
        super().__init__(res, side, trunc)
        self.b = key_bits_per_axis(res)
        self.keys = np.zeros(0, np.uint64)

    def integrate(self, depth, cam, world_to_eye):
        depth, w2e = f32(depth), f32(world_to_eye)
        n0 = self.keys.size
        cap = n0 + 8 * cam[0] * cam[1] + 1
        ok = np.zeros(cap, np.uint64)
        ov = np.zeros((cap, 2), np.float32)
        rk = np.ascontiguousarray(self.keys)
        rv = np.ascontiguousarray(self.values)
        n1 = lib().or64_integrate(C.byref(self.g), C.c_int(self.b), _p(depth), C.byref(cam_struct(cam)), _p(w2e),
                                  _p(rk), _p(rv), C.c_size_t(n0), _p(ok), _p(ov))
        self.keys = ok[:n1].copy()
        self.values = ov[:n1].copy()

    def mesh(self, with_indices=True):
        n = self.keys.size
        vcap, icap = 3 * n + 1, 15 * n + 1
        verts = np.zeros((vcap, 3), np.float32)
        idx = np.zeros(icap, np.uint32)
        nv, ni = C.c_size_t(), C.c_size_t()
        rc = lib().or64_mesh(C.byref(self.g), C.c_int(self.b), _p(self.keys), _p(self.values), C.c_size_t(n),
                             C.c_int(1 if with_indices else 0), _p(verts), C.c_size_t(vcap), _p(idx),
                             C.c_size_t(icap), C.byref(nv), C.byref(ni))
        assert rc == 0
        return verts[:nv.value].copy(), idx[:ni.value].copy()


def icp_align(depth, cam, e2w_guess, synth, synth_e2w, iters, fp64=False):
    """Returns (float pose (16,), double pose (16,), n_assoc of last step).
    fp64: sums, cross-covariance and Horn's matrix in double instead of the
    reference's float Kahan sums (the FP64 reference solution)."""
    depth, guess, se2w = f32(depth), f32(e2w_guess), f32(synth_e2w)
    synth = f32(synth)
    sh, sw = synth.shape[0], synth.shape[1]
    out = np.zeros(16, np.float32)
    outd = np.zeros(16, np.float64)
    st = _IcpStats()
    lib().or_icp_set_fp64(C.c_int(1 if fp64 else 0))
    lib().or_icp_align(_p(depth), C.byref(cam_struct(cam)), _p(guess), _p(synth), C.c_int(sw),
                       C.c_int(sh), _p(se2w), C.c_int(iters), _p(out), _p(outd), C.byref(st))
    lib().or_icp_set_fp64(C.c_int(0))
    return out, outd, st.n_assoc


def icp_associate(depth, cam, e2w, synth, synth_e2w):
    """One AlignStep's association under pose e2w: per source (rows, every
    4th column) the winner's linear target index (-1: none) and len^2."""
    depth, pose, se2w, synth = f32(depth), f32(e2w), f32(synth_e2w), f32(synth)
    sh, sw = synth.shape[0], synth.shape[1]
    n = ((cam[0] + 3) // 4) * cam[1]
    at = np.zeros(n, np.int64)
    l2 = np.zeros(n, np.float32)
    lib().or_icp_associate(_p(depth), C.byref(cam_struct(cam)), _p(pose), _p(synth), C.c_int(sw), C.c_int(sh),
                           _p(se2w), _p(at), _p(l2))
    return at, l2


def bin_points(points, world_to_clip, w, h):
    pts = f32(points)
    w2c = f32(world_to_clip)
    out = np.zeros((h, w, 3), np.float32)
    lib().or_bin(_p(pts), C.c_size_t(pts.size // 3), _p(w2c), _p(out), C.c_int(w), C.c_int(h))
    return out


def backproject(depth, cam, eye_to_world):
    """(h, w, 3) float32 world points of a frame; (0,0,0) where depth <= 0."""
    d = f32(depth)
    m = f32(eye_to_world)
    out = np.zeros((cam[1], cam[0], 3), np.float32)
    lib().or_backproject(_p(d), C.byref(cam_struct(cam)), _p(m), _p(out))
    return out
