"""ctypes wrapper of the reference's own CPU code (oracle/_ref/libkifi_ref.so,
built by oracle/build_ref.py).  Test and baseline infrastructure only.

Same conventions as oracle.cpu: matrices are float32 (16,) in kifi float4x4
(column-major) memory order; ``cam`` = (width, height, fx, fy, cx, cy,
znear, zfar).
"""
import ctypes as C
import os

import numpy as np

from . import build_ref

_lib = None


def available():
    return os.path.exists(build_ref.LIB)


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(build_ref.LIB)
        _lib.kref_volume_create.restype = C.c_void_p
        _lib.kref_volume_create.argtypes = [C.c_int, C.c_float, C.c_float]
        for f in ("kref_volume_destroy", "kref_volume_size"):
            getattr(_lib, f).argtypes = [C.c_void_p]
        _lib.kref_volume_size.restype = C.c_size_t
        _lib.kref_volume_export.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        _lib.kref_volume_insert.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t]
        _lib.kref_integrate.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int] + \
            [C.c_float] * 6 + [C.c_void_p]
        _lib.kref_splat.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int] + \
            [C.c_float] * 6 + [C.c_void_p, C.c_void_p]
        _lib.kref_splat.restype = C.c_size_t
        _lib.kref_sort_unique_expand.argtypes = [C.c_void_p, C.c_size_t, C.c_void_p]
        _lib.kref_sort_unique_expand.restype = C.c_size_t
        _lib.kref_radix_sort.argtypes = [C.c_void_p, C.c_size_t]
        _lib.kref_radix_sort_pairs.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t]
        _lib.kref_set_union.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p,
                                        C.c_void_p, C.c_size_t, C.c_void_p, C.c_void_p]
        _lib.kref_set_union.restype = C.c_size_t
        _lib.kref_kahan_sum.argtypes = [C.c_void_p, C.c_size_t]
        _lib.kref_kahan_sum.restype = C.c_float
        _lib.kref_partial_sum_exclusive.argtypes = [C.c_void_p, C.c_size_t]
        _lib.kref_mesh.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
        _lib.kref_mesh_fetch.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        _lib.kref_icp_align.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                                        C.c_int, C.c_int, C.c_void_p] + [C.c_float] * 6 + \
            [C.c_int, C.c_void_p]
        _lib.kref_bin.argtypes = [C.c_void_p, C.c_size_t, C.c_void_p, C.c_void_p, C.c_int,
                                  C.c_int]
        _lib.kref_eye_to_clip.argtypes = [C.c_int, C.c_int] + [C.c_float] * 6 + [C.c_void_p]
        _lib.kref_invert_transform.argtypes = [C.c_void_p, C.c_void_p]
        _lib.kref_depthstream_open.restype = C.c_void_p
        _lib.kref_depthstream_open.argtypes = [C.c_char_p]
        _lib.kref_depthstream_close.argtypes = [C.c_void_p]
        _lib.kref_depthstream_frame_count.argtypes = [C.c_void_p]
        _lib.kref_depthstream_next.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p,
                                               C.c_void_p, C.c_void_p]
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


class Volume:
    def __init__(self, res, side, trunc):
        self.h = lib().kref_volume_create(res, side, trunc)

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.kref_volume_destroy(self.h)
            self.h = None

    def size(self):
        return lib().kref_volume_size(self.h)

    def export(self):
        n = self.size()
        k = np.zeros(n, np.uint32)
        v = np.zeros((n, 2), np.float32)
        if n:
            lib().kref_volume_export(self.h, _p(k), _p(v))
        return k, v

    def insert(self, keys, values):
        k = np.ascontiguousarray(keys, np.uint32)
        v = np.ascontiguousarray(values, np.float32)
        lib().kref_volume_insert(self.h, _p(k), _p(v), k.size)

    def integrate(self, depth, cam, world_to_eye):
        d, m = f32(depth), f32(world_to_eye)
        lib().kref_integrate(self.h, _p(d), cam[0], cam[1], *cam[2:], _p(m))

    def splat(self, depth, cam, world_to_eye):
        d, m = f32(depth), f32(world_to_eye)
        out = np.zeros(cam[0] * cam[1] + 1, np.uint32)
        n = lib().kref_splat(self.h, _p(d), cam[0], cam[1], *cam[2:], _p(m), _p(out))
        return out[:n].copy()

    def mesh(self, with_indices=True):
        nv, ni = C.c_size_t(), C.c_size_t()
        lib().kref_mesh(self.h, 1 if with_indices else 0, C.byref(nv), C.byref(ni))
        verts = np.zeros((nv.value, 3), np.float32)
        idx = np.zeros(ni.value, np.uint32)
        lib().kref_mesh_fetch(self.h, _p(verts), _p(idx))
        return verts, idx


def sort_unique_expand(keys):
    k = np.ascontiguousarray(keys, np.uint32)
    out = np.zeros(8 * k.size + 1, np.uint32)
    n = lib().kref_sort_unique_expand(_p(k), k.size, _p(out))
    return out[:n].copy()


def radix_sort(keys):
    k = np.ascontiguousarray(keys, np.uint32).copy()
    lib().kref_radix_sort(_p(k), k.size)
    return k


def radix_sort_pairs(keys, vals):
    k = np.ascontiguousarray(keys, np.uint32).copy()
    v = np.ascontiguousarray(vals, np.uint32).copy()
    lib().kref_radix_sort_pairs(_p(k), _p(v), k.size)
    return k, v


def set_union(k1, v1, k2, v2):
    k1, v1, k2, v2 = (np.ascontiguousarray(x, dtype=np.int32) for x in (k1, v1, k2, v2))
    ko = np.full(k1.size + k2.size + 1, -1, np.int32)
    vo = np.full(k1.size + k2.size + 1, -1, np.int32)
    n = lib().kref_set_union(_p(k1), _p(v1), k1.size, _p(k2), _p(v2), k2.size, _p(ko), _p(vo))
    return ko[:n].copy(), vo[:n].copy()


def kahan_sum(x):
    x = f32(x)
    return float(lib().kref_kahan_sum(_p(x), x.size))


def partial_sum_exclusive(a):
    a = np.ascontiguousarray(a, np.int32).copy()
    lib().kref_partial_sum_exclusive(_p(a), a.size)
    return a


def icp_align(depth, cam, e2w_guess, synth, synth_e2w, iters):
    d, g, s, se = f32(depth), f32(e2w_guess), f32(synth), f32(synth_e2w)
    out = np.zeros(16, np.float32)
    lib().kref_icp_align(_p(d), cam[0], cam[1], _p(g), _p(s), s.shape[1], s.shape[0], _p(se),
                         *cam[2:], iters, _p(out))
    return out


def bin_points(points, world_to_clip, w, h):
    p, m = f32(points), f32(world_to_clip)
    out = np.zeros((h, w, 3), np.float32)
    lib().kref_bin(_p(p), p.size // 3, _p(m), _p(out), w, h)
    return out


def eye_to_clip(cam):
    out = np.zeros(16, np.float32)
    lib().kref_eye_to_clip(cam[0], cam[1], *cam[2:], _p(out))
    return out


def invert_transform(m):
    m = f32(m)
    out = np.zeros(16, np.float32)
    lib().kref_invert_transform(_p(m), _p(out))
    return out


def read_depthstream(path):
    """All frames of a .depth file via DepthStream: list of (depth (h,w), view (16,))."""
    h = lib().kref_depthstream_open(path.encode())
    try:
        frames = []
        cap = 4096 * 4096
        buf = np.zeros(cap, np.float32)
        w, hh = C.c_int(), C.c_int()
        view = np.zeros(16, np.float32)
        while lib().kref_depthstream_next(h, _p(buf), cap, C.byref(w), C.byref(hh), _p(view)):
            frames.append((buf[:w.value * hh.value].reshape(hh.value, w.value).copy(), view.copy()))
        return frames
    finally:
        lib().kref_depthstream_close(h)


def mesh2obj(verts, indices, path):
    """Mesher::Mesh2Obj (Mesher.cpp:50-78) of the reference on the given arrays."""
    v = np.ascontiguousarray(verts, np.float32).reshape(-1, 3)
    i = np.ascontiguousarray(indices, np.uint32).reshape(-1)
    lib().kref_mesh2obj(_p(v), C.c_size_t(v.shape[0]), _p(i), C.c_size_t(i.size), str(path).encode())
