"""Python mirror of kifi's fusion interface (denniskb/merge_fusion,
KinectFission/kifi), backed by libkifi_gpu.so through its C ABI.

Names, argument meanings and results follow the reference classes:

* ``DepthSensorParams``  -- KinectFission/kifi/DepthSensorParams.h:23-52
* ``Volume``             -- KinectFission/kifi/Volume.h:12-51
* ``Integrator``         -- KinectFission/kifi/Integrator.h:16-63
* ``Mesher``             -- KinectFission/kifi/Mesher.h:14-38

Matrices: a (16,) float array is taken in kifi's float4x4 memory order
(four columns, KinectFission/kifi/util/math.h:59-61); a (4, 4) array is taken
as the matrix itself (element [row, col]).
"""
import ctypes as C
import os

import numpy as np

from . import _lib
from ._lib import Camera, KifiError, VolumeDesc, check


def as_kifi_matrix(m):
    """(16,) float32 in kifi float4x4 memory order (column-major)."""
    a = np.asarray(m, dtype=np.float32)
    if a.shape == (4, 4):
        return np.ascontiguousarray(a.T).reshape(16)
    if a.shape == (16,):
        return np.ascontiguousarray(a)
    raise ValueError("expected a (16,) kifi matrix or a (4, 4) matrix")


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


class DepthSensorParams:
    """Camera intrinsics (DepthSensorParams.h:23-52)."""

    def __init__(self, resolution, focal_length, principal_point, sensible_range):
        self.resolution = (int(resolution[0]), int(resolution[1]))
        self.focal_length = (float(focal_length[0]), float(focal_length[1]))
        self.principal_point = (float(principal_point[0]), float(principal_point[1]))
        self.sensible_range = (float(sensible_range[0]), float(sensible_range[1]))

    def ResolutionPixels(self):
        return self.resolution

    def FocalLengthPixels(self):
        return self.focal_length

    def PrincipalPointPixels(self):
        return self.principal_point

    def SensibleRangeMeters(self):
        return self.sensible_range

    @staticmethod
    def KinectParams(resolution_640x480=True, near_mode=False):
        """DepthSensorParams::KinectParams (DepthSensorParams.cpp:67-82)."""
        w, h = (640, 480) if resolution_640x480 else (320, 240)
        fl = np.float32(571.26) if resolution_640x480 else np.float32(285.63)
        rng = (0.4, 3.0) if near_mode else (0.8, 4.0)
        return DepthSensorParams((w, h), (fl, fl), (w * 0.5, h * 0.5), rng)

    def camera(self):
        c = Camera()
        c.width, c.height = self.resolution
        c.fx, c.fy = self.focal_length
        c.cx, c.cy = self.principal_point
        c.znear_m, c.zfar_m = self.sensible_range
        return c

    def as_tuple(self):
        return (self.resolution[0], self.resolution[1]) + self.focal_length + \
            self.principal_point + self.sensible_range


class Volume:
    """Sparse TSDF volume resident on the GPU (Volume.h:12-51).

    ``Volume(resolution, sideLength, truncationMargin)``; the cube is centred
    at the world origin.  Voxels are (distance-sum, weight) pairs keyed by
    30-bit linear keys z<<20 | y<<10 | x up to 1024 voxels per axis, and by
    64-bit keys z<<2b | y<<b | x (b = max(10, log2 resolution)) beyond, or
    when ``key_bits=64``."""

    def __init__(self, resolution, side_length, truncation_margin, device=0, capacity=0,
                 stream=None, key_bits=0):
        self._h = None
        d = VolumeDesc()
        d.resolution = int(resolution)
        d.side_length_m = float(side_length)
        d.truncation_m = float(truncation_margin)
        d.initial_capacity = int(capacity)
        d.device = int(device)
        d.stream = stream
        d.key_bits = int(key_bits)
        h = C.c_void_p()
        check(_lib.load().kifi_volume_create(C.byref(d), C.byref(h)), "Volume")
        self._h = h
        kb, b = C.c_int(), C.c_int()
        check(_lib.load().kifi_volume_key_bits(h, C.byref(kb), C.byref(b)), "key_bits")
        self.key_bits, self.bits_per_axis = kb.value, b.value
        self._res = int(resolution)
        self._side = np.float32(side_length)
        self._trunc = np.float32(truncation_margin)

    def __del__(self):
        self.close()

    def close(self):
        if self._h is not None:
            _lib.load().kifi_volume_destroy(self._h)
            self._h = None

    @property
    def handle(self):
        return self._h

    # Volume.cpp:41-71
    def Resolution(self):
        return self._res

    def VoxelLength(self):
        return np.float32(self._side / np.float32(self._res))

    def SideLength(self):
        return self._side

    def TruncationMargin(self):
        return self._trunc

    def Minimum(self):
        return np.float32(-0.5) * self._side

    def Maximum(self):
        return np.float32(0.5) * self._side

    def size(self):
        n = C.c_size_t()
        check(_lib.load().kifi_volume_size(self._h, C.byref(n)), "size")
        return n.value

    def export(self, key_bits=None):
        """(keys (n,), values float32 (n, 2) = (distance-sum, weight)); keys
        uint32 or uint64 (``key_bits``, default the volume's own width)."""
        wide = (key_bits or self.key_bits) == 64
        n = self.size()
        keys = np.zeros(n + 1, np.uint64 if wide else np.uint32)
        vals = np.zeros((n + 1, 2), np.float32)
        got = C.c_size_t()
        fn = _lib.load().kifi_volume_export64 if wide else _lib.load().kifi_volume_export
        check(fn(self._h, _ptr(keys), _ptr(vals), n + 1, C.byref(got)), "export")
        return keys[:got.value].copy(), vals[:got.value].copy()

    def insert(self, keys, values=None):
        """flat_map::insert: union with sorted unique keys; resident voxels win.
        uint64 keys go through the 64-bit entry point, others as uint32."""
        wide = np.asarray(keys).dtype == np.uint64
        k = np.ascontiguousarray(keys, dtype=np.uint64 if wide else np.uint32)
        v = None if values is None else np.ascontiguousarray(values, dtype=np.float32)
        fn = _lib.load().kifi_volume_insert64 if wide else _lib.load().kifi_volume_insert
        check(fn(self._h, _ptr(k), None if v is None else _ptr(v), k.size), "insert")

    def clear(self):
        check(_lib.load().kifi_volume_clear(self._h), "clear")

    def reserve(self, capacity):
        check(_lib.load().kifi_volume_reserve(self._h, int(capacity)), "reserve")

    def sync(self):
        check(_lib.load().kifi_volume_sync(self._h), "sync")

    def stream(self):
        return _lib.load().kifi_volume_stream(self._h)

    def set_launch_mode(self, beside_tracking):
        """Launch shape of the fusion kernels: beside a tracking stream (short-lived CTAs, the
        merge build that holds fewer SM resources) or alone (the default).  Results are identical."""
        check(_lib.load().kifi_volume_set_launch_mode(self._h, 1 if beside_tracking else 0), "set_launch_mode")

    def autotune(self, depth_dev_ptr, depth_is_u16, camera_params, world_to_eye, force=False):
        """Measures and sets the persistent CTA counts of the fusion kernels
        on one device frame (kifi_volume_autotune); the volume is unchanged.
        Returns {"splat": n, "sort": n, "merge": n}."""
        cam = camera_params.camera()
        m = as_kifi_matrix(world_to_eye)
        out = np.zeros(3, np.int32)
        check(_lib.load().kifi_volume_autotune(self._h, C.c_void_p(depth_dev_ptr), 1 if depth_is_u16 else 0,
                                               C.byref(cam), _ptr(m), 1 if force else 0, _ptr(out)), "autotune")
        return {"splat": int(out[0]), "sort": int(out[1]), "merge": int(out[2])}

    def save(self, path):
        """Checkpoint: geometry, keys and voxels (no reference counterpart)."""
        check(_lib.load().kifi_volume_save(self._h, os.fsencode(path)), "save")

    @classmethod
    def load(cls, path, device=0):
        """A new volume holding exactly the voxels of a checkpoint."""
        h = C.c_void_p()
        lib = _lib.load()
        check(lib.kifi_volume_load(os.fsencode(path), int(device), C.byref(h)), "load")
        self = cls.__new__(cls)
        self._h = h
        with open(path, "rb") as f:
            hdr = f.read(20)
        self._res = int(np.frombuffer(hdr[8:12], np.int32)[0])
        self._side = np.frombuffer(hdr[12:16], np.float32)[0]
        self._trunc = np.frombuffer(hdr[16:20], np.float32)[0]
        kb, b = C.c_int(), C.c_int()
        check(lib.kifi_volume_key_bits(h, C.byref(kb), C.byref(b)), "key_bits")
        self.key_bits, self.bits_per_axis = kb.value, b.value
        return self


class Integrator:
    """Integrator::Integrate (Integrator.h:19-26)."""

    def Integrate(self, volume, frame, camera_params, world_to_eye):
        """frame: (h, w) float32 metres, or uint16 millimetres."""
        f = np.ascontiguousarray(frame)
        cam = camera_params.camera()
        if f.shape != (cam.height, cam.width):
            raise ValueError("frame shape does not match the camera resolution")
        m = as_kifi_matrix(world_to_eye)
        lib = _lib.load()
        if f.dtype == np.uint16:
            check(lib.kifi_integrate_u16(volume.handle, _ptr(f), C.byref(cam), _ptr(m)), "Integrate")
        else:
            f = np.ascontiguousarray(f, dtype=np.float32)
            check(lib.kifi_integrate_f32(volume.handle, _ptr(f), C.byref(cam), _ptr(m)), "Integrate")

    def IntegrateDevice(self, volume, depth_ptr, is_u16, camera_params, world_to_eye):
        """Asynchronous variant over a frame already in device memory."""
        cam = camera_params.camera()
        m = as_kifi_matrix(world_to_eye)
        check(_lib.load().kifi_integrate_device(volume.handle, C.c_void_p(depth_ptr),
                                                1 if is_u16 else 0, C.byref(cam), _ptr(m)),
              "IntegrateDevice")


class Mesher:
    """Mesher::Mesh (Mesher.h:17-18) and Mesher::Mesh2Obj (Mesher.h:20-25)."""

    @staticmethod
    def Mesh2Obj(vertices, indices, out_obj_file_name):
        v = np.ascontiguousarray(vertices, dtype=np.float32).reshape(-1, 3)
        i = np.ascontiguousarray(indices, dtype=np.uint32).reshape(-1)
        check(_lib.load().kifi_mesh_to_obj(_ptr(v), v.shape[0], _ptr(i), i.size,
                                           os.fsencode(out_obj_file_name)), "Mesh2Obj")

    def Mesh(self, volume, with_indices=True):
        """Returns (vertices float32 (V, 3), indices uint32 (I,)); without
        indices the vertices come in the reference's generation order."""
        lib = _lib.load()
        nv, ni = C.c_size_t(), C.c_size_t()
        st = lib.kifi_mesh(volume.handle, 1 if with_indices else 0, None, 0, None, 0,
                           C.byref(nv), C.byref(ni))
        if st not in (0, 4):
            check(st, "Mesh")
        verts = np.zeros((nv.value + 1, 3), np.float32)
        idx = np.zeros(ni.value + 1, np.uint32)
        check(lib.kifi_mesh(volume.handle, 1 if with_indices else 0, _ptr(verts), nv.value + 1,
                            _ptr(idx), ni.value + 1, C.byref(nv), C.byref(ni)), "Mesh")
        return verts[:nv.value].copy(), idx[:ni.value].copy()


class ICP:
    """ICP::Align (ICP.h:18-27) on the GPU.

    ``Align(rawDepthMap, eyeToWorldGuess, synthBuffer, synthEyeToWorld,
    cameraParams, iterations=4)`` -- the reference's parameter names say
    worldToEye but carry eye-to-world poses (ICP.cpp:12-15, :79); the
    reference fixes 4 iterations (ICP.cpp:22).  Returns the eye-to-world pose
    as a (16,) kifi matrix."""

    def __init__(self, device=0, stream=None):
        self._h = None
        h = C.c_void_p()
        check(_lib.load().kifi_icp_create(int(device), stream, C.byref(h)), "ICP")
        self._h = h

    def __del__(self):
        self.close()

    def close(self):
        if self._h is not None:
            _lib.load().kifi_icp_destroy(self._h)
            self._h = None

    @property
    def handle(self):
        return self._h

    def SetTarget(self, synth_points, synth_eye_to_world):
        p = np.ascontiguousarray(synth_points, dtype=np.float32)
        if p.ndim != 3 or p.shape[2] != 3:
            raise ValueError("target must be (h, w, 3)")
        m = as_kifi_matrix(synth_eye_to_world)
        check(_lib.load().kifi_icp_set_target(self._h, _ptr(p), p.shape[1], p.shape[0], _ptr(m)),
              "SetTarget")

    def SetTargetFromDepth(self, frame, camera_params, eye_to_world):
        f = np.ascontiguousarray(frame)
        u16 = f.dtype == np.uint16
        if not u16:
            f = np.ascontiguousarray(f, dtype=np.float32)
        cam = camera_params.camera()
        m = as_kifi_matrix(eye_to_world)
        check(_lib.load().kifi_icp_set_target_from_depth(self._h, _ptr(f), 0, 1 if u16 else 0,
                                                         C.byref(cam), _ptr(m)), "SetTargetFromDepth")

    def Align(self, raw_depth, eye_to_world_guess, synth_points, synth_eye_to_world,
              camera_params, iterations=4):
        self.SetTarget(synth_points, synth_eye_to_world)
        return self.AlignToTarget(raw_depth, eye_to_world_guess, camera_params, iterations)

    def AlignToTarget(self, raw_depth, eye_to_world_guess, camera_params, iterations=4):
        d = np.ascontiguousarray(raw_depth, dtype=np.float32)
        cam = camera_params.camera()
        g = as_kifi_matrix(eye_to_world_guess)
        out = np.zeros(16, np.float32)
        check(_lib.load().kifi_icp_align(self._h, _ptr(d), C.byref(cam), _ptr(g), int(iterations),
                                         _ptr(out)), "Align")
        return out

    def RecordAssociations(self, on=True):
        check(_lib.load().kifi_icp_record_associations(self._h, 1 if on else 0), "RecordAssociations")

    def Associations(self):
        """The last iteration's association per source (rows, every 4th
        column): (target index int64, -1 for none; len^2 float32)."""
        lib = _lib.load()
        n = C.c_size_t()
        lib.kifi_icp_associations(self._h, None, None, 0, C.byref(n))  # the count (capacity error ignored)
        idx = np.zeros(n.value, np.int64)
        l2 = np.zeros(n.value, np.float32)
        check(lib.kifi_icp_associations(self._h, _ptr(idx), _ptr(l2), n.value, C.byref(n)), "Associations")
        return idx, l2

    def Result(self):
        """(pose float (16,), pose double (16,), n_assoc per iteration, rms per iteration)."""
        pf = np.zeros(16, np.float32)
        pd = np.zeros(16, np.float64)
        na = np.zeros(64, np.int32)
        rms = np.zeros(64, np.float64)
        it = C.c_int()
        check(_lib.load().kifi_icp_result(self._h, _ptr(pf), _ptr(pd), _ptr(na), _ptr(rms), 64,
                                          C.byref(it)), "Result")
        n = min(it.value, 64)
        return pf, pd, na[:n].copy(), rms[:n].copy()


class Renderer:
    """Renderer::Bin (Renderer.h:23-29)."""

    def Bin(self, point_cloud, world_to_clip, width, height):
        p = np.ascontiguousarray(point_cloud, dtype=np.float32).reshape(-1, 3)
        m = as_kifi_matrix(world_to_clip)
        out = np.zeros((height, width, 3), np.float32)
        check(_lib.load().kifi_bin(_ptr(p), p.shape[0], _ptr(m), _ptr(out), int(width),
                                   int(height)), "Bin")
        return out


def radix_sort(keys, values=None):
    """util::radix_sort on the GPU (algorithm.h:63-134); uint64 keys sort
    with the 64-bit variant, anything else as uint32."""
    wide = np.asarray(keys).dtype == np.uint64
    k = np.ascontiguousarray(keys, dtype=np.uint64 if wide else np.uint32).copy()
    lib = _lib.load()
    if values is None:
        fn = lib.kifi_radix_sort_u64 if wide else lib.kifi_radix_sort_u32
        check(fn(_ptr(k), k.size), "radix_sort")
        return k
    v = np.ascontiguousarray(values, dtype=np.uint32).copy()
    fn = lib.kifi_radix_sort_pairs_u64 if wide else lib.kifi_radix_sort_pairs_u32
    check(fn(_ptr(k), _ptr(v), k.size), "radix_sort")
    return k, v


__all__ = ["DepthSensorParams", "Volume", "Integrator", "Mesher", "ICP", "Renderer", "radix_sort",
           "KifiError", "as_kifi_matrix"]


class DepthStream:
    """DepthStream (DepthStream.h:13-45): a .depth v1/v2 recording."""

    def __init__(self, file_name):
        self._h = None
        h = C.c_void_p()
        check(_lib.load().kifi_depthstream_open(os.fsencode(file_name), C.byref(h)), "DepthStream")
        self._h = h
        w, hh, u16, n = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        check(_lib.load().kifi_depthstream_info(h, C.byref(w), C.byref(hh), C.byref(u16), C.byref(n)),
              "DepthStream")
        self.width, self.height, self.texel_is_u16, self._n = w.value, hh.value, bool(u16.value), n.value

    def __del__(self):
        self.close()

    def close(self):
        if self._h is not None:
            _lib.load().kifi_depthstream_close(self._h)
            self._h = None

    def FrameCount(self):
        return self._n

    def NextFrame(self):
        """(frame float32 (height, width) metres, view (16,) kifi order), or
        None after the last frame (the reference returns false)."""
        frame = np.zeros((self.height, self.width), np.float32)
        view = np.zeros(16, np.float32)
        st = _lib.load().kifi_depthstream_next_frame(self._h, _ptr(frame), _ptr(view))
        if st == 10:  # KIFI_ERR_END_OF_STREAM
            return None
        check(st, "NextFrame")
        return frame, view

    def NextFrameDevice(self, depth_dev_ptr, cuda_stream=None):
        """Raw texels of the next frame into device memory (async on the
        stream); returns the view, or None after the last frame."""
        view = np.zeros(16, np.float32)
        st = _lib.load().kifi_depthstream_next_frame_device(self._h, C.c_void_p(depth_dev_ptr),
                                                            _ptr(view), cuda_stream)
        if st == 10:
            return None
        check(st, "NextFrameDevice")
        return view
