"""ctypes binding of libkifi_gpu.so (include/kifi_gpu.h).

Loading fails loudly when the library has not been built: there is no CPU
fallback for any entry point.
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libkifi_gpu.so")

KIFI_OK = 0
STATUS_NAMES = {
    0: "KIFI_OK", 1: "KIFI_ERR_INVALID_ARGUMENT", 2: "KIFI_ERR_OUT_OF_MEMORY", 3: "KIFI_ERR_CUDA",
    4: "KIFI_ERR_CAPACITY", 5: "KIFI_ERR_TIMEOUT", 6: "KIFI_ERR_UNSUPPORTED",
    7: "KIFI_ERR_NO_DEVICE", 8: "KIFI_ERR_IO", 9: "KIFI_ERR_FORMAT", 10: "KIFI_ERR_END_OF_STREAM",
}


# the status codes by name (KIFI_ERR_TIMEOUT, ...), as in include/kifi_gpu.h
globals().update({_name: _code for _code, _name in STATUS_NAMES.items()})


class KifiError(RuntimeError):
    def __init__(self, status, detail=""):
        self.status = status
        super().__init__("%s (%d): %s" % (STATUS_NAMES.get(status, "?"), status, detail))


class Camera(C.Structure):
    _fields_ = [("width", C.c_int), ("height", C.c_int), ("fx", C.c_float), ("fy", C.c_float),
                ("cx", C.c_float), ("cy", C.c_float), ("znear_m", C.c_float),
                ("zfar_m", C.c_float)]


class PipelineDesc(C.Structure):
    _fields_ = [("camera", Camera), ("resolution", C.c_int), ("side_length_m", C.c_float),
                ("truncation_m", C.c_float), ("icp_iterations", C.c_int), ("mesh_every", C.c_int),
                ("mesh_with_indices", C.c_int), ("initial_capacity", C.c_size_t),
                ("device", C.c_int), ("key_bits", C.c_int), ("closed_loop", C.c_int)]


class VolumeDesc(C.Structure):
    _fields_ = [("resolution", C.c_int), ("side_length_m", C.c_float),
                ("truncation_m", C.c_float), ("initial_capacity", C.c_size_t),
                ("device", C.c_int), ("stream", C.c_void_p), ("key_bits", C.c_int)]


# name -> (restype, argtypes); every exported symbol of include/kifi_gpu.h
SIGNATURES = {
    "kifi_status_string": (C.c_char_p, [C.c_int]),
    "kifi_last_error": (C.c_char_p, []),
    "kifi_device_count": (C.c_int, [C.POINTER(C.c_int)]),
    "kifi_volume_create": (C.c_int, [C.POINTER(VolumeDesc), C.POINTER(C.c_void_p)]),
    "kifi_volume_destroy": (C.c_int, [C.c_void_p]),
    "kifi_volume_size": (C.c_int, [C.c_void_p, C.POINTER(C.c_size_t)]),
    "kifi_volume_export": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t,
                                     C.POINTER(C.c_size_t)]),
    "kifi_volume_insert": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t]),
    "kifi_volume_export64": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t,
                                       C.POINTER(C.c_size_t)]),
    "kifi_volume_insert64": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t]),
    "kifi_volume_key_bits": (C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "kifi_icp_record_associations": (C.c_int, [C.c_void_p, C.c_int]),
    "kifi_icp_associations": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t, C.POINTER(C.c_size_t)]),
    "kifi_radix_sort_u64": (C.c_int, [C.c_void_p, C.c_size_t]),
    "kifi_radix_sort_pairs_u64": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t]),
    "kifi_volume_clear": (C.c_int, [C.c_void_p]),
    "kifi_volume_reserve": (C.c_int, [C.c_void_p, C.c_size_t]),
    "kifi_volume_sync": (C.c_int, [C.c_void_p]),
    "kifi_volume_stream": (C.c_void_p, [C.c_void_p]),
    "kifi_integrate_f32": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(Camera), C.c_void_p]),
    "kifi_integrate_u16": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(Camera), C.c_void_p]),
    "kifi_integrate_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.POINTER(Camera),
                                        C.c_void_p]),
    "kifi_mesh": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_size_t, C.c_void_p, C.c_size_t,
                            C.POINTER(C.c_size_t), C.POINTER(C.c_size_t)]),
    "kifi_radix_sort_u32": (C.c_int, [C.c_void_p, C.c_size_t]),
    "kifi_radix_sort_pairs_u32": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t]),
    "kifi_icp_create": (C.c_int, [C.c_int, C.c_void_p, C.POINTER(C.c_void_p)]),
    "kifi_icp_destroy": (C.c_int, [C.c_void_p]),
    "kifi_icp_stream": (C.c_void_p, [C.c_void_p]),
    "kifi_icp_set_target": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p]),
    "kifi_icp_set_target_from_depth": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_int,
                                                 C.POINTER(Camera), C.c_void_p]),
    "kifi_icp_align": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(Camera), C.c_void_p, C.c_int,
                                 C.c_void_p]),
    "kifi_icp_align_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.POINTER(Camera),
                                        C.c_void_p, C.c_int]),
    "kifi_icp_result": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                  C.c_int, C.POINTER(C.c_int)]),
    "kifi_gemm_bf16": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int,
                                 C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p]),
    "kifi_conv3x3s2_bf16": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_int,
                                      C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]),
    "kifi_volume_autotune": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.POINTER(Camera), C.c_void_p, C.c_int,
                                       C.c_void_p]),
    "kifi_proposer_create": (C.c_int, [C.c_int, C.c_int, C.POINTER(C.c_void_p)]),
    "kifi_proposer_destroy": (C.c_int, [C.c_void_p]),
    "kifi_proposer_param_count": (C.c_int, [C.c_void_p, C.POINTER(C.c_size_t)]),
    "kifi_proposer_set_params": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t]),
    "kifi_proposer_get_params": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t]),
    "kifi_proposer_make_input": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int,
                                           C.c_void_p]),
    "kifi_proposer_set_inputs": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int]),
    "kifi_proposer_get_inputs": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int]),
    "kifi_proposer_predict": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p]),
    "kifi_proposer_gradients": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]),
    "kifi_proposer_train_step": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_float, C.c_void_p]),
    "kifi_pipeline_set_graphs": (C.c_int, [C.c_void_p, C.c_int]),
    "kifi_pipeline_graph_stats": (C.c_int, [C.c_void_p, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)]),
    "kifi_depthstream_open": (C.c_int, [C.c_char_p, C.POINTER(C.c_void_p)]),
    "kifi_depthstream_close": (C.c_int, [C.c_void_p]),
    "kifi_depthstream_info": (C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                        C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "kifi_depthstream_next_frame": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "kifi_depthstream_next_frame_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "kifi_mesh_to_obj": (C.c_int, [C.c_void_p, C.c_size_t, C.c_void_p, C.c_size_t, C.c_char_p]),
    "kifi_volume_save": (C.c_int, [C.c_void_p, C.c_char_p]),
    "kifi_volume_load": (C.c_int, [C.c_char_p, C.c_int, C.POINTER(C.c_void_p)]),
    "kifi_radix_sort_pairs_u32_static": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p]),
    "kifi_icp_iteration_times": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                                           C.POINTER(C.c_int)]),
    "kifi_bin": (C.c_int, [C.c_void_p, C.c_size_t, C.c_void_p, C.c_void_p, C.c_int, C.c_int]),
    "kifi_mesh_device": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_size_t),
                                   C.POINTER(C.c_size_t), C.c_void_p, C.c_void_p]),
    "kifi_volume_set_profiling": (C.c_int, [C.c_void_p, C.c_int]),
    "kifi_volume_set_launch_mode": (C.c_int, [C.c_void_p, C.c_int]),
    "kifi_volume_stage_times": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(C.c_int)]),
    "kifi_volume_frame_log": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                                        C.POINTER(C.c_int)]),
    "kifi_pipeline_create": (C.c_int, [C.POINTER(PipelineDesc), C.POINTER(C.c_void_p)]),
    "kifi_pipeline_destroy": (C.c_int, [C.c_void_p]),
    "kifi_pipeline_volume": (C.c_void_p, [C.c_void_p]),
    "kifi_pipeline_icp": (C.c_void_p, [C.c_void_p]),
    "kifi_pipeline_integrate": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]),
    "kifi_pipeline_integrate_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]),
    "kifi_pipeline_sync": (C.c_int, [C.c_void_p, C.c_void_p]),
    "kifi_pipeline_mesh_counts": (C.c_int, [C.c_void_p, C.POINTER(C.c_size_t),
                                            C.POINTER(C.c_size_t)]),
    "kifi_pipeline_mesh_stats": (C.c_int, [C.c_void_p, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)]),
    "kifi_pipeline_join": (C.c_int, [C.c_void_p, C.c_void_p]),
    "kifi_sort_set_fault_injection": (C.c_int, [C.c_uint, C.c_ulonglong]),
    "kifi_batch_create": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_void_p)]),
    "kifi_batch_destroy": (C.c_int, [C.c_void_p]),
    "kifi_batch_step_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "kifi_batch_sync": (C.c_int, [C.c_void_p]),
    "kifi_batch_volume": (C.c_void_p, [C.c_void_p, C.c_int]),
    "kifi_batch_pose": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p]),
    "kifi_batch_stream": (C.c_void_p, [C.c_void_p]),
    "kifi_batch_set_profiling": (C.c_int, [C.c_void_p, C.c_int]),
    "kifi_batch_set_persistent": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "kifi_batch_step_times": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.POINTER(C.c_int)]),
    "kifi_volume_mesh_times": (C.c_int, [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int)]),
    "kifi_volume_mesh_stage_times": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(C.c_int)]),
    "kifi_pipeline_stage_times": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "kifi_icp_set_target_bin_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p, C.c_int,
                                                 C.c_int, C.c_void_p]),
}

_lib = None


def load():
    """The loaded library; raises OSError when it is missing."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise OSError("libkifi_gpu.so is not built (%s); run "
                          "`python -m merge_fusion_gb300.build`" % LIB_PATH)
        lib = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        _lib = lib
    return _lib


def check(status, what=""):
    if status != KIFI_OK:
        detail = load().kifi_last_error().decode(errors="replace")
        raise KifiError(status, (what + ": " if what else "") + detail)


def device_count():
    n = C.c_int(0)
    check(load().kifi_device_count(C.byref(n)))
    return n.value
