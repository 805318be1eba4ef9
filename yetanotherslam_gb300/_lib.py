"""ctypes binding of ``libyas_gb300.so`` (the C ABI of ``include/yas.h``).

The library is built in-tree by :mod:`yetanotherslam_gb300.build`; there is no
fallback implementation: if the shared object is missing or fails to load,
every entry point raises.
"""
from __future__ import annotations

import ctypes as C
import re
import threading
from pathlib import Path

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "_build" / "libyas_gb300.so"
HEADER = _PKG.parent / "include" / "yas.h"

YAS_OK = 0
STATUS = {
    0: "YAS_OK", 1: "YAS_ERR_BAD_ARG", 2: "YAS_ERR_OOM", 3: "YAS_ERR_CUDA", 4: "YAS_ERR_TABLE_FULL",
    5: "YAS_ERR_POOL_FULL", 6: "YAS_ERR_NUMERIC", 7: "YAS_ERR_TRACK_LOST", 8: "YAS_ERR_MESH_OVERFLOW",
    9: "YAS_ERR_STATE", 10: "YAS_ERR_COORD_RANGE", 11: "YAS_ERR_CAPACITY", 12: "YAS_ERR_TIMEOUT",
    13: "YAS_ERR_IO",
}
VOXEL_F32, VOXEL_F16, VOXEL_S24, VOXEL_S16 = 0, 1, 2, 3
TRACK_RGB, TRACK_ICP, TRACK_RGBD = 1, 2, 3


class YasError(RuntimeError):
    def __init__(self, code: int, where: str, detail: str = ""):
        self.code = code
        super().__init__(f"{where}: {STATUS.get(code, code)} {detail}".strip())


class Intrinsics(C.Structure):
    _fields_ = [("fx", C.c_float), ("fy", C.c_float), ("cx", C.c_float), ("cy", C.c_float)]


class Pose(C.Structure):
    _fields_ = [("m", C.c_double * 12)]


class MapConfig(C.Structure):
    _fields_ = [("hash_slots", C.c_int), ("max_blocks", C.c_int), ("voxel_size", C.c_float),
                ("trunc_dist", C.c_float), ("depth_min", C.c_float), ("depth_max", C.c_float),
                ("voxel_format", C.c_int), ("max_weight", C.c_int)]


class SessionConfig(C.Structure):
    _fields_ = [("width", C.c_int), ("height", C.c_int), ("K", Intrinsics), ("map", MapConfig),
                ("num_levels", C.c_int), ("iterations", C.c_int * 5), ("mode", C.c_int),
                ("depth_scale", C.c_float), ("max_step_translation", C.c_float), ("use_graph", C.c_int),
                ("fused_schedule", C.c_int)]


class ServerConfig(C.Structure):
    _fields_ = [("max_sessions", C.c_int), ("hbm_reserve_bytes", C.c_size_t), ("ring_frames", C.c_int),
                ("gn_per_session", C.c_int), ("gn_pixels_per_cta", C.c_int)]


class BatchTuning(C.Structure):
    _fields_ = [("march_warps_x", C.c_int), ("integrate_ctas", C.c_int), ("gn_pixels_per_cta", C.c_int),
                ("gn_per_session", C.c_int)]


class ServedResult(C.Structure):
    _fields_ = [("session", C.c_int), ("status", C.c_int), ("frame", C.c_longlong), ("latency_ms", C.c_double),
                ("Tcm", Pose)]


class ServerStats(C.Structure):
    _fields_ = [("frames", C.c_longlong), ("batches", C.c_longlong), ("mean_batch", C.c_double),
                ("p50_ms", C.c_double), ("p99_ms", C.c_double), ("max_ms", C.c_double), ("fps", C.c_double)]


class GnLevel(C.Structure):
    _fields_ = [("width", C.c_int), ("height", C.c_int), ("fx", C.c_float), ("fy", C.c_float), ("cx", C.c_float),
                ("cy", C.c_float), ("ref_intensity", C.c_void_p), ("ref_inv_depth", C.c_void_p),
                ("ref_vmap", C.c_void_p), ("ref_nmap", C.c_void_p), ("cur_intensity", C.c_void_p),
                ("cur_gx", C.c_void_p), ("cur_gy", C.c_void_p), ("cur_vmap", C.c_void_p), ("cur_nmap", C.c_void_p)]


_P = C.c_void_p
_PP = C.POINTER(C.c_void_p)
_I = C.c_int
_U = C.c_uint
_PU = C.POINTER(C.c_uint)
_PI = C.POINTER(C.c_int)

# name -> argtypes (restype int unless listed in _RESTYPE)
_SIGS = {
    "yas_status_string": [_I],
    "yas_version": [],
    "yas_map_config_default": [C.POINTER(MapConfig), _I, _I, C.c_float, C.c_float, _I],
    "yas_map_create": [_PP, C.POINTER(MapConfig), C.POINTER(Intrinsics), _P],
    "yas_map_create_ref": [_PP, _I, _I, _I, C.c_float, C.c_float, C.POINTER(Intrinsics), _P],
    "yas_map_destroy": [_P],
    "yas_map_reset": [_P],
    "yas_map_empty": [_P, _PI],
    "yas_map_fuse_depth": [_P, _P, _I, _I, _I, _I, C.POINTER(Pose)],
    "yas_map_check_visible": [_P, _I, _I, C.POINTER(Pose), _PU],
    "yas_map_num_visible": [_P, _PU],
    "yas_map_num_allocated": [_P, _PU],
    "yas_map_take_errors": [_P, _PU],
    "yas_map_export": [_P, _P, _P, _P, _U, _PU],
    "yas_map_import": [_P, _P, _P, _P, _U],
    "yas_map_export_visible": [_P, _P, _U, _PU],
    "yas_map_get_pose": [_P, C.POINTER(Pose)],
    "yas_map_set_pose": [_P, C.POINTER(Pose)],
    "yas_map_set_active": [_P, _I],
    "yas_map_is_active": [_P, _PI],
    "yas_map_hibernate": [_P],
    "yas_map_reactivate": [_P],
    "yas_map_is_hibernated": [_P, _PI],
    "yas_map_device_bytes": [_P, C.POINTER(C.c_size_t)],
    "yas_map_reserve": [_P, _I, _I],
    "yas_map_save": [_P, C.c_char_p],
    "yas_map_load": [_P, C.c_char_p],
    "yas_map_fuse_map": [_P, _P],
    "yas_map_swap": [_P, _P],
    "yas_map_reset_visible": [_P],
    "yas_copy_to_host": [_P, _I, _P, _I, _I, _I],
    "yas_tracker_set_reduction": [_P, _I],
    "yas_tracker_check_wait_limit": [_P, _PI],
    "yas_check_div_seeded": [_P, _P, _P, C.c_int],
    "yas_pyr_down_depth": [_P, _I, _I, _I, _P, _I, _I, _I, _P],
    "yas_depth_to_inv_depth": [_P, _I, _I, _I, _P, _I, _P],
    "yas_compute_vertex_map": [_P, _I, _I, _I, _P, _I, C.c_float, C.c_float, C.c_float, C.c_float, C.c_float, _P],
    "yas_compute_normal_map": [_P, _I, _I, _I, _P, _I, _P],
    "yas_image_gradient": [_P, _I, _I, _I, _P, _P, _I, _P],
    "yas_transform_reference_point": [_P, _I, _I, _I, _P, _I, _P, C.POINTER(Pose), _P],
    "yas_vmap_to_depth": [_P, _I, _I, _I, _P, _I, _P],
    "yas_canvas_create": [_PP, _I, _I, C.POINTER(Intrinsics), _P],
    "yas_canvas_destroy": [_P],
    "yas_canvas_clear": [_P],
    "yas_canvas_draw_triangles": [_P, _P, _P, C.c_uint, _I, C.POINTER(Pose), C.POINTER(Pose)],
    "yas_canvas_draw_mesh": [_P, _P, C.POINTER(Pose), C.POINTER(Pose)],
    "yas_canvas_read": [_P, _P, _I, _P, _I, _I],
    "yas_map_defuse_depth": [_P, _P, _I, _I, _I, _I, C.POINTER(Pose)],
    "yas_raycaster_create": [_PP, _I, _I, C.POINTER(Intrinsics), _P],
    "yas_raycaster_destroy": [_P],
    "yas_raycaster_raycast": [_P, _P, C.POINTER(Pose)],
    "yas_raycaster_vmap": [_P, _PP, _PI],
    "yas_raycaster_depth": [_P, _P, _I, _I],
    "yas_raycaster_num_visible": [_P, _PU],
    "yas_raycaster_num_rendering_blocks": [_P, _PU],
    "yas_raycaster_zrange": [_P, _P, _P],
    "yas_mesher_create": [_PP, _I, _P],
    "yas_mesher_destroy": [_P],
    "yas_mesher_meshify": [_P, _P, _PU],
    "yas_mesher_copy": [_P, _P, _P, _U],
    "yas_mesher_copy_cases": [_P, _P, _P, _U],
    "yas_tracker_create": [_PP, _I, _I, _P, _I, _P, _I, _P],
    "yas_tracker_destroy": [_P],
    "yas_tracker_set_reference_image": [_P, _P, _I, _I],
    "yas_tracker_set_tracking_image": [_P, _P, _I, _I],
    "yas_tracker_set_reference_depth": [_P, _P, _I, _I],
    "yas_tracker_set_tracking_depth": [_P, _P, _I, _I],
    "yas_tracker_set_reference_model": [_P, _P, _I],
    "yas_tracker_get_transform": [_P, C.POINTER(Pose), _I, C.POINTER(Pose)],
    "yas_tracker_swap_frame_buffer": [_P],
    "yas_tracker_is_good": [_P, _PI],
    "yas_tracker_set_schedule": [_P, _I],
    "yas_tracker_compute_step": [_P, _I, C.POINTER(Pose), _P, _P, _P],
    "yas_tracker_level_buffer": [_P, _I, _I, _PP, _PI, _PI, _PI],
    "yas_tracker_last_solve": [_P, _P, _P, _P, C.POINTER(Pose)],
    "yas_session_config_default": [C.POINTER(SessionConfig), _I, _I, C.POINTER(Intrinsics), _I, _I,
                                   C.c_float, C.c_float, _I],
    "yas_session_create": [_PP, C.POINTER(SessionConfig), _P],
    "yas_session_destroy": [_P],
    "yas_session_submit": [_P, _P, _P, _I],
    "yas_session_wait": [_P, C.POINTER(Pose), _PI],
    "yas_session_process_frame": [_P, _P, _P, _I, C.POINTER(Pose), _PI],
    "yas_session_map": [_P, _PP],
    "yas_session_tracker": [_P, _PP],
    "yas_session_raycaster": [_P, _PP],
    "yas_session_frame_count": [_P, _PI],
    "yas_session_new_submap": [_P, _PP],
    "yas_session_depth": [_P, _PP, _PI],
    "yas_session_kernels_per_frame": [_P, _PI],
    "yas_session_stream": [_P],
    "yas_session_profile_frame": [_P, _P, _P, _I, _P, _P, _I, _PI],
    "yas_mc_tables": [_P, _P, _P],
    "yas_render_scene": [_P, _P, _I, _I, _I, _P, _P, _I, _I, _P],
    "yas_gn_linearise_static": [C.POINTER(GnLevel), C.POINTER(Pose), _I, _P, _P],
    "yas_batch_tuning_default": [C.POINTER(BatchTuning)],
    "yas_batch_create": [_PP, _PP, _I, _P],
    "yas_batch_destroy": [_P],
    "yas_batch_set_tuning": [_P, C.POINTER(BatchTuning)],
    "yas_batch_get_tuning": [_P, C.POINTER(BatchTuning)],
    "yas_batch_step": [_P, _PP, _PP, _PI, _I],
    "yas_batch_wait": [_P, C.POINTER(Pose), _PI, C.POINTER(C.c_float)],
    "yas_batch_kernels_per_step": [_P, _PI],
    "yas_batch_autotune": [_P, _PP, _PP, _I, _I, C.POINTER(BatchTuning)],
    "yas_server_config_default": [C.POINTER(ServerConfig)],
    "yas_server_create": [_PP, C.POINTER(ServerConfig)],
    "yas_server_destroy": [_P],
    "yas_server_open_session": [_P, C.POINTER(SessionConfig), _PI],
    "yas_server_close_session": [_P, _I],
    "yas_server_suspend_session": [_P, _I],
    "yas_server_resume_session": [_P, _I],
    "yas_server_submit": [_P, _I, _P, _P],
    "yas_server_poll": [_P, C.POINTER(ServedResult), _I, _PI],
    "yas_server_drain": [_P, C.c_double],
    "yas_server_get_stats": [_P, C.POINTER(ServerStats)],
    "yas_server_reset_stats": [_P],
}
_RESTYPE = {"yas_status_string": C.c_char_p, "yas_version": C.c_char_p, "yas_session_stream": C.c_void_p}

_lock = threading.Lock()
_lib = None


def header_functions() -> list[str]:
    """Names of every ``YAS_API`` function declared in include/yas.h."""
    text = HEADER.read_text()
    return re.findall(r"YAS_API\s+[\w\s\*]+?\b(yas_\w+)\s*\(", text)


def load() -> C.CDLL:
    """Loads the native library (raises if it has not been built)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not LIB_PATH.exists():
            raise RuntimeError(f"native library missing: {LIB_PATH} (run __graft_entry__.build())")
        lib = C.CDLL(str(LIB_PATH))
        for name, args in _SIGS.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = _RESTYPE.get(name, C.c_int)
        _lib = lib
        return lib


def check(code: int, where: str) -> int:
    if code != YAS_OK:
        lib = load()
        raise YasError(code, where, lib.yas_status_string(code).decode())
    return code


def call(name: str, *args) -> int:
    """Calls ``name`` and raises :class:`YasError` on a non-zero status."""
    return check(getattr(load(), name)(*args), name)


def pose_from(mat) -> Pose:
    """Pose from a 3x4 or 4x4 array-like (row-major)."""
    import numpy as np
    m = np.asarray(mat, dtype=np.float64)[:3, :4].reshape(-1)
    p = Pose()
    for i in range(12):
        p.m[i] = float(m[i])
    return p


def pose_to(p: Pose):
    import numpy as np
    out = np.eye(4)
    out[:3, :4] = np.frombuffer(p.m, dtype=np.float64).reshape(3, 4)
    return out
