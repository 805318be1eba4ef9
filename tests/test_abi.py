"""The C ABI library: builds, loads, exports every declared symbol, and
rejects bad arguments on the host before touching the GPU (no compute calls
here, so this runs without a GPU)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from yetanotherslam_gb300 import _lib as L


def test_every_declared_function_is_exported_and_bound(native):
    names = L.header_functions()
    assert len(names) >= 60
    for n in names:
        assert hasattr(native, n), f"{n} declared in include/yas.h but not exported"
        assert n in L._SIGS, f"{n} has no ctypes signature"
    # and nothing is exported under the yas_ prefix that the header omits
    extra = set(L._SIGS) - set(names) - {"yas_mc_tables"}
    assert not extra, extra


def test_status_strings_and_version(native):
    assert native.yas_version().decode().startswith("yas-gb300")
    for code in L.STATUS:
        assert native.yas_status_string(code)
    assert native.yas_status_string(999) == b"unknown status"


def test_bad_arguments_rejected_on_host(native):
    K = L.Intrinsics(500.0, 500.0, 320.0, 240.0)
    h = C.c_void_p()
    cfg = L.MapConfig()
    assert native.yas_map_config_default(C.byref(cfg), 1000, 10, 0.01, 0.03, 1) == 0
    # non power-of-two slot count
    assert native.yas_map_create(C.byref(h), C.byref(cfg), C.byref(K), None) == 1
    cfg.hash_slots = 1024
    cfg.voxel_format = 7
    assert native.yas_map_create(C.byref(h), C.byref(cfg), C.byref(K), None) == 1
    cfg.voxel_format = 2
    cfg.max_weight = 1000  # S24 keeps an 8-bit weight
    assert native.yas_map_create(C.byref(h), C.byref(cfg), C.byref(K), None) == 1
    assert native.yas_map_create(None, C.byref(cfg), C.byref(K), None) == 1
    assert native.yas_map_destroy(None) == 1
    assert native.yas_map_create_ref(C.byref(h), 0, 10, 10, 0.01, 0.03, C.byref(K), None) == 1
    Kd = (C.c_double * 9)(500, 0, 320, 0, 500, 240, 0, 0, 1)
    assert native.yas_tracker_create(C.byref(h), 640, 480, Kd, 0, None, 3, None) == 1
    assert native.yas_tracker_create(C.byref(h), 640, 480, Kd, 6, None, 3, None) == 1
    assert native.yas_tracker_create(C.byref(h), 640, 480, Kd, 3, None, 0, None) == 1
    assert native.yas_tracker_create(C.byref(h), 8, 8, Kd, 3, None, 3, None) == 1  # level 2 is 2x2
    assert native.yas_raycaster_create(C.byref(h), 0, 480, C.byref(K), None) == 1
    assert native.yas_mesher_create(C.byref(h), 0, None) == 1
    sc = L.SessionConfig()
    assert native.yas_session_config_default(C.byref(sc), 640, 480, C.byref(K), 1 << 20, 1 << 16, 0.005,
                                             0.015, 1) == 0
    assert sc.num_levels == 3 and list(sc.iterations)[:3] == [10, 5, 3] and abs(sc.depth_scale - 0.001) < 1e-9
    assert native.yas_session_create(None, C.byref(sc), None) == 1


def test_pose_roundtrip():
    T = np.eye(4)
    T[:3, :3] = [[0, -1, 0], [1, 0, 0], [0, 0, 1]]
    T[:3, 3] = [1, 2, 3]
    assert np.array_equal(L.pose_to(L.pose_from(T)), T)
