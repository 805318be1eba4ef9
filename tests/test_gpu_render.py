"""Headless shading (RenderScene, RGBDFusion/src/ImageProc.cu:80-139) against
the oracle on the raycast model of a fused map.  Bar: every byte within 1 of
the oracle's (the specular term's powf may round differently on the device),
misses exactly (4, 2, 2, 255)."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

import oracle
from tests.helpers import sequence
from yetanotherslam_gb300 import _lib as L
from yetanotherslam_gb300 import rgbdfusion as rf
from yetanotherslam_gb300 import synth

pytestmark = pytest.mark.gpu


def test_render_scene_matches_oracle(cuda):
    import torch

    W, H = 320, 240
    K = synth.intrinsics(W, H)
    seq = sequence(3, 3, W, H)
    s = rf.Session(W, H, K, hash_slots=1 << 18, max_blocks=1 << 15)
    for rgb, d16, _, _ in seq:
        st, _ = s.process(rgb, d16)
        assert st == 0
    tr = C.c_void_p()
    L.call("yas_session_tracker", s.handle, C.byref(tr))
    ptrs = []
    for which in (8, 9):  # model (reference) vertex and normal maps, level 0
        p = C.c_void_p()
        w, h, pitch = C.c_int(), C.c_int(), C.c_int()
        L.call("yas_tracker_level_buffer", tr, 0, which, C.byref(p), C.byref(w), C.byref(h), C.byref(pitch))
        ptrs.append(p.value)
    # vertex map with misses as the raycaster writes them (NaN), planted in
    # a device copy of the model vertex map
    vmap = torch.as_tensor(rf.DeviceArray(ptrs[0], (H, W, 4), "<f4"), device="cuda").clone()
    vmap[: H // 4] = float("nan")
    nmap = torch.as_tensor(rf.DeviceArray(ptrs[1], (H, W, 4), "<f4"), device="cuda").clone()
    ptrs = [vmap.data_ptr(), nmap.data_ptr()]
    out = torch.zeros((H, W, 4), dtype=torch.uint8, device="cuda")
    light = (C.c_float * 3)(5.0, 5.0, 5.0)
    torch.cuda.synchronize()
    L.call("yas_render_scene", ptrs[0], ptrs[1], W, H, W * 16, light, out.data_ptr(), W * 4, 1, None)
    torch.cuda.synchronize()
    img = out.cpu().numpy()
    vm, nm = vmap.cpu().numpy(), nmap.cpu().numpy()
    ref = oracle.render_scene(vm, nm)
    d = np.abs(img.astype(np.int16) - ref.astype(np.int16))
    assert d.max() <= 1
    miss = np.isnan(vm[..., 0])
    assert miss.any() and (~miss).any()
    assert (img[miss] == np.array([4, 2, 2, 255], np.uint8)).all()
    # host output path
    host = np.zeros((H, W, 4), np.uint8)
    L.call("yas_render_scene", ptrs[0], ptrs[1], W, H, W * 16, light, host.ctypes.data, W * 4, 0, None)
    assert np.array_equal(host, img)
