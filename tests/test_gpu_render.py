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


def test_mesh_canvas_matches_oracle(cuda):
    """MapDrawer's mesh program (FullSystem/src/MapDrawer.cpp:13-58, 159-234) as a
    rasteriser: two submap meshes drawn into one z-buffer, bit-exact against
    the oracle's restatement (image and depth)."""
    W, H = 320, 240
    K = synth.intrinsics(W, H)
    seq = sequence(3, 4, W, H)
    s = rf.Session(W, H, K, hash_slots=1 << 18, max_blocks=1 << 15)
    T = None
    for rgb, d16, _, _ in seq:
        st, T = s.process(rgb, d16)
        assert st == 0
    me = rf.MeshEngine(2_000_000)
    pts, nrm, _, _ = me.Meshify(s.map())
    assert pts.shape[0] > 10000
    Tcw = np.linalg.inv(T)
    Tmw2 = np.eye(4)
    c, sn = np.cos(0.3), np.sin(0.3)
    Tmw2[:3, :3] = [[c, 0, sn], [0, 1, 0], [-sn, 0, c]]
    Tmw2[:3, 3] = [0.4, 0.05, 0.3]
    cv = rf.Canvas(W, H, K)
    cv.draw_mesh(me, np.eye(4), Tcw)
    cv.draw_triangles(pts, nrm, Tmw2, Tcw)
    rgba, depth = cv.read()
    keys = oracle.canvas_draw(pts, nrm, np.eye(4), Tcw, K, W, H)
    keys = oracle.canvas_draw(pts, nrm, Tmw2, Tcw, K, W, H, keys)
    ro, do = oracle.canvas_resolve(keys)
    assert np.array_equal(rgba, ro) and np.array_equal(depth, do)
    drawn = depth > 0
    assert drawn.mean() > 0.3 and (rgba[~drawn] == 255).all()
    assert len(np.unique(rgba[drawn][:, 0])) > 50
    cv.clear()
    rgba2, depth2 = cv.read()
    assert (rgba2 == 255).all() and not depth2.any()
