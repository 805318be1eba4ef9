"""The allocation-free linearisation entry point, yas_gn_linearise_static.

Some callers of this library cannot allocate device memory: a host
application that keeps the whole device-memory budget of its process, or code
running where cudaMalloc would synchronise the device or is not permitted
(a real-time frame callback).  This entry point takes the tracker's level
maps and an output buffer from the caller and keeps its own scratch in fixed
static device memory.  These tests call it through the C ABI, on two calls in
a row, since all calls share (and overwrite) the one scratch array, and check:

  * bit-identical H, b and statistics against yas_tracker_compute_step, which
    runs the same passes on the same grid with handle-owned scratch (the
    level intrinsics used here are exact in FP32, so both paths see the same
    camera constants);
  * the oracle's compute_step at the tracker parity tests' tolerance (every
    entry of H and b within 1e-3 of max|H|, max|b|);
  * that a warm call leaves the device's free memory unchanged.

The file name makes pytest collect it after every other test file.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

import oracle
from tests.helpers import rel_poses, sequence
from yetanotherslam_gb300 import _lib as L
from yetanotherslam_gb300 import rgbdfusion as rf
from yetanotherslam_gb300 import synth

pytestmark = pytest.mark.gpu


def _tracker(mode, W=320, H=240):
    fx, fy, cx, cy = synth.intrinsics(W, H)
    K = np.array([[fx, 0, cx], [0, fy, cy], [0, 0, 1.0]])
    seq = sequence(11, 2, W, H)
    g0, g1 = synth.gray_of(seq[0][0]), synth.gray_of(seq[1][0])
    tr = rf.RGBDTracking(W, H, K, bRGB=bool(mode & 1), bIcp=bool(mode & 2), num_levels=3, iterations=(10, 5, 3))
    m = rf.MapStruct(K)
    m.create_config(1 << 18, 1 << 15, 0.008, 0.024, rf.VOXEL_F32)
    m.Fuse(seq[0][2], np.eye(4))
    rc = rf.RayTraceEngine(W, H, K)
    rc.RayTrace(m, np.eye(4))
    tr.SetReferenceImage(g0)
    tr.SetReferenceDepth(seq[0][2])
    tr.SetTrackingImage(g1)
    tr.SetTrackingDepth(seq[1][2])
    tr.SetReferenceModel(rc.GetVMap())
    ot = oracle.Tracker(W, H, K, levels=3, iters=(10, 5, 3), mode=mode)
    ot.set_image(g0, True)
    ot.set_depth(seq[0][2], True)
    ot.set_image(g1, False)
    ot.set_depth(seq[1][2], False)
    ot.set_model(rc.GetVMap().numpy())
    gt = np.linalg.inv(rel_poses(seq)[1])
    return tr, ot, (fx, fy, cx, cy), gt, (m, rc)


def _level(tr, lvl, K):
    fx, fy, cx, cy = K
    s = float(1 << lvl)
    ptr = {w: tr.level_buffer(lvl, w).__cuda_array_interface__["data"][0] for w in range(10)}
    shape = tr.level_buffer(lvl, 0).__cuda_array_interface__["shape"]
    return L.GnLevel(shape[1], shape[0], fx / s, fy / s, cx / s, cy / s, ptr[6], ptr[7], ptr[8], ptr[9], ptr[0],
                     ptr[1], ptr[2], ptr[4], ptr[5])


@pytest.mark.parametrize("mode", [L.TRACK_RGBD, L.TRACK_RGB, L.TRACK_ICP])
def test_static_linearisation_matches_handle_path_twice(cuda, mode):
    import torch

    tr, ot, K, gt, keep = _tracker(mode)
    out = torch.zeros(46, dtype=torch.float64, device="cuda")
    perturb = np.eye(4)
    perturb[:3, 3] = [0.003, -0.002, 0.001]
    for lvl in (0, 1, 2):
        lv = _level(tr, lvl, K)
        for T in (gt, perturb @ gt):
            Hh, bh, sh = tr.compute_step(lvl, T)
            Ho, bo, so = ot.compute_step(lvl, T)
            for _ in range(2):  # two calls in a row share the static scratch
                out.fill_(np.nan)
                L.call("yas_gn_linearise_static", C.byref(lv), C.byref(L.pose_from(T)), mode, out.data_ptr(), None)
                torch.cuda.synchronize()
                o = out.cpu().numpy()
                Hs, bs, ss = o[:36].reshape(6, 6), o[36:42], o[42:46]
                assert np.array_equal(Hs, Hh), (lvl, np.abs(Hs - Hh).max())
                assert np.array_equal(bs, bh), (lvl, np.abs(bs - bh).max())
                assert np.array_equal(ss, sh, equal_nan=True), (lvl, ss, sh)  # stats[2] is NaN without RGB
                assert np.abs(Hs - Ho).max() <= 1e-3 * np.abs(Ho).max()
                assert np.abs(bs - bo).max() <= 1e-3 * max(np.abs(bo).max(), 1e-9)
                assert abs(ss[1] - so[1]) <= 2 + 1e-3 * so[1]


def test_static_linearisation_allocates_nothing(cuda):
    import torch

    tr, ot, K, gt, keep = _tracker(L.TRACK_RGBD)
    out = torch.zeros(46, dtype=torch.float64, device="cuda")
    lv = _level(tr, 0, K)
    pose = L.pose_from(gt)
    L.call("yas_gn_linearise_static", C.byref(lv), C.byref(pose), L.TRACK_RGBD, out.data_ptr(), None)
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(3):
        L.call("yas_gn_linearise_static", C.byref(lv), C.byref(pose), L.TRACK_RGBD, out.data_ptr(), None)
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0


def test_static_linearisation_rejects_oversized_levels(cuda):
    lv = L.GnLevel(1280, 720, 500.0, 500.0, 640.0, 360.0, *([1] * 9))
    code = L.load().yas_gn_linearise_static(C.byref(lv), C.byref(L.pose_from(np.eye(4))), L.TRACK_RGBD, 1, None)
    assert code == 11  # YAS_ERR_CAPACITY: no work is enqueued
