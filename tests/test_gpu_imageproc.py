"""ImageProc's free functions (RGBDFusion/include/ImageProc.h:8-24, kernels
ImageProc.cu:7-286) through the C ABI, against numpy restatements of the
reference kernels on the same device inputs.  Bar: bit-exact, and the pixels
the reference leaves unwritten keep their previous contents."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from tests.helpers import sequence
from yetanotherslam_gb300 import _lib as L
from yetanotherslam_gb300 import synth

pytestmark = pytest.mark.gpu
F = np.float32
SENT = F(7.25)


def _dev(a):
    import torch

    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _ptr(t):
    return t.data_ptr()


@pytest.fixture(scope="module")
def frame(cuda):
    W, H = 160, 120
    rgb, d16, dm, _ = sequence(3, 1, W, H)[0]
    gray = synth.gray_of(rgb).astype(F)
    return W, H, dm.astype(F), gray


def _inv(z):
    return np.where((z > F(0.2)) & (z < F(8.0)), F(1.0) / np.where(z == 0, F(1), z), F(0)).astype(F)


def test_depth_inverse_vertex_normal_maps(frame):
    import torch

    W, H, z, _ = frame
    fx, fy, cx, cy = synth.intrinsics(W, H)
    invfx, invfy = F(1.0 / fx), F(1.0 / fy)
    dz = _dev(z)
    di = torch.full((H, W), float(SENT), dtype=torch.float32, device="cuda")
    L.call("yas_depth_to_inv_depth", _ptr(dz), W, H, W * 4, _ptr(di), W * 4, None)
    inv = _inv(z)
    assert np.array_equal(di.cpu().numpy(), inv)
    # vertex map (cut-off 3 m), untouched xyz where invalid
    dv = torch.full((H, W, 4), float(SENT), dtype=torch.float32, device="cuda")
    L.call("yas_compute_vertex_map", _ptr(di), W, H, W * 4, _ptr(dv), W * 16, invfx, invfy, F(cx), F(cy), F(3.0), None)
    torch.cuda.synchronize()
    with np.errstate(divide="ignore"):
        zz = (F(1.0) / inv).astype(F)
    ok = (inv > 0) & (zz < F(3.0))
    xs, ys = np.meshgrid(np.arange(W, dtype=F), np.arange(H, dtype=F))
    ref = np.full((H, W, 4), SENT, F)
    ref[..., 0] = np.where(ok, zz * (xs - F(cx)) * invfx, SENT)
    ref[..., 1] = np.where(ok, zz * (ys - F(cy)) * invfy, SENT)
    ref[..., 2] = np.where(ok, zz, SENT)
    ref[..., 3] = np.where(ok, F(1), F(-1))
    vm = dv.cpu().numpy()
    assert np.array_equal(vm, ref)
    assert ok.mean() > 0.5
    # normal map
    dn = torch.full((H, W, 4), float(SENT), dtype=torch.float32, device="cuda")
    L.call("yas_compute_normal_map", _ptr(dv), W, H, W * 16, _ptr(dn), W * 16, None)
    nm = dn.cpu().numpy()
    v00, v01, v10 = vm[:-1, :-1], vm[:-1, 1:], vm[1:, :-1]
    good = (v00[..., 3] > 0) & (v01[..., 3] > 0) & (v10[..., 3] > 0)
    a, b = v10[..., :3] - v00[..., :3], v01[..., :3] - v00[..., :3]
    n = np.stack([a[..., 1] * b[..., 2] - a[..., 2] * b[..., 1], a[..., 2] * b[..., 0] - a[..., 0] * b[..., 2],
                  a[..., 0] * b[..., 1] - a[..., 1] * b[..., 0]], -1).astype(F)
    nn = ((n[..., 0] * n[..., 0] + n[..., 1] * n[..., 1]) + n[..., 2] * n[..., 2]).astype(F)
    inv_n = np.where(nn > 0, F(1) / np.sqrt(np.where(nn > 0, nn, F(1))), F(1)).astype(F)
    n = np.where((nn > 0)[..., None], n * inv_n[..., None], n).astype(F)
    exp = np.full((H, W, 4), SENT, F)
    exp[:-1, :-1, :3] = np.where(good[..., None], n, SENT)
    exp[..., 3] = -1.0
    exp[:-1, :-1, 3] = np.where(good, F(1), F(-1))
    assert np.array_equal(nm, exp)
    # VMapToDepth
    dd = torch.full((H, W), float(SENT), dtype=torch.float32, device="cuda")
    L.call("yas_vmap_to_depth", _ptr(dv), W, H, W * 16, _ptr(dd), W * 4, None)
    assert np.array_equal(dd.cpu().numpy(), np.where(vm[..., 3] > 0, vm[..., 2], F(0)))


def test_pyrdown_gradient_and_transformed_points(frame):
    import torch

    W, H, z, gray = frame
    inv = _inv(z)
    di = _dev(inv)
    w2, h2 = W // 2, H // 2
    dp = torch.full((h2, w2), float(SENT), dtype=torch.float32, device="cuda")
    L.call("yas_pyr_down_depth", _ptr(di), W, H, W * 4, _ptr(dp), w2, h2, w2 * 4, None)
    exp = np.full((h2, w2), SENT, F)
    exp[:-1, :-1] = inv[0:2 * (h2 - 1):2, 0:2 * (w2 - 1):2]
    assert np.array_equal(dp.cpu().numpy(), exp)
    # gradients
    dg = _dev(gray)
    gx = torch.full((H, W), float(SENT), dtype=torch.float32, device="cuda")
    gy = torch.full((H, W), float(SENT), dtype=torch.float32, device="cuda")
    L.call("yas_image_gradient", _ptr(dg), W, H, W * 4, _ptr(gx), _ptr(gy), W * 4, None)
    ex, ey = np.zeros((H, W), F), np.zeros((H, W), F)
    ex[1:-1, 1:-1] = (gray[1:-1, 2:] - gray[1:-1, :-2]) * F(0.5)
    ey[1:-1, 1:-1] = (gray[2:, 1:-1] - gray[:-2, 1:-1]) * F(0.5)
    assert np.array_equal(gx.cpu().numpy(), ex) and np.array_equal(gy.cpu().numpy(), ey)
    # TransformReferencePoint: R K^-1 in double, rounded to float; then FP32
    fx, fy, cx, cy = synth.intrinsics(W, H)
    K = np.array([[fx, 0, cx], [0, fy, cy], [0, 0, 1]], np.float64)
    T = np.eye(4)
    c, s = np.cos(0.05), np.sin(0.05)
    T[:3, :3] = [[c, 0, s], [0, 1, 0], [-s, 0, c]]
    T[:3, 3] = [0.02, -0.01, 0.03]
    dv = torch.full((H, W, 4), float(SENT), dtype=torch.float32, device="cuda")
    Kc = (C.c_double * 9)(*K.reshape(-1))
    L.call("yas_transform_reference_point", _ptr(di), W, H, W * 4, _ptr(dv), W * 16, Kc, C.byref(L.pose_from(T)), None)
    Ki = np.array([[1 / fx, 0, -cx / fx], [0, 1 / fy, -cy / fy], [0, 0, 1]])
    RK = np.array([[(T[i, 0] * Ki[0, j] + T[i, 1] * Ki[1, j]) + T[i, 2] * Ki[2, j] for j in range(3)]
                   for i in range(3)]).astype(F)
    t = T[:3, 3].astype(F)
    with np.errstate(divide="ignore"):
        zz = (F(1.0) / inv).astype(F)
    xs, ys = np.meshgrid(np.arange(W, dtype=F), np.arange(H, dtype=F))
    out = np.zeros((H, W, 4), F)
    for i in range(3):
        out[..., i] = ((RK[i, 0] * xs + RK[i, 1] * ys) + RK[i, 2]) * zz + t[i]
    out[..., 3] = 1.0
    out[inv <= 0] = [0, 0, 0, -1]
    assert np.array_equal(dv.cpu().numpy(), out)
