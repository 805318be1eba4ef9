"""Raycast and marching-cubes parity against the oracle on the same TSDF.

The GPU map is exported and imported into the oracle, so both sides read an
identical TSDF ("for a given TSDF").  Reference behaviour:
RGBDFusion/src/RayTraceEngine.cu:58-450, RGBDFusion/src/MeshEngine.cu:43-339.
Bars:
  * z-range tile maps: bit-exact (FP32 canonical projection);
  * raycast at 640x480: hit/miss differs on at most 20 pixels (measured 1-3
    of 307 200); on pixels both hit, |dz| <= 0.01 mm for 99.9 % of them
    (measured 1.9e-6 m) and > 1 mm on at most 20 pixels (measured 3-5).  The
    march is FP32 on the GPU and FP64 in the oracle, and the GPU jumps the
    samples inside unallocated blocks and before the pixel's near bound in one
    move where the oracle steps voxel by voxel, so a ray grazing a silhouette
    may step onto another surface on one side only;
  * marching cubes: multiset of (cube, case index) bit-exact; vertex
    positions within 1e-5 m; normals of triangles larger than 1e-7 m^2
    within 1e-3.
"""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from tests.helpers import rel_poses, sequence
from yetanotherslam_gb300 import rgbdfusion as rf
from yetanotherslam_gb300 import synth

pytestmark = pytest.mark.gpu


def _fused_map(fmt, W=640, H=480, n=5, vs=0.008):
    K = synth.intrinsics(W, H)
    seq = sequence(3, n, W, H)
    poses = rel_poses(seq)
    m = rf.MapStruct(K)
    m.create_config(1 << 20, 1 << 17, vs, 3 * vs, fmt)
    for i in range(n):
        m.Fuse(seq[i][2], poses[i])
    c, s, w = m.export()
    o = oracle.Map(vs, 3 * vs)
    o.import_blocks(c, s, w)
    return K, poses, m, o


@pytest.mark.parametrize("fmt", [rf.VOXEL_F32, rf.VOXEL_F16, rf.VOXEL_S16])
def test_raycast_matches_oracle(cuda, fmt):
    W, H = 640, 480
    K, poses, m, o = _fused_map(fmt)
    rc = rf.RayTraceEngine(W, H, K)
    T = poses[-1].copy()
    T[:3, 3] += np.array([0.01, -0.005, 0.008])
    rc.RayTrace(m, T)
    vg = rc.GetVMap().numpy()
    vo, zn, zf = o.raycast(W, H, K, T)
    gzn, gzf = rc.zrange()
    assert np.array_equal(gzn, zn) and np.array_equal(gzf, zf), "z-range tiles differ"
    hg, ho = vg[..., 3] > 0, vo[..., 3] > 0
    agree = (hg == ho).mean()
    both = hg & ho
    dz = np.abs(vg[..., 2][both] - vo[..., 2][both])
    print(f"raycast fmt {fmt}: hit/miss flips {int((hg != ho).sum())} of {hg.size}, |dz| p99.9 "
          f"{np.quantile(dz, 0.999):.3g} m, > 1 mm {int((dz > 1e-3).sum())}")
    assert hg.mean() > 0.5
    assert (hg != ho).sum() <= 20, f"hit agreement {agree:.6f}"
    assert np.quantile(dz, 0.999) <= 1e-5, f"p99.9 |dz| {np.quantile(dz, 0.999):.3g}"
    assert (dz > 1e-3).sum() <= 20, f"{(dz > 1e-3).sum()} pixels off by > 1 mm"
    # VMapToDepth (GetRayTracingResultDepth)
    d = rc.GetDepth()
    assert np.array_equal(d, np.where(hg, vg[..., 2], 0).astype(np.float32))


def test_raycast_of_empty_map_misses_everywhere(cuda):
    W, H = 64, 48
    K = synth.intrinsics(W, H)
    m = rf.MapStruct(K)
    m.create_config(1 << 12, 1 << 10, 0.01, 0.03, rf.VOXEL_F16)
    rc = rf.RayTraceEngine(W, H, K)
    rc.RayTrace(m, np.eye(4))
    v = rc.GetVMap().numpy()
    assert (v[..., 3] == -1).all()


def test_mc_tables_match_oracle(native):
    import ctypes as C

    edge = np.zeros(256, np.uint16)
    tri = np.zeros((256, 31), np.int8)
    cnt = np.zeros(256, np.uint8)
    native.yas_mc_tables(edge.ctypes.data, tri.ctypes.data, cnt.ctypes.data)
    e2, t2, c2 = oracle.mc_tables()
    assert np.array_equal(edge, e2) and np.array_equal(tri, t2) and np.array_equal(cnt, c2)


def _sorted_soup(pts, nrm, cases, cube):
    key = (cube[:, 0].astype(np.int64) + (1 << 20)) << 42 | (cube[:, 1].astype(np.int64) + (1 << 20)) << 21 | (
        cube[:, 2].astype(np.int64) + (1 << 20))
    order = np.argsort(key, kind="stable")
    return pts[order], nrm[order], cases[order], cube[order]


@pytest.mark.parametrize("fmt", [rf.VOXEL_F32, rf.VOXEL_S24, rf.VOXEL_S16])
def test_marching_cubes_matches_oracle(cuda, fmt):
    K, poses, m, o = _fused_map(fmt, n=3)
    me = rf.MeshEngine(4_000_000)
    pg, ng, cg, xg = me.Meshify(m)
    po, no, co, xo = o.mesh()
    assert me.N == 9 * pg.shape[0]
    assert pg.shape[0] == po.shape[0] > 10000
    pg, ng, cg, xg = _sorted_soup(pg, ng, cg, xg)
    po, no, co, xo = _sorted_soup(po, no, co, xo)
    assert np.array_equal(xg, xo) and np.array_equal(cg, co), "cube/case multisets differ"
    assert np.abs(pg - po).max() <= 1e-5
    # normals: a face normal's error is about the vertex error (FP32 rounding,
    # 1.2e-7 m at metre-scale coordinates) over the triangle's smallest
    # altitude, so the bound is 1e-4 + 5e-7 m / altitude; zero-area triangles
    # carry the zero normal on both sides
    t3 = po.reshape(-1, 3, 3).astype(np.float64)
    area2 = np.linalg.norm(np.cross(t3[:, 1] - t3[:, 0], t3[:, 2] - t3[:, 0]), axis=1)
    longest = np.max(np.stack([np.linalg.norm(t3[:, i] - t3[:, (i + 1) % 3], axis=1) for i in range(3)], 1), 1)
    nz = area2 > 0
    alt = np.where(nz, area2 / np.maximum(longest, 1e-30), 0.0)
    err = np.abs(ng - no).max(axis=1)
    assert (err[nz] <= 1e-4 + 5e-7 / alt[nz]).all(), float(np.max(err[nz] - 5e-7 / alt[nz]))
    assert (alt[nz] > 1e-4).mean() > 0.95  # the bound is tight on nearly all triangles


def test_mesh_overflow_is_reported(cuda):
    K, poses, m, o = _fused_map(rf.VOXEL_F16, W=320, H=240, n=1)
    me = rf.MeshEngine(100)
    pg, ng, cg, xg = me.Meshify(m)
    assert me.overflow and pg.shape[0] == 100
