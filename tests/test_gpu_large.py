"""The large-map pieces (multi-room loop sequence, de-/re-integration after a
pose correction, full-map marching cubes) on sizes the oracle finishes in
seconds.  The full 2000-frame 1280x720 / 4 mm run is bench.py --large.

Bars:
  * de-integrating frames last-in-first-out at the poses they were fused with
    gives back the map as it was before them: weights exact, TSDF within 1e-4
    of the truncation (undoing a running average multiplies the error already
    there by w / (w - 1) per removed frame, a product of the weight ratio, on
    top of the division's 2-ulp rounding), blocks allocated since then left
    empty; removing every
    frame leaves every weight at 0 (no voxel reached the weight cap).  (Blocks
    are never freed, so in any other order a frame's removal also reaches
    blocks allocated after it; those voxels it never observed have weight 0
    once the later frames are gone, and weight-0 voxels are skipped.)
  * de-/re-integration at corrected poses against the oracle doing the same:
    block set bit-exact, weights exact, TSDF within 1e-5 (F32 storage);
  * full-map marching cubes of the re-integrated map against the oracle's on
    the same TSDF: cube / case multisets bit-exact, vertices within 1e-5 m;
  * the 1280x720 tracker runs its whole schedule fused (residuals through
    global memory) and agrees with the per-iteration launches within the
    per-frame pose bar, 1e-4 (the two sum 0.9 M pixels in different orders).
"""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from tests.helpers import align_blocks, key_rows, pose_error
from yetanotherslam_gb300 import rgbdfusion as rf
from yetanotherslam_gb300 import synth

pytestmark = pytest.mark.gpu


def _rooms_frames(n, w, h, seed=5):
    sc = synth.Scene.rooms(seed=seed, loop_frames=2000)
    return [sc.render(i, w, h) for i in range(n)]


def _depth_m(d16):
    return d16.astype(np.float32) * np.float32(0.001)


def _correction(i, n):
    """A seeded correction spread along the trajectory (as a loop closure would)."""
    rng = np.random.default_rng(1800)
    xi = np.concatenate([rng.normal(0, 0.01, 3), rng.normal(0, np.radians(0.3), 3)]) * min(1.0, i / max(n - 1, 1))
    return oracle.se3_exp(xi)


def test_deintegration_last_in_first_out_is_exact(cuda):
    W, H, n, half = 320, 180, 40, 24
    K = synth.intrinsics(W, H)
    frames = _rooms_frames(n, W, H)
    s = rf.Session(W, H, K, hash_slots=1 << 20, max_blocks=1 << 17, voxel_size=0.004, voxel_format=rf.VOXEL_F32)
    poses, snap = [], None
    for i, f in enumerate(frames):
        st, T = s.process(f.rgb, f.depth)
        assert st == 0
        poses.append(T)
        if i == half - 1:
            snap = s.map().export()
    m = s.map()
    _, _, wn = m.export()
    assert wn.max() < 255 and snap[0].shape[0] > 100
    for i in range(n - 1, half - 1, -1):
        m.Defuse(_depth_m(frames[i].depth), poses[i])
    c, sd, w = m.export()
    k_snap, k_now = key_rows(snap[0]), key_rows(c)
    assert k_now.shape[0] > k_snap.shape[0]
    old = np.isin(k_now, k_snap)
    assert not w[~old].any()
    sa, wa, sb, wb = align_blocks(c[old], sd[old], w[old], *snap)
    assert np.array_equal(wa, wb)
    obs = wb > 0
    assert obs.sum() > 10000 and np.abs(sa[obs] - sb[obs]).max() <= 1e-4
    for i in range(half - 1, -1, -1):
        m.Defuse(_depth_m(frames[i].depth), poses[i])
    assert not m.export()[2].any()


def test_reintegration_at_corrected_poses_matches_oracle(cuda):
    W, H, n, vs = 160, 90, 12, 0.005
    K = synth.intrinsics(W, H)
    frames = _rooms_frames(n, W, H, seed=9)
    poses = [np.linalg.inv(frames[0].Twc) @ f.Twc for f in frames]
    fixed = [_correction(i, n) @ T for i, T in enumerate(poses)]
    m = rf.MapStruct(K)
    m.create_config(1 << 18, 1 << 15, vs, 3 * vs, rf.VOXEL_F32)
    o = oracle.Map(vs, 3 * vs)
    for f, T in zip(frames, poses):
        m.Fuse(_depth_m(f.depth), T)
        o.fuse(_depth_m(f.depth), K, T)
    for f, T, T2 in zip(frames, poses, fixed):
        m.Defuse(_depth_m(f.depth), T)
        m.Fuse(_depth_m(f.depth), T2)
        o.defuse(_depth_m(f.depth), K, T)
        o.fuse(_depth_m(f.depth), K, T2)
    cg, sg, wg = m.export()
    co, so, wo = o.export()
    sg, wg, so, wo = align_blocks(cg, sg, wg, co, so, wo)
    assert np.array_equal(wg, wo)
    obs = wo > 0
    assert obs.sum() > 10000 and np.abs(sg[obs] - so[obs]).max() <= 1e-5
    # full-map marching cubes on the same TSDF
    me = rf.MeshEngine(4_000_000)
    pg, _, kg, xg = me.Meshify(m)
    o2 = oracle.Map(vs, 3 * vs)
    c, sd, wt = m.export()
    o2.import_blocks(c, sd, wt)
    po, _, ko, xo = o2.mesh()

    def order(x, k):
        key = ((x[:, 0].astype(np.int64) + (1 << 20)) << 42) | ((x[:, 1].astype(np.int64) + (1 << 20)) << 21) | (
            x[:, 2].astype(np.int64) + (1 << 20))
        return np.lexsort((k, key))

    ig, io = order(xg, kg), order(xo, ko)
    assert pg.shape[0] == po.shape[0] > 1000
    assert np.array_equal(xg[ig], xo[io]) and np.array_equal(kg[ig], ko[io])
    assert np.abs(pg[ig] - po[io]).max() <= 1e-5


def test_hd_tracker_runs_fused_and_agrees_with_per_iteration(cuda):
    W, H, n = 1280, 720, 4
    K = synth.intrinsics(W, H)
    frames = _rooms_frames(n, W, H, seed=3)
    sa = rf.Session(W, H, K, hash_slots=1 << 21, max_blocks=1 << 18, voxel_size=0.004, fused_schedule=True)
    sb = rf.Session(W, H, K, hash_slots=1 << 21, max_blocks=1 << 18, voxel_size=0.004, fused_schedule=False)
    for f in frames:
        st_a, A = sa.process(f.rgb, f.depth)
        st_b, B = sb.process(f.rgb, f.depth)
        assert st_a == 0 and st_b == 0
        dt, dr = pose_error(A, B)
        assert dt <= 1e-4 and dr <= 1e-4, (dt, dr)
    assert sa.kernels_per_frame() < sb.kernels_per_frame() - 20
