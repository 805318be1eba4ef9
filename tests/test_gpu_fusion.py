"""Submap fusion, capacity growth and de-integration against the oracle.

Reference behaviour: RGBDFusion/src/VoxelMap.cu:173-199 (Swap), 213-444
(CreateBlockFunctor, MapStructFusionFunctor, Fuse(MapStruct*)), 446-515
(Reserve).  Bars:
  * block coordinate set after fusion: bit-exact (FP32 canonical allocation);
  * weights: exact; TSDF within 1e-5 of the truncation (F32 storage); with
    the reference's int16 storage (S16, the oracle keeping the same storage)
    within four int16 steps: each source map within two, plus one truncation
    of the blend;
  * reserve keeps every block's contents bit for bit;
  * de-integrating a frame matches the oracle's de-integration (weights exact,
    TSDF within 1e-5) and, on the blocks that existed when the frame was
    fused, gives back the map without that frame.
"""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from tests.helpers import align_blocks, sequence
from yetanotherslam_gb300 import rgbdfusion as rf
from yetanotherslam_gb300 import synth

pytestmark = pytest.mark.gpu

VS = 0.008


def _maps(K, slots=1 << 18, blocks=1 << 15, fmt=rf.VOXEL_F32):
    m = rf.MapStruct(K)
    m.create_config(slots, blocks, VS, 3 * VS, fmt)
    return m, oracle.Map(VS, 3 * VS, int16_sdf=fmt == rf.VOXEL_S16)


def _build(seq, frames, K, T_map, slots=1 << 18, blocks=1 << 15, fmt=rf.VOXEL_F32):
    """Submap with pose T_map (world), fused from `frames` of `seq`."""
    m, o = _maps(K, slots, blocks, fmt)
    m.SetPose(T_map)
    Tinv = np.linalg.inv(T_map)
    for i in frames:
        _, _, dm, Twc = seq[i]
        m.Fuse(dm, Tinv @ Twc)
        o.fuse(dm, K, Tinv @ Twc)
    return m, o


def _compare(m, o, tol=1e-5):
    cg, sg, wg = m.export()
    co, so, wo = o.export()
    sg, wg, so, wo = align_blocks(cg, sg, wg, co, so, wo)
    assert np.array_equal(wg, wo), "weights differ"
    obs = wo > 0
    assert np.abs(sg[obs] - so[obs]).max() <= tol
    return cg.shape[0]


@pytest.mark.parametrize("fmt", [rf.VOXEL_F32, rf.VOXEL_S16])
def test_fuse_map_matches_oracle(cuda, fmt):
    W, H = 320, 240
    K = synth.intrinsics(W, H)
    seq = sequence(21, 8, W, H)
    TA, TB = seq[0][3], seq[4][3]
    ma, oa = _build(seq, range(0, 4), K, TA, fmt=fmt)
    mb, ob = _build(seq, range(4, 8), K, TB, fmt=fmt)
    ma.FuseMap(mb)
    assert not oa.fuse_map(ob, TA, TB)
    n = _compare(ma, oa, tol=1e-5 if fmt == rf.VOXEL_F32 else 4.0 / 32767)
    assert n > 0 and mb.Empty()


def test_fuse_into_empty_map_takes_source(cuda):
    W, H = 160, 120
    K = synth.intrinsics(W, H)
    seq = sequence(22, 3, W, H)
    TB = seq[0][3]
    mb, _ = _build(seq, range(3), K, TB)
    ref = mb.export()
    ma, _ = _maps(K)
    ma.FuseMap(mb)
    got = ma.export()
    for a, b in zip(ref, got):
        assert np.array_equal(a, b)
    assert np.allclose(ma.GetPose(), TB) and mb.Empty()


def test_fuse_map_grows_a_small_destination(cuda):
    W, H = 320, 240
    K = synth.intrinsics(W, H)
    seq = sequence(23, 6, W, H)
    TA, TB = seq[0][3], seq[3][3]
    big, oa = _build(seq, range(0, 3), K, TA)
    c, sd, wt = big.export()
    ma = rf.MapStruct(K)  # a pool with room for A's blocks only
    ma.create_config(1 << 14, c.shape[0] + 64, VS, 3 * VS, rf.VOXEL_F32)
    ma.import_blocks(c, sd, wt)
    ma.SetPose(TA)
    mb, ob = _build(seq, range(3, 6), K, TB)
    ma.FuseMap(mb)  # more blocks than the destination's pool: grown and rehashed
    oa.fuse_map(ob, TA, TB)
    _compare(ma, oa)
    assert ma.take_errors() == 0


def test_reserve_keeps_contents(cuda):
    W, H = 320, 240
    K = synth.intrinsics(W, H)
    seq = sequence(24, 4, W, H)
    m, o = _build(seq, range(2), K, np.eye(4))
    before = m.export()
    m.Reserve(1 << 19, 1 << 16)
    after = m.export()
    for a, b in zip(before, after):
        assert np.array_equal(a, b)
    for i in (2, 3):  # the grown map keeps working
        _, _, dm, Twc = seq[i]
        m.Fuse(dm, Twc)
        o.fuse(dm, K, Twc)
    _compare(m, o)


def test_defuse_matches_oracle_and_undoes_a_frame(cuda):
    W, H = 320, 240
    K = synth.intrinsics(W, H)
    seq = sequence(25, 3, W, H)
    m, o = _build(seq, range(3), K, np.eye(4))
    _, _, dm, Twc = seq[1]
    m.Defuse(dm, Twc)
    o.defuse(dm, K, Twc)
    _compare(m, o)
    # On the blocks that frame 0 allocated (present when frame 1 was fused),
    # removing frame 1 gives the map fused from frames 0 and 2 alone.  Blocks
    # allocated later lose an observation they never had: de-integration is
    # exact only where the frame was fused.
    first, _ = _build(seq, [0], K, np.eye(4))
    b0 = {tuple(c) for c in first.export()[0]}
    ref, _ = _build(seq, [0, 2], K, np.eye(4))
    cg, sg, wg = m.export()
    cr, sr, wr = ref.export()
    at = {tuple(c): i for i, c in enumerate(cg)}
    checked = 0
    for j, c in enumerate(cr):
        if tuple(c) not in b0:
            continue
        i = at[tuple(c)]
        assert np.array_equal(wg[i], wr[j])
        obs = wr[j] > 0
        if obs.any():
            assert np.abs(sg[i][obs] - sr[j][obs]).max() <= 1e-5
        checked += 1
    assert checked == len(b0)


def test_swap_exchanges_storage_not_pose(cuda):
    """MapStruct::Swap (VoxelMap.cu:173-199): storage, grid and intrinsics
    change hands; each handle keeps its pose and active flag."""
    W, H = 160, 120
    K = synth.intrinsics(W, H)
    seq = sequence(5, 3, W, H)
    TA = np.eye(4)
    TB = np.eye(4)
    TB[:3, 3] = [0.5, 0.0, -0.25]
    a, _ = _build(seq, [0, 1], K, TA)
    b = rf.MapStruct(K)
    b.create_config(1 << 16, 1 << 14, 0.01, 0.03, rf.VOXEL_F16)
    b.SetPose(TB)
    b.SetActiveFlag(False)
    ea = a.export()
    a.Swap(b)
    assert a.Empty() and not b.Empty()
    for x, y in zip(b.export(), ea):
        assert np.array_equal(x, y)
    assert np.array_equal(a.GetPose(), TA) and np.array_equal(b.GetPose(), TB)
    assert a.isActive() and not b.isActive()
    # the grid moved with the storage: a now fuses as a 10 mm F16 map
    _, _, dm, Twc = seq[2]
    a.Fuse(dm, Twc)
    c, _, _ = a.export()
    ref = rf.MapStruct(K)
    ref.create_config(1 << 16, 1 << 14, 0.01, 0.03, rf.VOXEL_F16)
    ref.Fuse(dm, Twc)
    rc, _, _ = ref.export()
    assert a.take_errors() == 0 and ref.take_errors() == 0
    assert set(map(tuple, c.tolist())) == set(map(tuple, rc.tolist()))
