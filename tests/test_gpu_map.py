"""Parity of the voxel-hash map against the oracle, through the C ABI.

Reference behaviour: RGBDFusion/src/VoxelMap.cu:517-884 (allocation,
visibility, integration).  Bars:
  * allocated block coordinate set and visible set: bit-exact;
  * voxel weights: exact (integers);
  * TSDF (normalised by the truncation distance): F32 and S24 storage within
    1e-5, F16 storage within 1e-3 over these short sequences (weights <= 6),
    all against the FP64 oracle; S16 (the reference's int16 voxel) against
    the oracle keeping the same int16 storage: within three int16 steps
    (1e-4; an average computed in FP32 here and FP64 there can truncate to
    neighbouring steps, and the step then carries into later averages), and
    equal on at least 99 % of the observed voxels.
"""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from tests.helpers import align_blocks, rel_poses, sequence
from yetanotherslam_gb300 import _lib as L
from yetanotherslam_gb300 import rgbdfusion as rf
from yetanotherslam_gb300 import synth

pytestmark = pytest.mark.gpu

TOL = {rf.VOXEL_F32: 1e-5, rf.VOXEL_S24: 1e-5, rf.VOXEL_F16: 1e-3, rf.VOXEL_S16: 1e-4}


def _pair(fmt, K, vs=0.008, slots=1 << 20, blocks=1 << 17):
    m = rf.MapStruct(K)
    m.create_config(slots, blocks, vs, 3 * vs, fmt)
    o = oracle.Map(vs, 3 * vs, int16_sdf=fmt == rf.VOXEL_S16)
    return m, o


@pytest.mark.parametrize("fmt", [rf.VOXEL_F32, rf.VOXEL_F16, rf.VOXEL_S24, rf.VOXEL_S16])
def test_fuse_sequence_matches_oracle(cuda, fmt):
    W, H = 640, 480
    K = synth.intrinsics(W, H)
    seq = sequence(3, 6, W, H)
    poses = rel_poses(seq)
    m, o = _pair(fmt, K)
    for i, (rgb, d16, dm, _) in enumerate(seq):
        m.Fuse(dm, poses[i])
        o.fuse(dm, K, poses[i])
        # visible set of this fusion (MapStruct::visibleTable)
        vg = m.visible_coords()
        vo = o.visible(W, H, K, poses[i])
        assert {tuple(r) for r in vg} == {tuple(r) for r in vo}, f"frame {i}: visible sets differ"
        assert len(vg) == len(vo)
    assert m.take_errors() == 0
    cg, sg, wg = m.export()
    co, so, wo = o.export()
    sg, wg, so, wo = align_blocks(cg, sg, wg, co, so, wo)
    assert np.array_equal(wg, wo), "weights differ"
    obs = wo > 0
    err = np.abs(sg[obs] - so[obs])
    assert obs.sum() > 100000
    assert err.max() <= TOL[fmt], f"max TSDF error {err.max():.3g} (p99.9 {np.quantile(err, 0.999):.3g})"
    if fmt == rf.VOXEL_S16:
        assert (err == 0).mean() >= 0.99, f"equal on {(err == 0).mean():.4f} of the voxels"


def test_s16_word_is_the_reference_voxel(cuda):
    """S16 round trip of chosen values: the sdf comes back as
    (short)(s * 32767) / 32767 with the product in FP32 and truncation toward
    zero (PackFloat / UnPackFloat), the weight capped at 255."""
    rng = np.random.default_rng(5)
    n_blocks = 16
    n = n_blocks * 512
    s = rng.uniform(-1.0, 1.0, n).astype(np.float32)
    s[:8] = [0.0, -0.0, 1.0, -1.0, 1.0 / 32767, -1.0 / 32767, 0.5 / 32767, -1.5 / 32767]
    w = rng.integers(1, 300, n).astype(np.float32)
    coords = np.stack([np.arange(n_blocks), np.ones(n_blocks), np.zeros(n_blocks)], 1).astype(np.int32)
    m = rf.MapStruct(synth.intrinsics(64, 48))
    m.create_config(1 << 12, 1 << 8, 0.008, 0.024, rf.VOXEL_S16)
    m.import_blocks(coords, s.reshape(n_blocks, 512), w.reshape(n_blocks, 512))
    c, sd, wt = m.export()
    order = np.argsort(c[:, 0])
    got_s, got_w = sd[order].reshape(-1), wt[order].reshape(-1)
    q = np.trunc(s * np.float32(32767)).astype(np.int32)
    want = (q.astype(np.float32) / np.float32(32767)).astype(np.float32)
    assert np.array_equal(got_s, want)
    assert np.array_equal(got_w, np.minimum(w, 255))


def test_allocation_only_bit_exact_various_poses(cuda):
    """Allocation from a depth map at poses with arbitrary rotations."""
    W, H = 320, 240
    K = synth.intrinsics(W, H)
    seq = sequence(5, 3, W, H)
    rng = np.random.default_rng(0)
    m, o = _pair(rf.VOXEL_F32, K, vs=0.005)
    for k in range(4):
        a = rng.normal(size=3)
        a = a / np.linalg.norm(a) * rng.uniform(0, np.pi)
        th = np.linalg.norm(a)
        Wx = np.array([[0, -a[2], a[1]], [a[2], 0, -a[0]], [-a[1], a[0], 0]]) / th
        T = np.eye(4)
        T[:3, :3] = np.eye(3) + np.sin(th) * Wx + (1 - np.cos(th)) * Wx @ Wx
        T[:3, 3] = rng.uniform(-3, 3, size=3)
        dm = seq[k % 3][2]
        m.Fuse(dm, T)
        o.fuse(dm, K, T)
    cg, sg, wg = m.export()
    co, so, wo = o.export()
    sg, wg, so, wo = align_blocks(cg, sg, wg, co, so, wo)
    assert np.array_equal(wg, wo)
    assert np.abs(sg - so)[wo > 0].max() <= TOL[rf.VOXEL_F32]


def test_empty_nan_and_out_of_range_depth(cuda):
    W, H = 64, 48
    K = synth.intrinsics(W, H)
    m, o = _pair(rf.VOXEL_F16, K)
    for d in (np.zeros((H, W), np.float32), np.full((H, W), np.nan, np.float32),
              np.full((H, W), 5.0, np.float32), np.full((H, W), 0.05, np.float32)):
        m.Fuse(d, np.eye(4))
        o.fuse(d, K, np.eye(4))
    assert m.num_allocated() == 0 == o.num_blocks
    assert m.Empty()
    assert m.take_errors() == 0


def test_tiny_and_ragged_images(cuda):
    for W, H in [(1, 1), (7, 5), (33, 17)]:
        K = (30.0, 30.0, (W - 1) / 2, (H - 1) / 2)
        d = np.full((H, W), 1.2, np.float32)
        d[::2, ::3] = 0.7
        m, o = _pair(rf.VOXEL_F32, K, vs=0.004)
        m.Fuse(d, np.eye(4))
        o.fuse(d, K, np.eye(4))
        cg, sg, wg = m.export()
        co, so, wo = o.export()
        sg, wg, so, wo = align_blocks(cg, sg, wg, co, so, wo)
        assert np.array_equal(wg, wo)


def test_device_and_host_inputs_agree(cuda):
    import torch

    W, H = 320, 240
    K = synth.intrinsics(W, H)
    dm = sequence(3, 1, W, H)[0][2]
    a, _ = _pair(rf.VOXEL_F16, K)
    b, _ = _pair(rf.VOXEL_F16, K)
    a.Fuse(dm, np.eye(4))
    b.Fuse(torch.from_numpy(dm).cuda(), np.eye(4))
    torch.cuda.synchronize()
    ca, sa, wa = a.export()
    cb, sb, wb = b.export()
    sa, wa, sb, wb = align_blocks(ca, sa, wa, cb, sb, wb)
    assert np.array_equal(sa, sb) and np.array_equal(wa, wb)


def test_pool_exhaustion_reports_error(cuda):
    W, H = 320, 240
    K = synth.intrinsics(W, H)
    dm = sequence(3, 1, W, H)[0][2]
    m = rf.MapStruct(K)
    m.create_config(1 << 16, 64, 0.008, 0.024, rf.VOXEL_F16)
    m.Fuse(dm, np.eye(4))
    assert m.num_allocated() == 64
    bits = m.take_errors()
    assert bits & (1 << 5), "POOL_FULL not reported"
    assert m.take_errors() == 0  # cleared on read


def test_table_full_reports_error(cuda):
    W, H = 320, 240
    K = synth.intrinsics(W, H)
    dm = sequence(3, 1, W, H)[0][2]
    m = rf.MapStruct(K)
    m.create_config(64, 1 << 14, 0.008, 0.024, rf.VOXEL_F16)
    m.Fuse(dm, np.eye(4))
    assert m.num_allocated() == 64
    assert m.take_errors() & (1 << 4), "TABLE_FULL not reported"


def test_export_import_and_hibernate_roundtrip(cuda):
    W, H = 320, 240
    K = synth.intrinsics(W, H)
    seq = sequence(3, 2, W, H)
    poses = rel_poses(seq)
    m, _ = _pair(rf.VOXEL_S24, K)
    for i in range(2):
        m.Fuse(seq[i][2], poses[i])
    c0, s0, w0 = m.export()
    m.Hibernate()
    assert m.mbInHibernation
    m.ReActivate()
    c1, s1, w1 = m.export()
    assert np.array_equal(c0, c1) and np.array_equal(s0, s1) and np.array_equal(w0, w1)
    n = rf.MapStruct(K)
    n.create_config(1 << 16, 1 << 15, 0.008, 0.024, rf.VOXEL_S24)
    n.import_blocks(c0, s0, w0)
    c2, s2, w2 = n.export()
    s0a, w0a, s2a, w2a = align_blocks(c0, s0, w0, c2, s2, w2)
    assert np.array_equal(s0a, s2a) and np.array_equal(w0a, w2a)
    # fusing continues identically after a hibernate/reactivate cycle
    m.Fuse(seq[1][2], poses[1])
    n.Fuse(seq[1][2], poses[1])
    ca, sa, wa = m.export()
    cb, sb, wb = n.export()
    sa, wa, sb, wb = align_blocks(ca, sa, wa, cb, sb, wb)
    assert np.array_equal(sa, sb) and np.array_equal(wa, wb)


def _f16_word_model(s, w):
    """The FP16 voxel word as numpy computes it: the half (round to nearest
    even), a residual q of 1/256 of the half's ulp added to the half's FP32 bit
    pattern (q = 0 for a zero half; q = 128 at a normal half becomes -128 at the
    next half up in magnitude, 2^13 bit units further), the weight capped at 255."""
    s = s.astype(np.float32)
    h = s.astype(np.float16).astype(np.float32)
    hb = h.view(np.int32).astype(np.int64)
    d = (s.view(np.int32) & 0x7FFFFFFF).astype(np.int64) - (hb & 0x7FFFFFFF)
    q = (d + 16) >> 5
    up = (q > 127) & (np.abs(h) >= 2.0 ** -14)
    hb[up] += 8192
    q[up] -= 256
    q = np.clip(q, -128, 127)
    q[h == 0] = 0
    v = (hb + 32 * q).astype(np.int32).view(np.float32)
    return v, np.minimum(w, 255).astype(np.float32)


def test_f16_word_keeps_18_mantissa_bits(cuda):
    """FP16 storage round trip (import, export) of chosen values: bit-exact
    against the word's numpy model; within 2^-19 relative where the half is
    normal (|s| >= 2^-14: s rounded to 18 mantissa bits) and 2^-25 absolute
    below; signs and zeros kept."""
    rng = np.random.default_rng(77)
    n_blocks = 64
    n = n_blocks * 512
    s = rng.uniform(-1.0, 1.0, n).astype(np.float32)
    k = n // 8
    s[:k] = (rng.uniform(-1, 1, k) * 10.0 ** rng.uniform(-9, -4, k)).astype(np.float32)  # half subnormals
    e = rng.integers(-14, 1, k)  # next to powers of two, both sides
    s[k:2 * k] = (np.ldexp(1.0, e) * (1.0 + rng.uniform(-2e-3, 2e-3, k)) * rng.choice([-1, 1], k)).astype(np.float32)
    s[2 * k:2 * k + 6] = [0.0, -0.0, 1.0, -1.0, 2.0 ** -14, -(2.0 ** -24)]
    w = rng.integers(1, 300, n).astype(np.float32)
    coords = np.stack([np.arange(n_blocks), np.zeros(n_blocks), np.zeros(n_blocks)], 1).astype(np.int32)
    m = rf.MapStruct(synth.intrinsics(64, 48))
    m.create_config(1 << 12, 1 << 8, 0.008, 0.024, rf.VOXEL_F16)
    m.import_blocks(coords, s.reshape(n_blocks, 512), w.reshape(n_blocks, 512))
    c, sd, wt = m.export()
    order = np.argsort(c[:, 0])
    got_s, got_w = sd[order].reshape(-1), wt[order].reshape(-1)
    want_s, want_w = _f16_word_model(s, w)
    assert np.array_equal(got_s.view(np.int32), want_s.view(np.int32))
    assert np.array_equal(got_w, want_w)
    normal = np.abs(s) >= 2.0 ** -14
    err = np.abs(got_s.astype(np.float64) - s)
    assert np.all(err[normal] <= 2.0 ** -19 * np.abs(s[normal]))
    assert err[~normal].max() <= 2.0 ** -25
    assert np.all(np.signbit(got_s) == np.signbit(s))


def test_reset_clears_map(cuda):
    W, H = 160, 120
    K = synth.intrinsics(W, H)
    dm = sequence(3, 1, W, H)[0][2]
    m, _ = _pair(rf.VOXEL_F32, K)
    m.Fuse(dm, np.eye(4))
    assert m.num_allocated() > 0
    m.Reset()
    assert m.num_allocated() == 0 and m.Empty()
    m.Fuse(dm, np.eye(4))
    o = oracle.Map(0.008, 0.024)
    o.fuse(dm, K, np.eye(4))
    assert m.num_allocated() == o.num_blocks


@pytest.mark.parametrize("fmt", [rf.VOXEL_F32, rf.VOXEL_F16, rf.VOXEL_S16])
def test_submap_file_roundtrip(cuda, fmt, tmp_path):
    """SaveToFile / ReadFromFile: the round trip is bit-exact, the loaded map
    (grown from a small capacity) fuses on exactly as the original, a format
    mismatch is refused and a missing file reports YAS_ERR_IO."""
    W, H = 320, 240
    K = synth.intrinsics(W, H)
    seq = sequence(3, 4, W, H)
    poses = rel_poses(seq)
    a, _ = _pair(fmt, K)
    for i in range(3):
        a.Fuse(seq[i][2], poses[i])
    T = np.eye(4)
    T[:3, 3] = [0.1, -0.2, 0.3]
    a.SetPose(T)
    path = tmp_path / "submap.yas"
    a.SaveToFile(path)
    b = rf.MapStruct(K)
    b.create_config(1 << 10, 64, 0.008, 0.024, fmt)
    b.ReadFromFile(path)
    for x, y in zip(a.export(), b.export()):
        assert np.array_equal(x, y)
    assert np.array_equal(b.GetPose(), a.GetPose())
    a.Fuse(seq[3][2], poses[3])
    b.Fuse(seq[3][2], poses[3])
    ca, sa, wa = a.export()
    cb, sb, wb = b.export()
    sa, wa, sb, wb = align_blocks(ca, sa, wa, cb, sb, wb)
    assert np.array_equal(sa, sb) and np.array_equal(wa, wb)
    other = rf.MapStruct(K)
    other.create_config(1 << 14, 1 << 12, 0.008, 0.024, rf.VOXEL_S24)
    with pytest.raises(L.YasError) as e:
        other.ReadFromFile(path)
    assert e.value.code == 1
    with pytest.raises(L.YasError) as e:
        b.ReadFromFile(tmp_path / "missing.yas")
    assert e.value.code == 13
    before = b.export()
    raw = path.read_bytes()
    (tmp_path / "short.yas").write_bytes(raw[:-7])
    with pytest.raises(L.YasError) as e:
        b.ReadFromFile(tmp_path / "short.yas")
    assert e.value.code == 13
    # a header whose block count does not match the file's length
    bad = bytearray(raw)
    bad[44:48] = (0xFFFFFFF0).to_bytes(4, "little")
    (tmp_path / "big.yas").write_bytes(bytes(bad))
    with pytest.raises(L.YasError) as e:
        b.ReadFromFile(tmp_path / "big.yas")
    assert e.value.code == 13
    # the refused loads left b as it was
    for x, y in zip(b.export(), before):
        assert np.array_equal(x, y)
