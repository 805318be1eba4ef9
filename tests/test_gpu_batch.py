"""Batched keyframe submaps (yas_batch_*): many sessions of uneven resolution,
voxel size and length stepped as one graph with one batched GN launch.

Bars:
  * every session's poses within 5e-5 m / rad of the same session run alone
    through yas_session_process_frame (the batched GN partitions the pixels
    over fewer CTAs, so the summation order differs, and tracking through the
    map carries the difference from frame to frame).  Sessions against the
    oracle are held to the session bars in test_gpu_session.py; on some frames
    of some sequences FP32 residuals flip GetTransform's keep-the-better-
    estimate decision against the FP64 oracle, as the oracle's own FP32 build
    does (tests/precision_study.py), so that check is not repeated here on
    other seeds;
  * with a fixed GN share, a session's results are bit-identical alone in a
    batch and in the mix; they never depend on the march and integration
    launch shapes;
  * the autotuner returns one of its candidate shapes, leaves the batch's
    sessions untouched, and the tuned batch gives the results of a fresh batch
    with that tuning.
"""
from __future__ import annotations

import numpy as np
import pytest

from tests.helpers import pose_error, sequence
from yetanotherslam_gb300 import _lib as L
from yetanotherslam_gb300 import batching
from yetanotherslam_gb300 import rgbdfusion as rf
from yetanotherslam_gb300 import synth

pytestmark = pytest.mark.gpu

# (width, height, voxel, frames, seed): an uneven mix
MIX = [(320, 240, 0.008, 6, 3), (480, 360, 0.005, 4, 5), (640, 480, 0.005, 7, 7), (320, 240, 0.005, 3, 9)]


def _sessions(mix):
    return [rf.Session(w, h, synth.intrinsics(w, h), hash_slots=1 << 20, max_blocks=1 << 17, voxel_size=vs)
            for w, h, vs, _, _ in mix]


def _run_batch(mix, tuning=None):
    ss = _sessions(mix)
    b = batching.Batch(ss)
    if tuning is not None:
        b.tuning = tuning
    seqs = [sequence(seed, n, w, h) for w, h, _, n, seed in mix]
    poses = [[] for _ in mix]
    for f in range(max(m[3] for m in mix)):
        frames = [(q[f][0], q[f][1]) if f < len(q) else None for q in seqs]
        b.step(frames)
        P, st, ms = b.wait()
        assert ms > 0
        for i, fr in enumerate(frames):
            if fr is None:
                assert st[i] == -1 and np.isnan(P[i][:3]).all()
            else:
                assert st[i] == 0, (f, i, st[i])
                poses[i].append(P[i])
    return b, ss, poses


def test_batch_matches_sessions_run_alone(cuda):
    b, ss, poses = _run_batch(MIX)
    assert b.kernels_per_step() > 0
    for i, (w, h, vs, n, seed) in enumerate(MIX):
        alone = rf.Session(w, h, synth.intrinsics(w, h), hash_slots=1 << 20, max_blocks=1 << 17, voxel_size=vs)
        for f, (rgb, d16, _, _) in enumerate(sequence(seed, n, w, h)):
            st, T = alone.process(rgb, d16)
            assert st == 0
            dt, dr = pose_error(T, poses[i][f])
            assert dt <= 5e-5 and dr <= 5e-5, (i, f, dt, dr)


@pytest.mark.parametrize("per_session", [0, 1])
def test_session_result_is_the_same_alone_and_in_the_mix(cuda, per_session):
    # with a fixed GN share per resolution (the proportional default splits the
    # GPU by the step's mix, so it fixes the summation order per mix instead);
    # one GN launch per step or one per session give the same results
    fixed = batching.default_tuning()
    fixed.gn_pixels_per_cta = 32768
    fixed.gn_per_session = per_session
    _, _, mixed = _run_batch(MIX, fixed)
    for i in (0, 2):
        _, _, alone = _run_batch([MIX[i]], fixed)
        for A, B in zip(mixed[i], alone[0]):
            assert np.array_equal(A, B)
    if per_session:
        other = batching.default_tuning()
        other.gn_pixels_per_cta = 32768
        other.gn_per_session = 0
        _, _, one_launch = _run_batch(MIX, other)
        for i in range(len(MIX)):
            for A, B in zip(mixed[i], one_launch[i]):
                assert np.array_equal(A, B)


def test_launch_shapes_do_not_change_results(cuda):
    ta = batching.default_tuning()
    ta.march_warps_x, ta.integrate_ctas = 0, 152 * 4
    tb = batching.default_tuning()
    tb.march_warps_x, tb.integrate_ctas = 4, 152 * 16
    _, sa, pa = _run_batch(MIX[:3], ta)
    _, sb, pb = _run_batch(MIX[:3], tb)
    for i in range(3):
        for A, B in zip(pa[i], pb[i]):
            assert np.array_equal(A, B)
        ca, xa, wa = sa[i].map().export()
        cb, xb, wb = sb[i].map().export()
        ka, kb = np.lexsort(ca.T), np.lexsort(cb.T)
        assert np.array_equal(ca[ka], cb[kb]) and np.array_equal(xa[ka], xb[kb]) and np.array_equal(wa[ka], wb[kb])


def test_autotune_picks_a_candidate_and_leaves_sessions_untouched(cuda):
    mix = MIX[:3]
    ss = _sessions(mix)
    b = batching.Batch(ss)
    calib = []
    for w, h, vs, n, seed in mix:
        q = sequence(seed, 4, w, h)
        calib.append((np.stack([x[0] for x in q]), np.stack([x[1] for x in q])))
    t = b.autotune(calib)
    assert t.gn_pixels_per_cta in (0, 16384, 32768, 65536)
    assert t.march_warps_x in (0, 1, 2, 4)
    assert t.integrate_ctas in (152 * 4, 152 * 8, 152 * 16)
    assert t.gn_per_session in (0, 1)
    got = b.tuning
    assert (got.gn_pixels_per_cta, got.march_warps_x, got.integrate_ctas, got.gn_per_session) == (
        t.gn_pixels_per_cta, t.march_warps_x, t.integrate_ctas, t.gn_per_session)
    for s in ss:
        assert s.map().Empty()
    # the tuned batch steps as a fresh batch with that tuning
    seqs = [sequence(seed, n, w, h) for w, h, _, n, seed in mix]
    _, _, ref = _run_batch(mix, t)
    for f in range(3):
        b.step([(q[f][0], q[f][1]) for q in seqs])
        P, st, _ = b.wait()
        for i in range(3):
            assert st[i] == 0 and np.array_equal(P[i], ref[i][f])


def test_hibernated_session_is_refused(cuda):
    ss = _sessions(MIX[:2])
    b = batching.Batch(ss)
    seqs = [sequence(seed, 2, w, h) for w, h, _, _, seed in MIX[:2]]
    b.step([(q[0][0], q[0][1]) for q in seqs])
    b.wait()
    ss[1].map().Hibernate()
    with pytest.raises(L.YasError) as e:
        b.step([(q[1][0], q[1][1]) for q in seqs])
    assert e.value.code == 9
    ss[1].map().ReActivate()
    b.step([(q[1][0], q[1][1]) for q in seqs])
    _, st, _ = b.wait()
    assert (st == 0).all()
