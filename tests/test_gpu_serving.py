"""Served sessions (yas_server_*): continuous batching of many sessions' frames.

Bars:
  * a session's poses are bit-identical alone in the server and in a mix with
    other sessions of other resolutions (its work does not depend on its
    batch: fixed CTA share, own rows, own state), with a GN launch per session
    (the default) and with waiting sessions gathered into one batched launch;
  * served poses agree with the same sequence run through a standalone
    session within 1e-5 m / rad (same arithmetic per pixel, another fold
    order of the partial sums);
  * a session whose device footprint does not fit the free HBM minus the
    reserve is not admitted (YAS_ERR_OOM).
"""
from __future__ import annotations

import threading

import numpy as np
import pytest

from tests.helpers import pose_error, sequence
from yetanotherslam_gb300 import _lib as L
from yetanotherslam_gb300 import rgbdfusion as rf
from yetanotherslam_gb300 import serving, synth

pytestmark = pytest.mark.gpu

MAP = dict(hash_slots=1 << 18, max_blocks=1 << 15, voxel_size=0.008, voxel_format=rf.VOXEL_F16)


def _serve_alone(seq, W, H, gn_per_session=None):
    srv = serving.Server(hbm_reserve_bytes=1 << 30, gn_per_session=gn_per_session)
    sid = srv.open(W, H, synth.intrinsics(W, H), **MAP)
    poses = []
    for rgb, d16, _, _ in seq:
        assert srv.submit(sid, rgb, d16) == 0
        srv.drain()
        (r,) = srv.poll()
        assert r["status"] == 0 and r["session"] == sid
        poses.append(r["Tcm"])
    srv.close()
    return poses


@pytest.mark.parametrize("per_session", [True, False])
def test_served_sessions_same_alone_and_in_mix(cuda, per_session):
    """Eight sessions of three resolutions submit concurrently (their frames
    overlap on the device; gathered, batches of several sessions form and GN
    dispatch is deferred while one runs); every session's poses equal, bit for
    bit, its poses served alone."""
    n = 8
    specs = [(320, 240, 3), (160, 120, 5), (320, 240, 7), (640, 480, 9),
             (160, 120, 11), (640, 480, 13), (320, 240, 15), (160, 120, 17)]
    seqs = [sequence(seed, n, w, h) for w, h, seed in specs]
    alone = [_serve_alone(seq, w, h, per_session) for (w, h, _), seq in zip(specs, seqs)]

    srv = serving.Server(hbm_reserve_bytes=1 << 30, gn_per_session=per_session)
    sids = [srv.open(w, h, synth.intrinsics(w, h), **MAP) for w, h, _ in specs]

    def feed(s, frames):
        for rgb, d16, _, _ in frames:
            while srv.submit(s, rgb, d16) != 0:  # ring full: retry
                threading.Event().wait(0.0005)

    threads = [threading.Thread(target=feed, args=(sid, seq)) for sid, seq in zip(sids, seqs)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    srv.drain()
    results: dict[int, list] = {}
    for r in srv.poll(1024):
        results.setdefault(r["session"], []).append(r)
    st = srv.stats()
    srv.close()
    for sid, ref in zip(sids, alone):
        mine = sorted(results[sid], key=lambda r: r["frame"])
        assert [r["frame"] for r in mine] == list(range(n))
        for r, T in zip(mine, ref):
            assert r["status"] == 0
            assert np.array_equal(r["Tcm"], T), (sid, r["frame"])
    assert st["frames"] == len(specs) * n and st["p99_ms"] > 0.0


def test_per_session_gn_admission_beyond_co_resident_ctas(cuda):
    """Ten 640x480 sessions at once: their GN shares (16 CTAs each, 160 in all)
    exceed the 152 co-resident CTAs, so some frames' GN launches wait for
    others' to finish.  Every session's poses still equal, bit for bit, its
    poses served alone."""
    n, W, H = 4, 640, 480
    seeds = list(range(21, 31))
    seqs = [sequence(seed, n, W, H) for seed in seeds]
    alone = [_serve_alone(seq, W, H, True) for seq in seqs[:3]]
    srv = serving.Server(hbm_reserve_bytes=1 << 30, gn_per_session=True)
    sids = [srv.open(W, H, synth.intrinsics(W, H), **MAP) for _ in seeds]
    for k in range(n):
        for sid, seq in zip(sids, seqs):
            rgb, d16, _, _ = seq[k]
            while srv.submit(sid, rgb, d16) != 0:
                threading.Event().wait(0.0005)
    srv.drain()
    results: dict[int, list] = {}
    for r in srv.poll(1024):
        results.setdefault(r["session"], []).append(r)
    srv.close()
    assert all(r["status"] == 0 for rs in results.values() for r in rs)
    for sid, ref in zip(sids[:3], alone):
        mine = sorted(results[sid], key=lambda r: r["frame"])
        assert [r["frame"] for r in mine] == list(range(n))
        for r, T in zip(mine, ref):
            assert np.array_equal(r["Tcm"], T), (sid, r["frame"])


def test_served_matches_standalone_session(cuda):
    W, H, n = 320, 240, 8
    seq = sequence(3, n, W, H)
    served = _serve_alone(seq, W, H)
    s = rf.Session(W, H, synth.intrinsics(W, H), **MAP)
    for (rgb, d16, _, _), T in zip(seq, served):
        st, Ts = s.process(rgb, d16)
        assert st == 0
        dt, dr = pose_error(Ts, T)
        assert dt <= 1e-5 and dr <= 1e-5, (dt, dr)


def test_admission_by_free_hbm(cuda):
    srv = serving.Server(hbm_reserve_bytes=1 << 50)  # more than any GPU has
    with pytest.raises(L.YasError) as e:
        srv.open(320, 240, synth.intrinsics(320, 240), **MAP)
    assert e.value.code == 2  # YAS_ERR_OOM: not admitted
    srv.close()


def test_suspend_and_resume_session(cuda):
    """A suspended session's map leaves HBM; frames submitted meanwhile wait
    and, after resume, give the poses of an uninterrupted run."""
    import torch

    W, H, n = 320, 240, 6
    seq = sequence(3, n, W, H)
    alone = _serve_alone(seq, W, H)
    srv = serving.Server(hbm_reserve_bytes=1 << 30)
    sid = srv.open(W, H, synth.intrinsics(W, H), **MAP)
    for rgb, d16, _, _ in seq[:3]:
        assert srv.submit(sid, rgb, d16) == 0
        srv.drain()
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    srv.suspend(sid)
    free1 = torch.cuda.mem_get_info()[0]
    assert free1 - free0 >= (MAP["max_blocks"] * 512 * 4) // 2  # the voxel pool was released
    for rgb, d16, _, _ in seq[3:]:
        assert srv.submit(sid, rgb, d16) == 0
    srv.resume(sid)
    srv.drain()
    res = sorted(srv.poll(64), key=lambda r: r["frame"])
    srv.close()
    assert [r["frame"] for r in res] == list(range(n))
    for r, T in zip(res, alone):
        assert r["status"] == 0 and np.array_equal(r["Tcm"], T)
