"""The seeded synthetic generator (CPU): per-tile culled rendering equals
rendering every object for every pixel, bit for bit; the multi-room loop
closes and keeps every frame's motion within 2 cm and 1 degree."""
from __future__ import annotations

import numpy as np

from tests.helpers import pose_error
from yetanotherslam_gb300 import synth


def _same(sc, i, w, h):
    a = sc.render(i, w, h, clean=True)
    b = sc.render(i, w, h, clean=True, brute=True)
    (fa, ca), (fb, cb) = a, b
    assert np.array_equal(fa.rgb, fb.rgb) and np.array_equal(fa.depth, fb.depth) and np.array_equal(ca, cb)
    return fa


def test_culled_render_equals_brute_force():
    sc = synth.Scene(seed=3)
    for i in (0, 17):
        _same(sc, i, 320, 240)
    rooms = synth.Scene.rooms(seed=5, loop_frames=2000)
    for i in (0, 250, 777, 1500):
        f = _same(rooms, i, 320, 180)
        assert (f.depth > 0).mean() > 0.5


def test_room_loop_closes_with_small_steps():
    n = 2000
    sc = synth.Scene.rooms(seed=5, loop_frames=n)
    P = [sc.pose(i) for i in range(0, n + 1)]
    dt, dr = pose_error(P[0], P[n])
    assert dt < 1e-9 and dr < 1e-6
    steps = [pose_error(P[i], P[i + 1]) for i in range(0, n, 7)]
    assert max(s[0] for s in steps) < 0.02 and max(s[1] for s in steps) < np.radians(1.0)
