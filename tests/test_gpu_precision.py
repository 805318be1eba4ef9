"""Precision variants against the FP64 oracle on a short sequence
(tests/precision_study.py runs the full 300-frame, 640x480 / 5 mm study).

Bars:
  * per-frame tracking, open loop (the GPU tracker given the oracle's inputs
    of each frame): the motion estimate within 1e-4 m and 1e-4 rad of the
    oracle's with compensated sums, 1e-3 with plain sums;
  * sessions (closed loop through their own maps) over 24 frames: pose within
    3e-4 m / rad of the oracle's with compensated sums (the library's
    default), FP32 and FP16 TSDF alike, 1e-3 with plain FP32 sums (the
    reference's arithmetic).  Each frame tracks against the session's own
    raycast, so rounding that flips a rare ray's march decision, or
    GetTransform's keep-the-better-estimate decision, against the FP64 oracle
    carries into the later frames;
  * mapping with the oracle's poses: weights exactly equal; TSDF (normalised
    by the truncation) within 1e-5 for FP32 and S24 storage and within 1e-3
    (the stated TSDF bar) for FP16 storage, whose words keep the half's
    rounding residual in 1/256 of its ulp (19 significant bits; without it
    every write rounds to 11 bits and the error grows like a random walk over
    the observations); marching cubes with the oracle's case index on at
    least 99.99 % of cubes and vertices within 1e-4 of a voxel at the 99th
    percentile, for all three;
  * S16 (the reference's int16 voxel, PackFloat's truncation toward zero)
    against the oracle keeping the same int16 storage: weights equal, TSDF
    within 1e-4 (three int16 steps).  Its error against the FP64 map is
    reported, not barred: truncation loses every increment below one step.
"""
from __future__ import annotations

import pytest

from tests import precision_study as ps

pytestmark = pytest.mark.gpu


def test_precision_variants_against_oracle(cuda):
    vs = 0.008
    rep = ps.run(frames=24, W=320, H=240, voxel=vs, seed=11, mc_every=12, slots=1 << 19, blocks=1 << 16,
                 log=lambda *_: None)
    bad = []
    for red, p in rep["open_loop_vs_oracle"].items():
        bar = {"comp": 1e-4, "plain": 1e-3, "oracle_f64": 1e-7, "oracle_f32": 1e-3}[red]  # 1e-7: the arccos floor
        if not (p["t_m"]["max"] <= bar and p["r_rad"]["max"] <= bar and p["t_m"]["n"] == 23):
            bad.append(("open loop", red, p["t_m"]["max"], p["r_rad"]["max"]))
    for name, p in rep["pose_vs_oracle"].items():
        bar = 3e-4 if name.endswith("comp") else 1e-3
        if not (p["t_m"]["max"] <= bar and p["r_rad"]["max"] <= bar):
            bad.append(("pose", name, p["t_m"]["max"], p["r_rad"]["max"]))
    for chk in rep["checks"]:
        p16 = chk["s16_vs_int16_oracle"]
        if not (p16["weight_equal_frac"] == 1.0 and p16["max"] <= 1e-4 and p16["n"] > 100000):
            bad.append(("s16 parity", chk["frame"], p16["max"], p16["weight_equal_frac"]))
        for f, v in chk["mapping"].items():
            if f == "s16":  # the reference's int16 storage against FP64: reported, not a bar
                continue
            tsdf_bar, p99_bar, case_bar, vert_bar = ((1e-3, 1e-4, 0.9999, 1e-4) if f == "f16" else
                                                     (1e-5, 1e-5, 0.9999, 1e-4))
            t, m = v["tsdf"], v["mesh"]
            if not (t["weight_equal_frac"] == 1.0 and t["max"] <= tsdf_bar and t["p99"] <= p99_bar
                    and t["n"] > 100000):
                bad.append(("tsdf", chk["frame"], f, t["max"], t["weight_equal_frac"], t["n"]))
            if not (m["same_case_frac"] >= case_bar and m["p99"] <= vert_bar * vs):
                bad.append(("mesh", chk["frame"], f, m["same_case_frac"], m["p99"], m["max"]))
    assert not bad, (bad, ps.summary(rep))
