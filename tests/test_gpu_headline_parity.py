"""Tracking parity at the benchmark's own configuration, frame by frame.

Workload (the headline metric's): 640x480 frames of the seeded scene (seed 11,
as the precision study), 5 mm voxels, truncation 15 mm, 2^21 hash slots,
FP16 TSDF words, RGB+ICP over 3 levels with {10, 5, 3} Gauss-Newton
iterations, 30 frames.  Reference behaviour: Tracking::TrackRGBD
(FullSystem/src/Tracking.cpp:162-197) around RGBDTracking::GetTransform
(RGBDFusion/src/RGBDTracking.cu:152-214).  The FP64 oracle session runs the
same frames beside the library's session.  Bars, every frame:

  * open loop: the GPU tracker given exactly the oracle session's inputs of
    the frame (the previous frame as reference, the oracle's raycast at the
    previous pose as model) returns the oracle's motion estimate within
    1e-4 m and 1e-4 rad.  Both sides take the tracker's discrete decisions
    (pixels inside the image, ICP pairs and gates, the error that
    GetTransform's keep-the-better-estimate test compares) in FP32 at the
    same FP32 pose, so a near-tie of two iterations' errors is decided the
    same way;
  * closed loop: the F16 session's own motion estimate of each frame
    (T_prev^-1 T) within 1e-4 m and 1e-4 rad of the oracle session's, and
    its pose within 1e-3 m / rad of the oracle's after 30 frames (each side
    tracks against its own map, FP16 words here and FP64 there).
"""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from tests.helpers import pose_error
from yetanotherslam_gb300 import rgbdfusion as rf
from yetanotherslam_gb300 import synth

pytestmark = pytest.mark.gpu

W, H, VOXEL, SEED, FRAMES = 640, 480, 0.005, 11, 30


def test_bench_configuration_tracks_like_the_oracle_every_frame(cuda):
    import torch

    K = synth.intrinsics(W, H)
    K3 = np.array([[K[0], 0, K[2]], [0, K[1], K[3]], [0, 0, 1.0]])
    scene = synth.Scene(seed=SEED)
    sess = rf.Session(W, H, K, hash_slots=1 << 21, max_blocks=1 << 18, voxel_size=VOXEL, trunc_dist=3 * VOXEL,
                      voxel_format=rf.VOXEL_F16, num_levels=3, iterations=(10, 5, 3))
    orc = oracle.Session(W, H, K, VOXEL, 3 * VOXEL, kind="f64")
    tr = rf.RGBDTracking(W, H, K3, True, True, num_levels=3, iterations=(10, 5, 3))
    open_loop, closed_step = [], []
    prev_o = prev_g = prev_in = None
    for i in range(FRAMES):
        f = scene.render(i, W, H)
        gray = synth.gray_of(f.rgb)
        dm = f.depth.astype(np.float32) * np.float32(0.001)
        model = orc.map_raycast(prev_o) if prev_o is not None else None
        st_o, To = orc.frame(f.rgb, f.depth)
        st_g, Tg = sess.process(f.rgb, f.depth)
        assert st_o == 0 and st_g == 0, (i, st_o, st_g)
        if prev_o is not None:
            DT_o = np.linalg.inv(To) @ prev_o  # Tcm_i = Tcm_(i-1) DT^-1
            tr.SetReferenceImage(prev_in[0])
            tr.SetReferenceDepth(prev_in[1])
            tr.SetReferenceModel(torch.from_numpy(model).cuda())
            tr.SetTrackingImage(gray)
            tr.SetTrackingDepth(dm)
            open_loop.append(pose_error(DT_o, tr.GetTransform(np.eye(4), False)))
            closed_step.append(pose_error(np.linalg.inv(prev_o) @ To, np.linalg.inv(prev_g) @ Tg))
        prev_o, prev_g, prev_in = To, Tg, (gray, dm)
    ol, cs = np.array(open_loop), np.array(closed_step)
    report = (f"open loop t max {ol[:, 0].max():.3g} r max {ol[:, 1].max():.3g}; "
              f"closed loop step t max {cs[:, 0].max():.3g} r max {cs[:, 1].max():.3g}")
    assert (ol[:, 0] <= 1e-4).all() and (ol[:, 1] <= 1e-4).all(), (report, np.argmax(ol[:, 0]) + 1)
    assert (cs[:, 0] <= 1e-4).all() and (cs[:, 1] <= 1e-4).all(), (report, np.argmax(cs[:, 0]) + 1)
    dt, dr = pose_error(prev_o, prev_g)
    assert dt <= 1e-3 and dr <= 1e-3, (dt, dr, report)
    print(report)
    sess.close()
