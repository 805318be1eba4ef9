"""Precision study of the dense path against the FP64 host oracle.

Workload (the precision variant): a seeded synthetic sequence at 640x480,
5 mm voxels, truncation 3 voxels, 2^21 hash slots, 3-level RGB+ICP tracking
with {10, 5, 3} iterations, marching cubes every 50 frames.  Four GPU
sessions run the same frames:

  f32_comp   FP32 TSDF (float sdf + float weight), compensated FP32 sums
  f16_comp   FP16 TSDF (half sdf, its rounding residual, u8 weight), compensated FP32 sums
  f32_plain  FP32 TSDF,                            plain FP32 sums
  f16_plain  FP16 TSDF,                            plain FP32 sums

(compensated = TwoSum partial sums with double-float totals; plain = the
same order without error terms, the reference's arithmetic; the 6x6 solve
and the SE(3) update are double-float, 48 significant bits, in all four).  The oracle (FP64 restatement of the
reference's integrate / raycast / mesh / tracking math) runs the same frames.
Reported:

  * tracking, per variant: per-frame pose error against the oracle's pose
    (metres, radians); the session maps against the oracle session's on the
    voxels with equal weights (tracked poses differ slightly, so voxels at the
    edge of the truncation band can take one observation more or less);
  * mapping, per storage format: F32, F16 and S24 (24-bit fixed-point sdf +
    u8 weight, 4 B like F16) maps fused with the oracle's poses and the same
    depth, against an FP64 oracle map: TSDF error
    (normalised by the truncation) on the voxels both observe, and
    marching-cubes agreement (cubes whose case index matches, and the vertex
    error of their triangles in metres), at every mesh frame.

Usage: python -m tests.precision_study [--frames 300] [--out report.json]
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np
import torch

import oracle
from tests.helpers import key_rows, pose_error
from yetanotherslam_gb300 import rgbdfusion as rf
from yetanotherslam_gb300 import synth

VARIANTS = {
    "f32_comp": (rf.VOXEL_F32, True),
    "f16_comp": (rf.VOXEL_F16, True),
    "f32_plain": (rf.VOXEL_F32, False),
    "f16_plain": (rf.VOXEL_F16, False),
}


def _stats(x) -> dict:
    x = np.asarray(x, dtype=np.float64)
    if x.size == 0:
        return {"max": 0.0, "p99": 0.0, "p50": 0.0, "mean": 0.0, "n": 0}
    return {"max": float(x.max()), "p99": float(np.percentile(x, 99)), "p50": float(np.median(x)),
            "mean": float(x.mean()), "n": int(x.size)}


def tsdf_error(gpu, orc) -> dict:
    """Error of the GPU TSDF against the oracle's on the voxels both observe
    the same number of times (weights equal), and how many commonly observed
    voxels carry different weights."""
    cg, sg, wg = gpu
    co, so, wo = orc
    kg, ko = key_rows(cg), key_rows(co)
    common, ig, io = np.intersect1d(kg, ko, return_indices=True)
    sg, wg, so, wo = sg[ig], wg[ig], so[io], wo[io]
    both = (wg > 0) & (wo > 0)
    same = both & (wg == wo)
    d = np.abs(sg[same].astype(np.float64) - so[same])
    out = _stats(d)
    out.update(blocks_gpu=int(kg.size), blocks_oracle=int(ko.size), blocks_common=int(common.size),
               observed_both=int(both.sum()), weight_equal_frac=float(same.sum() / max(int(both.sum()), 1)),
               observed_differs=int(((wg > 0) != (wo > 0)).sum()))
    return out


def _cube_index(cube: np.ndarray):
    """Stable order by cube, and (key, first triangle, count) per cube."""
    key = key_rows(cube)
    order = np.argsort(key, kind="stable")
    ks = key[order]
    uniq, first, count = np.unique(ks, return_index=True, return_counts=True)
    return order, uniq, first, count


def mesh_error(gpu, orc) -> dict:
    """Cubes with the same case index in both soups, and their vertex error."""
    pg, _, cg, xg = gpu
    po, _, co, xo = orc
    og, ug, fg, ng = _cube_index(xg)
    oo, uo, fo, no = _cube_index(xo)
    common, ig, io = np.intersect1d(ug, uo, return_indices=True)
    case_g = cg[og][fg[ig]]
    case_o = co[oo][fo[io]]
    same = case_g == case_o
    ig, io = ig[same], io[same]
    cnt = ng[ig]
    total = int(cnt.sum())
    within = np.arange(total) - np.repeat(np.cumsum(cnt) - cnt, cnt)
    tg = og[np.repeat(fg[ig], cnt) + within]
    to = oo[np.repeat(fo[io], cnt) + within]
    d = np.abs(pg[tg].astype(np.float64) - po[to]).max(axis=1) if total else np.zeros(0)
    out = _stats(d)
    union = int(ug.size + uo.size - common.size)
    out.update(cubes_gpu=int(ug.size), cubes_oracle=int(uo.size), cubes_same_case=int(same.sum()),
               same_case_frac=float(same.sum() / max(union, 1)), triangles_gpu=int(pg.shape[0]),
               triangles_oracle=int(po.shape[0]))
    return out


def run(frames: int = 300, W: int = 640, H: int = 480, voxel: float = 0.005, seed: int = 11,
        mc_every: int = 50, slots: int = 1 << 21, blocks: int = 1 << 18, variants=None, log=print) -> dict:
    variants = variants or list(VARIANTS)
    K = synth.intrinsics(W, H)
    scene = synth.Scene(seed=seed)
    trunc = 3 * voxel
    # tracking: full sessions (RGB -> gray, u16 depth, pyramids, raycast, GN, fusion)
    sessions = {}
    for name in variants:
        fmt, comp = VARIANTS[name]
        s = rf.Session(W, H, K, hash_slots=slots, max_blocks=blocks, voxel_size=voxel, trunc_dist=trunc,
                       voxel_format=fmt)
        s.set_reduction(comp)
        sessions[name] = s
    orc = oracle.Session(W, H, K, voxel, trunc, kind="f64")
    # mapping: maps fused with the oracle's poses and the same depth, so the
    # TSDF and mesh differences are those of the storage and arithmetic alone
    maps = {}
    for fname, fmt in (("f32", rf.VOXEL_F32), ("f16", rf.VOXEL_F16), ("s24", rf.VOXEL_S24), ("s16", rf.VOXEL_S16)):
        m = rf.MapStruct(K)
        m.create_config(slots, blocks, voxel, trunc, fmt)
        maps[fname] = m
    omap = oracle.Map(voxel, trunc)
    # the reference's own int16 storage, restated in the oracle (parity of s16)
    omap16 = oracle.Map(voxel, trunc, int16_sdf=True)
    mesher = rf.MeshEngine(8_000_000)
    # open loop: standalone trackers given exactly the oracle session's inputs
    # of each frame (previous frame as reference, the oracle's raycast model)
    K3 = np.array([[K[0], 0, K[2]], [0, K[1], K[3]], [0, 0, 1]], np.float64)
    open_loop = {}
    for red, comp in (("comp", True), ("plain", False)):
        tr = rf.RGBDTracking(W, H, K3, True, True, num_levels=3, iterations=(10, 5, 3))
        tr.set_reduction(comp)
        open_loop[red] = tr
    # the oracle's own trackers on the same inputs: FP64 (must reproduce the
    # session's step) and its FP32 build (the reference's residual precision)
    oracle_ol = {k: oracle.Tracker(W, H, K3, levels=3, iters=(10, 5, 3), mode=3, kind=k) for k in ("f64", "f32")}
    ol_t = {r: [] for r in list(open_loop) + [f"oracle_{k}" for k in oracle_ol]}
    ol_r = {r: [] for r in ol_t}
    prev_in = None
    pose_t = {n: [] for n in variants}
    pose_r = {n: [] for n in variants}
    step_t = {n: [] for n in variants}
    step_r = {n: [] for n in variants}
    gt_t = {n: [] for n in variants}
    prev = {n: None for n in variants}
    prev_o = None
    checks = []
    T0inv = None
    t_start = time.time()
    for i in range(frames):
        f = scene.render(i, W, H)
        if T0inv is None:
            T0inv = np.linalg.inv(f.Twc)
        gray = synth.gray_of(f.rgb)
        dm = f.depth.astype(np.float32) * np.float32(0.001)
        if prev_o is not None:
            model_host = orc.map_raycast(prev_o)
            model = torch.from_numpy(model_host).cuda()
        st_o, To = orc.frame(f.rgb, f.depth)
        if prev_o is not None:
            DT_o = np.linalg.inv(To) @ prev_o  # Tcm_i = Tcm_(i-1) DT^-1
            torch.cuda.synchronize()
            for red, tr in open_loop.items():
                tr.SetReferenceImage(prev_in[0])
                tr.SetReferenceDepth(prev_in[1])
                tr.SetReferenceModel(model)
                tr.SetTrackingImage(gray)
                tr.SetTrackingDepth(dm)
                e_t, e_r = pose_error(DT_o, tr.GetTransform(np.eye(4), False))
                ol_t[red].append(e_t)
                ol_r[red].append(e_r)
            for k, otr in oracle_ol.items():
                otr.set_image(prev_in[0], True)
                otr.set_depth(prev_in[1], True)
                otr.set_model(model_host)
                otr.set_image(gray, False)
                otr.set_depth(dm, False)
                _, DT_k = otr.get_transform(np.eye(4), False)
                e_t, e_r = pose_error(DT_o, DT_k)
                ol_t[f"oracle_{k}"].append(e_t)
                ol_r[f"oracle_{k}"].append(e_r)
        prev_in = (gray, dm)
        gt = T0inv @ f.Twc
        for name, s in sessions.items():
            st, T = s.process(f.rgb, f.depth)
            if st != 0 or st_o != 0:
                raise RuntimeError(f"frame {i}: status {name}={st} oracle={st_o}")
            dt, dr = pose_error(To, T)
            pose_t[name].append(dt)
            pose_r[name].append(dr)
            gt_t[name].append(pose_error(gt, T)[0])
            if prev_o is not None:
                # this frame's motion estimate against the oracle's
                st_, sr_ = pose_error(np.linalg.inv(prev_o) @ To, np.linalg.inv(prev[name]) @ T)
                step_t[name].append(st_)
                step_r[name].append(sr_)
            prev[name] = T
        prev_o = To
        for m in maps.values():
            m.Fuse(dm, To)
        omap.fuse(dm, K, To)
        omap16.fuse(dm, K, To)
        if (i + 1) % mc_every == 0 or i + 1 == frames:
            row = {"frame": i + 1, "mapping": {}, "tracked": {}}
            o_exp, o_mesh = omap.export(), omap.mesh(8_000_000)
            for fname, m in maps.items():
                row["mapping"][fname] = {"tsdf": tsdf_error(m.export(), o_exp),
                                         "mesh": mesh_error(mesher.Meshify(m), o_mesh)}
            row["s16_vs_int16_oracle"] = tsdf_error(maps["s16"].export(), omap16.export())
            so_exp = orc.map_export()
            for name, s in sessions.items():
                row["tracked"][name] = {"tsdf": tsdf_error(s.map().export(), so_exp)}
            checks.append(row)
            log(f"frame {i + 1}/{frames}  {time.time() - t_start:.0f} s")
    return {
        "workload": {"frames": frames, "width": W, "height": H, "voxel_m": voxel, "trunc_m": trunc, "seed": seed,
                     "hash_slots": slots, "max_blocks": blocks, "mc_every": mc_every, "levels": 3,
                     "iterations": [10, 5, 3]},
        "pose_vs_oracle": {n: {"t_m": _stats(pose_t[n]), "r_rad": _stats(pose_r[n])} for n in variants},
        "frame_motion_vs_oracle": {n: {"t_m": _stats(step_t[n]), "r_rad": _stats(step_r[n])} for n in variants},
        "open_loop_vs_oracle": {r: {"t_m": _stats(ol_t[r]), "r_rad": _stats(ol_r[r])} for r in ol_t},
        "open_loop_t_m_per_frame": {r: [float(x) for x in ol_t[r]] for r in ol_t},
        "pose_vs_ground_truth_t_m": {n: _stats(gt_t[n]) for n in variants},
        "pose_t_m_per_frame": {n: [float(x) for x in pose_t[n]] for n in variants},
        "pose_r_rad_per_frame": {n: [float(x) for x in pose_r[n]] for n in variants},
        "checks": checks,
        "seconds": time.time() - t_start,
    }


def summary(report: dict) -> str:
    """Markdown tables of the report."""
    ck = report["checks"]
    lines = ["Per-frame tracking, open loop (a tracker given exactly the oracle session's inputs of each frame: "
             "previous frame as reference, the oracle's raycast as model; comp / plain are the GPU tracker's "
             "reductions, oracle_f64 / oracle_f32 the oracle's own tracker in FP64 and in FP32):", "",
             "| reduction | t max (m) | t p99 | t p50 | r max (rad) | r p99 |", "|---|---|---|---|---|---|"]
    for r, s in report["open_loop_vs_oracle"].items():
        s = dict(s)
        lines.append(f"| {r} | {s['t_m']['max']:.2e} | {s['t_m']['p99']:.2e} | {s['t_m']['p50']:.2e} | "
                     f"{s['r_rad']['max']:.2e} | {s['r_rad']['p99']:.2e} |")
    lines += ["", "Sessions against the oracle session: each frame's motion estimate (T_prev^-1 T), and the absolute pose "
             "(closed loop through the map); ground truth for scale:", "",
             "| variant | motion t max (m) | motion t p99 | motion r max (rad) | motion r p99 | pose t max (m) | "
             "pose t p50 | pose vs truth t max (m) |", "|---|---|---|---|---|---|---|---|"]
    for n, p in report["pose_vs_oracle"].items():
        s = report["frame_motion_vs_oracle"][n]
        g = report["pose_vs_ground_truth_t_m"][n]
        lines.append(f"| {n} | {s['t_m']['max']:.2e} | {s['t_m']['p99']:.2e} | {s['r_rad']['max']:.2e} | "
                     f"{s['r_rad']['p99']:.2e} | {p['t_m']['max']:.2e} | {p['t_m']['p50']:.2e} | {g['max']:.2e} |")
    lines += ["", "Mapping (the oracle's poses and depth; worst over the mesh frames):", "",
              "| storage | TSDF max (×trunc) | TSDF p99 | weights equal | MC same case | MC vertex max (m) | "
              "MC vertex p99 (m) |", "|---|---|---|---|---|---|---|"]
    for f in ck[-1]["mapping"]:
        tm = max(c["mapping"][f]["tsdf"]["max"] for c in ck)
        tp = max(c["mapping"][f]["tsdf"]["p99"] for c in ck)
        eq = min(c["mapping"][f]["tsdf"]["weight_equal_frac"] for c in ck)
        sc = min(c["mapping"][f]["mesh"]["same_case_frac"] for c in ck)
        vm = max(c["mapping"][f]["mesh"]["max"] for c in ck)
        vp = max(c["mapping"][f]["mesh"]["p99"] for c in ck)
        lines.append(f"| {f} | {tm:.2e} | {tp:.2e} | {eq:.4f} | {sc:.5f} | {vm:.2e} | {vp:.2e} |")
    p16 = [c["s16_vs_int16_oracle"] for c in ck]
    lines += ["", f"s16 against the oracle keeping the same int16 storage: TSDF max {max(x['max'] for x in p16):.2e}, "
              f"p99 {max(x['p99'] for x in p16):.2e}, weights equal {min(x['weight_equal_frac'] for x in p16):.4f}"]
    last = ck[-1]["mapping"]["f32"]
    lines += ["", f"final map: {last['tsdf']['blocks_oracle']} blocks, {last['mesh']['triangles_oracle']} "
              f"triangles (oracle); {report['seconds']:.0f} s"]
    return "\n".join(lines)


def main() -> None:
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--frames", type=int, default=300)
    ap.add_argument("--mc-every", type=int, default=50)
    ap.add_argument("--seed", type=int, default=11)
    ap.add_argument("--out", default="")
    a = ap.parse_args()
    rep = run(frames=a.frames, mc_every=a.mc_every, seed=a.seed)
    if a.out:
        with open(a.out, "w") as f:
            json.dump(rep, f, indent=1)
    print(summary(rep))


if __name__ == "__main__":
    main()
