"""Shared inputs and comparison helpers of the parity tests."""
from __future__ import annotations

import functools

import numpy as np

from yetanotherslam_gb300 import synth


@functools.lru_cache(maxsize=8)
def sequence(seed: int, n: int, w: int, h: int):
    """n frames of the seeded scene (rgb, depth u16, depth metres, Twc)."""
    sc = synth.Scene(seed=seed)
    out = []
    for i in range(n):
        f = sc.render(i, w, h)
        out.append((f.rgb, f.depth, (f.depth.astype(np.float32) * np.float32(0.001)), f.Twc))
    return out


def rel_poses(seq):
    """Camera -> first-camera poses (the map frame of a session started at frame 0)."""
    T0inv = np.linalg.inv(seq[0][3])
    return [T0inv @ s[3] for s in seq]


def key_rows(coords: np.ndarray) -> np.ndarray:
    """Sortable int64 keys of (n, 3) block coordinates."""
    c = coords.astype(np.int64) + (1 << 20)
    return (c[:, 0] << 42) | (c[:, 1] << 21) | c[:, 2]


def align_blocks(ca, sa, wa, cb, sb, wb):
    """Reorders both block sets by coordinate; asserts the coordinate sets are equal."""
    ka, kb = key_rows(ca), key_rows(cb)
    ia, ib = np.argsort(ka), np.argsort(kb)
    assert ka.shape == kb.shape, f"block counts differ: {ka.shape[0]} vs {kb.shape[0]}"
    assert np.array_equal(ka[ia], kb[ib]), "block coordinate sets differ"
    return sa[ia], wa[ia], sb[ib], wb[ib]


def pose_error(A: np.ndarray, B: np.ndarray) -> tuple[float, float]:
    """(translation m, rotation rad) of A^-1 B."""
    E = np.linalg.inv(A) @ B
    c = np.clip((np.trace(E[:3, :3]) - 1.0) / 2.0, -1.0, 1.0)
    return float(np.linalg.norm(E[:3, 3])), float(np.arccos(c))
