"""Batched keyframe submaps: ``yas_batch_*`` of ``include/yas.h``.

Many sessions (submaps of any resolution and voxel size) step together; one
step is one CUDA graph launch holding every active session's frame.  By
default (``gn_per_session = 1``) each session's whole Gauss-Newton schedule
is its own cooperative launch in that session's branch of the graph, so a
session's pose update and fusion start as soon as its own GN ends; with
``gn_per_session = 0`` one persistent cooperative launch runs every
session's schedule.  Both give the same results.  ``autotune`` picks the
launch shapes (and between these two modes) on scratch copies of the
sessions.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from .rgbdfusion import Session, _device_info


def default_tuning() -> L.BatchTuning:
    t = L.BatchTuning()
    L.call("yas_batch_tuning_default", C.byref(t))
    return t


class Batch:
    def __init__(self, sessions: list[Session], stream: int | None = None):
        self.sessions = list(sessions)
        n = len(self.sessions)
        arr = (C.c_void_p * n)(*[s.handle.value for s in self.sessions])
        self.handle = C.c_void_p()
        L.call("yas_batch_create", C.byref(self.handle), arr, n, stream)
        self._keep = []

    def close(self) -> None:
        if self.handle:
            L.call("yas_batch_destroy", self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def tuning(self) -> L.BatchTuning:
        t = L.BatchTuning()
        L.call("yas_batch_get_tuning", self.handle, C.byref(t))
        return t

    @tuning.setter
    def tuning(self, t: L.BatchTuning) -> None:
        L.call("yas_batch_set_tuning", self.handle, C.byref(t))

    def _ptrs(self, frames):
        n = len(self.sessions)
        rgb = (C.c_void_p * n)()
        dep = (C.c_void_p * n)()
        dev = None
        keep = []
        for i, fr in enumerate(frames):
            if fr is None:
                continue
            r, d = fr
            pr, _, dr, kr = _device_info(r)
            pd, _, dd, kd = _device_info(d if dr else np.ascontiguousarray(d, dtype=np.uint16))
            if dev is None:
                dev = dr
            if dr != dev or dd != dev:
                raise ValueError("a step's frames must all be on the host or all on the device")
            rgb[i], dep[i] = pr, pd
            keep += [kr, kd]
        return rgb, dep, int(bool(dev)), keep

    def step(self, frames) -> None:
        """frames[i]: (rgb, depth) of session i, or None to leave it idle this step."""
        n = len(self.sessions)
        if len(frames) != n:
            raise ValueError(f"{len(frames)} frames for {n} sessions")
        rgb, dep, dev, keep = self._ptrs(frames)
        active = (C.c_int * n)(*[0 if f is None else 1 for f in frames])
        self._keep = keep
        L.call("yas_batch_step", self.handle, rgb, dep, active, dev)

    def wait(self):
        """(poses (n,4,4), statuses (n,), device ms); idle sessions' entries are NaN / -1."""
        n = len(self.sessions)
        poses = (L.Pose * n)()
        st = (C.c_int * n)(*([-1] * n))
        for i in range(n):
            for k in range(12):
                poses[i].m[k] = float("nan")
        ms = C.c_float()
        L.call("yas_batch_wait", self.handle, poses, st, C.byref(ms))
        self._keep = []
        return np.stack([L.pose_to(p) for p in poses]), np.array(list(st)), ms.value

    def kernels_per_step(self) -> int:
        out = C.c_int()
        L.call("yas_batch_kernels_per_step", self.handle, C.byref(out))
        return out.value

    def autotune(self, calib) -> L.BatchTuning:
        """calib[i]: (rgb (f,h,w,3) u8, depth (f,h,w) u16) calibration frames of session i (f >= 3)."""
        n = len(self.sessions)
        f = {int(c[0].shape[0]) for c in calib}
        if len(f) != 1:
            raise ValueError("every session needs the same number of calibration frames")
        rgb, dep, dev, keep = self._ptrs(calib)
        out = L.BatchTuning()
        L.call("yas_batch_autotune", self.handle, rgb, dep, f.pop(), dev, C.byref(out))
        del keep
        return out
