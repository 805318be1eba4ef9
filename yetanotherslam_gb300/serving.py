"""Served SLAM sessions: the request server of ``include/yas.h`` (``yas_server_*``).

Frames of many sessions are submitted as they arrive; the server batches them
continuously on the GPU and returns per-frame results with their latency.
``gn_per_session`` (the default) gives every taken frame its own Gauss-Newton
launch on its session's stream; 0 gathers the waiting sessions into one
batched launch.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from .rgbdfusion import session_config


class Server:
    def __init__(self, max_sessions: int = 64, hbm_reserve_bytes: int = 4 << 30, ring_frames: int = 4,
                 gn_per_session: bool | None = None, gn_pixels_per_cta: int = 0):
        cfg = L.ServerConfig()
        L.call("yas_server_config_default", C.byref(cfg))
        cfg.max_sessions = max_sessions
        cfg.hbm_reserve_bytes = hbm_reserve_bytes
        cfg.ring_frames = ring_frames
        if gn_per_session is not None:
            cfg.gn_per_session = int(bool(gn_per_session))
        cfg.gn_pixels_per_cta = int(gn_pixels_per_cta)
        self.handle = C.c_void_p()
        L.call("yas_server_create", C.byref(self.handle), C.byref(cfg))
        self._sizes: dict[int, tuple[int, int]] = {}

    def open(self, width: int, height: int, K, **kw) -> int:
        """Admits a session (raises YasError YAS_ERR_OOM if its footprint does not fit the free HBM)."""
        cfg = session_config(width, height, K, **kw)
        sid = C.c_int()
        L.call("yas_server_open_session", self.handle, C.byref(cfg), C.byref(sid))
        self._sizes[sid.value] = (width, height)
        return sid.value

    def suspend(self, sid: int) -> None:
        """Moves the session's map to host memory (its frames wait until resume)."""
        L.call("yas_server_suspend_session", self.handle, sid)

    def resume(self, sid: int) -> None:
        L.call("yas_server_resume_session", self.handle, sid)

    def close_session(self, sid: int) -> None:
        L.call("yas_server_close_session", self.handle, sid)
        self._sizes.pop(sid, None)

    def submit(self, sid: int, rgb: np.ndarray, depth: np.ndarray) -> int:
        """Queues one frame; returns the status (0, or YAS_ERR_CAPACITY when the session's ring is full)."""
        w, h = self._sizes[sid]
        rgb = np.ascontiguousarray(rgb, dtype=np.uint8)
        depth = np.ascontiguousarray(depth, dtype=np.uint16)
        if rgb.size != w * h * 3 or depth.size != w * h:
            raise ValueError("frame size does not match the session")
        code = L.load().yas_server_submit(self.handle, sid, rgb.ctypes.data, depth.ctypes.data)
        if code not in (L.YAS_OK, 11):
            L.check(code, "yas_server_submit")
        return code

    def poll(self, capacity: int = 4096) -> list[dict]:
        buf = (L.ServedResult * capacity)()
        n = C.c_int()
        L.call("yas_server_poll", self.handle, buf, capacity, C.byref(n))
        return [{"session": r.session, "status": r.status, "frame": r.frame, "latency_ms": r.latency_ms,
                 "Tcm": L.pose_to(r.Tcm)} for r in buf[:n.value]]

    def drain(self, timeout_s: float = 30.0) -> None:
        L.call("yas_server_drain", self.handle, timeout_s)

    def stats(self) -> dict:
        s = L.ServerStats()
        L.call("yas_server_get_stats", self.handle, C.byref(s))
        return {k: getattr(s, k) for k, _ in L.ServerStats._fields_}

    def reset_stats(self) -> None:
        L.call("yas_server_reset_stats", self.handle)

    def close(self) -> None:
        if self.handle:
            L.call("yas_server_destroy", self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
