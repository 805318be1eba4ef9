"""Seeded synthetic RGB-D sequences (ctypes wrapper of ``csrc/synth.c``).

A :class:`Scene` is a box room with spheres and cuboids; :meth:`Scene.frames`
renders uint8 RGB, uint16 millimetre depth and the camera-to-world poses of a
smooth trajectory.  Intrinsics follow the configurations' convention:
fx = fy = 525, cx = 319.5, cy = 239.5 at 640x480, scaled with the resolution.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import build

_synth = None


def _load():
    global _synth
    if _synth is None:
        path = build.SYNTH
        if not path.exists():
            build.build_synth()
        lib = C.CDLL(str(path))
        lib.yas_synth_scene_size.restype = C.c_int
        lib.yas_synth_scene_init.argtypes = [C.c_void_p, C.c_uint64, C.c_int, C.c_int, C.c_double, C.c_double,
                                             C.c_double]
        lib.yas_synth_scene_init.restype = C.c_int
        lib.yas_synth_pose.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
        lib.yas_synth_pose.restype = None
        lib.yas_synth_render.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_double,
                                         C.c_double, C.c_double, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
        lib.yas_synth_render.restype = None
        lib.yas_synth_render_brute.argtypes = lib.yas_synth_render.argtypes
        lib.yas_synth_render_brute.restype = None
        lib.yas_synth_scene_init_rooms.argtypes = [C.c_void_p, C.c_uint64, C.c_int, C.c_double, C.c_double,
                                                   C.c_double, C.c_double, C.c_int]
        lib.yas_synth_scene_init_rooms.restype = C.c_int
        _synth = lib
    return _synth


def intrinsics(width: int, height: int) -> tuple[float, float, float, float]:
    """fx, fy, cx, cy for a resolution, scaled from 525/525/319.5/239.5 at 640x480."""
    s = width / 640.0
    return 525.0 * s, 525.0 * (height / 480.0), (width - 1) / 2.0, (height - 1) / 2.0


@dataclass
class Frame:
    rgb: np.ndarray      # (h, w, 3) uint8
    depth: np.ndarray    # (h, w) uint16 millimetres
    Twc: np.ndarray      # (4, 4) camera-to-world


class Scene:
    def __init__(self, seed: int = 1, n_spheres: int = 20, n_boxes: int = 10,
                 size: tuple[float, float, float] = (4.0, 3.0, 4.0)):
        lib = _load()
        self._buf = C.create_string_buffer(lib.yas_synth_scene_size())
        rc = lib.yas_synth_scene_init(self._buf, seed, n_spheres, n_boxes, *size)
        if rc != 0:
            raise RuntimeError(f"scene placement failed ({rc})")
        self.seed = seed

    @classmethod
    def rooms(cls, seed: int = 1, n_objects: int = 80, size: tuple[float, float, float] = (12.0, 4.0, 12.0),
              loop_radius: float = 4.5, loop_frames: int = 2000) -> "Scene":
        """Four rooms (interior walls with doorways) and a closed loop through them that
        returns to its start after `loop_frames` frames."""
        lib = _load()
        sc = cls.__new__(cls)
        sc._buf = C.create_string_buffer(lib.yas_synth_scene_size())
        rc = lib.yas_synth_scene_init_rooms(sc._buf, seed, n_objects, *size, loop_radius, loop_frames)
        if rc != 0:
            raise RuntimeError(f"scene placement failed ({rc})")
        sc.seed = seed
        return sc

    def pose(self, i: int) -> np.ndarray:
        out = np.zeros(12, dtype=np.float64)
        _load().yas_synth_pose(self._buf, i, out.ctypes.data)
        T = np.eye(4)
        T[:3, :4] = out.reshape(3, 4)
        return T

    def render(self, i: int, width: int = 640, height: int = 480, clean: bool = False, brute: bool = False):
        """Frame i; `brute` tests every object for every pixel (no per-tile culling; same output)."""
        fx, fy, cx, cy = intrinsics(width, height)
        Twc = self.pose(i)
        m = np.ascontiguousarray(Twc[:3, :4].reshape(-1))
        rgb = np.empty((height, width, 3), dtype=np.uint8)
        depth = np.empty((height, width), dtype=np.uint16)
        cl = np.empty((height, width), dtype=np.float32) if clean else None
        fn = _load().yas_synth_render_brute if brute else _load().yas_synth_render
        fn(self._buf, m.ctypes.data, width, height, fx, fy, cx, cy, i, rgb.ctypes.data, depth.ctypes.data,
           cl.ctypes.data if clean else None)
        f = Frame(rgb, depth, Twc)
        if clean:
            return f, cl
        return f

    def frames(self, n: int, width: int = 640, height: int = 480, start: int = 0) -> list[Frame]:
        return [self.render(start + i, width, height) for i in range(n)]


def gray_of(rgb: np.ndarray) -> np.ndarray:
    """BT.601 luma in 14-bit fixed point, the same rule the device ingest uses."""
    r = rgb[..., 0].astype(np.int32)
    g = rgb[..., 1].astype(np.int32)
    b = rgb[..., 2].astype(np.int32)
    return ((r * 4899 + g * 9617 + b * 1868 + 8192) >> 14).astype(np.uint8)
