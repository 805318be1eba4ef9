"""CPU oracle of the dense RGB-D path — TEST INFRASTRUCTURE ONLY.

Imported by ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg
of ``bench.py`` as the checker; the product (``yetanotherslam_gb300``) never
imports it.  See ``oracle.h`` for what is restated, in which precision, and
the parity-pinning status.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import build as _build

_libs: dict[str, C.CDLL] = {}

_P = C.c_void_p
_I = C.c_int
_F = C.c_float

_SIGS = {
    "orc_map_create": ([_F, _F, _F, _F, _I], _P),
    "orc_map_destroy": ([_P], None),
    "orc_map_set_storage": ([_P, _I], None),
    "orc_map_num_blocks": ([_P], _I),
    "orc_map_allocate": ([_P, _P, _I, _I, _P, _P], None),
    "orc_map_visible": ([_P, _I, _I, _P, _P, _P, _I], _I),
    "orc_map_fuse": ([_P, _P, _I, _I, _P, _P], _I),
    "orc_map_export": ([_P, _P, _P, _P], None),
    "orc_map_import": ([_P, _P, _P, _P, _I], None),
    "orc_raycast": ([_P, _I, _I, _P, _P, _P, _P, _P], None),
    "orc_mesh": ([_P, _P, _P, _P, _P, _I], _I),
    "orc_mc_tables": ([_P, _P, _P], None),
    "orc_tracker_create": ([_I, _I, _P, _I, _P, _I], _P),
    "orc_tracker_destroy": ([_P], None),
    "orc_tracker_set_image": ([_P, _P, _I], None),
    "orc_tracker_set_depth": ([_P, _P, _I], None),
    "orc_tracker_set_model": ([_P, _P], None),
    "orc_tracker_swap": ([_P], None),
    "orc_tracker_get_transform": ([_P, _P, _I, _P], _I),
    "orc_tracker_compute_step": ([_P, _I, _P, _P, _P, _P], None),
    "orc_tracker_level": ([_P, _I, _I, _P], None),
    "orc_session_create": ([_I, _I, _P, _F, _F, _I, _P, _I, _F, _F], _P),
    "orc_session_destroy": ([_P], None),
    "orc_session_frame": ([_P, _P, _P, _P], _I),
    "orc_session_map": ([_P], _P),
    "orc_session_tracker": ([_P], _P),
    "orc_map_defuse": ([_P, _P, _I, _I, _P, _P], _I),
    "orc_map_fuse_map": ([_P, _P, _P, _P], _I),
    "orc_render_scene": ([_P, _P, _I, _I, _P, _P], None),
    "orc_canvas_draw": ([_P, _P, C.c_uint, _P, _P, _P, _I, _I, _P], None),
    "orc_se3_exp": ([_P, _P], None),
    "orc_ldlt_solve6": ([_P, _P, _P], None),
    "orc_real_bytes": ([], _I),
}


def lib(kind: str = "f64") -> C.CDLL:
    """The checker (``f64``) or the FP32 multi-threaded baseline (``f32``)."""
    if kind not in _libs:
        l64, l32 = _build.build()
        cdll = C.CDLL(str(l64 if kind == "f64" else l32))
        for name, (args, res) in _SIGS.items():
            fn = getattr(cdll, name)
            fn.argtypes = args
            fn.restype = res
        _libs[kind] = cdll
    return _libs[kind]


def _ptr(a: np.ndarray):
    return a.ctypes.data


def _kvec(K) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(K, dtype=np.float32).reshape(4))


def _pose(T) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(T, dtype=np.float64)[:3, :4].reshape(12))


class Map:
    def __init__(self, voxel_size: float, trunc: float, depth_min: float = 0.1, depth_max: float = 3.0,
                 max_weight: int = 255, kind: str = "f64", int16_sdf: bool = False):
        """int16_sdf: every written sdf goes through the reference's int16 storage
        (PackFloat / UnPackFloat, VoxelStructUtils.h:6-14)."""
        self.L = lib(kind)
        self.h = self.L.orc_map_create(voxel_size, trunc, depth_min, depth_max, max_weight)
        if int16_sdf:
            self.L.orc_map_set_storage(self.h, 1)

    def __del__(self):
        if getattr(self, "h", None):
            self.L.orc_map_destroy(self.h)
            self.h = None

    @property
    def num_blocks(self) -> int:
        return self.L.orc_map_num_blocks(self.h)

    def allocate(self, depth: np.ndarray, K, Tcm) -> None:
        d = np.ascontiguousarray(depth, dtype=np.float32)
        self.L.orc_map_allocate(self.h, _ptr(d), d.shape[1], d.shape[0], _ptr(_kvec(K)), _ptr(_pose(Tcm)))

    def fuse(self, depth: np.ndarray, K, Tcm) -> int:
        d = np.ascontiguousarray(depth, dtype=np.float32)
        return self.L.orc_map_fuse(self.h, _ptr(d), d.shape[1], d.shape[0], _ptr(_kvec(K)), _ptr(_pose(Tcm)))

    def defuse(self, depth: np.ndarray, K, Tcm) -> int:
        d = np.ascontiguousarray(depth, dtype=np.float32)
        return self.L.orc_map_defuse(self.h, _ptr(d), d.shape[1], d.shape[0], _ptr(_kvec(K)), _ptr(_pose(Tcm)))

    def fuse_map(self, src: "Map", T_self, T_src) -> bool:
        """MapStruct::Fuse(MapStruct*); True if this map was empty and took src's storage."""
        a, b = _pose(T_self), _pose(T_src)
        return bool(self.L.orc_map_fuse_map(self.h, src.h, _ptr(a), _ptr(b)))

    def visible(self, cols: int, rows: int, K, Tcm) -> np.ndarray:
        out = np.zeros((max(self.num_blocks, 1), 3), dtype=np.int32)
        n = self.L.orc_map_visible(self.h, cols, rows, _ptr(_kvec(K)), _ptr(_pose(Tcm)), _ptr(out), out.shape[0])
        return out[:n]

    def export(self):
        n = self.num_blocks
        c = np.zeros((n, 3), dtype=np.int32)
        s = np.zeros((n, 512), dtype=np.float64)
        w = np.zeros((n, 512), dtype=np.float64)
        if n:
            self.L.orc_map_export(self.h, _ptr(c), _ptr(s), _ptr(w))
        return c, s, w

    def import_blocks(self, coords: np.ndarray, sdf: np.ndarray, wt: np.ndarray) -> None:
        c = np.ascontiguousarray(coords, dtype=np.int32)
        s = np.ascontiguousarray(sdf, dtype=np.float32)
        w = np.ascontiguousarray(wt, dtype=np.float32)
        self.L.orc_map_import(self.h, _ptr(c), _ptr(s), _ptr(w), c.shape[0])

    def raycast(self, w: int, h: int, K, Tcm):
        vmap = np.zeros((h, w, 4), dtype=np.float32)
        zw, zh = (w + 7) // 8, (h + 7) // 8
        zn = np.zeros((zh, zw), dtype=np.float32)
        zf = np.zeros((zh, zw), dtype=np.float32)
        self.L.orc_raycast(self.h, w, h, _ptr(_kvec(K)), _ptr(_pose(Tcm)), _ptr(vmap), _ptr(zn), _ptr(zf))
        return vmap, zn, zf

    def mesh(self, cap: int = 4_000_000):
        tris = np.zeros((cap, 9), dtype=np.float32)
        nrm = np.zeros((cap, 9), dtype=np.float32)
        cases = np.zeros(cap, dtype=np.int32)
        cube = np.zeros((cap, 3), dtype=np.int32)
        n = self.L.orc_mesh(self.h, _ptr(tris), _ptr(nrm), _ptr(cases), _ptr(cube), cap)
        n = min(n, cap)
        return tris[:n], nrm[:n], cases[:n], cube[:n]


def mc_tables():
    L = lib("f64")
    edge = np.zeros(256, dtype=np.uint16)
    tri = np.zeros((256, 31), dtype=np.int8)
    cnt = np.zeros(256, dtype=np.uint8)
    L.orc_mc_tables(_ptr(edge), _ptr(tri), _ptr(cnt))
    return edge, tri, cnt


class Tracker:
    def __init__(self, w: int, h: int, K33, levels: int = 3, iters=(10, 5, 3, 3, 3), mode: int = 3,
                 kind: str = "f64"):
        self.L = lib(kind)
        self.w, self.h = w, h
        Kd = np.ascontiguousarray(np.asarray(K33, dtype=np.float64).reshape(9))
        it = np.ascontiguousarray(np.asarray(list(iters) + [0] * (5 - len(iters)), dtype=np.int32)[:5])
        self.hdl = self.L.orc_tracker_create(w, h, _ptr(Kd), levels, _ptr(it), mode)
        self.levels = levels

    def __del__(self):
        if getattr(self, "hdl", None):
            self.L.orc_tracker_destroy(self.hdl)
            self.hdl = None

    def set_image(self, gray: np.ndarray, reference: bool) -> None:
        g = np.ascontiguousarray(gray, dtype=np.uint8)
        self.L.orc_tracker_set_image(self.hdl, _ptr(g), int(reference))

    def set_depth(self, depth: np.ndarray, reference: bool) -> None:
        d = np.ascontiguousarray(depth, dtype=np.float32)
        self.L.orc_tracker_set_depth(self.hdl, _ptr(d), int(reference))

    def set_model(self, vmap: np.ndarray) -> None:
        v = np.ascontiguousarray(vmap, dtype=np.float32)
        self.L.orc_tracker_set_model(self.hdl, _ptr(v))

    def swap(self) -> None:
        self.L.orc_tracker_swap(self.hdl)

    def get_transform(self, init=None, swap: bool = False):
        T0 = _pose(np.eye(4) if init is None else init)
        out = np.zeros(12, dtype=np.float64)
        st = self.L.orc_tracker_get_transform(self.hdl, _ptr(T0), int(swap), _ptr(out))
        T = np.eye(4)
        T[:3, :4] = out.reshape(3, 4)
        return st, T

    def compute_step(self, level: int, T):
        H = np.zeros(36)
        b = np.zeros(6)
        st = np.zeros(4)
        self.L.orc_tracker_compute_step(self.hdl, level, _ptr(_pose(T)), _ptr(H), _ptr(b), _ptr(st))
        return H.reshape(6, 6), b, st

    def level(self, level: int, which: int) -> np.ndarray:
        w, h = self.w >> level, self.h >> level
        k = 4 if which in (4, 5, 8, 9) else 1
        out = np.zeros((h, w, k) if k == 4 else (h, w), dtype=np.float32)
        self.L.orc_tracker_level(self.hdl, level, which, _ptr(out))
        return out


class Session:
    def __init__(self, w: int, h: int, K, voxel_size: float, trunc: float, levels: int = 3,
                 iters=(10, 5, 3, 3, 3), mode: int = 3, depth_scale: float = 0.001, max_step: float = 0.1,
                 kind: str = "f64", int16_sdf: bool = False):
        """int16_sdf: the session's map keeps the reference's int16 storage."""
        self.L = lib(kind)
        it = np.ascontiguousarray(np.asarray(list(iters) + [0] * (5 - len(iters)), dtype=np.int32)[:5])
        self.hdl = self.L.orc_session_create(w, h, _ptr(_kvec(K)), voxel_size, trunc, levels, _ptr(it), mode,
                                             depth_scale, max_step)
        if int16_sdf:
            self.L.orc_map_set_storage(self.L.orc_session_map(self.hdl), 1)
        self.w, self.h = w, h
        self.K = K

    def __del__(self):
        if getattr(self, "hdl", None):
            self.L.orc_session_destroy(self.hdl)
            self.hdl = None

    def frame(self, rgb: np.ndarray, depth: np.ndarray):
        r = np.ascontiguousarray(rgb, dtype=np.uint8)
        d = np.ascontiguousarray(depth, dtype=np.uint16)
        out = np.zeros(12)
        st = self.L.orc_session_frame(self.hdl, _ptr(r), _ptr(d), _ptr(out))
        T = np.eye(4)
        T[:3, :4] = out.reshape(3, 4)
        return st, T

    def map_raycast(self, Tcm):
        """Raycast of the session's map at Tcm (the model the next frame tracks against)."""
        m = Map.__new__(Map)
        m.L = self.L
        m.h = self.L.orc_session_map(self.hdl)
        try:
            return m.raycast(self.w, self.h, self.K, Tcm)[0]
        finally:
            m.h = None

    def map_mesh(self, cap: int = 4_000_000):
        """Marching cubes of the session's map (Map.mesh)."""
        m = Map.__new__(Map)
        m.L = self.L
        m.h = self.L.orc_session_map(self.hdl)
        try:
            return m.mesh(cap)
        finally:
            m.h = None

    def map_export(self):
        m = Map.__new__(Map)
        m.L = self.L
        m.h = self.L.orc_session_map(self.hdl)
        try:
            return m.export()
        finally:
            m.h = None


def canvas_draw(pts: np.ndarray, nrm: np.ndarray, Tmw, Tcw, K, w: int, h: int, keys: np.ndarray | None = None):
    """MapDrawer's mesh program as a rasteriser: draws an (n, 9) triangle soup into
    the 64-bit z-buffer `keys` (new, all empty, when None); returns keys."""
    if keys is None:
        keys = np.full((h, w), np.iinfo(np.uint64).max, dtype=np.uint64)
    p = np.ascontiguousarray(pts, dtype=np.float32)
    n = np.ascontiguousarray(nrm, dtype=np.float32)
    k4 = np.ascontiguousarray(np.asarray(K, dtype=np.float32).reshape(-1)[:4])
    lib().orc_canvas_draw(_ptr(p), _ptr(n), p.shape[0], _ptr(_pose(Tmw)), _ptr(_pose(Tcw)), _ptr(k4), w, h, _ptr(keys))
    return keys


def canvas_resolve(keys: np.ndarray):
    """(rgba (h, w, 4) uint8 on a white background, depth (h, w) float32, 0 where empty)."""
    empty = keys == np.iinfo(np.uint64).max
    lo = np.where(empty, np.uint64(0xFFFFFFFF), keys & np.uint64(0xFFFFFFFF)).astype(np.uint32)
    rgba = lo.view(np.uint8).reshape(keys.shape + (4,))
    depth = np.where(empty, np.uint32(0), (keys >> np.uint64(32)).astype(np.uint32)).view(np.float32)
    return rgba, depth


def render_scene(vmap: np.ndarray, nmap: np.ndarray, light=(5.0, 5.0, 5.0)) -> np.ndarray:
    """RenderScene: (h, w, 4) float vertex/normal maps -> (h, w, 4) uint8."""
    v = np.ascontiguousarray(vmap, dtype=np.float32)
    n = np.ascontiguousarray(nmap, dtype=np.float32)
    h, w = v.shape[:2]
    out = np.zeros((h, w, 4), np.uint8)
    lt = np.asarray(light, dtype=np.float32)
    lib().orc_render_scene(_ptr(v), _ptr(n), w, h, _ptr(lt), _ptr(out))
    return out


def se3_exp(xi) -> np.ndarray:
    x = np.ascontiguousarray(np.asarray(xi, dtype=np.float64))
    out = np.zeros(12)
    lib("f64").orc_se3_exp(_ptr(x), _ptr(out))
    T = np.eye(4)
    T[:3, :4] = out.reshape(3, 4)
    return T


def ldlt_solve(A, b) -> np.ndarray:
    a = np.ascontiguousarray(np.asarray(A, dtype=np.float64).reshape(36))
    bb = np.ascontiguousarray(np.asarray(b, dtype=np.float64))
    x = np.zeros(6)
    lib("f64").orc_ldlt_solve6(_ptr(a), _ptr(bb), _ptr(x))
    return x
