"""Python mirror of YetAnotherSLAM's RGBDFusion classes over the C ABI.

Class and method names follow the reference (RGBDFusion/include/VoxelMap.h,
RayTraceEngine.h, MeshEngine.h, RGBDTracking.h) so code written against the
reference reads the same.  Images are numpy arrays (host) or CUDA tensors
(device, anything exposing ``__cuda_array_interface__``); poses are 4x4 (or
3x4) numpy arrays in the reference's conventions (``Tcm``: camera -> map).
Every call goes to ``libyas_gb300``; there is no Python fallback.
"""
from __future__ import annotations

import ctypes as C
import math
import sys

import numpy as np

from . import _lib as L

VOXEL_F32, VOXEL_F16, VOXEL_S24, VOXEL_S16 = L.VOXEL_F32, L.VOXEL_F16, L.VOXEL_S24, L.VOXEL_S16
TRACK_RGB, TRACK_ICP, TRACK_RGBD = L.TRACK_RGB, L.TRACK_ICP, L.TRACK_RGBD


def _intr(K) -> L.Intrinsics:
    K = np.asarray(K, dtype=np.float64)
    if K.shape == (3, 3):
        fx, fy, cx, cy = K[0, 0], K[1, 1], K[0, 2], K[1, 2]
    else:
        fx, fy, cx, cy = K.reshape(4)
    return L.Intrinsics(fx, fy, cx, cy)


def _device_info(a):
    """(pointer, pitch_bytes, on_device, object to keep alive) of an image argument."""
    torch = sys.modules.get("torch")
    if torch is not None and isinstance(a, torch.Tensor) and a.is_cuda:
        # the tensor's own accessors: building its __cuda_array_interface__
        # dict costs several microseconds per image and frame
        if a.requires_grad:
            a = a.detach()
        es = a.element_size()
        row = math.prod(a.shape[1:]) * es if a.is_contiguous() else a.stride(0) * es
        return a.data_ptr(), row, 1, a
    cai = getattr(a, "__cuda_array_interface__", None)
    if cai is not None:
        ptr = cai["data"][0]
        shape = cai["shape"]
        strides = cai.get("strides")
        itemsize = np.dtype(cai["typestr"]).itemsize
        row = strides[0] if strides else math.prod(shape[1:]) * itemsize
        return ptr, row, 1, a
    arr = np.ascontiguousarray(a)
    return arr.ctypes.data, arr.strides[0], 0, arr


class DeviceArray:
    """Borrowed view of library-owned device memory (``__cuda_array_interface__``)."""

    def __init__(self, ptr: int, shape, typestr: str, owner=None):
        self.__cuda_array_interface__ = {"shape": tuple(shape), "typestr": typestr, "data": (ptr, False),
                                         "version": 3, "strides": None}
        self._owner = owner

    def torch(self):
        import torch
        return torch.as_tensor(self, device="cuda")

    def numpy(self) -> np.ndarray:
        return self.torch().cpu().numpy()


class MapStruct:
    """MapStruct (VoxelMap.h:32-144): one voxel-hash TSDF submap."""

    def __init__(self, K, stream: int | None = None):
        self.K = _intr(K)
        self.handle = C.c_void_p()
        self._stream = stream
        self.voxelSize = 0.0
        self.truncationDist = 0.0

    # MapStruct::create(hashTableSize, bucketSize, voxelBlockSize, voxelSize, truncationDist)
    def create(self, hashTableSize: int, bucketSize: int, voxelBlockSize: int, voxelSize: float,
               truncationDist: float, voxel_format: int = VOXEL_F32) -> None:
        if voxel_format == VOXEL_F32:
            L.call("yas_map_create_ref", C.byref(self.handle), hashTableSize, bucketSize, voxelBlockSize,
                   voxelSize, truncationDist, C.byref(self.K), self._stream)
        else:
            slots = 1
            while slots < max(hashTableSize, 2 * voxelBlockSize):
                slots <<= 1
            self.create_config(slots, voxelBlockSize, voxelSize, truncationDist, voxel_format)
        self.voxelSize, self.truncationDist = voxelSize, truncationDist

    def create_config(self, hash_slots: int, max_blocks: int, voxel_size: float, trunc_dist: float,
                      voxel_format: int = VOXEL_F16, depth_min: float = 0.1, depth_max: float = 3.0,
                      max_weight: int = 255) -> None:
        cfg = L.MapConfig()
        L.call("yas_map_config_default", C.byref(cfg), hash_slots, max_blocks, voxel_size, trunc_dist,
               voxel_format)
        cfg.depth_min, cfg.depth_max, cfg.max_weight = depth_min, depth_max, max_weight
        L.call("yas_map_create", C.byref(self.handle), C.byref(cfg), C.byref(self.K), self._stream)
        self.voxelSize, self.truncationDist = voxel_size, trunc_dist

    def Release(self) -> None:
        if self.handle:
            L.call("yas_map_destroy", self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.Release()
        except Exception:
            pass

    def Reset(self) -> None:
        L.call("yas_map_reset", self.handle)

    def Empty(self) -> bool:
        out = C.c_int()
        L.call("yas_map_empty", self.handle, C.byref(out))
        return bool(out.value)

    # MapStruct::Fuse(GpuMat depth, SE3d Tcm)
    def Fuse(self, depth, Tcm) -> None:
        ptr, pitch, dev, keep = _device_info(depth)
        h, w = depth.shape[:2]
        L.call("yas_map_fuse_depth", self.handle, ptr, w, h, pitch, dev, C.byref(L.pose_from(Tcm)))

    # MapStruct::Fuse(MapStruct*): fuse another submap into this one (src is left empty)
    def FuseMap(self, src: "MapStruct") -> None:
        L.call("yas_map_fuse_map", self.handle, src.handle)

    # MapStruct::Swap(MapStruct*): exchange storage; each keeps its pose and flag
    def Swap(self, other: "MapStruct") -> None:
        L.call("yas_map_swap", self.handle, other.handle)

    # MapStruct::Reserve(hashTableSize, bucketSize, voxelBlockSize)
    def Reserve(self, hash_slots: int, max_blocks: int) -> None:
        L.call("yas_map_reserve", self.handle, hash_slots, max_blocks)

    # MapStruct::SaveToFile / ReadFromFile
    def SaveToFile(self, path: str) -> None:
        L.call("yas_map_save", self.handle, str(path).encode())

    def ReadFromFile(self, path: str) -> None:
        L.call("yas_map_load", self.handle, str(path).encode())

    def Defuse(self, depth, Tcm) -> None:
        """Removes the observation of `depth` at Tcm (re-integration after a pose correction)."""
        ptr, pitch, dev, keep = _device_info(depth)
        h, w = depth.shape[:2]
        L.call("yas_map_defuse_depth", self.handle, ptr, w, h, pitch, dev, C.byref(L.pose_from(Tcm)))

    def CheckNumVisibleBlocks(self, cols: int, rows: int, Tcm) -> int:
        out = C.c_uint()
        L.call("yas_map_check_visible", self.handle, cols, rows, C.byref(L.pose_from(Tcm)), C.byref(out))
        return out.value

    def GetNumVisibleBlocks(self) -> int:
        out = C.c_uint()
        L.call("yas_map_num_visible", self.handle, C.byref(out))
        return out.value

    def ResetNumVisibleBlocks(self) -> None:
        L.call("yas_map_reset_visible", self.handle)

    def num_allocated(self) -> int:
        out = C.c_uint()
        L.call("yas_map_num_allocated", self.handle, C.byref(out))
        return out.value

    def take_errors(self) -> int:
        out = C.c_uint()
        L.call("yas_map_take_errors", self.handle, C.byref(out))
        return out.value

    def export(self):
        """(coords (n,3) int32, sdf (n,512) float32, weight (n,512) float32) in pool order."""
        n = C.c_uint()
        L.call("yas_map_export", self.handle, None, None, None, 0, C.byref(n))
        cnt = n.value
        coords = np.zeros((cnt, 3), dtype=np.int32)
        sdf = np.zeros((cnt, 512), dtype=np.float32)
        wt = np.zeros((cnt, 512), dtype=np.float32)
        if cnt:
            L.call("yas_map_export", self.handle, coords.ctypes.data, sdf.ctypes.data, wt.ctypes.data, cnt,
                   C.byref(n))
        return coords, sdf, wt

    def import_blocks(self, coords, sdf, wt) -> None:
        c = np.ascontiguousarray(coords, dtype=np.int32)
        s = np.ascontiguousarray(sdf, dtype=np.float32)
        w = np.ascontiguousarray(wt, dtype=np.float32)
        L.call("yas_map_import", self.handle, c.ctypes.data, s.ctypes.data, w.ctypes.data, c.shape[0])

    def visible_coords(self) -> np.ndarray:
        n = C.c_uint()
        L.call("yas_map_export_visible", self.handle, None, 0, C.byref(n))
        out = np.zeros((n.value, 3), dtype=np.int32)
        if n.value:
            L.call("yas_map_export_visible", self.handle, out.ctypes.data, n.value, C.byref(n))
        return out

    def GetPose(self) -> np.ndarray:
        p = L.Pose()
        L.call("yas_map_get_pose", self.handle, C.byref(p))
        return L.pose_to(p)

    def SetPose(self, Tcw) -> None:
        L.call("yas_map_set_pose", self.handle, C.byref(L.pose_from(Tcw)))

    def SetActiveFlag(self, flag: bool) -> None:
        L.call("yas_map_set_active", self.handle, int(flag))

    def isActive(self) -> bool:
        out = C.c_int()
        L.call("yas_map_is_active", self.handle, C.byref(out))
        return bool(out.value)

    def Hibernate(self) -> None:
        L.call("yas_map_hibernate", self.handle)

    def ReActivate(self) -> None:
        L.call("yas_map_reactivate", self.handle)

    @property
    def mbInHibernation(self) -> bool:
        out = C.c_int()
        L.call("yas_map_is_hibernated", self.handle, C.byref(out))
        return bool(out.value)


class RayTraceEngine:
    """RayTraceEngine (RayTraceEngine.h:11-49)."""

    def __init__(self, w: int, h: int, K, stream: int | None = None):
        self.w, self.h = w, h
        self.handle = C.c_void_p()
        L.call("yas_raycaster_create", C.byref(self.handle), w, h, C.byref(_intr(K)), stream)

    def __del__(self):
        try:
            if self.handle:
                L.call("yas_raycaster_destroy", self.handle)
                self.handle = C.c_void_p()
        except Exception:
            pass

    def RayTrace(self, pMapStruct: MapStruct, Tcm) -> None:
        L.call("yas_raycaster_raycast", self.handle, pMapStruct.handle, C.byref(L.pose_from(Tcm)))

    def GetVMap(self) -> DeviceArray:
        ptr = C.c_void_p()
        pitch = C.c_int()
        L.call("yas_raycaster_vmap", self.handle, C.byref(ptr), C.byref(pitch))
        return DeviceArray(ptr.value, (self.h, self.w, 4), "<f4", self)

    def GetDepth(self) -> np.ndarray:
        out = np.zeros((self.h, self.w), dtype=np.float32)
        L.call("yas_raycaster_depth", self.handle, out.ctypes.data, out.strides[0], 0)
        return out

    def GetNumVisibleBlock(self) -> int:
        out = C.c_uint()
        L.call("yas_raycaster_num_visible", self.handle, C.byref(out))
        return out.value

    def zrange(self):
        zw, zh = (self.w + 7) // 8, (self.h + 7) // 8
        zn = np.zeros((zh, zw), dtype=np.float32)
        zf = np.zeros((zh, zw), dtype=np.float32)
        L.call("yas_raycaster_zrange", self.handle, zn.ctypes.data, zf.ctypes.data)
        return zn, zf


class MeshEngine:
    """MeshEngine (MeshEngine.h:8-24)."""

    def __init__(self, MaxNumTriangle: int, stream: int | None = None):
        self.handle = C.c_void_p()
        L.call("yas_mesher_create", C.byref(self.handle), MaxNumTriangle, stream)
        self.N = 0

    def __del__(self):
        try:
            if self.handle:
                L.call("yas_mesher_destroy", self.handle)
                self.handle = C.c_void_p()
        except Exception:
            pass

    def Meshify(self, pMapStruct: MapStruct):
        """Returns (points (n,9), normals (n,9), cases (n,), cube_xyz (n,3)); N = 9 n as the reference."""
        n = C.c_uint()
        code = L.load().yas_mesher_meshify(self.handle, pMapStruct.handle, C.byref(n))
        if code not in (L.YAS_OK, 8):
            L.check(code, "yas_mesher_meshify")
        cnt = n.value
        pts = np.zeros((cnt, 9), dtype=np.float32)
        nrm = np.zeros((cnt, 9), dtype=np.float32)
        cases = np.zeros(cnt, dtype=np.int32)
        cube = np.zeros((cnt, 3), dtype=np.int32)
        if cnt:
            L.call("yas_mesher_copy", self.handle, pts.ctypes.data, nrm.ctypes.data, cnt)
            L.call("yas_mesher_copy_cases", self.handle, cases.ctypes.data, cube.ctypes.data, cnt)
        self.N = 9 * cnt
        self.overflow = code == 8
        return pts, nrm, cases, cube


class RGBDTracking:
    """RGBDTracking (RGBDTracking.h:9-107)."""

    def __init__(self, w: int, h: int, K, bRGB: bool = True, bIcp: bool = True, num_levels: int = 5,
                 iterations=(10, 5, 3, 3, 3), stream: int | None = None):
        K = np.asarray(K, dtype=np.float64).reshape(3, 3)
        mode = (TRACK_RGB if bRGB else 0) | (TRACK_ICP if bIcp else 0)
        self.w, self.h, self.levels = w, h, num_levels
        it = (C.c_int * 5)(*(list(iterations) + [0] * 5)[:5])
        Kc = (C.c_double * 9)(*K.reshape(-1))
        self.handle = C.c_void_p()
        L.call("yas_tracker_create", C.byref(self.handle), w, h, Kc, num_levels, it, mode, stream)

    def __del__(self):
        try:
            if self.handle:
                L.call("yas_tracker_destroy", self.handle)
                self.handle = C.c_void_p()
        except Exception:
            pass

    def _img(self, fn: str, img):
        ptr, pitch, dev, keep = _device_info(img)
        L.call(fn, self.handle, ptr, pitch, dev)

    def SetReferenceImage(self, imGray) -> None:
        self._img("yas_tracker_set_reference_image", imGray)

    def SetTrackingImage(self, imGray) -> None:
        self._img("yas_tracker_set_tracking_image", imGray)

    def SetReferenceDepth(self, imDepth) -> None:
        self._img("yas_tracker_set_reference_depth", np.asarray(imDepth, dtype=np.float32)
                  if not hasattr(imDepth, "__cuda_array_interface__") else imDepth)

    def SetTrackingDepth(self, imDepth) -> None:
        self._img("yas_tracker_set_tracking_depth", np.asarray(imDepth, dtype=np.float32)
                  if not hasattr(imDepth, "__cuda_array_interface__") else imDepth)

    def SetReferenceModel(self, vmap) -> None:
        ptr, pitch, dev, keep = _device_info(vmap)
        if not dev:
            raise ValueError("SetReferenceModel expects a device vertex map")
        L.call("yas_tracker_set_reference_model", self.handle, ptr, pitch)

    def GetTransform(self, init=None, bSwapBuffer: bool = False) -> np.ndarray:
        out = L.Pose()
        init = np.eye(4) if init is None else init
        code = L.load().yas_tracker_get_transform(self.handle, C.byref(L.pose_from(init)), int(bSwapBuffer),
                                                  C.byref(out))
        if code not in (L.YAS_OK, 6):
            L.check(code, "yas_tracker_get_transform")
        return L.pose_to(out)

    def SwapFrameBuffer(self) -> None:
        L.call("yas_tracker_swap_frame_buffer", self.handle)

    def set_schedule(self, fused: bool) -> None:
        """Whole schedule in one cooperative launch (True) or two launches per iteration."""
        L.call("yas_tracker_set_schedule", self.handle, int(fused))

    def set_reduction(self, compensated: bool) -> None:
        """Compensated FP32 sums with double-float totals (True) or plain FP32 sums (False)."""
        L.call("yas_tracker_set_reduction", self.handle, int(compensated))

    def check_wait_limit(self) -> int:
        """Runs the fused schedule with one of two CTAs missing, so its bounded
        waits run out (about 1 s); returns the status it reports
        (YAS_ERR_TIMEOUT, 12, when the limit works)."""
        out = C.c_int()
        L.call("yas_tracker_check_wait_limit", self.handle, C.byref(out))
        return out.value

    def IsTrackingGood(self) -> bool:
        out = C.c_int()
        L.call("yas_tracker_is_good", self.handle, C.byref(out))
        return bool(out.value)

    def compute_step(self, level: int, T):
        H = np.zeros(36)
        b = np.zeros(6)
        st = np.zeros(4)
        L.call("yas_tracker_compute_step", self.handle, level, C.byref(L.pose_from(T)), H.ctypes.data,
               b.ctypes.data, st.ctypes.data)
        return H.reshape(6, 6), b, st

    def last_solve(self):
        """(H 6x6, b, update x, estimate 4x4) of the last Gauss-Newton solve."""
        H = np.zeros(36)
        b = np.zeros(6)
        x = np.zeros(6)
        est = L.Pose()
        L.call("yas_tracker_last_solve", self.handle, H.ctypes.data, b.ctypes.data, x.ctypes.data, C.byref(est))
        return H.reshape(6, 6), b, x, L.pose_to(est)

    def level_buffer(self, level: int, which: int) -> DeviceArray:
        ptr = C.c_void_p()
        w, h, p = C.c_int(), C.c_int(), C.c_int()
        L.call("yas_tracker_level_buffer", self.handle, level, which, C.byref(ptr), C.byref(w), C.byref(h),
               C.byref(p))
        shape = (h.value, w.value, 4) if which in (4, 5, 8, 9) else (h.value, w.value)
        return DeviceArray(ptr.value, shape, "<f4", self)


def session_config(width: int, height: int, K, hash_slots: int = 1 << 20, max_blocks: int = 1 << 17,
                   voxel_size: float = 0.008, trunc_dist: float | None = None, voxel_format: int = VOXEL_F16,
                   num_levels: int = 3, iterations=(10, 5, 3, 3, 3), mode: int = TRACK_RGBD,
                   depth_scale: float = 0.001, use_graph: bool = True, fused_schedule: bool = True) -> L.SessionConfig:
    """yas_session_config of a session (the reference's constants unless given)."""
    cfg = L.SessionConfig()
    trunc = 3 * voxel_size if trunc_dist is None else trunc_dist
    L.call("yas_session_config_default", C.byref(cfg), width, height, C.byref(_intr(K)), hash_slots,
           max_blocks, voxel_size, trunc, voxel_format)
    cfg.num_levels = num_levels
    for i in range(5):
        cfg.iterations[i] = list(iterations)[i] if i < len(iterations) else 0
    cfg.mode = mode
    cfg.depth_scale = depth_scale
    cfg.use_graph = int(use_graph)
    cfg.fused_schedule = int(fused_schedule)
    return cfg


class Session:
    """One SLAM session's per-frame dense pipeline (Tracking::TrackRGBD's dense calls)."""

    def __init__(self, width: int, height: int, K, hash_slots: int = 1 << 20, max_blocks: int = 1 << 17,
                 voxel_size: float = 0.008, trunc_dist: float | None = None, voxel_format: int = VOXEL_F16,
                 num_levels: int = 3, iterations=(10, 5, 3, 3, 3), mode: int = TRACK_RGBD,
                 depth_scale: float = 0.001, use_graph: bool = True, stream: int | None = None,
                 fused_schedule: bool = True):
        cfg = session_config(width, height, K, hash_slots, max_blocks, voxel_size, trunc_dist, voxel_format,
                             num_levels, iterations, mode, depth_scale, use_graph, fused_schedule)
        self.cfg = cfg
        self.width, self.height = width, height
        self.handle = C.c_void_p()
        L.call("yas_session_create", C.byref(self.handle), C.byref(cfg), stream)
        # per-frame calls, looked up once
        lib = L.load()
        self._submit_fn, self._wait_fn = lib.yas_session_submit, lib.yas_session_wait
        self._pose, self._status = L.Pose(), C.c_int()

    def close(self):
        if self.handle:
            L.call("yas_session_destroy", self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, rgb, depth) -> None:
        rp, _, rdev, k1 = _device_info(rgb)
        dp, _, ddev, k2 = _device_info(depth)
        if rdev != ddev:
            raise ValueError("rgb and depth must both be host or both be device arrays")
        self._keep = (k1, k2)
        L.check(self._submit_fn(self.handle, rp, dp, rdev), "yas_session_submit")

    def wait(self):
        L.check(self._wait_fn(self.handle, C.byref(self._pose), C.byref(self._status)), "yas_session_wait")
        return self._status.value, L.pose_to(self._pose)

    def process(self, rgb, depth):
        """Tracks and fuses one frame; returns (status, Tcm 4x4)."""
        self.submit(rgb, depth)
        return self.wait()

    @property
    def stream(self) -> int:
        return L.load().yas_session_stream(self.handle) or 0

    def kernels_per_frame(self) -> int:
        out = C.c_int()
        L.call("yas_session_kernels_per_frame", self.handle, C.byref(out))
        return out.value

    def map(self) -> MapStruct:
        h = C.c_void_p()
        L.call("yas_session_map", self.handle, C.byref(h))
        m = MapStruct.__new__(MapStruct)
        m.handle = h
        m.K = self.cfg.K
        m._stream = None
        m.voxelSize = self.cfg.map.voxel_size
        m.truncationDist = self.cfg.map.trunc_dist
        m._borrowed = True
        m.Release = lambda: None
        return m

    def new_submap(self) -> MapStruct:
        """CreateNewKeyFrame's submap switch: returns the previous submap (owned by the caller)."""
        h = C.c_void_p()
        L.call("yas_session_new_submap", self.handle, C.byref(h))
        m = MapStruct.__new__(MapStruct)
        m.handle = h
        m.K = self.cfg.K
        m._stream = None
        m.voxelSize = self.cfg.map.voxel_size
        m.truncationDist = self.cfg.map.trunc_dist
        return m

    def set_reduction(self, compensated: bool) -> None:
        """Gauss-Newton totals of the session's tracker: compensated FP32 with FP64
        totals (True, the default) or plain FP32 sums (False)."""
        h = C.c_void_p()
        L.call("yas_session_tracker", self.handle, C.byref(h))
        L.call("yas_tracker_set_reduction", h, int(compensated))


class Canvas:
    """Headless drawing of submap meshes (MapDrawer's mesh program) into an RGBA image."""

    def __init__(self, width: int, height: int, K, stream: int | None = None):
        self.w, self.h = width, height
        self.handle = C.c_void_p()
        L.call("yas_canvas_create", C.byref(self.handle), width, height, C.byref(_intr(K)), stream)

    def __del__(self):
        try:
            if self.handle:
                L.call("yas_canvas_destroy", self.handle)
                self.handle = C.c_void_p()
        except Exception:
            pass

    def clear(self) -> None:
        L.call("yas_canvas_clear", self.handle)

    def draw_mesh(self, mesher: MeshEngine, Tmw, Tcw) -> None:
        """The mesher's last mesh, placed by Tmw (submap -> world) and seen from Tcw (world -> camera)."""
        L.call("yas_canvas_draw_mesh", self.handle, mesher.handle, C.byref(L.pose_from(Tmw)), C.byref(L.pose_from(Tcw)))

    def draw_triangles(self, points, normals, Tmw, Tcw) -> None:
        p = np.ascontiguousarray(points, dtype=np.float32)
        n = np.ascontiguousarray(normals, dtype=np.float32)
        L.call("yas_canvas_draw_triangles", self.handle, p.ctypes.data, n.ctypes.data, p.shape[0], 0,
               C.byref(L.pose_from(Tmw)), C.byref(L.pose_from(Tcw)))

    def read(self):
        """(rgba (h, w, 4) uint8, depth (h, w) float32 metres, 0 where empty)."""
        rgba = np.zeros((self.h, self.w, 4), np.uint8)
        depth = np.zeros((self.h, self.w), np.float32)
        L.call("yas_canvas_read", self.handle, rgba.ctypes.data, self.w * 4, depth.ctypes.data, self.w * 4, 0)
        return rgba, depth
