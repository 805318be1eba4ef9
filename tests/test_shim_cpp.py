"""The C++ class layer (include/yas_rgbdfusion.hpp): FullSystem-style code
keeps RGBDFusion's class and method names (VoxelMap.h:32-144,
RayTraceEngine.h:11-49, MeshEngine.h:8-24, RGBDTracking.h:9-107) and links
against libyas_gb300.

tests/cpp/shim_tracking.cpp runs the dense calls of
Tracking::StereoInitialization / TrackRGBD (FullSystem/src/Tracking.cpp:139-197)
and the MapStruct calls of MapDrawer and CreateNewKeyFrame through the header.
Bars: it compiles warning-free and links (CPU); its poses are bit-identical to
the same calls made through the Python class mirror, and every other result
(visible counts, raycast depth, mesh, file round trip, swap, fusion, shading,
hibernation, errors) equals the Python side's or its documented value (GPU).
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np
import pytest

from tests.helpers import pose_error, rel_poses, sequence

ROOT = Path(__file__).resolve().parent.parent
DRIVER = ROOT / "tests" / "cpp" / "shim_tracking.cpp"
FLAGS = ["-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror", "-ffp-contract=off"]


def _compile(out: Path, extra=()) -> Path:
    from yetanotherslam_gb300 import build

    lib_dir = build.LIB.parent
    cmd = ["g++", *FLAGS, *extra, f"-I{ROOT / 'include'}", str(DRIVER), f"-L{lib_dir}", "-lyas_gb300",
           f"-Wl,-rpath,{lib_dir}", "-o", str(out)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


def test_shim_compiles_and_links(native, tmp_path):
    _compile(tmp_path / "shim_tracking")
    # the header alone, without the global names, in its own translation unit
    tu = tmp_path / "tu.cpp"
    tu.write_text('#define YAS_SHIM_NO_GLOBAL_NAMES\n#include "yas_rgbdfusion.hpp"\n'
                  "int main() { yas::shim::SE3d T; return (int)T.inverse().m[0] - 1; }\n")
    r = subprocess.run(["g++", *FLAGS, "-fsyntax-only", f"-I{ROOT / 'include'}", str(tu)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


# --- the C++ SE3d stand-in's arithmetic, operation for operation ----------
def _mul(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    r = np.eye(4)
    for i in range(3):
        for j in range(3):
            r[i, j] = float(a[i, 0]) * float(b[0, j]) + float(a[i, 1]) * float(b[1, j]) + float(a[i, 2]) * float(b[2, j])
        r[i, 3] = (float(a[i, 0]) * float(b[0, 3]) + float(a[i, 1]) * float(b[1, 3]) + float(a[i, 2]) * float(b[2, 3])
                   + float(a[i, 3]))
    return r


def _inv(a: np.ndarray) -> np.ndarray:
    r = np.eye(4)
    r[:3, :3] = a[:3, :3].T
    for i in range(3):
        r[i, 3] = -(float(r[i, 0]) * float(a[0, 3]) + float(r[i, 1]) * float(a[1, 3]) + float(r[i, 2]) * float(a[2, 3]))
    return r


def _seq_sum(v: np.ndarray) -> float:
    v = np.asarray(v, dtype=np.float64).ravel()
    return float(np.cumsum(v)[-1]) if v.size else 0.0


def _parse(path: Path) -> dict:
    out = {}
    for line in path.read_text().splitlines():
        key, *vals = line.split()
        if key == "pose":
            out.setdefault("pose", []).append((int(vals[1]), np.array([float(x) for x in vals[2:]])))
        else:
            out[key] = vals
    return out


@pytest.mark.gpu
def test_shim_tracking_matches_python_classes(cuda, tmp_path):
    from yetanotherslam_gb300 import _lib as L
    from yetanotherslam_gb300 import rgbdfusion as rf
    from yetanotherslam_gb300 import synth

    W, H, n = 320, 240, 10
    fx, fy, cx, cy = synth.intrinsics(W, H)
    seq = sequence(3, n, W, H)
    grays = [synth.gray_of(rgb) for rgb, _, _, _ in seq]
    frames = tmp_path / "frames.bin"
    with open(frames, "wb") as f:
        f.write(np.array([W, H, n], np.int32).tobytes())
        f.write(np.array([fx, fy, cx, cy], np.float32).tobytes())
        for g, (_, _, dm, _) in zip(grays, seq):
            f.write(np.ascontiguousarray(g, np.uint8).tobytes())
            f.write(np.ascontiguousarray(dm, np.float32).tobytes())
    exe = _compile(tmp_path / "shim_tracking")
    out = tmp_path / "out.txt"
    r = subprocess.run([str(exe), str(frames), str(out), str(tmp_path)], capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, (r.stdout, r.stderr, out.read_text() if out.exists() else "")
    got = _parse(out)

    # the same calls through the Python mirror
    K3 = np.array([[fx, 0, cx], [0, fy, cy], [0, 0, 1]], np.float64)
    K4 = np.float32([fx, fy, cx, cy])
    tr = rf.RGBDTracking(W, H, K3, True, True, num_levels=3, iterations=(10, 5, 3))
    rt = rf.RayTraceEngine(W, H, K4)
    me = rf.MeshEngine(1 << 21)
    ms = rf.MapStruct(K4)
    ms.create(1 << 18, 4000, 1 << 15, 0.008, 0.024)
    Tcp = np.eye(4)
    poses = []
    for i, (g, (_, _, dm, _)) in enumerate(zip(grays, seq)):
        st = 0
        if i == 0:
            tr.SetReferenceImage(g)
            tr.SetReferenceDepth(dm)
            ms.Fuse(dm, Tcp)
        else:
            rt.RayTrace(ms, Tcp)
            tr.SetReferenceModel(rt.GetVMap())
            tr.SetTrackingImage(g)
            tr.SetTrackingDepth(dm)
            DT = tr.GetTransform(np.eye(4), True)
            if np.sqrt(DT[0, 3] ** 2 + DT[1, 3] ** 2 + DT[2, 3] ** 2) > 0.1:
                st = 7
            else:
                Tcp = _mul(Tcp, _inv(DT))
                ms.Fuse(dm, Tcp)
        poses.append((st, Tcp.copy()))

    assert len(got["pose"]) == n
    gt = rel_poses(seq)
    for i, ((st_c, Tc), (st_p, Tp)) in enumerate(zip(got["pose"], poses)):
        assert st_c == st_p == 0, i
        assert np.array_equal(Tc, Tp[:3, :4].reshape(-1)), f"frame {i}"
        et, er = pose_error(gt[i], Tp)
        assert et < 0.05 and er < 0.02
    assert got["good"] == ["1"]
    assert int(got["visible"][0]) == ms.GetNumVisibleBlocks() > 0

    rt.RayTrace(ms, Tcp)
    assert [int(x) for x in got["raytracer"]] == [rt.GetNumVisibleBlock(), _num_rendering(L, rt)]
    depth = rt.GetDepth()
    pos = depth[depth > 0]
    assert float(got["depth"][0]) == _seq_sum(pos) and int(got["depth"][1]) == pos.size > 0

    pts, _, _, _ = me.Meshify(ms)
    assert int(got["mesh"][0]) == pts.size > 0 and got["mesh"][1] == "1"
    # same triangles; the pool order (concurrent allocation) and so the soup's
    # order differ between processes, which moves the sum's last bits
    assert abs(float(got["mesh"][2]) - _seq_sum(pts.reshape(-1))) <= 1e-12 * abs(_seq_sum(pts.reshape(-1)))
    assert got["mesh_deleted"] == ["0", "0"]
    assert got["hibernate"] == ["1", "0", "0", "1"]
    na, nb, tz = got["file"]
    assert int(na) == int(nb) == ms.num_allocated() and float(tz) == 1.0
    assert got["swap"] == ["0", "1", "1"]
    assert int(got["fuse_map"][0]) == int(na) and got["fuse_map"][1] == "1"

    vm, nm = tr.level_buffer(0, 8), tr.level_buffer(0, 9)
    img = np.zeros((H, W, 4), np.uint8)
    L.call("yas_render_scene", vm.__cuda_array_interface__["data"][0], nm.__cuda_array_interface__["data"][0], W, H,
           W * 16, None, img.ctypes.data, W * 4, 0, None)
    assert got["render"] == [str(W), str(H), str(int(img.astype(np.uint64).sum()))]
    assert got["raw_depth"] == ["1"]
    assert got["vmap_to_depth"] == ["1"]
    for name in ("curr_image.pfm", "last_image.pfm", "gx.pfm", "gy.pfm"):
        data = (tmp_path / name).read_bytes()
        head = f"Pf\n{W} {H}\n-1.0\n".encode()
        assert data.startswith(head) and len(data) == len(head) + W * H * 4
    assert got["error"] == ["9"]  # YAS_ERR_STATE: the map was never created


def _num_rendering(L, rt) -> int:
    out = C.c_uint()
    L.call("yas_raycaster_num_rendering_blocks", rt.handle, C.byref(out))
    return out.value


# --- FullSystem's own types: the YAS_SHIM_SOPHUS / YAS_SHIM_OPENCV branches --
FS_DRIVER = ROOT / "tests" / "cpp" / "shim_fullsystem.cpp"
STANDIN = ROOT / "tests" / "cpp" / "standin"


def _cuda_root() -> Path:
    import shutil

    nvcc = shutil.which("nvcc")
    return Path(nvcc).resolve().parent.parent if nvcc else Path("/usr/local/cuda")


def _compile_fullsystem(out: Path) -> Path:
    """The FullSystem-typed driver against the header with both reference-type
    branches on, and the stand-in Eigen / Sophus / OpenCV headers (the
    stand-in GpuMat links the CUDA runtime for its copies, as OpenCV does)."""
    from yetanotherslam_gb300 import build

    lib_dir = build.LIB.parent
    cuda = _cuda_root()
    cudalib = cuda / "lib64" if (cuda / "lib64").exists() else cuda / "lib"
    cmd = ["g++", *FLAGS, "-DYAS_SHIM_SOPHUS", "-DYAS_SHIM_OPENCV", f"-I{STANDIN}", f"-I{ROOT / 'include'}",
           f"-I{cuda / 'include'}", str(FS_DRIVER), f"-L{lib_dir}", "-lyas_gb300", f"-L{cudalib}", "-lcudart",
           f"-Wl,-rpath,{lib_dir}", f"-Wl,-rpath,{cudalib}", "-o", str(out)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


def test_fullsystem_typed_shim_compiles_and_links(native, tmp_path):
    """Tracking.cpp's calls with Sophus::SE3d, Eigen::Matrix3f/3d, cv::Mat and
    cv::cuda::GpuMat (VoxelMap.h:32-144, RGBDTracking.h:9-107) compile
    warning-free against the header's YAS_SHIM_SOPHUS and YAS_SHIM_OPENCV
    branches and link against libyas_gb300."""
    _compile_fullsystem(tmp_path / "shim_fullsystem")


@pytest.mark.gpu
def test_fullsystem_typed_shim_tracks_like_python_classes(cuda, tmp_path):
    from yetanotherslam_gb300 import rgbdfusion as rf
    from yetanotherslam_gb300 import synth

    W, H, n = 320, 240, 10
    fx, fy, cx, cy = synth.intrinsics(W, H)
    seq = sequence(3, n, W, H)
    grays = [synth.gray_of(rgb) for rgb, _, _, _ in seq]
    frames = tmp_path / "frames.bin"
    with open(frames, "wb") as f:
        f.write(np.array([W, H, n], np.int32).tobytes())
        f.write(np.array([fx, fy, cx, cy], np.float32).tobytes())
        for g, (_, _, dm, _) in zip(grays, seq):
            f.write(np.ascontiguousarray(g, np.uint8).tobytes())
            f.write(np.ascontiguousarray(dm, np.float32).tobytes())
    exe = _compile_fullsystem(tmp_path / "shim_fullsystem")
    out = tmp_path / "out.txt"
    r = subprocess.run([str(exe), str(frames), str(out)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, (r.stdout, r.stderr, out.read_text() if out.exists() else "")
    got = _parse(out)

    # the same calls through the Python mirror (FullSystem's 5-level tracker,
    # create(5000, 4000, 4500, 0.01, 0.03))
    K3 = np.array([[fx, 0, cx], [0, fy, cy], [0, 0, 1]], np.float64)
    K4 = np.float32([fx, fy, cx, cy])
    tr = rf.RGBDTracking(W, H, K3, True, True)
    rt = rf.RayTraceEngine(W, H, K4)
    me = rf.MeshEngine(1 << 21)
    ms = rf.MapStruct(K4)
    ms.create(5000, 4000, 4500, 0.01, 0.03)
    Tcp = np.eye(4)
    poses = []
    for i, (g, (_, _, dm, _)) in enumerate(zip(grays, seq)):
        st = 0
        if i == 0:
            tr.SetReferenceImage(g)
            tr.SetReferenceDepth(dm)
            ms.Fuse(dm, Tcp)
        else:
            rt.RayTrace(ms, Tcp)
            tr.SetReferenceModel(rt.GetVMap())
            tr.SetTrackingImage(g)
            tr.SetTrackingDepth(dm)
            DT = tr.GetTransform(np.eye(4), True)
            if np.sqrt(DT[0, 3] ** 2 + DT[1, 3] ** 2 + DT[2, 3] ** 2) > 0.1:
                st = 7
            else:
                Tcp = _mul(Tcp, _inv(DT))
                ms.Fuse(dm, Tcp)
        poses.append((st, Tcp.copy()))

    assert len(got["pose"]) == n
    gt = rel_poses(seq)
    for i, ((st_c, Tc), (st_p, Tp)) in enumerate(zip(got["pose"], poses)):
        assert st_c == st_p == 0, i
        assert np.abs(Tc - Tp[:3, :4].reshape(-1)).max() <= 1e-12, f"frame {i}"
        et, er = pose_error(gt[i], Tp)
        assert et < 0.05 and er < 0.02
    assert got["good"] == ["1"]
    depth = rt.GetDepth()
    pos = depth[depth > 0]
    assert float(got["keyframe_depth"][0]) == _seq_sum(pos) and int(got["keyframe_depth"][1]) == pos.size > 0
    pts, _, _, _ = me.Meshify(ms)
    assert int(got["mesh"][0]) == pts.size > 0 and got["mesh"][1] == "1"
    sw = got["switch"]
    assert sw[:2] == ["0", "1"]
    assert np.allclose([float(x) for x in sw[2:]], Tcp[:3, 3], atol=1e-12)
