"""In-tree build of the native libraries.

* ``libyas_gb300.so`` — the CUDA kernels and the C ABI of ``include/yas.h``,
  compiled for sm_103a only (one ``-gencode``), one nvcc process per
  translation unit in parallel, linked with the static CUDA runtime.
* ``libyas_synth.so`` — the seeded synthetic RGB-D scene generator (host C).

Outputs go to ``yetanotherslam_gb300/_build/`` (git-ignored).  Everything is
rebuilt from source on the machine that runs it; a build is skipped only when
every output is newer than every input.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
INCLUDE = ROOT / "include"

CUDA_SOURCES = ["map.cu", "raycast.cu", "mesh.cu", "imgproc.cu", "tracker.cu", "capi.cu", "session.cu", "server.cu", "fusion.cu", "batch.cu", "canvas.cu"]
NVCC_FLAGS = [
    "-gencode", "arch=compute_103a,code=sm_103a",
    "-lineinfo", "-O3", "-std=c++17",
    "--expt-relaxed-constexpr",
    "-Xcompiler", "-fPIC,-fvisibility=hidden,-ffp-contract=off,-O2",
    "-I", str(INCLUDE),
]

LIB = BUILD / "libyas_gb300.so"
SYNTH = BUILD / "libyas_synth.so"


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libyas_gb300")


def _stale(out: Path, inputs: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(p.stat().st_mtime > t for p in inputs)


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def build_cuda(verbose: bool = False, force: bool = False) -> Path:
    BUILD.mkdir(parents=True, exist_ok=True)
    headers = sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + [INCLUDE / "yas.h"]
    srcs = [CSRC / s for s in CUDA_SOURCES]
    if not force and not _stale(LIB, srcs + headers + [Path(__file__)]):
        return LIB
    nvcc = _nvcc()
    objs = []
    jobs = []
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        for s in srcs:
            o = BUILD / (s.stem + ".o")
            objs.append(o)
            cmd = [nvcc, *NVCC_FLAGS, "-c", str(s), "-o", str(o)]
            if verbose:
                cmd.insert(1, "-Xptxas=-v")
            jobs.append(ex.submit(_run, cmd))
        for j in jobs:
            j.result()
    tmp = LIB.with_suffix(".so.tmp")
    _run([nvcc, "-shared", "-gencode", "arch=compute_103a,code=sm_103a", "-cudart", "static",
          *map(str, objs), "-o", str(tmp), "-Xlinker", "--exclude-libs,ALL"])
    os.replace(tmp, LIB)
    return LIB


def build_synth(force: bool = False) -> Path:
    BUILD.mkdir(parents=True, exist_ok=True)
    src = CSRC / "synth.c"
    if not force and not _stale(SYNTH, [src, Path(__file__)]):
        return SYNTH
    cc = os.environ.get("CC", "gcc")
    tmp = SYNTH.with_suffix(".so.tmp")
    _run([cc, "-O2", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
          str(src), "-o", str(tmp), "-lm"])
    os.replace(tmp, SYNTH)
    return SYNTH


def build_all(verbose: bool = False, force: bool = False) -> None:
    build_synth(force=force)
    build_cuda(verbose=verbose, force=force)


if __name__ == "__main__":
    build_all(verbose="-v" in sys.argv, force="-f" in sys.argv)
    print(LIB)
