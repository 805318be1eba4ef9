"""Build recipe of the CPU oracle (test infrastructure only).

Two shared libraries from the same C sources:

* ``_build/liboracle64.so`` — the checker: ``real`` = double, FP32-exact
  discrete decisions (``-ffp-contract=off``), sums in a fixed order.
* ``_build/liboracle32.so`` — the timed CPU baseline: ``real`` = float,
  OpenMP over all host cores (parallel sums where the checker keeps a fixed
  order).

The reference's own dense path is not built here: it needs OpenCV with its
CUDA modules, Eigen, Sophus, g2o and Pangolin, none of which is installed,
so ``oracle/_ref`` stays empty.
"""
from __future__ import annotations

import os
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
SOURCES = ["oracle_map.c", "oracle_track.c"]
LIB64 = BUILD / "liboracle64.so"
LIB32 = BUILD / "liboracle32.so"

_COMMON = ["-std=c11", "-fPIC", "-shared", "-ffp-contract=off", "-fopenmp", "-D_GNU_SOURCE"]


def _stale(out: Path, inputs: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(p.stat().st_mtime > t for p in inputs)


def _compile(out: Path, extra: list[str]) -> None:
    cc = os.environ.get("CC", "gcc")
    tmp = out.with_suffix(".so.tmp")
    cmd = [cc, *_COMMON, *extra, *(str(HERE / s) for s in SOURCES), "-o", str(tmp), "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, out)


def build(force: bool = False) -> tuple[Path, Path]:
    BUILD.mkdir(parents=True, exist_ok=True)
    inputs = [HERE / s for s in SOURCES] + [HERE / "oracle.h", Path(__file__)]
    if force or _stale(LIB64, inputs):
        _compile(LIB64, ["-O2", "-DORACLE_REAL=double"])
    if force or _stale(LIB32, inputs):
        _compile(LIB32, ["-O3", "-DORACLE_REAL=float", "-DORACLE_PARALLEL_SUMS=1"])
    return LIB64, LIB32


if __name__ == "__main__":
    print(build(force=True))
