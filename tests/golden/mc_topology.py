"""Marching-cubes topology of a triangle table, and the fixture that pins it.

The reference's table (RGBDFusion/utils/TriangleTable.h:8-279, edgeTable and
triTable) is not copied into this project: the table used here is generated
from cube topology.  What a table must share with the reference for the
surfaces to be the same is its topology, per case index:

  * the edge mask (which cube edges carry a vertex),
  * the number of triangles,
  * the oriented iso-polygons: the triangles of a case, glued along their
    shared edges, form polygons whose boundary loops (directed cycles of edge
    indices) fix where the surface runs, how ambiguous faces are resolved and
    which side faces inward.

Only the choice of diagonals inside a polygon is left open.  ``topology``
computes these three from any table; ``digest`` reduces them to SHA-256 sums,
which ``tests/golden/mc_topology.json`` holds for the reference's table, so
the pin travels without the reference.

Usage (regenerates the fixture from the reference's source file):
    python -m tests.golden.mc_topology /path/to/RGBDFusion/utils/TriangleTable.h
"""
from __future__ import annotations

import hashlib
import json
import re
import sys
from collections import Counter
from pathlib import Path

FIXTURE = Path(__file__).resolve().parent / "mc_topology.json"


def parse_reference_table(path) -> tuple[list[int], list[list[tuple[int, int, int]]]]:
    """edgeTable (256 ints) and triTable (256 triangle lists) of a C header
    written as the reference writes its table."""
    txt = Path(path).read_text()
    e0 = txt.index("edgeTable")
    t0 = txt.index("triTable")
    edge = [int(x, 0) for x in re.findall(r"0x[0-9a-fA-F]+|\b\d+\b", txt[txt.index("{", e0):t0])][:256]
    body = txt[txt.index("{", t0):]
    nums = [int(x) for x in re.findall(r"-?\d+", body)][: 256 * 16]
    if len(edge) != 256 or len(nums) != 256 * 16:
        raise ValueError(f"{path}: not a 256-case marching-cubes table")
    tris = []
    for c in range(256):
        row = nums[16 * c: 16 * c + 16]
        tris.append(triangles(row))
    return edge, tris


def triangles(row) -> list[tuple[int, int, int]]:
    """Triangles of one table row (edge-index triples up to the first -1)."""
    out = []
    for i in range(0, len(row) - 2, 3):
        if row[i] < 0:
            break
        out.append((int(row[i]), int(row[i + 1]), int(row[i + 2])))
    return out


def boundary_loops(tris) -> list[tuple[int, ...]]:
    """Directed boundary loops of a case's triangles, each rotated to start at
    its smallest edge index, sorted.  A directed edge (a, b) of a triangle is on
    the boundary when no triangle of the case has (b, a)."""
    directed = Counter()
    for t in tris:
        for k in range(3):
            directed[(t[k], t[(k + 1) % 3])] += 1
    succ = {}
    for (a, b), n in directed.items():
        if (b, a) in directed:
            continue
        if n != 1 or a in succ:
            raise ValueError(f"non-manifold triangle set {tris}")
        succ[a] = b
    loops = []
    seen = set()
    for s in sorted(succ):
        if s in seen:
            continue
        loop, x = [], s
        while x not in seen:
            seen.add(x)
            loop.append(x)
            x = succ[x]
        i = loop.index(min(loop))
        loops.append(tuple(loop[i:] + loop[:i]))
    return sorted(loops)


def topology(edge, tris) -> dict:
    """Per-case edge masks, triangle counts and oriented boundary loops."""
    return {
        "edge": [int(e) for e in edge],
        "count": [len(t) for t in tris],
        "loops": [[list(l) for l in boundary_loops(t)] for t in tris],
    }


def _sha(obj) -> str:
    return hashlib.sha256(json.dumps(obj, separators=(",", ":")).encode()).hexdigest()


def digest(topo: dict) -> dict:
    return {k: _sha(v) for k, v in topo.items()}


def main(argv) -> None:
    if len(argv) != 2:
        raise SystemExit(__doc__)
    edge, tris = parse_reference_table(argv[1])
    out = {
        "source": "RGBDFusion/utils/TriangleTable.h:8-279 (edgeTable, triTable) of the reference",
        "made_by": "python -m tests.golden.mc_topology <path of that file>",
        "sha256": digest(topology(edge, tris)),
        "cases_with_polygons": sum(1 for t in tris if t),
        "triangles": sum(len(t) for t in tris),
    }
    FIXTURE.write_text(json.dumps(out, indent=1) + "\n")
    print(json.dumps(out, indent=1))


if __name__ == "__main__":
    main(sys.argv)
