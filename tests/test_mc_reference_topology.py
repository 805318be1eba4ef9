"""Marching-cubes topology pinned to the reference's own triangle table.

The table here is generated from cube topology (the library's
``build_mc_tables`` and the oracle's independent generator), not copied from
RGBDFusion/utils/TriangleTable.h:8-279.  These tests pin it to that table
(MeshEngine.cu:43-269 indexes it with the same corner and edge numbering):

  * per case index: the edge mask, the triangle count and the oriented
    boundary loops of the iso-polygons are the reference's;
  * against ``tests/golden/mc_topology.json`` (SHA-256 of those three lists
    made from the reference's file by ``tests/golden/mc_topology.py``), which
    runs everywhere;
  * against the reference's file itself, parsed at test time, when the
    reference tree is present (skipped otherwise), with per-case messages.

Diagonals inside a polygon are not pinned: the reference fans many of its
polygons from vertices that follow no order of the edge indices and splits
40 of its hexagons without a common apex, a choice made case by case in its
table, while the generator here fans every loop from its lowest edge.  The
vertices (edge crossings) and the polygon outlines are the same.
"""
from __future__ import annotations

import json
import os
from pathlib import Path

import numpy as np
import pytest

import oracle
from tests.golden import mc_topology as mt

REFERENCE_TABLE = Path(os.environ.get("YAS_REFERENCE_ROOT", "/root/reference")) / "RGBDFusion/utils/TriangleTable.h"


def _generated():
    """(edge, triangle lists) of the oracle's generator and of the library's."""
    out = []
    edge, tri, cnt = oracle.mc_tables()
    out.append(("oracle", edge, [mt.triangles(tri[c]) for c in range(256)], cnt))
    return out


def _library_tables(native):
    edge = np.zeros(256, np.uint16)
    tri = np.zeros((256, 31), np.int8)
    cnt = np.zeros(256, np.uint8)
    native.yas_mc_tables(edge.ctypes.data, tri.ctypes.data, cnt.ctypes.data)
    return ("library", edge, [mt.triangles(tri[c]) for c in range(256)], cnt)


def test_generated_topology_matches_reference_fixture(native):
    fx = json.loads(mt.FIXTURE.read_text())
    for name, edge, tris, cnt in _generated() + [_library_tables(native)]:
        assert [len(t) for t in tris] == [int(c) for c in cnt], name
        d = mt.digest(mt.topology(edge, tris))
        for k in ("edge", "count", "loops"):
            assert d[k] == fx["sha256"][k], f"{name}: {k} differs from the reference table's"
        assert sum(len(t) for t in tris) == fx["triangles"]


def test_generated_topology_matches_reference_source():
    if not REFERENCE_TABLE.exists():
        pytest.skip("the reference tree is not on this machine")
    r_edge, r_tris = mt.parse_reference_table(REFERENCE_TABLE)
    ref = mt.topology(r_edge, r_tris)
    # the committed fixture was made from this file
    assert mt.digest(ref) == json.loads(mt.FIXTURE.read_text())["sha256"]
    _, edge, tris, _ = _generated()[0]
    gen = mt.topology(edge, tris)
    for c in range(256):
        assert gen["edge"][c] == ref["edge"][c], f"case {c}: edge mask"
        assert gen["count"][c] == ref["count"][c], f"case {c}: triangle count"
        assert gen["loops"][c] == ref["loops"][c], f"case {c}: polygons {gen['loops'][c]} vs {ref['loops'][c]}"
    # how far the diagonals agree: cases whose triangle sets are equal up to
    # the rotation of each triangle's vertex list (recorded, not a bar)
    def canon(t):
        i = t.index(min(t))
        return t[i:] + t[:i]

    same = sum(sorted(map(canon, a)) == sorted(map(canon, b)) for a, b in zip(tris, r_tris))
    assert same >= 98
