"""Known-answer tests that pin the CPU oracle (no GPU).

The reference ships no tests or golden vectors for its dense path, so the
oracle is pinned here against analytic answers and independent numpy
restatements: plane and sphere TSDFs, exact plane raycasts, watertight and
consistently oriented sphere meshes, the marching-cubes table's topology,
the LDL^T solve and SE(3) exponential, the Gaussian pyramid, BT.601 luma,
FP32 block allocation, and recovery of a known camera motion.
"""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from yetanotherslam_gb300 import synth

CORNER = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]])
EDGE = np.array([[0, 1], [1, 2], [2, 3], [3, 0], [4, 5], [5, 6], [6, 7], [7, 4], [0, 4], [1, 5], [2, 6], [3, 7]])


def _plane_depth(W, H, z):
    return np.full((H, W), z, dtype=np.float32)


def test_plane_tsdf_matches_analytic():
    W, H = 64, 48
    K = (60.0, 60.0, 31.5, 23.5)
    vs, tr = 0.01, 0.03
    m = oracle.Map(vs, tr)
    m.fuse(_plane_depth(W, H, 1.5), K, np.eye(4))
    c, s, w = m.export()
    assert c.shape[0] > 0
    li = np.arange(512)
    lx, ly, lz = li & 7, (li >> 3) & 7, li >> 6
    z = ((c[:, 2:3] * 8 + lz[None, :]).astype(np.float32) * np.float32(vs)).astype(np.float64)
    obs = w > 0
    expect = np.minimum(1.0, (1.5 - z) / tr)
    assert np.abs(s[obs] - expect[obs]).max() < 1e-6
    # every observed voxel lies in front of (or within the truncation behind) the plane
    assert (z[obs] <= 1.5 + tr + 1e-6).all()
    # weights: one observation
    assert np.all(w[obs] == 1)


def test_plane_raycast_depth_exact():
    W, H = 64, 48
    K = (60.0, 60.0, 31.5, 23.5)
    m = oracle.Map(0.01, 0.03)
    for _ in range(3):
        m.fuse(_plane_depth(W, H, 1.234), K, np.eye(4))
    v, zn, zf = m.raycast(W, H, K, np.eye(4))
    hit = v[..., 3] > 0
    assert hit[4:-4, 4:-4].all()
    err = np.abs(v[..., 2] - 1.234)
    # head-on rays land on the plane exactly
    assert err[20:28, 28:36].max() < 1e-5
    # oblique rays: the two fixed correction moves of sdf*trunc along the ray
    # (RayTraceEngine.cu:436-448) undershoot by (1 - cos)^2 of the start offset
    assert err[hit].max() < 5e-4


def _sphere_blocks(r, vs, tr, centre=(0.0, 0.0, 0.0)):
    nb = int(np.ceil((r + 2 * tr) / (8 * vs))) + 1
    rng = np.arange(-nb, nb)
    bx, by, bz = np.meshgrid(rng, rng, rng, indexing="ij")
    coords = np.stack([bx.ravel(), by.ravel(), bz.ravel()], 1).astype(np.int32)
    li = np.arange(512)
    loc = np.stack([li & 7, (li >> 3) & 7, li >> 6], 1)
    p = (coords[:, None, :] * 8 + loc[None, :, :]) * vs - np.asarray(centre)
    d = np.linalg.norm(p, axis=2)
    sdf = np.clip((d - r) / tr, -1, 1).astype(np.float32)
    wt = np.ones_like(sdf)
    return coords, sdf, wt


def test_sphere_mesh_on_surface_watertight_oriented():
    vs, tr, r = 0.01, 0.03, 0.2
    m = oracle.Map(vs, tr)
    m.import_blocks(*_sphere_blocks(r, vs, tr))
    tris, nrm, cases, cube = m.mesh()
    assert tris.shape[0] > 1000
    v = tris.reshape(-1, 3)
    assert np.abs(np.linalg.norm(v, axis=1) - r).max() < 0.05 * vs
    # normals point to the inside (sdf < 0): towards the centre; degenerate
    # triangles (a vertex collapsed onto a grid corner where sdf ~ 0) carry the
    # zero normal
    t3 = tris.reshape(-1, 3, 3)
    area = np.linalg.norm(np.cross(t3[:, 1] - t3[:, 0], t3[:, 2] - t3[:, 0]), axis=1)
    c = t3.mean(1)
    assert (np.sum(nrm[area > 0, :3] * c[area > 0], axis=1) < 0).all()
    assert (nrm[area == 0] == 0).all()
    # watertight + consistently oriented: every directed edge is matched by its reverse
    edge, tri, cnt = oracle.mc_tables()
    counts = {}
    gid = []
    order = 0
    for q, (cs, p) in enumerate(zip(cases, cube)):
        # index of this triangle within its cube: count previous triangles with the same cube
        order = order + 1 if q > 0 and np.array_equal(cube[q - 1], p) else 0
        es = tri[cs][3 * order:3 * order + 3]
        ids = []
        for e in es:
            a, b = p + CORNER[EDGE[e][0]], p + CORNER[EDGE[e][1]]
            ids.append(tuple(sorted((tuple(a), tuple(b)))))
        gid.append(ids)
    for ids in gid:
        for j in range(3):
            key = (ids[j], ids[(j + 1) % 3])
            counts[key] = counts.get(key, 0) + 1
    for (a, b), n in counts.items():
        assert n == 1 and counts.get((b, a), 0) == 1, "open or inconsistently oriented edge"


def test_mc_table_topology():
    edge, tri, cnt = oracle.mc_tables()
    for c in range(256):
        signs = [(c >> i) & 1 for i in range(8)]
        mask = sum(1 << e for e in range(12) if signs[EDGE[e][0]] != signs[EDGE[e][1]])
        assert edge[c] == mask
        assert edge[c] == edge[255 - c]
        t = tri[c]
        n = int(cnt[c])
        assert np.all(t[3 * n:] == -1) and np.all(t[:3 * n] >= 0)
        used = set(int(e) for e in t[:3 * n])
        assert used == {e for e in range(12) if (mask >> e) & 1}
        # the boundary of the triangle set runs along cube faces only
        directed = {}
        for k in range(n):
            a = t[3 * k:3 * k + 3]
            for j in range(3):
                u, v = int(a[j]), int(a[(j + 1) % 3])
                if directed.get((v, u), 0):
                    directed[(v, u)] -= 1
                else:
                    directed[(u, v)] = directed.get((u, v), 0) + 1
        for (u, v), k in directed.items():
            if k == 0:
                continue
            cu = {EDGE[u][0], EDGE[u][1]}
            cv = {EDGE[v][0], EDGE[v][1]}
            face = any(all(CORNER[x][ax] == sd for x in cu | cv) for ax in range(3) for sd in (0, 1))
            assert face, f"case {c}: boundary segment {u}->{v} crosses the cube interior"
    assert int(cnt.max()) <= 10
    # single inside corner: one triangle whose normal points at that corner
    for i in range(8):
        c = 1 << i
        assert cnt[c] == 1
        e = tri[c][:3]
        P = []
        for ed in e:
            a, b = CORNER[EDGE[ed][0]], CORNER[EDGE[ed][1]]
            P.append((a + b) / 2.0)
        n = np.cross(P[1] - P[0], P[2] - P[0])
        assert np.dot(n, CORNER[i] - np.mean(P, axis=0)) > 0


def test_ldlt_solve_against_numpy():
    rng = np.random.default_rng(1)
    for _ in range(50):
        A = rng.normal(size=(6, 6))
        A = A @ A.T + 1e-3 * np.eye(6)
        b = rng.normal(size=6)
        x = oracle.ldlt_solve(A, b)
        assert np.allclose(x, np.linalg.solve(A, b), rtol=1e-8, atol=1e-10)
    assert np.array_equal(oracle.ldlt_solve(np.zeros((6, 6)), np.ones(6)), np.zeros(6))
    # rank-deficient PSD: finite (pseudo-inverse on the zero pivot)
    J = rng.normal(size=(3, 6))
    assert np.all(np.isfinite(oracle.ldlt_solve(J.T @ J, rng.normal(size=6))))
    # NaN on the first pivot: identity transpositions, that pivot pseudo-inverted to 0
    A = np.eye(6)
    A[0, 0] = np.nan
    assert np.array_equal(oracle.ldlt_solve(A, np.ones(6)), [0, 1, 1, 1, 1, 1])
    # NaN in the right-hand side propagates (the tracker's failure signal)
    assert np.isnan(oracle.ldlt_solve(np.eye(6), [np.nan, 0, 0, 0, 0, 0])[0])


def test_se3_exp_against_expm():
    scipy_linalg = pytest.importorskip("scipy.linalg")
    rng = np.random.default_rng(2)
    for scale in (1.0, 1e-3, 1e-7, 0.0):
        for _ in range(10):
            xi = rng.normal(size=6) * scale
            v, w = xi[:3], xi[3:]
            M = np.zeros((4, 4))
            M[:3, :3] = [[0, -w[2], w[1]], [w[2], 0, -w[0]], [-w[1], w[0], 0]]
            M[:3, 3] = v
            assert np.allclose(oracle.se3_exp(xi), scipy_linalg.expm(M), atol=1e-12)


def test_pyramid_and_gradients_against_numpy():
    W, H = 64, 48
    rng = np.random.default_rng(3)
    g = rng.integers(0, 256, size=(H, W), dtype=np.uint8)
    t = oracle.Tracker(W, H, np.array([[50, 0, 31.5], [0, 50, 23.5], [0, 0, 1.0]]), levels=3, mode=3)
    t.set_image(g, False)
    k = np.array([1, 4, 6, 4, 1], dtype=np.float64) / 16
    img = g.astype(np.float64)
    for lvl in range(3):
        got = t.level(lvl, 0)
        assert np.abs(got - img).max() < 1e-3
        gx = np.zeros_like(img)
        gy = np.zeros_like(img)
        gx[1:-1, 1:-1] = (img[1:-1, 2:] - img[1:-1, :-2]) * 0.5
        gy[1:-1, 1:-1] = (img[2:, 1:-1] - img[:-2, 1:-1]) * 0.5
        assert np.abs(t.level(lvl, 1) - gx).max() < 1e-3
        assert np.abs(t.level(lvl, 2) - gy).max() < 1e-3
        p = np.pad(img, 2, mode="reflect")  # numpy "reflect" == reflect-101
        v = sum(k[i] * p[i:i + img.shape[0], :] for i in range(5))
        hsm = sum(k[i] * v[:, i:i + img.shape[1]] for i in range(5))
        img = hsm[::2, ::2]


def test_bt601_fixed_point_luma():
    rng = np.random.default_rng(4)
    rgb = rng.integers(0, 256, size=(100, 100, 3), dtype=np.uint8)
    g = synth.gray_of(rgb).astype(np.float64)
    f = rgb[..., 0] * 0.299 + rgb[..., 1] * 0.587 + rgb[..., 2] * 0.114
    # 14-bit coefficients 4899/9617/1868 differ from 0.299/0.587/0.114 by < 2.5e-5 each
    assert np.abs(g - f).max() <= 0.5 + 255 * 5e-5


def _np_block_set(depth, K, T, vs, tr, dmin=0.1, dmax=3.0):
    """Independent numpy restatement of the FP32 allocation (VoxelMap.cu:549-651)."""
    f32 = np.float32
    R = T[:3, :3].astype(f32)
    t = T[:3, 3].astype(f32)
    invfx, invfy = f32(1.0 / np.float64(np.float32(K[0]))), f32(1.0 / np.float64(np.float32(K[1])))
    cx, cy = f32(K[2]), f32(K[3])
    half = f32(tr) * f32(0.5)
    out = set()
    H, W = depth.shape
    for y in range(H):
        for x in range(W):
            d = depth[y, x]
            if np.isnan(d) or d < f32(dmin) or d > f32(dmax):
                continue
            dn = max(f32(dmin), f32(d - half))
            df = min(f32(dmax), f32(d + half))
            if dn >= df:
                continue
            ends = []
            for z in (dn, df):
                p = [f32(f32(invfx * f32(f32(x) - cx)) * z), f32(f32(invfy * f32(f32(y) - cy)) * z), z]
                q = [f32(f32(f32(f32(R[i, 0] * p[0]) + f32(R[i, 1] * p[1])) + f32(R[i, 2] * p[2])) + t[i]) for i in range(3)]
                ends.append([int(np.floor(f32(qi / f32(vs)))) >> 3 for qi in q])
            s, e = ends
            d3 = [e[i] - s[i] for i in range(3)]
            inc = [-1 if v < 0 else 1 for v in d3]
            ad = [abs(v) for v in d3]
            if ad[0] >= ad[1] and ad[0] >= ad[2]:
                M, a1, a2 = 0, 1, 2
            elif ad[1] >= ad[0] and ad[1] >= ad[2]:
                M, a1, a2 = 1, 0, 2
            else:
                M, a1, a2 = 2, 1, 0
            cur = list(s)
            e1, e2 = 2 * ad[a1] - 1, 2 * ad[a2] - 1
            out.add(tuple(cur))
            for _ in range(ad[M]):
                if e1 > 0:
                    cur[a1] += inc[a1]
                    e1 -= 2 * ad[M]
                if e2 > 0:
                    cur[a2] += inc[a2]
                    e2 -= 2 * ad[M]
                e1 += 2 * ad[a1]
                e2 += 2 * ad[a2]
                cur[M] += inc[M]
                out.add(tuple(cur))
    return out


def test_allocation_against_numpy_restatement():
    W, H = 40, 30
    K = synth.intrinsics(W, H)
    sc = synth.Scene(seed=5)
    f = sc.render(3, W, H)
    depth = f.depth.astype(np.float32) * np.float32(0.001)
    T = np.eye(4)
    a = 0.7
    T[:3, :3] = [[np.cos(a), 0, np.sin(a)], [0, 1, 0], [-np.sin(a), 0, np.cos(a)]]
    T[:3, 3] = [0.31, -1.2, 2.05]
    for vs, tr in ((0.004, 0.012), (0.01, 0.05)):
        m = oracle.Map(vs, tr)
        m.allocate(depth, K, T)
        c, _, _ = m.export()
        assert {tuple(r) for r in c} == _np_block_set(depth, K, T, vs, tr)


def test_known_motion_recovered():
    """Photometric (and RGB+ICP) on an occluder-free room, ICP on the object
    scene (a bare room is nearly one plane: point-to-plane ICP is degenerate)."""
    W, H = 160, 120
    fx, fy, cx, cy = synth.intrinsics(W, H)
    K = np.array([[fx, 0, cx], [0, fy, cy], [0, 0, 1.0]])
    for mode, (ns, nb) in ((1, (0, 0)), (3, (0, 0)), (2, (20, 10))):
        sc = synth.Scene(seed=1, n_spheres=ns, n_boxes=nb)
        f0, c0 = sc.render(0, W, H, clean=True)
        f1, c1 = sc.render(1, W, H, clean=True)
        t = oracle.Tracker(W, H, K, levels=3, iters=(10, 5, 3), mode=mode)
        t.set_image(synth.gray_of(f0.rgb), True)
        t.set_depth(c0, True)
        t.set_image(synth.gray_of(f1.rgb), False)
        t.set_depth(c1, False)
        t.set_model(_vmap_of(c0, K))
        st, T = t.get_transform(np.eye(4))
        gt = np.linalg.inv(f1.Twc) @ f0.Twc
        E = np.linalg.inv(gt) @ T
        assert st == 0
        assert np.linalg.norm(E[:3, 3]) < 1.5e-3, (mode, np.linalg.norm(E[:3, 3]))


def _vmap_of(depth, K):
    H, W = depth.shape
    ys, xs = np.mgrid[0:H, 0:W]
    z = depth.astype(np.float32)
    v = np.zeros((H, W, 4), np.float32)
    v[..., 0] = (xs - K[0, 2]) / K[0, 0] * z
    v[..., 1] = (ys - K[1, 2]) / K[1, 1] * z
    v[..., 2] = z
    v[..., 3] = np.where((z > 0.2) & (z < 3.0), 1.0, -1.0)
    return v


def test_oracle_fuse_map_identity_and_defuse_kat():
    """Fusing a map into an identical copy at the same pose doubles every
    weight (below the cap) and keeps every sdf whose eight-voxel cell is fully
    observed; de-integrating a frame right after fusing it restores the map.
    The voxel size is a power of two (2^-7 m), so voxel -> metres -> voxel is
    exact in FP32 and the identity maps every voxel onto itself."""
    from yetanotherslam_gb300 import synth
    from tests.helpers import sequence

    W, H = 160, 120
    K = synth.intrinsics(W, H)
    seq = sequence(31, 2, W, H)
    vs = 2.0 ** -7
    a = oracle.Map(vs, 3 * vs)
    b = oracle.Map(vs, 3 * vs)
    for _, _, dm, T in seq:
        a.fuse(dm, K, T)
        b.fuse(dm, K, T)
    ca, sa, wa = a.export()
    assert not a.fuse_map(b, np.eye(4), np.eye(4))
    assert b.num_blocks == 0
    c2, s2, w2 = a.export()
    assert np.array_equal(ca, c2)
    moved = w2 != wa
    assert moved.any()
    assert np.array_equal(w2[moved], np.minimum(2 * wa[moved], 255))
    assert np.abs(s2[moved] - sa[moved]).max() < 1e-12
    d = oracle.Map(vs, 3 * vs)
    d.fuse(seq[0][2], K, seq[0][3])
    c0, s0, w0 = d.export()
    d.fuse(seq[1][2], K, seq[1][3])
    d.defuse(seq[1][2], K, seq[1][3])
    c1, s1, w1 = d.export()
    n0 = c0.shape[0]
    assert np.array_equal(c1[:n0], c0) and np.array_equal(w1[:n0], w0)
    obs = w0 > 0
    assert np.abs(s1[:n0][obs] - s0[obs]).max() < 1e-12
