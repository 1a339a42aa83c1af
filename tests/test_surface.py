"""The marching-cubes surface (Particles::getSurfacePrims, particles.cpp:352-385) on the CPU:
the library's triangulation table, and the FP64 restatement against the reference's own
surface (tests/golden/surface_*.npz from tests/golden/make_surface_golden.py)."""
from __future__ import annotations

import os
from collections import Counter

import numpy as np
import pytest

from tests.golden.make_golden import params_from_json

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")

# corners and edges as generateGridCell (particles.cpp:309-323) and polygonise number them
CORNER = [(0, 0, 0), (0, 1, 0), (1, 1, 0), (1, 0, 0), (0, 0, 1), (0, 1, 1), (1, 1, 1), (1, 0, 1)]
EDGE = [(0, 1), (1, 2), (2, 3), (3, 0), (4, 5), (5, 6), (6, 7), (7, 4), (0, 4), (1, 5), (2, 6), (3, 7)]


@pytest.fixture(scope="module")
def table():
    from fluid_gb300 import build, pbf

    build.build_cuda()
    return pbf.mc_table()


def _faces():
    out = []
    for axis in range(3):
        for side in (0, 1):
            u, v = (axis + 1) % 3, (axis + 2) % 3
            cyc = []
            for cu, cv in ((0, 0), (1, 0), (1, 1), (0, 1)):
                cyc += [c for c in range(8) if CORNER[c][axis] == side and CORNER[c][u] == cu and CORNER[c][v] == cv]
            out.append(cyc)
    return out


def _edge(a, b):
    return next(e for e, (p, q) in enumerate(EDGE) if {p, q} == {a, b})


def _generate(ci):
    """The table's rule, written again here: on a face with four crossing edges the
    segments cut off the corners below the iso level; loops from the lowest unused edge;
    a fan from the first vertex sharing no face with a non-adjacent loop vertex."""
    faces = _faces()
    face_edges = [{_edge(f[k], f[(k + 1) % 4]) for k in range(4)} for f in faces]
    inside = [(ci >> k) & 1 for k in range(8)]
    partner = {}
    for f in faces:
        es = [_edge(f[k], f[(k + 1) % 4]) for k in range(4)]
        cross = [k for k in range(4) if inside[f[k]] != inside[f[(k + 1) % 4]]]
        pairs = [(es[cross[0]], es[cross[1]])] if len(cross) == 2 else (
            [(es[(k + 3) % 4], es[k]) for k in range(4) if inside[f[k]]] if len(cross) == 4 else [])
        for a, b in pairs:
            partner.setdefault(a, []).append(b)
            partner.setdefault(b, []).append(a)
    tris, used = [], set()
    for start in range(12):
        if start not in partner or start in used:
            continue
        loop, prev, cur = [], None, start
        while True:
            loop.append(cur)
            used.add(cur)
            nxt = partner[cur][0] if (prev is None or partner[cur][0] != prev) else partner[cur][1]
            prev, cur = cur, nxt
            if cur == start:
                break
        k = len(loop)
        apex = next(a for a in range(k) if all(
            not any(loop[a] in fe and loop[(a + i) % k] in fe for fe in face_edges) for i in range(2, k - 1)))
        r = loop[apex:] + loop[:apex]
        tris += [(r[0], r[i], r[i + 1]) for i in range(1, k - 1)]
    return tris


def test_table_is_the_documented_rule(table):
    edges, ntri, tri = table
    for ci in range(256):
        want = _generate(ci)
        assert ntri[ci] == len(want) <= 5, ci
        assert [tuple(tri[ci, 3 * t:3 * t + 3]) for t in range(ntri[ci])] == want, ci
        inside = [(ci >> k) & 1 for k in range(8)]
        mask = sum(1 << e for e, (a, b) in enumerate(EDGE) if inside[a] != inside[b])
        assert edges[ci] == mask
        assert set(tri[ci, :3 * ntri[ci]].tolist()) == {e for e in range(12) if mask >> e & 1}


def test_table_closes_the_surface(table):
    """On random fields every mesh edge off the grid boundary belongs to exactly two triangles."""
    _, ntri, tri = table
    n = 7
    for seed in range(10):
        val = np.random.default_rng(seed).uniform(-1, 1, (n + 1, n + 1, n + 1))
        count = Counter()
        for ix in range(n):
            for iy in range(n):
                for iz in range(n):
                    ci = sum(1 << k for k in range(8)
                             if val[ix + CORNER[k][0], iy + CORNER[k][1], iz + CORNER[k][2]] < 0)
                    for t in range(ntri[ci]):
                        vs = []
                        for e in tri[ci, 3 * t:3 * t + 3]:
                            a, b = EDGE[e]
                            vs.append(tuple(sorted(tuple(np.add((ix, iy, iz), CORNER[c])) for c in (a, b))))
                        for p, q in ((0, 1), (1, 2), (2, 0)):
                            count[tuple(sorted((vs[p], vs[q])))] += 1

        def on_boundary(e):
            pts = [p for v in e for p in v]
            return any(all(p[a] == 0 for p in pts) or all(p[a] == n for p in pts) for a in range(3))

        assert all(c == 2 for e, c in count.items() if not on_boundary(e)), seed


def _area(t):
    return 0.5 * np.linalg.norm(np.cross(t[:, 1] - t[:, 0], t[:, 2] - t[:, 0]), axis=1).sum()


@pytest.mark.parametrize("name", ["surface_p_default_0step", "surface_p_default_3step"])
def test_restatement_matches_the_reference_surface(table, oracle_lib, name):
    """The FP64 restatement with this library's table against the reference's surface: the
    same vertices (edge crossings) and normals bit for bit, the same triangle count in
    every cube, the surface area within 1e-3 (the tables may split a cube's non-planar
    polygon along other diagonals: 4e-6 on the loaded particles, 1.5e-4 after 3 steps)."""
    _, ntri, tri = table
    g = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    prm = params_from_json(str(g["params"]))
    o = oracle_lib.surface(g["pos"], prm, ntri, tri)
    rv = {tuple(p): tuple(m) for p, m in zip(g["xyz"].reshape(-1, 3), g["nrm"].reshape(-1, 3))}
    ov = {tuple(p): tuple(m) for p, m in zip(o["xyz"].reshape(-1, 3), o["nrm"].reshape(-1, 3))}
    assert rv == ov
    assert Counter(g["cube"].tolist()) == Counter(o["cube"].tolist())
    ra, oa = _area(g["xyz"]), _area(o["xyz"])
    print(f"{name}: {len(g['cube'])} triangles, {len(rv)} vertices, area reference {ra:.6f} here {oa:.6f}")
    assert abs(ra - oa) <= 1e-3 * ra
