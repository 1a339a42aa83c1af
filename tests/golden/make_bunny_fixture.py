"""Extract the collider triangles of the reference's bunny scene into tests/golden/cbbunny.npz.

Reads ``dae/sky/CBbunny.dae`` of the reference checkout (path as the first argument or in
``PBF_REFERENCE_DIR``) and writes every mesh of its visual scene in world coordinates the
way the reference's COLLADA loader places them (src/collada/collada.cpp:160-200 and
:244-348): the scene's up-axis correction (Z_UP: x -> -x, y <-> z) times each node's
matrix times the vertex. Stored: ``vertices`` (V, 3) float64, ``triangles`` (T, 3) int32
indices, ``mesh_of`` (T,) int32 (0 = the bunny) and ``names``; the GPU machine reads only the
npz. Usage: ``python tests/golden/make_bunny_fixture.py <reference_dir>``.
"""
from __future__ import annotations

import os
import sys
import xml.etree.ElementTree as ET
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
NS = {"c": "http://www.collada.org/2005/11/COLLADASchema"}


def up_axis_transform(root) -> np.ndarray:
    up = root.find("c:asset/c:up_axis", NS).text.strip()
    m = np.eye(4)
    if up == "Z_UP":
        m[1, 1], m[1, 2], m[2, 1], m[2, 2], m[0, 0] = 0.0, 1.0, 1.0, 0.0, -1.0
    elif up == "X_UP":
        m[0, 0], m[0, 1], m[1, 0], m[1, 1], m[2, 2] = 0.0, 1.0, 1.0, 0.0, -1.0
    return m


def geometry_triangles(geom) -> tuple[np.ndarray, np.ndarray]:
    mesh = geom.find("c:mesh", NS)
    sources = {s.get("id"): np.array(s.find("c:float_array", NS).text.split(), dtype=np.float64)
               for s in mesh.findall("c:source", NS)}
    verts = mesh.find("c:vertices", NS)
    pos_src = verts.find("c:input[@semantic='POSITION']", NS).get("source")[1:]
    pos = sources[pos_src].reshape(-1, 3)
    poly = mesh.find("c:polylist", NS)
    inputs = poly.findall("c:input", NS)
    stride = max(int(i.get("offset")) for i in inputs) + 1
    voff = int(next(i for i in inputs if i.get("semantic") == "VERTEX").get("offset"))
    vcount = np.array(poly.find("c:vcount", NS).text.split(), dtype=np.int64)
    p = np.array(poly.find("c:p", NS).text.split(), dtype=np.int64).reshape(-1, stride)[:, voff]
    tris, k = [], 0
    for c in vcount:  # fan-triangulate polygons (the scene's are triangles and quads)
        for j in range(1, c - 1):
            tris.append((p[k], p[k + j], p[k + j + 1]))
        k += c
    return pos, np.array(tris, dtype=np.int64)


def main(argv) -> int:
    ref_dir = argv[1] if len(argv) > 1 else os.environ.get("PBF_REFERENCE_DIR")
    if not ref_dir:
        raise SystemExit("usage: make_bunny_fixture.py <reference_dir> (or set PBF_REFERENCE_DIR)")
    root = ET.parse(Path(ref_dir) / "dae" / "sky" / "CBbunny.dae").getroot()
    up = up_axis_transform(root)
    geoms = {g.get("id"): g for g in root.findall("c:library_geometries/c:geometry", NS)}
    verts, tris, mesh_of, names = [], [], [], []
    for node in root.findall("c:library_visual_scenes/c:visual_scene/c:node", NS):
        inst = node.find("c:instance_geometry", NS)
        if inst is None:
            continue
        mat = np.array(node.find("c:matrix", NS).text.split(), dtype=np.float64).reshape(4, 4)
        pos, t = geometry_triangles(geoms[inst.get("url")[1:]])
        world = (up @ mat @ np.c_[pos, np.ones(len(pos))].T).T[:, :3]
        tris.append(t + sum(len(v) for v in verts))
        verts.append(world)
        mesh_of.append(np.full(len(t), len(names), dtype=np.int32))
        names.append(node.get("name"))
    order = sorted(range(len(names)), key=lambda k: names[k] != "Mesh")  # the bunny first
    V = np.concatenate(verts)
    T = np.concatenate([tris[k] for k in order]).astype(np.int32)
    M = np.concatenate([np.full(len(tris[k]), i, dtype=np.int32) for i, k in enumerate(order)])
    np.savez_compressed(HERE / "cbbunny.npz", vertices=V, triangles=T, mesh_of=M,
                        names=np.array([names[k] for k in order]))
    b = V[np.unique(T[M == 0])]
    print(f"cbbunny.npz: {len(T)} triangles ({int((M == 0).sum())} bunny), bunny bounds {b.min(0)} .. {b.max(0)}")
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv))
