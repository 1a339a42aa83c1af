"""Collider primitives besides the box walls on the GPU: spheres, meshes above the old
1,024-triangle limit (walked through the host-built hierarchy), and the reference's own
bunny scene (dae/sky/CBbunny.dae, 28,576 triangles).

Each is compared with the FP64 restatement (pinned bit for bit to the reference build on
the sphere and 2,048-triangle golden cases by tests/test_oracle_golden.py), one step on
the GPU's own neighbour sets, with the bars of the ramp case: positions 1e-5, velocities
and densities 1e-4 (a stop keeps 4 FP32 ulps from the surface where the reference keeps
1e-11, which moves stopped particles by ~5e-7).
"""
from __future__ import annotations

import os

import numpy as np
import pytest

from fluid_gb300 import scenes
from fluid_gb300.params import PBF_FLAG_GRAPH, PBF_FLAG_STATS
from tests.golden.make_golden import SPHERE, params_from_json, sphere_scene, wavy_floor, wavy_scene
from tests.helpers import rel_err

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


@pytest.fixture(scope="module")
def pbf():
    from fluid_gb300 import pbf as mod

    mod.lib()
    return mod


def _f32(a):
    return np.asarray(a, dtype=np.float32).astype(np.float64)


def bunny_triangles():
    g = np.load(os.path.join(GOLDEN, "cbbunny.npz"))
    t = g["triangles"][g["mesh_of"] == 0]
    return g["vertices"][t].reshape(-1, 9)


def _against_oracle(pbf, oracle_lib, name, pos, vel, prm, mesh=None, spheres=None, steps=1):
    pos, vel = _f32(pos), _f32(vel)
    with pbf.Simulator(pos, vel, prm.with_(flags=PBF_FLAG_STATS)) as sim:
        if mesh is not None:
            sim.set_collider_mesh(mesh)
        if spheres is not None:
            sim.set_collider_spheres(spheres)
        sim.time_step(prm.dt, 1)
        x, v, rho, st = sim.positions(), sim.velocities(), sim.densities(), sim.stats()
        nb = sim.neighbors()
    with pbf.Simulator(pos, vel, prm) as sim:
        sim.time_step(prm.dt, 1)
        x_free = sim.positions()
    oracle_lib.set_mesh(None if mesh is None else np.asarray(mesh, dtype=np.float32).astype(np.float64))
    oracle_lib.set_spheres(None if spheres is None else np.asarray(spheres, dtype=np.float32).astype(np.float64))
    try:
        ref = oracle_lib.step(pos, vel, prm, 1, given_neighbors=nb)
    finally:
        oracle_lib.set_mesh(None)
        oracle_lib.set_spheres(None)
    e = {"pos": rel_err(x, ref["pos"]), "vel": rel_err(v, ref["vel"]), "rho": rel_err(rho, ref["density"])}
    moved = float(np.abs(x - x_free).max())
    print(f"{name}: GPU vs FP64 on identical sets {e}; the collider moves particles by {moved:.2e}")
    assert st["error_flags"] == 0
    assert moved > 1e-3, "the collider must change this step"
    assert e["pos"] < 1e-5 and e["vel"] < 1e-4 and e["rho"] < 1e-4, e
    return x


def test_sphere_matches_oracle(pbf, oracle_lib):
    """A block falling onto a sphere (stops and slides on its curved surface)."""
    p, v, prm = sphere_scene()
    x = _against_oracle(pbf, oracle_lib, "sphere", p, v, prm, spheres=SPHERE)
    c, r = SPHERE[0, :3], SPHERE[0, 3]
    assert np.linalg.norm(x - c, axis=1).min() >= r - 1e-6  # nothing passed into the sphere


def test_mesh_of_2048_triangles_matches_oracle(pbf, oracle_lib):
    """A block falling onto a wavy floor of 2,048 triangles (twice the old limit)."""
    p, v, prm = wavy_scene()
    _against_oracle(pbf, oracle_lib, "wavy floor (2048 triangles)", p, v, prm, mesh=wavy_floor())


def test_bunny_scene_matches_oracle(pbf, oracle_lib):
    """The reference's bunny (28,576 triangles, in the Cornell box of dae/sky/CBbunny.dae):
    a 6^3 block just above its ears, falling into them."""
    tri = bunny_triangles()
    assert len(tri) == 28576
    s = 0.025
    p = scenes.lattice(6, 6, 6, s, corner=(0.0, 0.785, 0.05))
    p += scenes.uniform(17, p.size, -0.0005, 0.0005).reshape(p.shape)
    v = np.zeros_like(p)
    v[:, 1] = -4.0
    prm = scenes.physical_params(0.05, s, box_lo=(-1.0, 0.0, -1.0), box_hi=(1.0, 1.5, 1.0))
    _against_oracle(pbf, oracle_lib, "bunny", p, v, prm, mesh=tri)


def test_bunny_rollout_runs_and_replays(pbf):
    """4,096 particles poured onto the bunny for 40 steps: no error flag, finite state,
    graph replay bit-identical to stream-ordered launches, and the collider changes the flow."""
    tri = bunny_triangles()
    s = 0.03
    p = _f32(scenes.lattice(16, 16, 16, s, corner=(-0.24, 0.85, -0.24)))
    v = np.zeros_like(p)
    prm = scenes.physical_params(0.06, s, box_lo=(-1.0, 0.0, -1.0), box_hi=(1.0, 1.5, 1.0), max_neighbors=256)
    outs = []
    for flags in (PBF_FLAG_STATS, PBF_FLAG_STATS | PBF_FLAG_GRAPH):
        with pbf.Simulator(p, v, prm.with_(flags=flags)) as sim:
            sim.set_collider_mesh(tri)
            sim.time_step(prm.dt, 40)
            outs.append((sim.positions(), sim.velocities(), sim.stats()["error_flags"]))
    with pbf.Simulator(p, v, prm) as sim:
        sim.time_step(prm.dt, 40)
        free = sim.positions()
    (x, vv, err), (x2, v2, err2) = outs
    assert err == err2 == 0
    assert np.all(np.isfinite(x)) and np.all(np.isfinite(vv))
    assert np.array_equal(x, x2) and np.array_equal(vv, v2)
    print(f"bunny rollout: mean |x - x_without_bunny| {np.abs(x - free).mean():.3e}")
    assert np.abs(x - free).mean() > 1e-2


def test_collider_sphere_arguments(pbf):
    sc = scenes.block4096(1)
    with pbf.Simulator(_f32(sc.pos), _f32(sc.vel), sc.params) as sim:
        with pytest.raises(pbf.PbfError):
            sim.set_collider_spheres(np.array([[0.5, 0.5, 0.5, 0.0]]))  # radius must be positive
        with pytest.raises(pbf.PbfError):
            sim.set_collider_spheres(np.array([[0.5, np.nan, 0.5, 0.1]]))
        with pytest.raises(pbf.PbfError):
            sim.set_collider_spheres(np.tile([0.5, 0.5, 0.5, 0.1], (1025, 1)))
        sim.set_collider_spheres(SPHERE)
        sim.time_step(sc.params.dt, 1)
        sim.set_collider_spheres(None)
        sim.time_step(sc.params.dt, 1)
