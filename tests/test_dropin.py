"""The drop-in boundary with the reference's own types and callers.

tests/dropin/particles.h replaces the reference's src/particles.h with the GB300 facade
over the reference's CGL::Vector3D and CGL::Color, and keeps its renderer-typed members
(BVHAccel* bvh, the Primitive* surface, getSurfacePrims(double, double, BSDF*)). It is
compiled against the reference's headers and linked with the reference's BVHAccel,
MarchingTriangle, BSDF and CGL objects (tests/dropin/build_dropin.py), and
tests/dropin/dropin_main.cpp drives it as Application::load_particles and the PathTracer's
keys m, c and h do. Its results must be bit-identical to the same library driven from
Python, and its loaded densities and first step within 1e-5 of the FP64 oracle.
"""
from __future__ import annotations

import subprocess

import numpy as np
import pytest

from fluid_gb300 import scenes
from fluid_gb300.params import PBF_FLAG_STATS
from tests.helpers import rel_err


@pytest.fixture(scope="module")
def dropin():
    from tests.dropin import build_dropin

    if not build_dropin.available():
        pytest.skip("the reference's staged headers and objects (oracle/_ref) are not built")
    return str(build_dropin.build())


def test_params_string_matches_the_reference(dropin):
    """Particles' constructor prints paramsString() (particles.h:114-116, particles.cpp:420-438)."""
    from oracle import ref_runner

    if not ref_runner.available():
        pytest.skip("reference build not available")
    ours = subprocess.run([dropin, "--params-string"], capture_output=True, text=True, check=True).stdout
    ref = subprocess.run([str(ref_runner.DRIVER), "--params-string"], capture_output=True, text=True,
                         check=True).stdout
    assert ours == ref and "Newton steps: 12" in ours


def _read(path):
    with open(path, "rb") as f:
        assert f.read(8) == b"PBFDROP1"
        n, steps, surf = np.frombuffer(f.read(24), dtype=np.int64)
        t = np.frombuffer(f.read(8), dtype=np.float64)[0]
        x = np.frombuffer(f.read(12 * n), dtype=np.float32).reshape(n, 3)
        v = np.frombuffer(f.read(12 * n), dtype=np.float32).reshape(n, 3)
        rho = np.frombuffer(f.read(4 * n), dtype=np.float32)
    return {"n": int(n), "steps": int(steps), "surface": int(surf), "time": float(t), "pos": x, "vel": v,
            "density": rho}


@pytest.mark.gpu
def test_reference_callers_drive_the_gpu_step(dropin, tmp_path, oracle_lib):
    from fluid_gb300 import pbf

    sc = scenes.block4096(1)
    xml = tmp_path / "block.xml"
    scenes.write_xml(xml, sc.pos, sc.vel, sc.params.rest_density, sc.params)
    r = subprocess.run([dropin, str(xml), str(tmp_path)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    assert "Fluid simulation parameters" in r.stdout
    st = {k: _read(tmp_path / f"{k}.bin") for k in ("load", "m", "c", "h")}

    # the same library from Python, on the loader's inputs: <density> goes through stof
    prm = sc.params.with_(rest_density=float(np.float32(sc.params.rest_density)), flags=PBF_FLAG_STATS)
    pos32 = sc.pos.astype(np.float32).astype(np.float64)
    vel32 = sc.vel.astype(np.float32).astype(np.float64)
    dt = prm.dt
    with pbf.Simulator(pos32, vel32, prm) as sim:
        load = sim.estimate_densities()
        sim.time_step(dt, 1)
        m = (sim.positions(), sim.velocities(), sim.densities())
        # key c: the reference's loop, simulate_time accumulated in double
        t0 = t = dt
        n_c = 0
        while t < t0 + 1:
            t += dt
            n_c += 1
        sim.time_step(dt, n_c)
        c = (sim.positions(), sim.velocities(), sim.densities())
        sx, _ = sim.surface()
        sim.time_step(dt, 1)
        h = (sim.positions(), sim.velocities(), sim.densities())

    assert np.array_equal(st["load"]["density"], load)
    for name, ref in (("m", m), ("c", c), ("h", h)):
        for k, a in zip(("pos", "vel", "density"), ref):
            assert np.array_equal(st[name][k], a), (name, k)
    assert st["c"]["steps"] == n_c and st["c"]["time"] == t
    assert st["h"]["surface"] == len(sx) > 0

    # and against the FP64 oracle: the load-time densities and the first step
    ref_load = oracle_lib.estimate_densities(pos32, prm)
    ref_m = oracle_lib.step(pos32, vel32, prm, steps=1)
    e = {"load": rel_err(st["load"]["density"], ref_load), "pos": rel_err(st["m"]["pos"], ref_m["pos"]),
         "vel": rel_err(st["m"]["vel"], ref_m["vel"]), "rho": rel_err(st["m"]["density"], ref_m["density"])}
    print(f"drop-in vs FP64: {e}; {n_c} steps in the one-second loop; {len(sx)} surface triangles")
    assert all(v < 1e-5 for v in e.values()), e
