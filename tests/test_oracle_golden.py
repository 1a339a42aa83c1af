"""The FP64 restatement oracle against golden vectors made by the reference's own step.

The fixtures in tests/golden/ were produced by tests/golden/make_golden.py, which runs
the reference's src/particles.cpp (built headless by oracle/ref/build_ref.py). These
tests pin the oracle: it must reproduce the reference bit for bit.
"""
from __future__ import annotations

import glob
import os

import numpy as np
import pytest

from tests.golden.make_golden import params_from_json

# reference-step vectors of make_golden.py (the finite-difference fixture of the adjoint
# workload, the surface and the render fixtures and the bunny scene's triangles are read
# by their own tests)
GOLDEN = sorted(p for p in glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz"))
                if not os.path.basename(p).startswith(("adjoint_", "surface_", "render_", "cbbunny")))


def _case_id(path):
    return os.path.basename(path).replace(".npz", "")


@pytest.fixture(params=GOLDEN, ids=_case_id)
def golden(request, oracle_lib):
    g = np.load(request.param)
    oracle_lib.set_mesh(g["mesh"] if "mesh" in g.files else None)  # collider triangles of the case
    oracle_lib.set_spheres(g["spheres"] if "spheres" in g.files else None)  # and its spheres
    yield g
    oracle_lib.set_mesh(None)
    oracle_lib.set_spheres(None)


def test_golden_files_present():
    names = {_case_id(p) for p in GOLDEN}
    assert {"block4096_mass_1step", "p_default_1step", "block512_mass_20step", "sphere_block512_2step",
            "wavyfloor2048_block512_2step"} <= names


def test_oracle_matches_reference_bitwise(golden, oracle_lib):
    """Jacobi-order reference step == restatement, every bit (particles.cpp:250-297)."""
    prm = params_from_json(str(golden["params"]))
    steps = int(golden["steps"])
    out = oracle_lib.step(golden["pos_in"], golden["vel_in"], prm, steps=steps, neighbors=True, threads=4)
    for key in ("pos", "vel", "density"):
        np.testing.assert_array_equal(out[key], golden[key], err_msg=key)
    np.testing.assert_array_equal(out["nbr_offsets"], golden["nbr_offsets"])
    np.testing.assert_array_equal(out["nbr_idx"], golden["nbr_idx"])


def test_oracle_positions_match_literal_reference_after_one_step(golden, oracle_lib):
    """The unmodified Particles::timeStep differs from the Jacobi order only in velocities.

    Positions and densities after ONE step do not depend on the XSPH order
    (particles.cpp:285-288): x is x* before that pass and density is recomputed from x*.
    """
    if int(golden["steps"]) != 1:
        pytest.skip("after the first step the literal velocities feed back into positions")
    prm = params_from_json(str(golden["params"]))
    out = oracle_lib.step(golden["pos_in"], golden["vel_in"], prm, steps=1)
    np.testing.assert_array_equal(out["pos"], golden["literal_pos"])
    np.testing.assert_array_equal(out["density"], golden["literal_density"])


def test_load_time_density_matches_reference(golden, oracle_lib):
    """Particles::estimateDensities (particles.cpp:440-444), self term included."""
    prm = params_from_json(str(golden["params"]))
    d = oracle_lib.estimate_densities(golden["pos_in"], prm, threads=2)
    np.testing.assert_array_equal(d, golden["load_density"])


def test_oracle_thread_count_independent(oracle_lib):
    oracle_lib.set_mesh(None)
    g = np.load(GOLDEN[0])
    prm = params_from_json(str(g["params"]))
    a = oracle_lib.step(g["pos_in"], g["vel_in"], prm, steps=1, threads=1)
    b = oracle_lib.step(g["pos_in"], g["vel_in"], prm, steps=1, threads=3)
    for key in ("pos", "vel", "density"):
        np.testing.assert_array_equal(a[key], b[key])


def test_density_at_points_matches_bruteforce(oracle_lib):
    """Particles::estimateDensityAt (particles.cpp:446-453) against a numpy poly6 sum."""
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "p_default_1step.npz"))
    prm = params_from_json(str(g["params"]))
    pos = g["pos_in"]
    rng = np.random.default_rng(0)
    pts = pos[rng.integers(0, len(pos), 16)] + rng.uniform(-0.1, 0.1, (16, 3))
    got = oracle_lib.estimate_density_at(pos, pts, prm)
    r2 = ((pos[None, :, :] - pts[:, None, :]) ** 2).sum(-1)
    w = np.where(r2 < prm.h2, 1.56668147106 * (prm.h2 - r2) ** 3 / prm.h ** 9, 0.0)
    np.testing.assert_allclose(got, w.sum(1), rtol=1e-12)
