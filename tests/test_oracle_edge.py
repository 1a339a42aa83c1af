"""The FP64 restatement against the reference's own step on tiny edge-case inputs.

A lone particle (no neighbours: density 0, lambda = 1 / EPSILON, no correction), a pair
inside and a pair outside the kernel radius, a particle thrown into a wall corner (stop
and slide, particles.cpp:87-132) and one crossing the clip plane y = 1.49, and a tight
cluster: the restatement reproduces the reference build bit for bit on each, over
several steps.
"""
from __future__ import annotations

import numpy as np
import pytest

from fluid_gb300.params import REFERENCE_DEFAULTS

CASES = {
    "one": ([[0.0, 0.5, 0.0]], [[0.0, 0.0, 0.0]]),
    "pair_inside_h": ([[0.0, 0.5, 0.0], [0.1, 0.5, 0.0]], [[0.0, 0.0, 0.0], [0.0, 0.0, 0.0]]),
    "pair_outside_h": ([[0.0, 0.5, 0.0], [0.8, 0.5, 0.0]], [[0.0, 0.0, 0.0], [0.0, 0.0, 0.0]]),
    "wall_corner": ([[0.97, 0.03, -0.97]], [[3.0, -4.0, -2.0]]),
    "clip_plane": ([[0.2, 1.45, 0.1]], [[0.5, 6.0, 0.0]]),
    "cluster": ([[0.05 * (k % 2), 0.3 + 0.05 * ((k // 2) % 2), 0.05 * (k // 4)] for k in range(8)],
                [[0.1, 0.0, -0.1]] * 8),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_restatement_matches_reference_on_tiny_inputs(name, oracle_lib):
    from oracle import ref_runner

    if not ref_runner.available():
        pytest.skip("reference build not available")
    pos, vel = (np.asarray(a, dtype=np.float64) for a in CASES[name])
    prm = REFERENCE_DEFAULTS
    oracle_lib.set_mesh(None)
    ref = ref_runner.run(pos, vel, prm, steps=3, mode="jacobi")
    out = oracle_lib.step(pos, vel, prm, steps=3)
    for key in ("pos", "vel", "density"):
        np.testing.assert_array_equal(out[key], ref[key], err_msg=key)
    assert np.all(np.isfinite(out["pos"]))
