"""The FP64 reference gradient (oracle/pbf_oracle_adj.c) against FP64 central finite
differences of the FP64 restatement, on the CPU.

The step is differentiated with its neighbour sets fixed (the finite differences run on
the same sets) and every collision with its active set fixed; the differences use a
step small enough that no perturbation changes an active set. Bar: 1e-5 normwise
relative error over the checked coordinates (the FD truncation error is ~1e-7 here).
"""
from __future__ import annotations

import numpy as np
import pytest

from tests.helpers import adjoint_corner_scene, adjoint_fall_scene, adjoint_free_scene, rel_err

TOL = 1e-5


def _setup(oracle, p, v, prm, seed=0):
    o = oracle.step(p, v, prm, 1, neighbors=True)
    nb = (o["nbr_offsets"], o["nbr_idx"])
    rng = np.random.default_rng(seed)
    gx = rng.standard_normal(p.shape)
    gv = rng.standard_normal(p.shape)
    return o, nb, gx, gv


def _loss(oracle, p, v, prm, nb, gx, gv):
    r = oracle.step(p, v, prm, 1, given_neighbors=nb)
    return float((gx * r["pos"]).sum() + (gv * r["vel"]).sum())


def _fd(oracle, p, v, prm, nb, gx, gv, coords, eps):
    out = []
    for which, i, k in coords:
        a = [p.copy(), v.copy()]
        b = [p.copy(), v.copy()]
        a[which][i, k] += eps
        b[which][i, k] -= eps
        out.append((_loss(oracle, *a, prm, nb, gx, gv) - _loss(oracle, *b, prm, nb, gx, gv)) / (2 * eps))
    return np.array(out)


def test_recorded_forward_is_the_restatement_bit_for_bit(oracle_lib):
    p, v, prm = adjoint_fall_scene()
    o, nb, gx, gv = _setup(oracle_lib, p, v, prm)
    a = oracle_lib.step_adjoint(p, v, prm, gx, gv, given_neighbors=nb)
    assert np.array_equal(a["pos"], o["pos"]) and np.array_equal(a["vel"], o["vel"])
    # the search inside the adjoint finds the same sets as the step
    b = oracle_lib.step_adjoint(p, v, prm, gx, gv)
    assert np.array_equal(a["gx"], b["gx"]) and np.array_equal(a["gv"], b["gv"])


@pytest.mark.parametrize("scene", ["fall", "corner"])
def test_one_step_gradient_matches_central_differences(oracle_lib, scene):
    p, v, prm = adjoint_fall_scene() if scene == "fall" else adjoint_corner_scene()
    o, nb, gx, gv = _setup(oracle_lib, p, v, prm, seed=1)
    a = oracle_lib.step_adjoint(p, v, prm, gx, gv, given_neighbors=nb)
    kinds = a["kinds"]
    assert kinds[2] + kinds[3] + kinds[7] > 0  # stops happened in the prediction or the iterations
    if scene == "corner":
        assert kinds[3] > 0 and kinds[4] > 0  # slides and second stops
    rng = np.random.default_rng(2)
    n = p.shape[0]
    coords = [(t % 2, int(rng.integers(n)), int(rng.integers(3))) for t in range(64)]
    fd = _fd(oracle_lib, p, v, prm, nb, gx, gv, coords, 1e-7)
    an = np.array([(a["gx"] if w == 0 else a["gv"])[i, k] for w, i, k in coords])
    err = rel_err(an, fd)
    print(f"{scene}: kinds {kinds.tolist()} adjoint vs FD normwise {err:.2e}")
    assert err < TOL


def test_rest_density_gradient_matches_central_difference(oracle_lib):
    p, v, prm = adjoint_fall_scene()
    o, nb, gx, gv = _setup(oracle_lib, p, v, prm, seed=3)
    a = oracle_lib.step_adjoint(p, v, prm, gx, gv, given_neighbors=nb)
    d = 1e-6 * prm.rest_density
    lp = _loss(oracle_lib, p, v, prm.with_(rest_density=prm.rest_density + d), nb, gx, gv)
    lm = _loss(oracle_lib, p, v, prm.with_(rest_density=prm.rest_density - d), nb, gx, gv)
    fd = (lp - lm) / (2 * d)
    print(f"d loss / d rho0: adjoint {a['grho0']:.9e} FD {fd:.9e}")
    assert abs(a["grho0"] - fd) <= TOL * abs(fd)


def test_checkpointed_rollout_gradient_matches_central_differences(oracle_lib):
    """Five steps, neighbour sets searched again in every step of the FD rollouts: the
    free block has no collision, and its kernels vanish smoothly at h, so the rollout
    is differentiable and the checkpointed reverse matches the differences. The
    dynamics amplify perturbations about 3x per step, so the rollout is close to
    linear only for tiny perturbations: the differences use eps = 1e-8 (at 1e-6 the
    second-order terms already reach 1e-2 of the derivative after 5 steps)."""
    p, v, prm = adjoint_free_scene(6)
    steps = 5
    rng = np.random.default_rng(4)
    gx = rng.standard_normal(p.shape)
    gv = rng.standard_normal(p.shape)
    a = oracle_lib.rollout_adjoint(p, v, prm, steps, gx, gv)

    def loss(pp, vv):
        r = oracle_lib.step(pp, vv, prm, steps)
        return float((gx * r["pos"]).sum() + (gv * r["vel"]).sum())

    n = p.shape[0]
    fd, an = [], []
    for t in range(32):
        w, i, k = t % 2, int(rng.integers(n)), int(rng.integers(3))
        A = [p.copy(), v.copy()]
        B = [p.copy(), v.copy()]
        A[w][i, k] += 1e-8
        B[w][i, k] -= 1e-8
        fd.append((loss(*A) - loss(*B)) / 2e-8)
        an.append((a["gx"] if w == 0 else a["gv"])[i, k])
    err = rel_err(an, fd)
    print(f"5-step rollout adjoint vs FD normwise {err:.2e}")
    assert err < TOL
