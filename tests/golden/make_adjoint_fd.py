"""FP64 central finite differences of the adjoint workload, for tests/test_gpu_adjoint.py.

Workload (the adjoint configuration): the 32^3 block of ``scenes.adjoint_32k`` (h = 0.05,
4 iterations), loss = mean squared distance of the final positions to a target rollout
made from the same state with the initial velocities perturbed by N(0, 0.1^2) noise
(``scenes.normal(seed, 3n, 0.1, stream=7)``), gradient with respect to the initial
velocities and the rest density. For every horizon T in ``HORIZONS`` this stores, for
64 random velocity coordinates, the FP64 central difference of the loss (eps = 1e-4,
neighbour sets searched in every step as in the forward) and the FP64 reference
gradient (oracle.rollout_adjoint), plus both for the rest density (eps = 1e-4 rho0).

Runs the FP64 oracle on the CPU only (a few minutes on 8 cores); the GPU machine reads
the committed ``adjoint_32k_fd.npz``. Usage: ``python tests/golden/make_adjoint_fd.py``.
"""
from __future__ import annotations

import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))

from fluid_gb300 import scenes  # noqa: E402
from oracle import oracle  # noqa: E402

HORIZONS = (1, 2, 30)
EPS = 1e-4
COORDS = 64
OUT = HERE / "adjoint_32k_fd.npz"


def workload(seed: int = 5):
    sc = scenes.adjoint_32k(seed)
    pos = sc.pos.astype(np.float32).astype(np.float64)
    vel = sc.vel.astype(np.float32).astype(np.float64)
    noise = scenes.normal(seed, vel.size, 0.1, stream=7).reshape(vel.shape)
    vt = (vel + noise).astype(np.float32).astype(np.float64)
    return pos, vel, vt, sc.params


def main() -> None:
    pos, vel, vt, prm = workload()
    n = pos.shape[0]
    rng = np.random.default_rng(2024)
    coords = rng.choice(3 * n, COORDS, replace=False)
    out = {"coords": coords, "horizons": np.array(HORIZONS), "eps": EPS}
    for T in HORIZONS:
        t0 = time.time()
        target = oracle.step(pos, vt, prm, T)["pos"]

        def loss(v, p=prm):
            return float(((oracle.step(pos, v, p, T)["pos"] - target) ** 2).mean())

        fin = oracle.step(pos, vel, prm, T)["pos"]
        gx = 2.0 * (fin - target) / fin.size
        ref = oracle.rollout_adjoint(pos, vel, prm, T, gx, np.zeros_like(gx))
        fd = np.empty(COORDS)
        for q, c in enumerate(coords):
            a, b = vel.copy(), vel.copy()
            a.flat[c] += EPS
            b.flat[c] -= EPS
            fd[q] = (loss(a) - loss(b)) / (2 * EPS)
        d = EPS * prm.rest_density
        fd_r = (loss(vel, prm.with_(rest_density=prm.rest_density + d)) -
                loss(vel, prm.with_(rest_density=prm.rest_density - d))) / (2 * d)
        out[f"fd_{T}"] = fd
        out[f"ref_{T}"] = ref["gv"].flat[coords]
        out[f"fd_rho0_{T}"] = fd_r
        out[f"ref_rho0_{T}"] = ref["grho0"]
        out[f"loss_{T}"] = loss(vel)
        err = np.linalg.norm(out[f"ref_{T}"] - fd) / np.linalg.norm(fd)
        print(f"T={T}: loss {out[f'loss_{T}']:.4e} reference gradient vs FD {err:.2e} "
              f"rho0 {ref['grho0']:.4e} vs {fd_r:.4e} ({time.time() - t0:.0f} s)", flush=True)
    np.savez(OUT, **out)
    print(f"wrote {OUT}")


if __name__ == "__main__":
    main()
