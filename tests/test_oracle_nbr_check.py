"""The C neighbour-set check (orc_nbr_check_fp32) that the large-scene GPU parity tests use.

It must agree with the numpy restatement of the FP32 predicate (tests/helpers.py) on a
jittered lattice with pairs at the knife edge, and it must notice a pair that a list
misses or holds in excess. Mistakes are planted in the lists handed to the check, on the
CPU.
"""
from __future__ import annotations

import numpy as np

from fluid_gb300 import scenes
from tests.helpers import neighbor_sets_fp32


def _points():
    s = 0.05
    p = scenes.lattice(10, 9, 8, s, corner=(0.1, 0.2, 0.3))
    p += scenes.uniform(21, p.size, -0.002, 0.002).reshape(p.shape)
    # a few pairs at exactly the radius along x (exact in FP32: 0.1 apart at dyadic-ish values)
    edge = np.array([[0.5, 0.75, 0.25], [0.6, 0.75, 0.25], [0.5, 0.875, 0.25]], dtype=np.float64)
    return np.concatenate([p, edge]).astype(np.float32)


def test_check_agrees_with_numpy_predicate(oracle_lib):
    x = _points()
    h2 = 0.01
    off, ids = neighbor_sets_fp32(x, h2)
    r = oracle_lib.check_neighbors_fp32(x, h2, off, ids.astype(np.uint32))
    assert r == {"bad": 0, "missing": 0, "extra": 0, "first": -1}
    assert off[-1] > 10 * len(x)


def test_check_reports_planted_mistakes(oracle_lib):
    x = _points()
    h2 = 0.01
    off, ids = neighbor_sets_fp32(x, h2)
    ids = ids.astype(np.uint32)
    # drop the first neighbour of particle 7
    drop = off[7]
    ids_m = np.delete(ids, drop)
    off_m = off.copy()
    off_m[8:] -= 1
    r = oracle_lib.check_neighbors_fp32(x, h2, off_m, ids_m)
    assert r["bad"] == 1 and r["missing"] == 1 and r["extra"] == 0 and r["first"] == 7
    # replace a neighbour of particle 3 by a far particle (one missing, one extra)
    ids_x = ids.copy()
    far = int(np.argmax(np.linalg.norm(x - x[3], axis=1)))
    ids_x[off[3]] = far
    seg = np.sort(ids_x[off[3]:off[4]])
    ids_x[off[3]:off[4]] = seg
    r = oracle_lib.check_neighbors_fp32(x, h2, off, ids_x)
    assert r["bad"] == 1 and r["missing"] == 1 and r["extra"] == 1 and r["first"] == 3


def test_check_empty(oracle_lib):
    r = oracle_lib.check_neighbors_fp32(np.zeros((0, 3), np.float32), 0.01, np.zeros(1, np.int64),
                                        np.zeros(0, np.uint32))
    assert r["bad"] == 0 and r["first"] == -1
