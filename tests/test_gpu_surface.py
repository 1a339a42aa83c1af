"""GPU surface (pbf_surface) against the FP64 restatement with the same triangulation table.

The restatement is pinned to the reference's own surface by tests/test_surface.py (same
vertices and normals bit for bit, same triangles per cube). Here the FP32 GPU field may
differ from the FP64 one by ~1e-6 relative, so: the same triangles in the same order,
vertices within 1e-5 (absolute; the cubes are 0.05-0.15 wide) and unit normals within 2e-3.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np
import pytest

from fluid_gb300 import scenes
from tests.golden.make_golden import params_from_json

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


@pytest.fixture(scope="module")
def pbf():
    from fluid_gb300 import pbf as mod

    mod.lib()
    return mod


def _f32(a):
    return np.asarray(a, dtype=np.float32).astype(np.float64)


def _case(name):
    if name == "block4096":
        sc = scenes.block4096(1)
        return _f32(sc.pos), sc.params, dict(lo=sc.params.box_lo, hi=sc.params.box_hi)
    g = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    return _f32(g["pos"]), params_from_json(str(g["params"])), {}


@pytest.mark.parametrize("name", ["surface_p_default_0step", "surface_p_default_3step", "block4096"])
def test_surface_matches_fp64_restatement(pbf, oracle_lib, name):
    pos, prm, bounds = _case(name)
    edges, ntri, tri = pbf.mc_table()
    with pbf.Simulator(pos, np.zeros_like(pos), prm) as sim:
        xyz, nrm = sim.surface(**bounds)
        xyz2, nrm2 = sim.surface(**bounds)
    assert np.array_equal(xyz, xyz2) and np.array_equal(nrm, nrm2)
    o = oracle_lib.surface(pos, prm, ntri, tri, **bounds)
    assert len(xyz) == len(o["xyz"]) > 100
    dv = np.abs(xyz - o["xyz"]).max()
    dn = np.abs(nrm - o["nrm"]).max()
    print(f"{name}: {len(xyz)} triangles; vertices max |GPU - FP64| {dv:.2e}, normals {dn:.2e}")
    assert dv < 1e-5 and dn < 2e-3


def test_surface_capacity_and_empty(pbf):
    pos, prm, _ = _case("surface_p_default_0step")
    with pbf.Simulator(pos, np.zeros_like(pos), prm) as sim:
        xyz, nrm = sim.surface()
        L = pbf.lib()
        cap = 17
        part = np.zeros((cap, 3, 3), dtype=np.float32)
        pn = np.zeros((cap, 3, 3), dtype=np.float32)
        count = ctypes.c_size_t(0)
        rc = L.pbf_surface(sim._h, 0.95 * prm.rest_density, 0.5 * prm.h, None, None,
                           part.ctypes.data_as(pbf.P), pn.ctypes.data_as(pbf.P), cap, ctypes.byref(count))
        assert rc == 0 and count.value == len(xyz)
        assert np.array_equal(part, xyz[:cap]) and np.array_equal(pn, nrm[:cap])
        empty, _ = sim.surface(iso=1e30)
        assert len(empty) == 0
        with pytest.raises(pbf.PbfError):
            sim.surface(step=-1.0)
