"""pbf_density_noalloc: the density estimate for callers that cannot allocate device memory.

Some hosts cannot let a library call cudaMalloc: their device memory belongs to another
framework's caching allocator, or their loop must never stall on the device
synchronization that cudaMalloc/cudaFree can cause. pbf_density_noalloc serves them with
caller-owned device buffers and one fixed scratch array inside the library. These tests
call it through the C ABI (device buffers made here by the caller, which is allowed) and
compare it with the handle-based pbf_estimate_densities on the same input, twice in a
row with different inputs, since every call reuses the scratch array the last call left.
The file sorts last so that a run stopping at the first failure has run everything else.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np
import pytest

from fluid_gb300 import scenes
from tests.golden.make_golden import params_from_json
from tests.helpers import rel_err

pytestmark = pytest.mark.gpu

GOLDEN_DIR = os.path.join(os.path.dirname(__file__), "golden")
TOL = 1e-5  # the one-step tolerance of the parity tests


@pytest.fixture(scope="module")
def pbf():
    from fluid_gb300 import pbf as mod

    mod.lib()
    return mod


def _noalloc(pbf, prm, pos32):
    import torch

    x = torch.from_numpy(np.ascontiguousarray(pos32, dtype=np.float32)).cuda()
    rho = torch.full((pos32.shape[0],), float("nan"), dtype=torch.float32, device="cuda")
    cp = prm.to_c()
    stream = torch.cuda.current_stream().cuda_stream
    rc = pbf.lib().pbf_density_noalloc(ctypes.byref(cp), pos32.shape[0], ctypes.c_void_p(x.data_ptr()),
                                       ctypes.c_void_p(rho.data_ptr()), ctypes.c_void_p(stream))
    assert rc == 0, pbf.lib().pbf_last_error(None).decode()
    torch.cuda.synchronize()
    return rho.cpu().numpy()


def _with_handle(pbf, prm, pos32):
    with pbf.Simulator(pos32, None, prm) as sim:
        return sim.estimate_densities()


def _cases():
    g = np.load(os.path.join(GOLDEN_DIR, "p_default_1step.npz"))
    sc = scenes.block4096(1)
    return [(params_from_json(str(g["params"])), g["pos_in"].astype(np.float32)),
            (sc.params, sc.pos.astype(np.float32))]


def test_noalloc_matches_handle_path_on_consecutive_calls(pbf, oracle_lib):
    cases = _cases()
    order = [0, 1, 0]  # the third call runs on what the second left in the scratch array
    for k in order:
        prm, pos = cases[k]
        got = _noalloc(pbf, prm, pos)
        want = _with_handle(pbf, prm, pos)
        ref = oracle_lib.estimate_densities(pos.astype(np.float64), prm)  # the FP64 restatement
        err, err64 = rel_err(got, want), rel_err(got, ref)
        print(f"case {k}: n={len(pos)} rel err vs pbf_estimate_densities {err:.2e}, vs FP64 {err64:.2e}")
        assert np.all(np.isfinite(got))
        assert err < TOL and err64 < TOL


def _largest_case():
    """65,536 particles (the particle limit) with h such that the unit box needs 64^3 =
    262,144 cells of size h (the cell limit): the scratch layout's offsets and the scan's
    tile count at their largest."""
    h = 0.0162
    prm = scenes.physical_params(h, h / 2)
    pos = scenes.lattice(64, 32, 32, h / 2, corner=(0.2, 0.0, 0.3))
    pos += scenes.uniform(29, pos.size, -1e-4, 1e-4).reshape(pos.shape)
    return prm, pos.astype(np.float32)


def test_noalloc_at_its_limits(pbf, oracle_lib):
    from tests.helpers import scene_grid

    prm, pos = _largest_case()
    _, _, dims = scene_grid(prm, prm.box_lo, prm.box_hi)
    assert len(pos) == 65536 and int(np.prod(dims)) == 262144
    for _ in range(2):
        got = _noalloc(pbf, prm, pos)
        want = _with_handle(pbf, prm, pos)
        ref = oracle_lib.estimate_densities(pos.astype(np.float64), prm)
        err, err64 = rel_err(got, want), rel_err(got, ref)
        print(f"limits: rel err vs pbf_estimate_densities {err:.2e}, vs FP64 {err64:.2e}")
        assert err < TOL and err64 < TOL


def test_noalloc_dense_cell(pbf):
    """300 particles in about one cell (more than the 256 whose order the call fixes):
    within the tolerance of the handle path, call after call."""
    rng = np.random.default_rng(8)
    prm = scenes.physical_params(0.1, 0.05)
    pos = np.stack([rng.uniform(0.41, 0.49, 300), rng.uniform(0.01, 0.09, 300),
                    rng.uniform(0.41, 0.49, 300)], 1).astype(np.float32)
    want = _with_handle(pbf, prm, pos)
    for _ in range(2):
        assert rel_err(_noalloc(pbf, prm, pos), want) < TOL


def test_noalloc_empty_and_host_pointers(pbf):
    lib = pbf.lib()
    prm = scenes.block4096(1).params
    cp = prm.to_c()
    assert lib.pbf_density_noalloc(ctypes.byref(cp), 0, None, None, None) == 0
    # host memory is refused before any device work
    x = np.zeros((10, 3), dtype=np.float32)
    r = np.zeros(10, dtype=np.float32)
    rc = lib.pbf_density_noalloc(ctypes.byref(cp), 10, x.ctypes.data_as(ctypes.c_void_p),
                                 r.ctypes.data_as(ctypes.c_void_p), None)
    assert rc == 1 and b"device" in lib.pbf_last_error(None)


def test_noalloc_rejects_inputs_beyond_its_limits(pbf):
    lib = pbf.lib()
    prm = scenes.block4096(1).params
    cp = prm.to_c()
    dummy = ctypes.c_void_p(16)  # never dereferenced: the size check comes first
    rc = lib.pbf_density_noalloc(ctypes.byref(cp), 65537, dummy, dummy, None)
    assert rc == 1
    assert b"PBF_NOALLOC_MAX_PARTICLES" in lib.pbf_last_error(None)
    fine = prm.with_(h=0.002, h2=0.000004)  # 500^3 cells of size h over the unit box
    cp = fine.to_c()
    rc = lib.pbf_density_noalloc(ctypes.byref(cp), 10, dummy, dummy, None)
    assert rc == 1
    assert b"PBF_NOALLOC_MAX_CELLS" in lib.pbf_last_error(None)
