"""GPU parity: the CUDA step through the C ABI against the FP64 oracle and the golden vectors.

Tolerances: after one step, positions, velocities and densities within
1e-5 normwise relative error of the FP64 reference step in the order-independent XSPH form;
neighbour sets and cell ids bit-exact against a host check that evaluates the same FP32
predicate on the same FP32 x*. Every test also reports the FP32-vs-FP64 error it saw.
"""
from __future__ import annotations

import os

import numpy as np
import pytest

from fluid_gb300 import scenes
from fluid_gb300.params import PBF_FLAG_GRAPH, PBF_FLAG_KEEP_PREDICTED, PBF_FLAG_STATS
from tests.golden.make_golden import params_from_json
from tests.helpers import cells_fp32, csr_sets, neighbor_sets_fp32, rel_err

pytestmark = pytest.mark.gpu

TOL_1STEP = 1e-5
GOLDEN_DIR = os.path.join(os.path.dirname(__file__), "golden")


@pytest.fixture(scope="module")
def pbf():
    from fluid_gb300 import pbf as mod

    mod.lib()
    return mod


def _f32(a):
    return np.asarray(a, dtype=np.float32).astype(np.float64)


def _run_gpu(pbf, pos, vel, prm, steps=1, **kw):
    with pbf.Simulator(pos, vel, prm, **kw) as sim:
        sim.time_step(prm.dt, steps)
        return sim.positions(), sim.velocities(), sim.densities(), sim.stats()


def test_one_step_block4096_matches_oracle(pbf, oracle_lib):
    sc = scenes.block4096(1)
    pos, vel = _f32(sc.pos), _f32(sc.vel)
    x, v, rho, st = _run_gpu(pbf, pos, vel, sc.params)
    ref = oracle_lib.step(pos, vel, sc.params, steps=1)
    ex, ev, er = rel_err(x, ref["pos"]), rel_err(v, ref["vel"]), rel_err(rho, ref["density"])
    print(f"block4096 1 step FP32 vs FP64: pos {ex:.2e} vel {ev:.2e} rho {er:.2e}")
    assert ex < TOL_1STEP and ev < TOL_1STEP and er < TOL_1STEP
    assert st["error_flags"] == 0
    assert abs(st["mean_density"] - ref["density"].mean()) / ref["density"].mean() < 1e-5
    assert abs(st["mean_density_iter0"] - ref["mean_density_iter0"][0]) / ref["mean_density_iter0"][0] < 1e-5


def _golden(name):
    g = np.load(os.path.join(GOLDEN_DIR, f"{name}.npz"))
    return g, params_from_json(str(g["params"]))


def test_golden_block4096_one_step(pbf):
    """Against the reference's own output (FP64 inputs) on the jittered config-1 block."""
    g, prm = _golden("block4096_mass_1step")
    x, v, rho, st = _run_gpu(pbf, g["pos_in"], g["vel_in"], prm)
    ex, ev, er = rel_err(x, g["pos"]), rel_err(v, g["vel"]), rel_err(rho, g["density"])
    print(f"block4096 vs reference: pos {ex:.2e} vel {ev:.2e} rho {er:.2e}")
    assert ex < TOL_1STEP and ev < TOL_1STEP and er < TOL_1STEP


def _fp64_sensitivity(oracle_lib, g, prm, sets):
    """How much the FP64 reference step itself moves when only its inputs are rounded to FP32."""
    a = oracle_lib.step(g["pos_in"], g["vel_in"], prm, 1, given_neighbors=sets)
    b = oracle_lib.step(_f32(g["pos_in"]), _f32(g["vel_in"]), prm, 1, given_neighbors=sets)
    return {k: rel_err(b[k], a[k]) for k in ("pos", "vel", "density")}, b


@pytest.mark.parametrize("name", ["p_default_1step", "spheresp_default_1step"])
def test_golden_lattice_fixtures_on_identical_neighbor_sets(pbf, oracle_lib, name):
    """The reference's own particle files are exact lattices: pairs sit at exactly r = H, so
    neighbour membership is a knife edge (the FP64 step moves by 2e-3 when its inputs are
    rounded to FP32). Compare on identical sets: the GPU's FP32 sets (checked bit-exact
    against the host predicate) fed to the FP64 oracle on the same FP32 inputs. The bar is
    1e-5, or 10x the FP64 step's own sensitivity to input rounding where that is larger
    (the spheres file: 12 undamped Jacobi iterations over ~110 neighbours)."""
    g, prm = _golden(name)
    prm = prm.with_(flags=PBF_FLAG_STATS | PBF_FLAG_KEEP_PREDICTED)
    with pbf.Simulator(g["pos_in"], g["vel_in"], prm) as sim:
        sim.time_step(prm.dt, 1)
        x, v, rho = sim.positions(), sim.velocities(), sim.densities()
        off, ids = sim.neighbors()
        xs = sim.predicted()
    e_off, e_ids = neighbor_sets_fp32(xs, prm.h2)
    assert np.array_equal(off, e_off) and np.array_equal(ids.astype(np.int64), e_ids)
    sens, ref = _fp64_sensitivity(oracle_lib, g, prm, (off, ids))
    got = {"pos": rel_err(x, ref["pos"]), "vel": rel_err(v, ref["vel"]), "density": rel_err(rho, ref["density"])}
    print(f"{name}: GPU vs FP64 on identical sets {got}; FP64 sensitivity to FP32 inputs {sens}")
    for k in got:
        assert got[k] < max(TOL_1STEP, 10 * sens[k]), k
    # and the reference's own output differs from the oracle only through the set knife edge
    full = oracle_lib.step(g["pos_in"], g["vel_in"], prm, 1)
    assert np.array_equal(full["pos"], g["pos"])


def _ensemble(oracle_lib, pos, vel, prm, steps, members=3, seed=0):
    """FP64 and FP32 oracle rollouts from FP32-rounded inputs perturbed by about one ulp."""
    rng = np.random.default_rng(seed)
    base = _f32(pos)
    out = []
    for fp32 in (False, True):
        for k in range(members):
            p = base if k == 0 else base * (1 + rng.uniform(-6e-8, 6e-8, base.shape))
            out.append(oracle_lib.step(p, _f32(vel), prm, steps, fp32=fp32))
    return out


def _density_error(rho, prm):
    c = np.abs(np.asarray(rho, dtype=np.float64) / prm.rest_density - 1)
    return c.mean(), np.percentile(c, 99)


@pytest.mark.parametrize("name", ["block512_mass_20step", "block512_ref_4step", "p_default_3step"])
def test_golden_rollouts_statistics(pbf, oracle_lib, name):
    """Multi-step rollouts are chaotic (FP32 rounding of the inputs alone moves the FP64
    rollout by percent after ten steps), so they are compared by density-constraint
    statistics against an ensemble of FP64 and FP32 oracle rollouts from ulp-perturbed
    inputs. Horizons stay at or below 20 steps: beyond that the clumping rate of the
    reference's formulation depends on the arithmetic precision itself."""
    g, prm = _golden(name)
    steps = int(g["steps"])
    x, v, rho, st = _run_gpu(pbf, g["pos_in"], g["vel_in"], prm, steps=steps)
    ens = _ensemble(oracle_lib, g["pos_in"], g["vel_in"], prm, steps)
    means = np.array([_density_error(e["density"], prm)[0] for e in ens])
    p99s = np.array([_density_error(e["density"], prm)[1] for e in ens])
    m, p99 = _density_error(rho, prm)
    ref_m, _ = _density_error(g["density"], prm)
    print(f"{name}: mean|C| gpu {m:.4f} ensemble {means.min():.4f}..{means.max():.4f} reference {ref_m:.4f}; "
          f"p99|C| gpu {p99:.4f} ensemble {p99s.min():.4f}..{p99s.max():.4f}")
    margin = max(means.max() - means.min(), 0.1 * means.mean()) + 1e-3
    assert means.min() - margin <= m <= means.max() + margin
    margin99 = max(p99s.max() - p99s.min(), 0.25 * p99s.mean()) + 1e-3
    assert p99s.min() - margin99 <= p99 <= p99s.max() + margin99
    assert np.all(np.isfinite(x))


def test_neighbor_sets_and_cells_bitexact(pbf, oracle_lib):
    sc = scenes.block4096(1)
    prm = sc.params.with_(flags=PBF_FLAG_STATS | PBF_FLAG_KEEP_PREDICTED)
    pos, vel = _f32(sc.pos), _f32(sc.vel)
    with pbf.Simulator(pos, vel, prm) as sim:
        sim.time_step(prm.dt, 1)
        xs = sim.predicted()
        off, ids = sim.neighbors()
        cells = sim.cells()
    e_off, e_ids = neighbor_sets_fp32(xs, prm.h2)
    assert np.array_equal(off, e_off)
    assert np.array_equal(ids.astype(np.int64), e_ids)
    assert np.array_equal(cells.astype(np.int64), cells_fp32(xs, prm))
    # against the FP64 reference sets: only pairs within rounding of the radius may differ
    ref = oracle_lib.step(pos, vel, sc.params, steps=1, neighbors=True, predicted=True)
    a, b = csr_sets(off, ids), csr_sets(ref["nbr_offsets"], ref["nbr_idx"])
    diff = sum(len(s ^ t) for s, t in zip(a, b))
    print(f"neighbour pairs differing FP32 vs FP64: {diff} of {len(ids)}")
    assert diff <= 1e-4 * len(ids) + 2
    assert rel_err(xs, ref["pred"]) < 1e-6


def test_crowded_cells_sort_deterministically(pbf):
    """600 particles inside about one cell of size h (a compressed clump): the cell sort
    takes its block-wide path (cells over 32 particles); the step is bit-identical from run
    to run and the neighbour sets match the host FP32 check."""
    rng = np.random.default_rng(8)
    prm = scenes.physical_params(0.1, 0.05, max_neighbors=1023,
                                 flags=PBF_FLAG_STATS | PBF_FLAG_KEEP_PREDICTED)
    pos = np.stack([rng.uniform(0.41, 0.49, 600), rng.uniform(0.01, 0.09, 600), rng.uniform(0.41, 0.49, 600)], 1)
    pos = _f32(pos)
    vel = np.zeros_like(pos)
    runs = []
    for _ in range(3):
        with pbf.Simulator(pos, vel, prm) as sim:
            sim.time_step(prm.dt, 1)
            runs.append((sim.positions(), sim.velocities(), sim.densities(), sim.predicted(), sim.neighbors()))
    for r in runs[1:]:
        for a, b in zip(runs[0][:4], r[:4]):
            assert np.array_equal(a, b)
    off, ids = runs[0][4]
    e_off, e_ids = neighbor_sets_fp32(runs[0][3], prm.h2)
    assert np.array_equal(off, e_off) and np.array_equal(ids.astype(np.int64), e_ids)
    assert np.diff(off).max() > 400


def test_determinism_and_graph_replay(pbf):
    sc = scenes.block4096(2)
    pos, vel = _f32(sc.pos), _f32(sc.vel)
    runs = []
    for flags in (PBF_FLAG_STATS, PBF_FLAG_STATS, PBF_FLAG_STATS | PBF_FLAG_GRAPH):
        x, v, rho, _ = _run_gpu(pbf, pos, vel, sc.params.with_(flags=flags), steps=5)
        runs.append((x, v, rho))
    for r in runs[1:]:
        for a, b in zip(runs[0], r):
            assert np.array_equal(a, b)


def test_profiled_graph_replay_matches_and_times_every_phase(pbf):
    """Profiling inside graph replay (phase events as graph nodes, one graph per event set
    and buffer parity): same results as plain launches, and every phase timed."""
    sc = scenes.block4096(3)
    pos, vel = _f32(sc.pos), _f32(sc.vel)
    ref = _run_gpu(pbf, pos, vel, sc.params.with_(flags=PBF_FLAG_STATS), steps=6)
    with pbf.Simulator(pos, vel, sc.params.with_(flags=PBF_FLAG_STATS | PBF_FLAG_GRAPH)) as sim:
        sim.set_profiling(True)
        sim.time_step(sc.params.dt, 3)
        sim.set_profiling(False)
        sim.time_step(sc.params.dt, 1)
        sim.set_profiling(True)
        sim.time_step(sc.params.dt, 2)
        ph = sim.phase_times()
        out = (sim.positions(), sim.velocities(), sim.densities())
    for a, b in zip(ref[:3], out):
        assert np.array_equal(a, b)
    for name in ("predict", "neighbors", "lambda", "deltap", "xsph", "vorticity"):
        ms, launches = ph[name]
        assert ms > 0 and launches > 0, name
    assert ph["lambda"][1] == 5 * sc.params.iters


def test_rollout_block4096_density_error(pbf, oracle_lib):
    """20-step config-1 rollout: density-constraint statistics against the oracle ensemble."""
    sc = scenes.block4096(1)
    x, v, rho, st = _run_gpu(pbf, _f32(sc.pos), _f32(sc.vel), sc.params, steps=20)
    ens = _ensemble(oracle_lib, sc.pos, sc.vel, sc.params, 20)
    means = np.array([_density_error(e["density"], sc.params)[0] for e in ens])
    m, _ = _density_error(rho, sc.params)
    print(f"block4096 20 steps: mean|C| gpu {m:.4f} ensemble {means.min():.4f}..{means.max():.4f}")
    margin = max(means.max() - means.min(), 0.1 * means.mean()) + 1e-3
    assert means.min() - margin <= m <= means.max() + margin
    assert np.all(np.isfinite(x)) and st["error_flags"] == 0


def test_estimate_densities_and_density_at(pbf, oracle_lib):
    g = np.load(os.path.join(GOLDEN_DIR, "p_default_1step.npz"))
    prm = params_from_json(str(g["params"]))
    pos = g["pos_in"]
    with pbf.Simulator(pos, g["vel_in"], prm) as sim:
        d = sim.estimate_densities()
        rng = np.random.default_rng(3)
        pts = pos[rng.integers(0, len(pos), 64)] + rng.uniform(-0.2, 0.2, (64, 3))
        q = sim.estimate_density_at(pts)
        # after a density query the simulator still steps like a fresh one
        sim.time_step(prm.dt, 1)
        x = sim.positions()
    assert rel_err(d, g["load_density"]) < 1e-5
    ref_q = oracle_lib.estimate_density_at(_f32(pos), _f32(pts), prm)
    assert rel_err(q, ref_q) < 1e-5
    # a step after the queries equals a step of a fresh simulator (the queries re-sort only)
    with pbf.Simulator(pos, g["vel_in"], prm) as fresh:
        fresh.time_step(prm.dt, 1)
        assert np.array_equal(fresh.positions(), x)


def test_batched_equals_separate(pbf):
    """A batch of independent scenes gives bit-identical results to stepping each alone."""
    b = scenes.batched_256(seed=9, n_scenes=6, lo=500, hi=3000)
    pos, vel = _f32(b.pos), _f32(b.vel)
    with pbf.Simulator(pos, vel, b.params, counts=b.counts, boxes=b.boxes) as sim:
        sim.time_step(b.params.dt, 3)
        xb, vb = sim.positions(), sim.velocities()
    off = 0
    for c in b.counts:
        x, v, _, _ = _run_gpu(pbf, pos[off:off + c], vel[off:off + c], b.params, steps=3)
        assert np.array_equal(x, xb[off:off + c])
        assert np.array_equal(v, vb[off:off + c])
        off += c


def test_batch_with_empty_scenes(pbf):
    """Scenes without particles (first, in the middle, last) take no slots: the batch steps
    the others to the same bits as a batch of only them."""
    b = scenes.batched_256(seed=4, n_scenes=3, lo=500, hi=2000)
    pos, vel = _f32(b.pos), _f32(b.vel)
    with pbf.Simulator(pos, vel, b.params, counts=b.counts, boxes=b.boxes) as sim:
        sim.time_step(b.params.dt, 2)
        x0, v0 = sim.positions(), sim.velocities()
    counts = [0, b.counts[0], 0, 0, b.counts[1], b.counts[2], 0]
    boxes = [b.boxes[0], b.boxes[0], b.boxes[1], b.boxes[2], b.boxes[1], b.boxes[2], b.boxes[2]]
    with pbf.Simulator(pos, vel, b.params, counts=counts, boxes=boxes) as sim:
        sim.time_step(b.params.dt, 2)
        assert np.array_equal(sim.positions(), x0) and np.array_equal(sim.velocities(), v0)


def test_empty_and_tiny(pbf):
    prm = scenes.physical_params(0.1, 0.05)
    with pbf.Simulator(np.zeros((0, 3)), None, prm) as sim:
        sim.time_step(prm.dt, 2)
        assert sim.positions().shape == (0, 3)
    x, v, rho, _ = _run_gpu(pbf, np.array([[0.5, 0.5, 0.5]]), np.zeros((1, 3)), prm, steps=1)
    assert rho[0] == 0.0
    assert abs(v[0, 1] - (-9.8 / 60)) < 1e-6


def test_invalid_arguments(pbf):
    prm = scenes.physical_params(0.1, 0.05)
    with pytest.raises(pbf.PbfError) as e:
        pbf.Simulator(np.zeros((4, 3)), None, prm.with_(h=-1.0))
    assert e.value.status == 1
    with pytest.raises(pbf.PbfError):
        pbf.Simulator(np.zeros((4, 3)), None, prm.with_(max_neighbors=2))


def test_neighbor_capacity_is_reported(pbf):
    sc = scenes.block4096(1)
    prm = sc.params.with_(max_neighbors=8)
    with pbf.Simulator(_f32(sc.pos), _f32(sc.vel), prm) as sim:
        with pytest.raises(pbf.PbfError) as e:
            sim.time_step(prm.dt, 1)
        assert e.value.status == 5


def test_list_capacity_does_not_change_results(pbf):
    """A slot's list words lie in groups of four: a capacity just above the largest list (its
    last group partly used), an odd one and a large one give the same bits."""
    sc = scenes.block4096(2)
    pos, vel = _f32(sc.pos), _f32(sc.vel)
    with pbf.Simulator(pos, vel, sc.params.with_(max_neighbors=256, flags=PBF_FLAG_STATS)) as sim:
        sim.time_step(sc.params.dt, 1)
        mx = sim.stats()["max_neighbors"]
    assert mx > 8
    outs = []
    for cap in (mx, mx + 1, mx + 7, 256):
        with pbf.Simulator(pos, vel, sc.params.with_(max_neighbors=cap, flags=PBF_FLAG_STATS)) as sim:
            sim.time_step(sc.params.dt, 1)
            assert sim.stats()["error_flags"] == 0, cap
            outs.append((sim.positions(), sim.velocities(), sim.densities(), sim.neighbors()))
    for o in outs[1:]:
        for a, b in zip(o[:3], outs[0][:3]):
            assert np.array_equal(a, b)
        assert np.array_equal(o[3][0], outs[0][3][0]) and np.array_equal(o[3][1], outs[0][3][1])


def _capacity_params(h, s, hi):
    return scenes.physical_params(h, s, box_lo=(0.0, 0.0, 0.0), box_hi=hi, clip_planes=(),
                                  clamp_lo=(0.0, 0.0, 0.0), clamp_hi=hi)


def test_slab_offset_limit_is_reported(pbf):
    """A list entry holds a 14-bit offset into its slab's three rows of cells. Rows of 990
    cells at ~16 particles a cell (15,000 slots a row) overflow it: the step must fail with
    PBF_ERR_CAPACITY, not store a wrapped offset."""
    h, s = 0.01, 0.004
    p = scenes.lattice(2470, 7, 7, s, corner=(0.002, 0.002, 0.002))
    prm = _capacity_params(h, s, (9.9, 0.032, 0.032))
    with pbf.Simulator(_f32(p), np.zeros_like(p), prm) as sim:
        with pytest.raises(pbf.PbfError) as e:
            sim.time_step(prm.dt, 1)
    assert e.value.status == 5 and "row" in str(e.value)


def test_row_candidate_limit_is_reported(pbf):
    """5,000 particles inside one cell: more candidates in a row than the build scans
    (4,096); the step must fail with PBF_ERR_CAPACITY."""
    h, s = 0.1, 0.05
    rng = np.random.default_rng(3)
    p = rng.uniform(0.52, 0.58, (5000, 3))
    prm = _capacity_params(h, s, (1.0, 1.0, 1.0)).with_(max_neighbors=1024)
    with pbf.Simulator(_f32(p), np.zeros_like(p), prm) as sim:
        with pytest.raises(pbf.PbfError) as e:
            sim.time_step(prm.dt, 1)
    assert e.value.status == 5


def test_autotune_keeps_state_and_results(pbf):
    """The autotuner restores the state it timed on; launch shapes never change results."""
    sc = scenes.block4096(3)
    with pbf.Simulator(_f32(sc.pos), _f32(sc.vel), sc.params) as sim:
        sim.time_step(sc.params.dt, 2)
        x0 = sim.positions()
        best = sim.autotune(sc.params.dt, reps=2)
        assert all(best[k] in (64, 128, 256, 512) for k in ("block_predict", "block_nbr", "block_solve",
                                                              "block_misc"))
        assert best["gather_depth"] in (4, 8) and best["list_stream"] in (0, 1)
        assert np.array_equal(sim.positions(), x0)
        sim.time_step(sc.params.dt, 3)
        xa = sim.positions()
    with pbf.Simulator(_f32(sc.pos), _f32(sc.vel), sc.params) as sim:
        sim.set_tuning(block_nbr=512, block_solve=64, block_predict=128, block_misc=64)
        sim.time_step(sc.params.dt, 5)
        assert np.array_equal(sim.positions(), xa)


@pytest.mark.parametrize("scene", ["block4096", "batched", "crowded"])
def test_kernel_forms_give_identical_bits(pbf, scene):
    """Every tuning form (gather depth 4 and 8, cached and streaming list loads, every block
    size) visits each particle's neighbours in the same order and rounds every operation
    explicitly: the neighbour lists and three steps of state are bit-identical across forms."""
    if scene == "block4096":
        sc = scenes.block4096(5)
        pos, vel, prm, kw = _f32(sc.pos), _f32(sc.vel), sc.params, {}
    elif scene == "batched":
        b = scenes.batched_256(seed=9, n_scenes=5, lo=500, hi=3000)
        pos, vel, prm, kw = _f32(b.pos), _f32(b.vel), b.params, {"counts": b.counts, "boxes": b.boxes}
    else:
        rng = np.random.default_rng(8)
        prm = scenes.physical_params(0.1, 0.05, max_neighbors=1023)
        pos = _f32(np.stack([rng.uniform(0.41, 0.49, 600), rng.uniform(0.01, 0.09, 600),
                             rng.uniform(0.41, 0.49, 600)], 1))
        vel, kw = np.zeros_like(pos), {}
    forms = [dict(gather_depth=8, list_stream=0, block_nbr=128, block_solve=128),
             dict(gather_depth=8, list_stream=1, block_nbr=128, block_solve=128),
             dict(gather_depth=4, list_stream=0, block_nbr=128, block_solve=128),
             dict(gather_depth=4, list_stream=1, block_nbr=64, block_solve=256),
             dict(gather_depth=8, list_stream=1, block_nbr=512, block_solve=512),
             dict(gather_depth=4, list_stream=0, block_nbr=256, block_solve=64)]
    outs = []
    for f in forms:
        with pbf.Simulator(pos, vel, prm.with_(flags=PBF_FLAG_STATS), **kw) as sim:
            sim.set_tuning(**f)
            sim.time_step(prm.dt, 1)
            nb = sim.neighbors()
            sim.time_step(prm.dt, 2)
            outs.append((nb, sim.positions(), sim.velocities(), sim.densities(), sim.stats()["error_flags"]))
    for o in outs[1:]:
        assert np.array_equal(o[0][0], outs[0][0][0]) and np.array_equal(o[0][1], outs[0][0][1])
        for a, b in zip(o[1:4], outs[0][1:4]):
            assert np.array_equal(a, b)
        assert o[4] == outs[0][4] == 0


def test_tuning_arguments(pbf):
    sc = scenes.block4096(1)
    with pbf.Simulator(_f32(sc.pos), _f32(sc.vel), sc.params) as sim:
        for bad in (dict(gather_depth=6), dict(gather_depth=0), dict(list_stream=-1), dict(block_nbr=100)):
            with pytest.raises(pbf.PbfError):
                sim.set_tuning(**bad)
        t = sim.tuning()
        assert t["gather_depth"] in (4, 8) and t["list_stream"] in (0, 1)


def test_collider_mesh_matches_oracle(pbf, oracle_lib):
    """A block dropped onto a two-triangle ramp (pbf_set_collider_mesh) against the FP64
    restatement with the same triangles (pinned to the reference build by
    tests/golden/ramp_block512_2step.npz), one step on identical neighbour sets. The GPU
    backs off 4 FP32 ulps from a triangle where the reference backs off 1e-11, which
    moves stopped particles by ~5e-7."""
    from tests.golden.make_golden import RAMP, ramp_scene

    p, v, prm = ramp_scene()
    pos, vel = _f32(p), _f32(v)
    ramp = RAMP.astype(np.float32)
    with pbf.Simulator(pos, vel, prm) as sim:
        sim.set_collider_mesh(ramp)
        sim.time_step(prm.dt, 1)
        x, v1, rho = sim.positions(), sim.velocities(), sim.densities()
        nb = sim.neighbors()
    with pbf.Simulator(pos, vel, prm) as sim:
        sim.time_step(prm.dt, 1)
        x_free = sim.positions()
    oracle_lib.set_mesh(ramp.astype(np.float64))
    try:
        ref = oracle_lib.step(pos, vel, prm, 1, given_neighbors=nb)
    finally:
        oracle_lib.set_mesh(None)
    ex, ev, er = rel_err(x, ref["pos"]), rel_err(v1, ref["vel"]), rel_err(rho, ref["density"])
    moved = np.abs(x - x_free).max()
    print(f"ramp 1 step FP32 vs FP64: pos {ex:.2e} vel {ev:.2e} rho {er:.2e}; ramp moves particles by {moved:.2e}")
    assert moved > 1e-3
    assert ex < 1e-5 and ev < 1e-4 and er < 1e-4
    assert np.all(x[:, 1] >= ref["pos"][:, 1].min() - 1e-5)


def test_collider_mesh_arguments(pbf):
    import torch

    sc = scenes.block4096(1)
    with pbf.Simulator(_f32(sc.pos), _f32(sc.vel), sc.params) as sim:
        with pytest.raises(pbf.PbfError):
            sim.set_collider_mesh(np.zeros((1, 9), dtype=np.float32))  # degenerate
        with pytest.raises(pbf.PbfError):
            sim.set_collider_mesh(np.ones((1025, 9), dtype=np.float32))
        from tests.golden.make_golden import RAMP

        sim.set_collider_mesh(RAMP)
        x = torch.zeros((sim.n, 3), dtype=torch.float32, device="cuda")
        r = torch.zeros(1, dtype=torch.float64, device="cuda")
        with pytest.raises(pbf.PbfError):  # the adjoint takes the box collider only
            sim.adjoint_step_device(sc.params.dt, None, None, None, None, x.data_ptr(), x.data_ptr(), r.data_ptr())
        sim.set_collider_mesh(None)
        sim.time_step(sc.params.dt, 1)


def test_get_state_matches_the_single_getters(pbf):
    """pbf_get_state (one reordering pass, one wait) returns what pbf_get_positions,
    pbf_get_velocities and pbf_get_densities return one by one; NULL arrays are skipped."""
    import ctypes

    sc = scenes.block4096(3)
    with pbf.Simulator(_f32(sc.pos), _f32(sc.vel), sc.params) as sim:
        sim.time_step(sc.params.dt, 2)
        x, v, rho = sim.positions(), sim.velocities(), sim.densities()
        n = len(x)
        xs, vs, rs = (np.zeros((n, 3), np.float32), np.zeros((n, 3), np.float32), np.zeros(n, np.float32))
        L = pbf.lib()
        assert L.pbf_get_state(sim._h, xs.ctypes.data_as(pbf.P), vs.ctypes.data_as(pbf.P),
                               rs.ctypes.data_as(pbf.P)) == 0
        assert np.array_equal(xs, x) and np.array_equal(vs, v) and np.array_equal(rs, rho)
        v2 = np.zeros((n, 3), np.float32)
        assert L.pbf_get_state(sim._h, None, v2.ctypes.data_as(pbf.P), None) == 0
        assert np.array_equal(v2, v)
        assert L.pbf_get_state(sim._h, None, None, None) == 0


@pytest.mark.gpu
def test_page_locked_host_buffers_match_pageable_ones(pbf):
    """pbf_set_state / pbf_get_state with page-locked host buffers (views into the middle
    of one larger page-locked block) carry the same state, bit for bit, as with pageable
    ones."""
    import torch

    sc = scenes.block4096(4)
    n = len(sc.pos)
    L = pbf.lib()
    x0, v0 = _f32(sc.pos), _f32(sc.vel)
    outs = []
    for pinned in (False, True):
        with pbf.Simulator(x0, v0, sc.params) as sim:
            if pinned:
                blk = torch.zeros(3 * n * 4 + 64, dtype=torch.float32, pin_memory=True).numpy()
                xh, vh = blk[16:16 + 3 * n].reshape(n, 3), blk[32 + 3 * n:32 + 6 * n].reshape(n, 3)
                xo = blk[48 + 6 * n:48 + 9 * n].reshape(n, 3)
                ro = blk[48 + 9 * n:48 + 10 * n]
            else:
                xh, vh, xo, ro = (np.zeros((n, 3), np.float32), np.zeros((n, 3), np.float32),
                                  np.zeros((n, 3), np.float32), np.zeros(n, np.float32))
            xh[:] = x0
            vh[:] = v0
            assert L.pbf_set_state(sim._h, xh.ctypes.data_as(pbf.P), vh.ctypes.data_as(pbf.P)) == 0
            sim.time_step(sc.params.dt, 1)
            assert L.pbf_get_state(sim._h, xo.ctypes.data_as(pbf.P), vh.ctypes.data_as(pbf.P),
                                   ro.ctypes.data_as(pbf.P)) == 0
            outs.append((xo.copy(), vh.copy(), ro.copy()))
    for a, b in zip(*outs):
        assert np.array_equal(a, b)
    assert np.all(np.isfinite(outs[1][0])) and not np.array_equal(outs[1][0], x0)
