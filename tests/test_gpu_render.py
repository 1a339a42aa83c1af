"""GPU path tracer (pbf_render) against the CPU restatement of the reference's PathTracer.

The restatement is pinned byte for byte to the reference's own frames by
tests/test_render_oracle.py. Here both draw the same random numbers (a function of
seed, pixel, sample and draw index), trace the same triangles (the scene plus the
surface pbf_surface returns) and differ in arithmetic: FP32 on the GPU, FP64 geometry in
the restatement, and secondary rays start at 1e-4 on the GPU against the reference's
1e-11. A path whose Russian-roulette or glass coin lands within rounding of its
probability, or that grazes an edge, can turn differently, so the bars are on the bulk of
the pixels and on the frame's mean, written in each test.
"""
from __future__ import annotations

import os

import numpy as np
import pytest

from fluid_gb300 import render as R
from tests.golden.make_golden import params_from_json
from tests.golden.make_render_golden import camera_from_json, scene_from_arrays

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


@pytest.fixture(scope="module")
def pbf():
    from fluid_gb300 import pbf as mod

    mod.lib()
    return mod


def _case(name):
    g = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    return g, scene_from_arrays(g), camera_from_json(str(g["camera"])), params_from_json(str(g["params"]))


def _gpu(pbf, g, scene, cam, prm, W, H, aa, depth, area, seed, surface=True):
    pos = np.asarray(g["pos"], dtype=np.float32)
    with pbf.Simulator(pos, np.zeros_like(pos), prm) as sim:
        sim.set_render_scene(scene)
        out = sim.render(cam, W, H, aa, depth, area, seed=seed, fluid_surface=surface)
        again = sim.render(cam, W, H, aa, depth, area, seed=seed, fluid_surface=surface)
        sx, sn = sim.surface() if surface else (np.zeros((0, 3, 3)), np.zeros((0, 3, 3)))
    assert np.array_equal(out["hdr"], again["hdr"]) and np.array_equal(out["rgba"], again["rgba"])
    return out, sx.astype(np.float64), sn.astype(np.float64)


def _compare(name, a, b, frac_bar, mean_bar):
    d = np.abs(a - b).max(-1)
    scale = np.maximum(np.abs(b).max(-1), 1e-2)
    close = d <= 1e-3 * scale + 1e-4
    mean_rel = abs(a.mean() - b.mean()) / max(b.mean(), 1e-6)
    print(f"{name}: {close.mean() * 100:.2f}% of pixels within 1e-3, frame means {a.mean():.5f} / {b.mean():.5f} "
          f"(rel {mean_rel:.2e}), max |diff| {d.max():.3e}")
    assert close.mean() >= frac_bar and mean_rel <= mean_bar


@pytest.mark.parametrize("name", ["render_p_default", "render_p_default_aa4", "render_materials"])
def test_render_matches_restatement(pbf, oracle_lib, name):
    from oracle import oracle

    g, scene, cam, prm = _case(name)
    W, H, aa, depth, area, seed = (int(v) for v in g["settings"])
    out, sx, sn = _gpu(pbf, g, scene, cam, prm, W, H, aa, depth, area, seed)
    assert out["stats"]["surface_triangles"] == len(sx) > 100
    ref = oracle.render(scene, cam, sx, sn, W, H, aa, depth, area, oracle.RNG_COUNTER, seed)
    # bars: 99% of pixels within 1e-3 relative, the frame mean within 1e-3
    _compare(name, out["hdr"], ref["hdr"], 0.99, 1e-3)


def test_deterministic_lights_match_closely(pbf, oracle_lib):
    """Point and directional lights, one ray per pixel, no bounce: no random numbers, so
    every pixel is the same function on both sides (bar: 99.5% within 1e-3, mean 1e-4)."""
    from oracle import oracle

    g, scene, cam, prm = _case("render_p_default")
    scene.lights = [R.Light(R.POINT, (1.5, 1.2, 1.0), position=(-0.3, 1.2, 0.4)),
                    R.Light(R.DIRECTIONAL, (0.4, 0.4, 0.5), direction=(0.2, -1.0, -0.3))]
    out, sx, sn = _gpu(pbf, g, scene, cam, prm, 64, 48, 1, 0, 1, 5)
    ref = oracle.render(scene, cam, sx, sn, 64, 48, 1, 0, 1, oracle.RNG_COUNTER, 5)
    _compare("deterministic", out["hdr"], ref["hdr"], 0.995, 1e-4)
    assert out["hdr"].max() > 0.05


def _tessellate(scene, k):
    """Every triangle split into k * k smaller ones (same surface, more triangles)."""
    tri, nrm, ids = [], [], []
    for t, n, m in zip(scene.tri, scene.nrm, scene.tri_mat):
        for i in range(k):
            for j in range(k - i):
                corners = [(i, j), (i + 1, j), (i, j + 1)]
                if j + 1 < k - i:
                    corners2 = [(i + 1, j), (i + 1, j + 1), (i, j + 1)]
                else:
                    corners2 = None
                for cs in (corners, corners2):
                    if cs is None:
                        continue
                    tri.append([t[0] + (t[1] - t[0]) * a / k + (t[2] - t[0]) * b / k for a, b in cs])
                    nrm.append([n[0], n[0], n[0]])
                    ids.append(m)
    return R.RenderScene(np.array(tri), np.array(nrm), np.array(ids), scene.materials, scene.lights)


def test_scene_hierarchy_matches_restatement(pbf, oracle_lib):
    """A scene of more than 32 triangles gets its own hierarchy (the walls tessellated
    into 160 triangles each); bars as the fixture cases."""
    from oracle import oracle

    g, scene, cam, prm = _case("render_materials")
    big = _tessellate(scene, 4)
    assert len(big.tri) == 16 * len(scene.tri)
    W, H, aa, depth, area, seed = (int(v) for v in g["settings"])
    out, sx, sn = _gpu(pbf, g, big, cam, prm, W, H, aa, depth, area, seed)
    assert out["stats"]["triangles"] == len(big.tri) + len(sx)
    ref = oracle.render(big, cam, sx, sn, W, H, aa, depth, area, oracle.RNG_COUNTER, seed)
    _compare("tessellated scene", out["hdr"], ref["hdr"], 0.99, 1e-3)


def test_tonemap_and_small_scenes(pbf):
    """The 8-bit frame is toColor of the HDR frame (rows flipped); a scene of one
    triangle and an empty scene render."""
    g, scene, cam, prm = _case("render_p_default")
    out, _, _ = _gpu(pbf, g, scene, cam, prm, 40, 30, 2, 2, 2, 3)
    h = out["hdr"][::-1]
    v = np.power(h * np.float32(np.sqrt(2.0)), np.float32(1 / 2.2)).astype(np.float32)
    want = (np.minimum(v, 1.0) * 255).astype(np.int32)
    assert np.abs(out["rgba"][..., :3].astype(np.int32) - want).max() <= 1 and (out["rgba"][..., 3] == 255).all()
    one = R.RenderScene(scene.tri[:1], scene.nrm[:1], np.zeros(1, np.int64), scene.materials[:1],
                        [R.Light(R.POINT, (1, 1, 1), position=(0.0, 1.0, 2.0))])
    a, _, _ = _gpu(pbf, g, one, cam, prm, 24, 18, 1, 1, 1, 1, surface=False)
    assert a["stats"]["triangles"] == 1 and a["hdr"].max() > 0
    empty = R.RenderScene(np.zeros((0, 3, 3)), np.zeros((0, 3, 3)), np.zeros(0, np.int64), [], [])
    e, _, _ = _gpu(pbf, g, empty, cam, prm, 24, 18, 1, 1, 1, 1, surface=False)
    assert e["stats"]["triangles"] == 0 and e["hdr"].max() == 0


def test_render_rejects_bad_arguments(pbf):
    g, scene, cam, prm = _case("render_p_default")
    pos = np.asarray(g["pos"], dtype=np.float32)
    with pbf.Simulator(pos, np.zeros_like(pos), prm) as sim:
        sim.set_render_scene(scene)
        with pytest.raises(pbf.PbfError):
            sim.render(cam, 0, 10)
        with pytest.raises(pbf.PbfError):
            sim.render(cam, 10, 10, ns_aa=0)
        bad = R.RenderScene(scene.tri, scene.nrm, scene.tri_mat, scene.materials, scene.lights)
        bad.materials = bad.materials[:1]
        with pytest.raises(pbf.PbfError):
            sim.set_render_scene(bad)


def test_sample_batches_give_the_same_frame(pbf):
    """With a 1 MiB path buffer the 16 samples per pixel are traced in 16 batches and
    summed batch by batch; the frame is bit-identical to the one-batch frame."""
    g, scene, cam, prm = _case("render_materials")
    pos = np.asarray(g["pos"], dtype=np.float32)
    with pbf.Simulator(pos, np.zeros_like(pos), prm) as sim:
        sim.set_render_scene(scene)
        one = sim.render(cam, 256, 192, 16, 2, 2, seed=4)
        many = sim.render(cam, 256, 192, 16, 2, 2, seed=4, path_buffer_mib=1)
    assert one["hdr"].max() > 0
    assert np.array_equal(one["hdr"], many["hdr"]) and np.array_equal(one["rgba"], many["rgba"])
