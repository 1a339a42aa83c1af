"""The path tracer's CPU restatement (oracle/pbf_oracle_pt.c) against frames of the
reference's own PathTracer::render_to_file (tests/golden/render_*.npz, made by
tests/golden/make_render_golden.py): with the reference's random numbers (rand() after
srand(seed), one render thread, tiles in queue order) every byte of every frame is
the same, and so is the camera the reference placed."""
from __future__ import annotations

import glob
import os

import numpy as np
import pytest

from tests.golden.make_render_golden import camera_from_json, scene_from_arrays

CASES = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "render_*.npz")))


@pytest.fixture(scope="module")
def orc():
    from oracle import oracle

    oracle.build()
    return oracle


def _id(p):
    return os.path.basename(p)[:-4]


def test_fixtures_present():
    assert {"render_p_default", "render_p_default_aa4", "render_materials"} <= {_id(p) for p in CASES}


@pytest.mark.parametrize("path", CASES, ids=_id)
def test_restatement_reproduces_reference_frame(orc, path):
    g = np.load(path)
    W, H, ns_aa, depth, ns_area, seed = (int(v) for v in g["settings"])
    scene, cam = scene_from_arrays(g), camera_from_json(str(g["camera"]))
    out = orc.render(scene, cam, g["surf_xyz"], g["surf_nrm"], W, H, ns_aa, depth, ns_area, orc.RNG_STD, seed)
    fr = out["frame"]
    assert np.array_equal(fr["pos"], g["cam_position"])
    assert np.array_equal(fr["c2w"][1], g["cam_up"]) and fr["vfov"] == float(g["cam_vfov"])
    diff = np.abs(out["rgba"].astype(int) - g["rgba"].astype(int))
    print(f"{_id(path)}: {W}x{H}, {len(g['surf_xyz'])} surface triangles, "
          f"{int((diff.max(-1) > 0).sum())} pixels differ")
    assert np.array_equal(out["rgba"], g["rgba"])


def test_counter_random_numbers_are_per_pixel(orc):
    """With the counter draws (the GPU renderer's) a pixel's value does not depend on the
    order pixels are rendered in: any thread count gives the same frame."""
    g = np.load(CASES[0])
    scene, cam = scene_from_arrays(g), camera_from_json(str(g["camera"]))
    a = orc.render(scene, cam, g["surf_xyz"], g["surf_nrm"], 32, 24, 2, 2, 2, orc.RNG_COUNTER, 11, threads=1)
    b = orc.render(scene, cam, g["surf_xyz"], g["surf_nrm"], 32, 24, 2, 2, 2, orc.RNG_COUNTER, 11, threads=3)
    assert np.array_equal(a["hdr"], b["hdr"]) and a["hdr"].max() > 0
