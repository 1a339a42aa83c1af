"""The C++ facade and pbf_run on the GPU: key semantics, dumps, parity with the oracle."""
from __future__ import annotations

import subprocess
from pathlib import Path

import numpy as np
import pytest

from fluid_gb300 import scenes
from tests.golden.make_golden import params_from_json
from tests.helpers import rel_err

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parents[1]
GOLDEN = ROOT / "tests" / "golden"


@pytest.fixture(scope="module")
def pbf_run():
    from fluid_gb300 import build

    return str(build.RUN_BIN)


def read_frame(path):
    b = Path(path).read_bytes()
    assert b[:8] == b"PBFFRAME"
    n = int(np.frombuffer(b, np.int64, 1, 8)[0])
    t = float(np.frombuffer(b, np.float64, 1, 16)[0])
    x = np.frombuffer(b, np.float32, 3 * n, 24).reshape(n, 3)
    rho = np.frombuffer(b, np.float32, n, 24 + 12 * n)
    return t, x, rho


def test_windowless_one_step_matches_oracle(pbf_run, tmp_path, oracle_lib):
    sc = scenes.block4096(1)
    f = tmp_path / "block.xml"
    pos32 = sc.pos.astype(np.float32).astype(np.float64)
    scenes.write_xml(f, pos32, sc.vel, sc.params.rest_density, sc.params)
    out = tmp_path / "frames"
    r = subprocess.run([pbf_run, "-p", str(f), "-d", str(sc.params.dt * 0.5), "-o", str(out), "--quiet"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    frames = sorted(out.glob("frame_*.bin"))
    assert len(frames) == 2  # the state before and after the one step the -d interval needs
    t0, x0, rho0 = read_frame(frames[0])
    t1, x1, rho1 = read_frame(frames[1])
    assert t0 == 0.0 and t1 == pytest.approx(sc.params.dt)
    prm = sc.params.with_(rest_density=float(np.float32(sc.params.rest_density)))
    ref = oracle_lib.step(pos32, sc.vel, prm, 1)
    assert rel_err(x1, ref["pos"]) < 1e-5
    assert rel_err(rho1, ref["density"]) < 1e-5
    load = oracle_lib.estimate_densities(pos32, prm)
    assert rel_err(rho0, load) < 1e-5  # Application::load_particles ends with estimateDensities


def test_reference_fixture_keys(pbf_run, tmp_path):
    """The reference's own particles file through keys m and c (p.xml: rho0 150, H 0.3)."""
    g = np.load(GOLDEN / "p_default_1step.npz")
    prm = params_from_json(str(g["params"]))
    f = tmp_path / "p.xml"
    scenes.write_xml(f, g["pos_in"], g["vel_in"], prm.rest_density, prm)
    r = subprocess.run([pbf_run, "-p", str(f), "-k", "mc"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    # key m: one step; key c: steps until one more second has passed (63 steps of 0.016)
    assert r.stderr.count("Time: ") == 1 + 63
    assert r.stdout.count("avg rho: ") == 64
    assert "Time: 0 => 0.016" in r.stderr


def read_obj(path):
    v, vn, f = [], [], []
    for line in Path(path).read_text().splitlines():
        if line.startswith("v "):
            v.append([float(t) for t in line.split()[1:]])
        elif line.startswith("vn "):
            vn.append([float(t) for t in line.split()[1:]])
        elif line.startswith("f "):
            f.append([int(t.split("//")[0]) - 1 for t in line.split()[1:]])
    return np.array(v), np.array(vn), np.array(f)


def test_surface_dumps_match_the_surface_call(pbf_run, tmp_path):
    """pbf_run --surface writes the surface updateSurface builds (the reference's rendering
    input) for every dumped frame; it is the Simulator.surface of the same state."""
    from fluid_gb300 import pbf

    g = np.load(GOLDEN / "surface_p_default_0step.npz")
    prm = params_from_json(str(g["params"]))
    pos = g["pos"].astype(np.float32).astype(np.float64)
    f = tmp_path / "p.xml"
    scenes.write_xml(f, pos, np.zeros_like(pos), prm.rest_density, prm)
    out = tmp_path / "frames"
    r = subprocess.run([pbf_run, "-p", str(f), "-d", str(prm.dt * 0.5), "-o", str(out), "--surface", "--quiet"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    objs = sorted(out.glob("frame_*.obj"))
    assert len(objs) == 2
    v, vn, fc = read_obj(objs[0])
    with pbf.Simulator(pos, np.zeros_like(pos), prm.with_(rest_density=float(np.float32(prm.rest_density)))) as sim:
        xyz, nrm = sim.surface()
    assert len(fc) == len(xyz) > 100
    assert np.abs(v.reshape(-1, 3, 3) - xyz).max() < 1e-5
    assert np.abs(vn.reshape(-1, 3, 3) - nrm).max() < 1e-5


def test_path_traced_frames(pbf_run, tmp_path):
    """pbf_run -f renders the loaded state (the reference's windowless -f) through the C++
    PathTracer facade: the PNG is the frame Simulator.render gives for the same state,
    scene and settings; -d renders one PNG per dumped frame."""
    from fluid_gb300 import pbf
    from fluid_gb300 import render as R
    from oracle.ref_runner import read_png

    g = np.load(GOLDEN / "surface_p_default_0step.npz")
    prm = params_from_json(str(g["params"]))
    pos = g["pos"].astype(np.float32).astype(np.float64)
    f = tmp_path / "p.xml"
    scenes.write_xml(f, pos, np.zeros_like(pos), prm.rest_density, prm)
    png = tmp_path / "one.png"
    r = subprocess.run([pbf_run, "-p", str(f), "-f", str(png), "-r", "64", "48", "-s", "2", "-m", "2", "-l", "2",
                        "--quiet"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    img = read_png(png)
    assert img.shape == (48, 64, 4)
    scene, cam = R.cornell_box(prm.box_lo, prm.box_hi)
    with pbf.Simulator(pos, np.zeros_like(pos), prm.with_(rest_density=float(np.float32(prm.rest_density)))) as sim:
        sim.set_render_scene(scene)
        want = sim.render(cam, 64, 48, 2, 2, 2, seed=1, hdr=False)["rgba"]
    assert np.array_equal(img, want) and img[..., :3].max() > 0
    out = tmp_path / "frames"
    r = subprocess.run([pbf_run, "-p", str(f), "-d", str(prm.dt * 0.5), "-o", str(out), "-r", "32", "24", "--quiet"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    pngs = sorted(out.glob("frame_*.png"))
    assert len(pngs) == 2 and all(read_png(p).shape == (24, 32, 4) for p in pngs)
