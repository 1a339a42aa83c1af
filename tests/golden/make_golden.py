"""Generate the golden vectors in tests/golden/ by running the reference's own PBF step.

Runs where the reference checkout and its headless build exist (oracle/ref/build_ref.py);
the GPU machine only reads the committed ``*.npz`` files. Each case stores its inputs,
its parameters (JSON) and the outputs of the reference step in both orders:

* ``jacobi`` — the reference's Particle methods with an order-independent XSPH pass
  (oracle/ref/ref_driver.cpp, mode 1): what the oracle restatement and the CUDA path
  compute;
* ``literal`` — the reference's unmodified ``Particles::timeStep`` (mode 0).

Usage: ``python tests/golden/make_golden.py <reference_dir> [case ...]`` (or the reference
directory in ``PBF_REFERENCE_DIR``); with case names, only those cases are made.
"""
from __future__ import annotations

import dataclasses
import json
import os
import sys
import xml.etree.ElementTree as ET
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))

from fluid_gb300 import scenes  # noqa: E402
from fluid_gb300.params import PbfParams  # noqa: E402
from oracle import ref_runner  # noqa: E402

# The reference's Cornell box scene (dae/sky/CBempty.dae): walls x = +-1, floor y = 0,
# ceiling y = 1.5, back z = -1, open front z = +1 (clipped by particles.cpp:57-65).
CORNELL = dict(box_lo=(-1.0, 0.0, -1.0), box_hi=(1.0, 1.5, 1.0), box_open_mask=1 << 5)


def load_reference_xml(path: Path):
    """Application::load_particles (application.cpp:302-344): density via stof, pos/v triples."""
    root = ET.parse(path).getroot()
    rho0 = float(np.float32(float(root.find("density").text)))
    pos, vel = [], []
    for p in root.find("ps").findall("particle"):
        pos.append([float(t) for t in p.find("pos").text.split()])
        vel.append([float(t) for t in p.find("v").text.split()])
    return np.array(pos), np.array(vel), rho0


def save_case(name: str, pos, vel, params: PbfParams, steps: int, neighbors: bool = True, mesh=None,
              spheres=None) -> None:
    jac = ref_runner.run(pos, vel, params, steps=steps, mode="jacobi", neighbors=neighbors,
                         load_density=True, mesh=mesh, spheres=spheres)
    lit = ref_runner.run(pos, vel, params, steps=steps, mode="literal", mesh=mesh, spheres=spheres)
    data = dict(
        params=json.dumps(dataclasses.asdict(params)),
        steps=np.int64(steps),
        pos_in=pos, vel_in=vel,
        pos=jac["pos"], vel=jac["vel"], density=jac["density"],
        load_density=jac["load_density"],
        literal_pos=lit["pos"], literal_vel=lit["vel"], literal_density=lit["density"],
    )
    if mesh is not None:
        data["mesh"] = np.asarray(mesh, dtype=np.float64).reshape(-1, 9)
    if spheres is not None:
        data["spheres"] = np.asarray(spheres, dtype=np.float64).reshape(-1, 4)
    if neighbors:
        data["nbr_offsets"] = jac["nbr_offsets"].astype(np.int32)
        data["nbr_idx"] = jac["nbr_idx"].astype(np.int32)
    np.savez_compressed(HERE / f"{name}.npz", **data)
    print(f"{name}: n={pos.shape[0]} steps={steps}")


# A slanted ramp of two triangles across the [0,1]^3 box (collider mesh besides the walls).
RAMP = np.array([[0.05, 0.25, 0.0, 0.95, 0.05, 0.0, 0.95, 0.05, 1.0],
                 [0.05, 0.25, 0.0, 0.95, 0.05, 1.0, 0.05, 0.25, 1.0]])


def ramp_scene():
    """8^3 block (s = 0.05, h = 0.1) just above the ramp, moving down and along x: its
    lowest layer reaches the ramp in the first step."""
    s = 0.05
    p = scenes.lattice(8, 8, 8, s, corner=(0.3, 0.20, 0.3))
    p += scenes.uniform(5, p.size, -0.001, 0.001).reshape(p.shape)
    v = np.zeros_like(p)
    v[:, 0] = 0.3
    v[:, 1] = -3.0
    return p, v, scenes.physical_params(0.1, s)


def mesh_case():
    p, v, prm = ramp_scene()
    save_case("ramp_block512_2step", p, v, prm, 2, mesh=RAMP)


# A solid sphere resting on the floor of the [0,1]^3 box.
SPHERE = np.array([[0.5, 0.2, 0.5, 0.22]])


def sphere_scene():
    """8^3 block (s = 0.05, h = 0.1) over the sphere, falling and drifting in x: its lowest
    layer reaches the sphere in the first step (stops and slides on its curved surface)."""
    s = 0.05
    p = scenes.lattice(8, 8, 8, s, corner=(0.3, 0.45, 0.3))
    p += scenes.uniform(9, p.size, -0.001, 0.001).reshape(p.shape)
    v = np.zeros_like(p)
    v[:, 0] = 0.4
    v[:, 1] = -4.0
    return p, v, scenes.physical_params(0.1, s)


def wavy_floor(n: int = 32) -> np.ndarray:
    """A height-field floor over [0,1]^2 of 2 n^2 triangles (2,048 for n = 32):
    y = 0.1 + 0.05 sin(6 pi x) cos(6 pi z), normals facing up."""
    g = np.linspace(0.0, 1.0, n + 1)
    X, Z = np.meshgrid(g, g, indexing="ij")
    Y = 0.1 + 0.05 * np.sin(6 * np.pi * X) * np.cos(6 * np.pi * Z)
    P = np.stack([X, Y, Z], -1)
    tris = []
    for i in range(n):
        for k in range(n):
            a, b, c, d = P[i, k], P[i + 1, k], P[i + 1, k + 1], P[i, k + 1]
            tris.append(np.concatenate([a, d, c]))  # (d - a) x (c - a) points up
            tris.append(np.concatenate([a, c, b]))
    return np.array(tris)


def wavy_scene():
    """8^3 block (s = 0.05, h = 0.1) falling onto the wavy floor of 2,048 triangles."""
    s = 0.05
    p = scenes.lattice(8, 8, 8, s, corner=(0.3, 0.17, 0.3))
    p += scenes.uniform(13, p.size, -0.001, 0.001).reshape(p.shape)
    v = np.zeros_like(p)
    v[:, 1] = -3.0
    v[:, 2] = 0.5
    return p, v, scenes.physical_params(0.1, s)


def sphere_case():
    p, v, prm = sphere_scene()
    save_case("sphere_block512_2step", p, v, prm, 2, spheres=SPHERE)


def wavy_case():
    p, v, prm = wavy_scene()
    save_case("wavyfloor2048_block512_2step", p, v, prm, 2, mesh=wavy_floor())


def params_from_json(text: str) -> PbfParams:
    d = json.loads(text)
    for k, v in d.items():
        if isinstance(v, list):
            d[k] = tuple(tuple(x) if isinstance(x, list) else x for x in v)
    return PbfParams(**d)


def main(argv):
    ref_dir = argv[1] if len(argv) > 1 else os.environ.get("PBF_REFERENCE_DIR")
    if not ref_dir:
        raise SystemExit("usage: make_golden.py <reference_dir> [case ...] (or set PBF_REFERENCE_DIR)")
    reference = Path(ref_dir)
    if not ref_runner.available():
        raise SystemExit("build the reference driver first: python oracle/ref/build_ref.py")
    only = set(argv[2:])
    if only:
        for name in sorted(only):
            {"sphere": sphere_case, "wavy": wavy_case, "ramp": mesh_case}[name]()
        return

    sc = scenes.block4096(1, scale="mass")
    save_case("block4096_mass_1step", sc.pos, sc.vel, sc.params, 1)

    s = 0.05
    p = scenes.lattice(8, 8, 8, s)
    p += scenes.uniform(7, p.size, -0.001, 0.001).reshape(p.shape)
    # Raw reference constants: the unnormalised XSPH term makes this fluid blow up
    # within a few steps; 4 steps still run inside the box with wall contacts.
    save_case("block512_ref_4step", p, np.zeros_like(p), scenes.physical_params(0.1, s, scale="ref"), 4)
    # Scale-consistent constants: a 20-step collapse against the floor and walls (past about
    # 20 steps the clumping rate of the reference's formulation depends on the precision).
    save_case("block512_mass_20step", p, np.zeros_like(p), scenes.physical_params(0.1, s), 20)

    mesh_case()
    sphere_case()
    wavy_case()

    for xml_name, steps in (("p.xml", 1), ("p.xml", 3), ("spheres_p.xml", 1)):
        pos, vel, rho0 = load_reference_xml(reference / "particles" / xml_name)
        prm = PbfParams(rest_density=rho0, **CORNELL)
        stem = xml_name.replace(".xml", "").replace("_p", "p")
        save_case(f"{stem}_default_{steps}step", pos, vel, prm, steps)


if __name__ == "__main__":
    main(sys.argv)
