"""Generate tests/golden/surface_*.npz: the reference's own surface triangles.

Runs the reference's headless build (oracle/ref/build_ref.py) with its surface flag: the
loop of Particles::getSurfacePrims (particles.cpp:352-385) over the reference's
generateGridCell, polygonise (marching.cpp) and getVertexNormal, with updateSurface's
arguments (isolevel 0.95 rest density, step 0.5 H) and the reference's fixed bounds.
Each case stores the particle positions the surface was taken from, the parameters
(JSON) and the triangles (xyz, nrm as (T, 3, 3), the cube index of each).

Usage: ``python tests/golden/make_surface_golden.py [reference_dir]``.
"""
from __future__ import annotations

import dataclasses
import json
import os
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parents[1]))

from fluid_gb300.params import PbfParams  # noqa: E402
from oracle import ref_runner  # noqa: E402
from tests.golden.make_golden import CORNELL, load_reference_xml  # noqa: E402


def save(name: str, pos, vel, params: PbfParams, steps: int) -> None:
    out = ref_runner.run(pos, vel, params, steps=steps, mode="jacobi", surface=True)
    src = pos if steps == 0 else out["pos"]
    np.savez_compressed(HERE / f"{name}.npz", params=json.dumps(dataclasses.asdict(params)), steps=np.int64(steps),
                        pos=src, xyz=out["surf_xyz"], nrm=out["surf_nrm"], cube=out["surf_cube"])
    print(f"{name}: n={pos.shape[0]} steps={steps} triangles={len(out['surf_cube'])}")


def main(argv):
    ref_dir = argv[1] if len(argv) > 1 else os.environ.get("PBF_REFERENCE_DIR")
    if not ref_dir:
        raise SystemExit(f"usage: {Path(argv[0]).name} <reference_dir> (or set PBF_REFERENCE_DIR)")
    reference = Path(ref_dir)
    if not ref_runner.available():
        raise SystemExit("build the reference driver first: python oracle/ref/build_ref.py")
    pos, vel, rho0 = load_reference_xml(reference / "particles" / "p.xml")
    prm = PbfParams(rest_density=rho0, **CORNELL)
    save("surface_p_default_0step", pos, vel, prm, 0)
    save("surface_p_default_3step", pos, vel, prm, 3)


if __name__ == "__main__":
    main(sys.argv)
