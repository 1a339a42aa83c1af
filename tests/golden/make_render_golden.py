"""Generate tests/golden/render_*.npz: frames of the reference's own path tracer.

Runs the reference's headless renderer (oracle/_ref/pbf_ref_render, built by
oracle/ref/build_ref.py): PathTracer::render_to_file (src/pathtracer.cpp) on one worker
thread after srand(seed), over a Cornell box (fluid_gb300.render.cornell_box) and the
surface of the reference's default particles (particles/p.xml). Each case stores the
scene arrays, the camera description and its frame as the reference placed it, the
render settings, the particles and parameters, the reference's fluid surface
triangles and the 8-bit frame it wrote (RGBA, PNG row order).

Usage: ``python tests/golden/make_render_golden.py [reference_dir]``.
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

from fluid_gb300 import render as R  # noqa: E402
from fluid_gb300.params import PbfParams  # noqa: E402
from oracle import ref_runner  # noqa: E402
from tests.golden.make_golden import CORNELL, load_reference_xml  # noqa: E402


def scene_arrays(scene: R.RenderScene) -> dict:
    return {
        "tri": scene.tri, "nrm": scene.nrm, "tri_mat": scene.tri_mat,
        "mat_kind": np.array([m.kind for m in scene.materials], dtype=np.int64),
        "mat_c1": np.array([m.c1 for m in scene.materials], dtype=np.float64).reshape(-1, 3),
        "mat_c2": np.array([m.c2 for m in scene.materials], dtype=np.float64).reshape(-1, 3),
        "mat_ior": np.array([m.ior for m in scene.materials], dtype=np.float64),
        "light_kind": np.array([l.kind for l in scene.lights], dtype=np.int64),
        "light_vec": np.array([[l.radiance, l.position, l.direction, l.dim_x, l.dim_y] for l in scene.lights],
                              dtype=np.float64).reshape(-1, 5, 3),
    }


def scene_from_arrays(g) -> R.RenderScene:
    mats = [R.Material(int(k), tuple(c1), tuple(c2), float(ior))
            for k, c1, c2, ior in zip(g["mat_kind"], g["mat_c1"], g["mat_c2"], g["mat_ior"])]
    lights = [R.Light(int(k), *[tuple(v) for v in vec]) for k, vec in zip(g["light_kind"], g["light_vec"])]
    return R.RenderScene(g["tri"], g["nrm"], g["tri_mat"], mats, lights)


def camera_from_json(text: str) -> R.CameraDesc:
    return R.CameraDesc(**json.loads(text))


def save(name: str, scene, cam, pos, params: PbfParams, W: int, H: int, ns_aa: int, max_depth: int, ns_area: int,
         seed: int) -> None:
    out = ref_runner.render(scene, cam, pos, params, W, H, ns_aa=ns_aa, max_depth=max_depth, ns_area_light=ns_area,
                            seed=seed)
    np.savez_compressed(HERE / f"{name}.npz", params=json.dumps(dataclasses.asdict(params)),
                        camera=json.dumps(dataclasses.asdict(cam)), pos=pos,
                        settings=np.array([W, H, ns_aa, max_depth, ns_area, seed], dtype=np.int64),
                        rgba=out["rgba"], surf_xyz=out["surf_xyz"], surf_nrm=out["surf_nrm"],
                        cam_position=out["position"], cam_up=out["up"], cam_vfov=np.float64(out["vfov"]),
                        **scene_arrays(scene))
    print(f"{name}: {W}x{H} aa {ns_aa} depth {max_depth} area {ns_area}: {len(out['surf_xyz'])} surface "
          f"triangles, mean {out['rgba'][..., :3].mean():.1f}, {out['seconds']:.1f} s")


def main(argv):
    ref_dir = argv[1] if len(argv) > 1 else os.environ.get("PBF_REFERENCE_DIR")
    if not ref_dir:
        raise SystemExit(f"usage: {Path(argv[0]).name} <reference_dir> (or set PBF_REFERENCE_DIR)")
    reference = Path(ref_dir)
    if not ref_runner.render_available():
        raise SystemExit("build the reference renderer first: python oracle/ref/build_ref.py")
    pos, _, rho0 = load_reference_xml(reference / "particles" / "p.xml")
    prm = PbfParams(rest_density=rho0, **CORNELL)
    lo, hi = prm.box_lo, prm.box_hi
    # the reference's defaults: 1 camera ray per pixel, depth 1, 1 area-light sample
    scene, cam = R.cornell_box(lo, hi)
    save("render_p_default", scene, cam, pos, prm, 64, 48, 1, 1, 1, 1)
    save("render_p_default_aa4", scene, cam, pos, prm, 48, 36, 4, 3, 4, 2)
    scene, cam = R.cornell_box(lo, hi, glass_block=True)
    scene.lights = [R.Light(R.POINT, (1.5, 1.2, 1.0), position=(-0.3, 1.2, 0.2)),
                    R.Light(R.DIRECTIONAL, (0.4, 0.4, 0.5), direction=(0.2, -1.0, -0.3)),
                    R.Light(R.HEMISPHERE, (0.1, 0.1, 0.12))] + scene.lights
    scene.materials.append(R.Material(R.EMISSION, (2.0, 1.0, 0.5)))
    scene.materials.append(R.Material(R.REFRACTION, (1.0, 1.0, 1.0), ior=1.33))
    scene.tri_mat[0:2] = len(scene.materials) - 2  # emissive floor
    scene.tri_mat[4:6] = len(scene.materials) - 1  # back wall with the reference's black RefractionBSDF
    save("render_materials", scene, cam, pos, prm, 48, 36, 2, 4, 2, 3)


if __name__ == "__main__":
    main(sys.argv)
