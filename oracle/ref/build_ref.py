"""Recipe: build the reference's own PBF step headless (test infrastructure: the oracle).

Two stages, both writing only under ``oracle/_ref/`` (git-ignored):

1. ``stage(reference)`` — needs the reference checkout: its directory is an argument
   (``--reference DIR`` on the command line) or ``PBF_REFERENCE_DIR``; without either,
   staging stops with an error. Copies the reference files the step needs, unmodified, into
   ``oracle/_ref/src/`` and writes ``particles_param.cpp``: the reference's
   ``src/particles.cpp`` with its parameter ``#define`` block (lines 20-44) and the
   gravity literal (line 180) rewritten mechanically into references to the runtime
   globals of ``oracle/ref/ref_params.h``, plus one appended helper that re-runs the
   static initialiser of ``Particle::tensile_instability_scale`` (line 151) after the
   globals are set. Nothing else in the step is touched.
2. ``compile()`` — needs only the staged tree, so it also runs on a machine without
   the reference checkout. Compiles the staged translation units with the driver
   ``oracle/ref/ref_driver.cpp`` and ``oracle/ref/gl_link_stubs.cpp`` into
   ``oracle/_ref/pbf_ref_driver``, and with the path tracer's units and
   ``oracle/ref/ref_render.cpp`` into ``oracle/_ref/pbf_ref_render``, with
   ``g++ -O3 -std=gnu++11 -ffp-contract=off`` (contraction off so x86-64 and aarch64
   round identically).

Usage: ``python oracle/ref/build_ref.py [--reference DIR] [--stage-only|--compile-only]``.
"""
from __future__ import annotations

import os
import re
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
ORACLE = HERE.parent
OUT = ORACLE / "_ref"
STAGE = OUT / "src"
DRIVER = OUT / "pbf_ref_driver"
RENDER = OUT / "pbf_ref_render"

def reference_dir() -> Path | None:
    """The reference checkout named by ``PBF_REFERENCE_DIR``, or None."""
    d = os.environ.get("PBF_REFERENCE_DIR")
    return Path(d) if d else None

# Translation units of the reference that the step links against.
REF_TUS = [
    "src/bvh.cpp",
    "src/bbox.cpp",
    "src/static_scene/marching_triangle.cpp",
    "src/static_scene/sphere.cpp",
    "src/marching.cpp",
    "src/bsdf.cpp",
    "src/sampler.cpp",
    "CGL/src/vector3D.cpp",
    "CGL/src/color.cpp",
    "CGL/src/spectrum.cpp",
    "CGL/src/matrix3x3.cpp",
]
# Further translation units of the renderer driver (the path tracer and what it links).
RENDER_TUS = [
    "src/pathtracer.cpp",
    "src/static_scene/light.cpp",
    "src/static_scene/environment_light.cpp",
    "src/camera.cpp",
    "CGL/src/lodepng.cpp",
]
# Header trees the step's includes reach.
REF_HEADER_DIRS = ["src", "CGL/include"]

# particles.cpp:20-44 parameter block -> runtime globals (ref_params.h).
PARAM_DEFINES = {
    "DEFAULT_DELTA_T": "pbf_ref_dt",
    "H": "pbf_ref_h",
    "H2": "pbf_ref_h2",
    "NEWTON_NUM_STEPS": "pbf_ref_iters",
    "EPSILON": "pbf_ref_epsilon",
    "K": "pbf_ref_k",
    "VORTICITY_EPSILON": "pbf_ref_vort_eps",
    "C": "pbf_ref_xsph_c",
}
GRAVITY_LINE = "velocity.y -= 10 * delta_t;"
STATIC_LINE = (
    "double Particle::tensile_instability_scale = "
    "1.0 / poly6_kernel(Vector3D(0, 0, 0.1 * H));"
)
REINIT = (
    "\n  // appended by oracle/ref/build_ref.py: re-run the static initialiser above\n"
    "  // once the runtime parameter globals are set.\n"
    "  void pbf_ref_reinit_statics() {\n"
    "    Particle::tensile_instability_scale = 1.0 / poly6_kernel(Vector3D(0, 0, 0.1 * H));\n"
    "  }\n"
)


def rewrite_particles(text: str) -> str:
    """Mechanical rewrite of the parameter block; fails loudly on any mismatch."""
    for name, glob in PARAM_DEFINES.items():
        pat = re.compile(rf"^#define {name} [^\n]+$", re.M)
        hits = pat.findall(text)
        if len(hits) != 1:
            raise RuntimeError(f"expected one '#define {name}' in particles.cpp, found {len(hits)}")
        text = pat.sub(f"#define {name} ({glob})", text)
    if not re.search(r"^#define N 4$", text, re.M):
        raise RuntimeError("expected '#define N 4' (tensile exponent) in particles.cpp")
    if text.count(GRAVITY_LINE) != 1:
        raise RuntimeError("gravity literal not found exactly once in particles.cpp")
    text = text.replace(GRAVITY_LINE, "velocity.y -= pbf_ref_gravity * delta_t;")
    if text.count(STATIC_LINE) != 1:
        raise RuntimeError("tensile_instability_scale initialiser not found in particles.cpp")
    text = text.replace(STATIC_LINE, STATIC_LINE + REINIT)
    return '#include "ref_params.h"\n' + text


def stage(reference: Path | None = None) -> None:
    reference = reference or reference_dir()
    if reference is None:
        raise FileNotFoundError("no reference checkout given: pass its directory or set PBF_REFERENCE_DIR")
    if not (reference / "src" / "particles.cpp").is_file():
        raise FileNotFoundError(f"reference checkout not found at {reference}")
    if STAGE.exists():
        shutil.rmtree(STAGE)
    STAGE.mkdir(parents=True)
    for d in REF_HEADER_DIRS:
        for src in (reference / d).rglob("*.h"):
            dst = STAGE / src.relative_to(reference)
            dst.parent.mkdir(parents=True, exist_ok=True)
            shutil.copy2(src, dst)
    for tu in REF_TUS + RENDER_TUS:
        dst = STAGE / tu
        dst.parent.mkdir(parents=True, exist_ok=True)
        shutil.copy2(reference / tu, dst)
    text = (reference / "src" / "particles.cpp").read_text()
    (STAGE / "src" / "particles_param.cpp").write_text(rewrite_particles(text))


def staged() -> bool:
    return (STAGE / "src" / "particles_param.cpp").is_file()


def compile(jobs: int = 8, cxx: str = "g++") -> Path:
    if not staged():
        raise FileNotFoundError("reference sources are not staged under oracle/_ref/src")
    obj_dir = OUT / "obj"
    obj_dir.mkdir(parents=True, exist_ok=True)
    flags = [
        "-O3", "-std=gnu++11", "-ffp-contract=off", "-w",
        "-include", "cstdint", "-DGLEW_NO_GLU",
        "-I", str(HERE / "shim"), "-I", str(HERE),
        "-I", str(STAGE / "CGL" / "include"), "-I", str(STAGE / "CGL" / "include" / "CGL"),
        "-I", str(STAGE / "src"),
    ]
    common = [STAGE / tu for tu in REF_TUS] + [
        STAGE / "src" / "particles_param.cpp",
        HERE / "gl_link_stubs.cpp",
    ]
    render = [STAGE / tu for tu in RENDER_TUS] + [HERE / "ref_render.cpp"]
    sources = common + [HERE / "ref_driver.cpp"] + render

    def cc(src: Path) -> Path:
        obj = obj_dir / (src.name.replace(".cpp", ".o"))
        if obj.exists() and obj.stat().st_mtime >= src.stat().st_mtime:
            return obj
        subprocess.run([cxx, *flags, "-c", str(src), "-o", str(obj)], check=True)
        return obj

    with ThreadPoolExecutor(max_workers=jobs) as ex:
        objs = dict(zip(sources, ex.map(cc, sources)))
    base = [str(objs[s]) for s in common]
    subprocess.run([cxx, "-o", str(DRIVER), *base, str(objs[HERE / "ref_driver.cpp"])], check=True)
    subprocess.run([cxx, "-o", str(RENDER), *base, *(str(objs[s]) for s in render), "-pthread"], check=True)
    return DRIVER


def main(argv: list[str]) -> int:
    if "--compile-only" not in argv:
        ref = Path(argv[argv.index("--reference") + 1]) if "--reference" in argv else None
        stage(ref)
    if "--stage-only" not in argv:
        print(compile())
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv[1:]))
