"""Recipe: build ``tests/dropin/_build/pbf_dropin`` (test infrastructure).

The drop-in replacement header ``tests/dropin/particles.h`` and its driver
``dropin_main.cpp`` are compiled against the reference's own headers and linked with the
reference's own BVHAccel, MarchingTriangle, BSDF and CGL objects, as staged and compiled
under ``oracle/_ref/`` by ``oracle/ref/build_ref.py`` (headless; the drawing routines
those objects reference are the link-time stubs that abort if reached), and with this
library's ``libpbf.so`` / ``libpbf_host.so``. Nothing of the reference's particles.cpp is
linked: the facade replaces it.
"""
from __future__ import annotations

import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
REF = ROOT / "oracle" / "_ref"
STAGE = REF / "src"
OBJ = REF / "obj"
LIB = ROOT / "fluid_gb300" / "_lib"
OUT = HERE / "_build" / "pbf_dropin"
# the reference's translation units the replacement header's callers link against
REF_OBJS = ["bvh.o", "bbox.o", "marching_triangle.o", "bsdf.o", "sampler.o", "vector3D.o", "color.o",
            "spectrum.o", "matrix3x3.o", "gl_link_stubs.o"]


def available() -> bool:
    return (STAGE / "src" / "bvh.h").is_file() and all((OBJ / o).is_file() for o in REF_OBJS)


def build(force: bool = False) -> Path:
    if not available():
        raise FileNotFoundError("the reference's staged headers and objects (oracle/_ref) are not built")
    if str(ROOT) not in sys.path:
        sys.path.insert(0, str(ROOT))
    from fluid_gb300 import build as native

    native.build()
    srcs = [HERE / "dropin_main.cpp", HERE / "particles.h", ROOT / "fluid_gb300" / "host" / "pbf_particles.h"]
    deps = srcs + [OBJ / o for o in REF_OBJS] + [LIB / "libpbf.so", LIB / "libpbf_host.so"]
    if not force and OUT.exists() and all(OUT.stat().st_mtime >= d.stat().st_mtime for d in deps):
        return OUT
    OUT.parent.mkdir(parents=True, exist_ok=True)
    cmd = ["g++", "-O2", "-std=gnu++17", "-w", "-include", "cstdint", "-DGLEW_NO_GLU",
           "-I", str(ROOT / "oracle" / "ref" / "shim"), "-I", str(STAGE / "CGL" / "include"),
           "-I", str(STAGE / "CGL" / "include" / "CGL"), "-I", str(STAGE / "src"), "-I", str(ROOT / "include"),
           "-I", str(ROOT / "fluid_gb300" / "host"), "-I", str(HERE),
           str(HERE / "dropin_main.cpp"), *(str(OBJ / o) for o in REF_OBJS),
           "-L", str(LIB), "-lpbf_host", "-lpbf", f"-Wl,-rpath,{LIB}", "-o", str(OUT)]
    subprocess.run(cmd, check=True)
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
