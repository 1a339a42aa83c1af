"""In-tree build of the native parts: ``libpbf.so`` (CUDA, sm_103a) and the C++ host tools.

Sources are compiled in parallel with ``nvcc -gencode arch=compute_103a,code=sm_103a``
(and ``g++`` for host-only C++), outputs land in ``fluid_gb300/_lib/`` (git-ignored).
A target is rebuilt when any of its sources or headers is newer than it.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
HOST = PKG / "host"
OUT = PKG / "_lib"
INCLUDE = ROOT / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-Xcompiler", "-fvisibility=hidden", "-I", str(INCLUDE)]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-Wall", "-I", str(INCLUDE), "-I", str(HOST)]

LIB = OUT / "libpbf.so"
HOST_LIB = OUT / "libpbf_host.so"
RUN_BIN = OUT / "pbf_run"


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise FileNotFoundError("nvcc not found")


def cuda_sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu"))


def _headers() -> list[Path]:
    return sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + sorted(INCLUDE.glob("*.h"))


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(r.stdout + r.stderr)
        raise RuntimeError(f"build step failed: {' '.join(cmd[:3])} ... ({r.returncode})")


def build_cuda(jobs: int = 8, force: bool = False) -> Path:
    OUT.mkdir(parents=True, exist_ok=True)
    obj_dir = OUT / "obj"
    obj_dir.mkdir(exist_ok=True)
    headers = _headers()
    srcs = cuda_sources()
    compiler = nvcc()

    def compile_one(src: Path) -> Path:
        obj = obj_dir / (src.stem + ".o")
        if force or _stale(obj, [src, *headers]):
            _run([compiler, *ARCH, *NVCC_FLAGS, "-c", str(src), "-o", str(obj)])
        return obj

    with ThreadPoolExecutor(max_workers=jobs) as ex:
        objs = list(ex.map(compile_one, srcs))
    if force or _stale(LIB, objs):
        tmp = LIB.with_suffix(".so.tmp")
        _run([compiler, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcuda"])
        os.replace(tmp, LIB)
    return LIB


def build_host(jobs: int = 8, force: bool = False) -> list[Path]:
    """C++ host side: the Particles facade (libpbf_host.so) and the pbf_run driver."""
    if not HOST.exists():
        return []
    OUT.mkdir(parents=True, exist_ok=True)
    lib_srcs = sorted(p for p in HOST.glob("*.cpp") if p.name != "pbf_run.cpp")
    hdrs = sorted(HOST.glob("*.h")) + sorted(INCLUDE.glob("*.h"))
    outs = []
    if lib_srcs and (force or _stale(HOST_LIB, [*lib_srcs, *hdrs, LIB])):
        _run(["g++", *CXX_FLAGS, "-shared", "-o", str(HOST_LIB), *map(str, lib_srcs),
              "-L", str(OUT), "-lpbf", f"-Wl,-rpath,$ORIGIN"])
    if lib_srcs:
        outs.append(HOST_LIB)
    run_src = HOST / "pbf_run.cpp"
    if run_src.exists() and (force or _stale(RUN_BIN, [run_src, *hdrs, HOST_LIB])):
        _run(["g++", *CXX_FLAGS, "-o", str(RUN_BIN), str(run_src), "-L", str(OUT), "-lpbf_host", "-lpbf",
              f"-Wl,-rpath,$ORIGIN"])
    if run_src.exists():
        outs.append(RUN_BIN)
    return outs


def build(force: bool = False) -> list[Path]:
    lib = build_cuda(force=force)
    return [lib, *build_host(force=force)]


if __name__ == "__main__":
    for p in build(force="--force" in sys.argv):
        print(p)
