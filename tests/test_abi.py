"""The C ABI library: loads without a GPU, exports every declared symbol, and its struct
layouts match the ctypes mirrors. No compute calls here."""
from __future__ import annotations

import ctypes
import re
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
HEADERS = sorted((ROOT / "include").glob("*.h"))


@pytest.fixture(scope="module")
def libpbf():
    from fluid_gb300 import build, pbf

    build.build_cuda()
    return pbf.lib()


def declared_functions():
    names = []
    for h in HEADERS:
        text = h.read_text()
        names += re.findall(r"^PBF_API [^;]*?\b(pbf_\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_headers_declare_functions():
    names = declared_functions()
    assert "pbf_create" in names and "pbf_step" in names and len(names) >= 20


def test_every_declared_symbol_is_exported(libpbf):
    out = subprocess.run(["nm", "-D", "--defined-only", str(ROOT / "fluid_gb300" / "_lib" / "libpbf.so")],
                         capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r" T (pbf_\w+)", out))
    missing = [n for n in declared_functions() if n not in exported]
    assert not missing, missing
    for n in declared_functions():
        assert hasattr(libpbf, n)


def test_abi_version(libpbf):
    from fluid_gb300.pbf import ABI_VERSION

    header = (ROOT / "include" / "pbf.h").read_text()
    assert int(re.search(r"#define PBF_ABI_VERSION (\d+)", header).group(1)) == ABI_VERSION
    assert libpbf.pbf_abi_version() == ABI_VERSION


def test_default_params_are_the_reference_constants(libpbf):
    from fluid_gb300.params import REFERENCE_DEFAULTS
    from fluid_gb300.pbf import default_params_c

    c = default_params_c()
    r = REFERENCE_DEFAULTS.to_c()
    for name, _ in c._fields_:
        a, b = getattr(c, name), getattr(r, name)
        if hasattr(a, "__len__"):
            assert list(a) == list(b), name
        else:
            assert a == b, name
    # particles.cpp:24-44, 180
    assert (c.h, c.h2, c.iters, c.epsilon, c.scorr_k, c.scorr_n) == (0.3, 0.09, 12, 2.0, 0.0001, 4)
    assert (c.vort_eps, c.xsph_c, c.dt, tuple(c.gravity)) == (0.001, 0.001, 0.016, (0.0, -10.0, 0.0))


def test_last_error_without_handle(libpbf):
    assert isinstance(libpbf.pbf_last_error(None), bytes)


def test_struct_layout_matches_header(tmp_path):
    """Compile a C probe against include/pbf.h and compare sizeof/offsetof with ctypes."""
    from fluid_gb300.params import CParams
    from fluid_gb300.pbf import CStats

    fields_p = [f for f, _ in CParams._fields_]
    fields_s = [f for f, _ in CStats._fields_]
    src = ["#include <stdio.h>", "#include <stddef.h>", '#include "pbf.h"', "int main(void){"]
    src.append('printf("%zu\\n", sizeof(pbf_params));')
    src += [f'printf("%zu\\n", offsetof(pbf_params, {f}));' for f in fields_p]
    src.append('printf("%zu\\n", sizeof(pbf_stats));')
    src += [f'printf("%zu\\n", offsetof(pbf_stats, {f}));' for f in fields_s]
    src.append("return 0;}")
    c = tmp_path / "probe.c"
    c.write_text("\n".join(src))
    exe = tmp_path / "probe"
    subprocess.run(["gcc", "-I", str(ROOT / "include"), "-o", str(exe), str(c)], check=True)
    vals = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    expect = [ctypes.sizeof(CParams)] + [getattr(CParams, f).offset for f in fields_p]
    expect += [ctypes.sizeof(CStats)] + [getattr(CStats, f).offset for f in fields_s]
    assert vals == expect


def test_create_rejects_bad_arguments_before_any_device_work(libpbf):
    """pbf_batch_create validates its arguments on the host first (no GPU is touched):
    a NULL out pointer, no scenes, NULL xyz with particles, or a count of 2^31 or more
    (also where the sum over scenes would wrap) give PBF_ERR_INVALID and a message."""
    from fluid_gb300.pbf import default_params_c

    prm = default_params_c()
    out = ctypes.c_void_p()
    SizeArr = ctypes.c_size_t * 2
    L = libpbf
    xyz = (ctypes.c_float * 6)()
    invalid = 1  # PBF_ERR_INVALID
    header = (ROOT / "include" / "pbf.h").read_text()
    assert re.search(r"PBF_ERR_INVALID\s*=\s*1\b", header)
    args = lambda n_scenes, counts, x, o: (ctypes.byref(prm), n_scenes, counts, None, None, x, None, 0, o)
    assert L.pbf_batch_create(*args(1, SizeArr(2, 0), xyz, None)) == invalid
    assert L.pbf_batch_create(*args(0, SizeArr(2, 0), xyz, ctypes.byref(out))) == invalid
    assert L.pbf_batch_create(*args(1, SizeArr(2, 0), None, ctypes.byref(out))) == invalid
    assert L.pbf_batch_create(*args(1, SizeArr(1 << 31, 0), xyz, ctypes.byref(out))) == invalid
    wrap = SizeArr((1 << 64) - 1, 2)  # sums to 1 modulo 2^64
    assert L.pbf_batch_create(*args(2, wrap, xyz, ctypes.byref(out))) == invalid
    assert b"2^31" in L.pbf_last_error(None)
    assert not out.value
