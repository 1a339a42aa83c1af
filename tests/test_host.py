"""C++ host side without a GPU: the particle-file loader behind pbf_run --parse-only.

Application::load_particles (application.cpp:302-344) is the reference's loader: a
missing file gives an empty simulator, an XML error exits, <density> goes through stof.
"""
from __future__ import annotations

import subprocess
from pathlib import Path

import numpy as np
import pytest

from fluid_gb300 import scenes

ROOT = Path(__file__).resolve().parents[1]
GOLDEN = ROOT / "tests" / "golden"


@pytest.fixture(scope="module")
def pbf_run():
    from fluid_gb300 import build

    build.build_cuda()
    build.build_host()
    return str(build.RUN_BIN)


def _parse(pbf_run, path):
    r = subprocess.run([pbf_run, "-p", str(path), "--parse-only"], capture_output=True, text=True)
    return r.returncode, r.stdout


def test_reference_format_round_trip(pbf_run, tmp_path):
    sc = scenes.block4096(1)
    f = tmp_path / "block.xml"
    scenes.write_xml(f, sc.pos, sc.vel, sc.params.rest_density, sc.params)
    rc, out = _parse(pbf_run, f)
    assert rc == 0, out
    fields = out.split()
    assert fields[1] == "4096"
    assert float(fields[3]) == pytest.approx(float(np.float32(sc.params.rest_density)), rel=1e-8)  # stof
    assert float(fields[5]) == pytest.approx(sc.params.h) and fields[7] == "4"
    assert fields[-1] == "file"


def test_reference_style_file_without_params(pbf_run, tmp_path):
    f = tmp_path / "p.xml"
    f.write_text("""<?xml version="1.0"?>
<!-- written like particles/pgen.py -->
<particles>
  <density>700.0</density>
  <ps>
    <particle><pos>-0.9 0.1 0.9</pos><v>0 -1 0</v></particle>
    <particle attr="ignored"><pos> 1e-1 2.5E-1  0.3 </pos><v>0 0 0</v></particle>
  </ps>
  <fs/>
</particles>""")
    rc, out = _parse(pbf_run, f)
    assert rc == 0
    assert out.split()[1] == "2" and out.split()[3] == "700" and out.split()[-1] == "default"


def test_missing_file_gives_empty_simulator(pbf_run, tmp_path):
    rc, out = _parse(pbf_run, tmp_path / "nope.xml")
    assert rc == 0
    assert "[Warning]" in out and "particles 0" in out


@pytest.mark.parametrize("text,why", [
    ("<particles><density>1</density>", "unterminated"),
    ("<particles><ps></particles>", "mismatched"),
    ("<particles><density>1 &bogus;</density></particles>", "entity"),
    ("<scene></scene>", "not a particles file"),
    ("<particles><ps><particle><v>0 0 0</v></particle></ps></particles>", "pos"),
])
def test_malformed_files_are_rejected(pbf_run, tmp_path, text, why):
    f = tmp_path / "bad.xml"
    f.write_text(text)
    rc, out = _parse(pbf_run, f)
    assert rc == 1
    assert why in out


def test_entities_and_cdata(pbf_run, tmp_path):
    f = tmp_path / "e.xml"
    f.write_text("<particles><density><![CDATA[250]]></density><ps>"
                 "<particle><pos>0.5 0.5 0.5</pos><v>0 0 0</v></particle></ps></particles>")
    rc, out = _parse(pbf_run, f)
    assert rc == 0 and out.split()[3] == "250"
