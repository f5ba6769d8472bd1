"""The plugin translation unit of INTEGRATION.md (the binding a mantaflow
maintainer adds in place of the hot-path plugins) type-checks against
include/mantagpu.h: its code block is compiled with g++ -fsyntax-only, the
reference's own headers replaced by tests/plugin_tu/manta_mock.h (they need
the reference's CMake build and code generator).  Runs without a GPU."""
import os
import re
import shutil
import subprocess

import pytest

from tests.conftest import ROOT


def _tu_source(name="source/plugin/gpu_path.cpp"):
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    blocks = re.findall(r"```cpp\n(.*?)```", text, flags=re.S)
    tu = [b for b in blocks if name in b]
    assert len(tu) == 1
    return tu[0]


def test_plugin_tu_is_complete():
    src = _tu_source()
    for name in ("advectSemiLagrange", "resetPhiInObs", "setWallBcs", "addBuoyancy", "addGravity",
                 "addGravityNoScale", "setOpenBound", "resetOutflow", "extrapolateMACSimple", "extrapolateLsSimple",
                 "solvePressure", "computePressureRhs", "solvePressureSystem", "correctVelocity", "releaseMG"):
        assert re.search(r"PYTHON\(\) void %s\(" % name, src), name
    assert "..." not in src
    flip = _tu_source("source/plugin/gpu_flip.cpp")
    for name in ("mapPartsToMAC", "mapMACToParts", "flipVelocityUpdate", "mapPartsToGrid", "mapPartsToGridVec3",
                 "mapGridToParts", "mapGridToPartsVec3"):
        assert re.search(r"PYTHON\(\) void %s\(" % name, flip), name


@pytest.mark.parametrize("unit", ["source/plugin/gpu_path.cpp", "source/plugin/gpu_flip.cpp"])
def test_plugin_tu_compiles(tmp_path, unit):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not found")
    src = _tu_source(unit)
    for h in ("grid.h", "levelset.h", "particle.h"):
        src = src.replace('#include "%s"' % h, "")
    src = '#include "manta_mock.h"\n' + src
    f = tmp_path / os.path.basename(unit)
    f.write_text(src)
    r = subprocess.run([gxx, "-std=c++17", "-fsyntax-only", "-Wall", "-I", os.path.join(ROOT, "include"),
                        "-I", os.path.join(ROOT, "tests", "plugin_tu"), str(f)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
