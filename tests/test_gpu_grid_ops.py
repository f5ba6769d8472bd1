"""Grid members and library housekeeping on the GPU: Grid::swap, copyFrom,
setConst / clear, getMaxAbs / getMax / getMin (grid.cpp:99-110, 303-330),
join (knJoinReal, grid.cpp:303-311) against the oracle, countCells, the
per-family profiling entries, the launch counter, and mg_shutdown followed
by a fresh mg_init in a process of its own.
"""
import ctypes as C
import os
import subprocess
import sys

import numpy as np
import pytest

from oracle import oracle as og
from tests.conftest import ROOT

pytestmark = pytest.mark.gpu

m = pytest.importorskip("mantaflow_gb300")
from mantaflow_gb300 import _lib  # noqa: E402


def _solver(shape):
    nz, ny, nx = shape
    return m.Solver(name="ops", gridSize=m.vec3(nx, ny, nz), dim=3 if nz > 1 else 2)


@pytest.mark.parametrize("shape", [(12, 14, 16), (1, 20, 18)])
def test_swap_copy_const_and_norms(shape):
    rng = np.random.default_rng(1)
    s = _solver(shape)
    a, b = s.create(m.RealGrid), s.create(m.RealGrid)
    va = (rng.random(shape, dtype=np.float32) - 0.7).astype(np.float32)
    vb = (rng.random(shape, dtype=np.float32) * 3).astype(np.float32)
    m.copyArrayToGridReal(va, a)
    m.copyArrayToGridReal(vb, b)
    a.swap(b)
    assert np.array_equal(a.numpy(), vb) and np.array_equal(b.numpy(), va)
    assert b.getMaxAbs() == float(np.max(np.abs(va)))
    assert b.getMax() == float(va.max()) and b.getMin() == float(va.min())
    a.copyFrom(b)
    assert np.array_equal(a.numpy(), va)
    a.setConst(2.5)
    assert np.all(a.numpy() == np.float32(2.5))
    a.clear()
    assert not np.any(a.numpy())
    v = s.create(m.MACGrid)
    v.setConst(m.vec3(1, -2, 3))
    got = v.numpy()
    assert np.all(got[..., 0] == 1) and np.all(got[..., 1] == -2) and np.all(got[..., 2] == 3)


@pytest.mark.parametrize("keepMax", [True, False])
def test_join_against_oracle(keepMax):
    shape = (10, 12, 14)
    rng = np.random.default_rng(2)
    va = (rng.random(shape, dtype=np.float32) - 0.5).astype(np.float32)
    vb = (rng.random(shape, dtype=np.float32) - 0.5).astype(np.float32)
    s = _solver(shape)
    a, b = s.create(m.RealGrid), s.create(m.RealGrid)
    m.copyArrayToGridReal(va, a)
    m.copyArrayToGridReal(vb, b)
    a.join(b, keepMax=keepMax)
    want = va.copy()
    og.join_real(want, vb, keepMax)
    assert np.array_equal(a.numpy(), want)


def test_count_cells():
    shape = (16, 18, 20)
    f = np.zeros(shape, np.int32)
    og.init_domain(f, 0)
    og.fill_grid(f)
    og.set_open_bound(f, 0, "Y")
    s = _solver(shape)
    flags = s.create(m.FlagGrid)
    m.copyArrayToGridReal(f, flags)
    assert flags.countCells(m.FlagFluid) == int(np.count_nonzero(f & og.FLUID))
    assert flags.countCells(m.FlagObstacle, bnd=1) == int(np.count_nonzero(f[1:-1, 1:-1, 1:-1] & og.OBSTACLE))


def test_profiling_and_launch_counter():
    n = 24
    s = _solver((n, n, n))
    flags, vel, dens = s.create(m.FlagGrid), s.create(m.MACGrid), s.create(m.RealGrid)
    flags.initDomain(boundaryWidth=0)
    flags.fillGrid()
    m.copyArrayToGridReal(np.random.default_rng(3).random((n, n, n), dtype=np.float32), dens)
    L = _lib.load()
    c0 = C.c_longlong()
    _lib.check(L.mg_launch_count(C.byref(c0)))
    _lib.check(L.mg_profile_reset(s._h))
    _lib.check(L.mg_profile_enable(s._h, 1))
    m.advectSemiLagrange(flags=flags, vel=vel, grid=dens, order=2)
    m.addBuoyancy(flags=flags, density=dens, vel=vel, gravity=m.vec3(0, -1e-3, 0))
    _lib.check(L.mg_profile_enable(s._h, 0))
    cap = 64
    cnt = C.c_int(cap)
    names = (C.c_char_p * cap)()
    ms = (C.c_double * cap)()
    lns = (C.c_longlong * cap)()
    _lib.check(L.mg_profile_read(s._h, C.byref(cnt), names, ms, lns))
    fams = {names[q].decode(): (ms[q], lns[q]) for q in range(cnt.value)}
    assert "add_buoyancy" in fams and fams["add_buoyancy"][1] == 1 and fams["add_buoyancy"][0] > 0
    assert any(k.startswith("advect") for k in fams)
    c1 = C.c_longlong()
    _lib.check(L.mg_launch_count(C.byref(c1)))
    assert c1.value - c0.value >= 3


_SHUTDOWN = r"""
import ctypes as C, sys
import numpy as np
sys.path.insert(0, sys.argv[1])
from mantaflow_gb300 import _lib
L = _lib.load()
_lib.check(L.mg_init(0))
s = C.c_void_p(); g = C.c_void_p()
_lib.check(L.mg_solver_create(8, 8, 8, 3, C.byref(s)))
_lib.check(L.mg_grid_create(s, 0, C.byref(g)))
_lib.check(L.mg_shutdown())
# handles of the old library state are refused, not used
rc = L.mg_grid_set_const(g, 1.0, 0.0, 0.0)
assert rc != 0, rc
_lib.check(L.mg_init(0))
_lib.check(L.mg_solver_create(8, 8, 8, 3, C.byref(s)))
_lib.check(L.mg_grid_create(s, 0, C.byref(g)))
_lib.check(L.mg_grid_set_const(g, 1.5, 0.0, 0.0))
a = np.zeros(512, np.float32)
_lib.check(L.mg_grid_download(g, a.ctypes.data_as(C.c_void_p), a.nbytes))
assert np.all(a == 1.5)
_lib.check(L.mg_shutdown())
print("ok")
"""


def test_shutdown_and_reinit_in_a_fresh_process():
    r = subprocess.run([sys.executable, "-c", _SHUTDOWN, ROOT], capture_output=True, text=True, timeout=300,
                       env=dict(os.environ))
    assert r.returncode == 0 and r.stdout.strip().endswith("ok"), r.stdout + r.stderr
