"""mg_advect_semi_lagrange_noalloc (fixed device scratch, no allocation)
against mg_advect_semi_lagrange (pooled temporaries), both through the C ABI.

The file is collected last so that it also runs after every other GPU test
in the same process; it must pass alone in a fresh process as well.  Both
entry points launch the same kernels on the same inputs, so the results are
held to the other advection tests' bound (1e-6 relative, 99.9% bit-identical)
on two calls in a row.
"""
import ctypes

import numpy as np
import pytest

from tests.conftest import golden_path

pytestmark = pytest.mark.gpu

m = pytest.importorskip("mantaflow_gb300")
from mantaflow_gb300 import _lib  # noqa: E402


def close(got, want, what, rel=1e-6, min_exact=0.999):
    got = np.asarray(got, np.float64)
    want = np.asarray(want, np.float64)
    assert got.shape == want.shape, what
    diff = np.abs(got - want)
    assert float(np.max(diff - rel * np.maximum(1.0, np.abs(want)))) <= 0.0, "%s: max diff %g" % (what, diff.max())
    assert np.mean(got == want) >= min_exact, what


def solver_bytes(s):
    b = ctypes.c_size_t(0)
    assert _lib.load().mg_solver_memory(s._h, ctypes.byref(b)) == 0
    return b.value


def setup(g, kind):
    nz, ny, nx = g["flags"].shape
    s = m.Solver(name="noalloc", gridSize=m.vec3(nx, ny, nz), dim=3)
    s.timestep = float(g["dt"])
    flags = s.create(m.FlagGrid)
    m.copyArrayToGridReal(g["flags"], flags)
    vel = s.create(m.MACGrid)
    m.copyArrayToGridReal(g["vel"], vel)
    if kind == "real":
        tgt = s.create(m.RealGrid)
        m.copyArrayToGridReal(g["dens"], tgt)
    elif kind == "vec3":
        tgt = s.create(m.VecGrid)
        m.copyArrayToGridReal(g["vec3"], tgt)
    else:
        tgt = vel
    return s, flags, vel, tgt


# (grid kind, order, clampMode, orderSpace)
CASES = [("real", 2, 2, 1), ("real", 1, 1, 2), ("vec3", 2, 1, 1), ("mac", 2, 2, 1), ("mac", 1, 1, 1)]


@pytest.mark.parametrize("kind,order,clamp,ospace", CASES)
def test_noalloc_matches_pooled(kind, order, clamp, ospace):
    g = np.load(golden_path("advect_3d"), allow_pickle=False)
    L = _lib.load()
    sa, fa, va, ta = setup(g, kind)
    sb, fb, vb, tb = setup(g, kind)
    for call in range(2):
        rc = L.mg_advect_semi_lagrange(fa._h, va._h, ta._h, order, 1.0, ospace, 0, -1, clamp, 1)
        assert rc == 0, L.mg_last_error().decode()
        before = solver_bytes(sb)
        rc = L.mg_advect_semi_lagrange_noalloc(fb._h, vb._h, tb._h, order, 1.0, ospace, 0, -1, clamp, 1)
        assert rc == 0, L.mg_last_error().decode()
        assert solver_bytes(sb) == before, "the no-alloc entry point grew the solver's memory"
        close(tb.numpy(), ta.numpy(), "%s order %d call %d" % (kind, order, call + 1))
        if kind != "mac":
            close(vb.numpy(), va.numpy(), "velocity unchanged, call %d" % (call + 1), rel=0.0, min_exact=1.0)


def test_noalloc_rejects_oversized_grid():
    L = _lib.load()
    s = m.Solver(name="big", gridSize=m.vec3(160, 160, 160), dim=3)  # 4,096,000 cells > 3,145,728
    flags = s.create(m.FlagGrid)
    vel = s.create(m.MACGrid)
    dens = s.create(m.RealGrid)
    rc = L.mg_advect_semi_lagrange_noalloc(flags._h, vel._h, dens._h, 2, 1.0, 1, 0, -1, 2, 1)
    assert rc == 1  # MG_ERR_ARG
    assert "fixed scratch" in L.mg_last_error().decode()
    # a MAC grid of 1,048,576 cells fits, one of 110^3 (3,993,000 floats) does not
    s2 = m.Solver(name="mac", gridSize=m.vec3(110, 110, 110), dim=3)
    f2 = s2.create(m.FlagGrid)
    v2 = s2.create(m.MACGrid)
    assert L.mg_advect_semi_lagrange_noalloc(f2._h, v2._h, v2._h, 2, 1.0, 1, 0, -1, 2, 1) == 1
