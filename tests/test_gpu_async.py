"""Asynchronous grid transfers (mg_grid_upload_async / download_async /
mg_solver_wait_copies): round trips of Real and MAC grids, and a pipelined
plume sequence -- each step's upload and downloads queued without waiting,
the next step computing while results stream out -- that must give the same
bits as the synchronous transfers."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

m = pytest.importorskip("mantaflow_gb300")
from mantaflow_gb300 import _lib  # noqa: E402


def _pinned(L, nfloat):
    p = C.c_void_p()
    _lib.check(L.mg_host_alloc(4 * nfloat, C.byref(p)))
    return p, np.ctypeslib.as_array((C.c_float * nfloat).from_address(p.value))


def test_async_round_trip():
    L = _lib.load()
    n = 24
    s = m.Solver(name="rt", gridSize=m.vec3(n, n + 3, n - 2), dim=3)
    rng = np.random.default_rng(3)
    for kind, comps in ((m.RealGrid, 1), (m.MACGrid, 3)):
        g = s.create(kind)
        cnt = n * (n + 3) * (n - 2) * comps
        pin_in, a = _pinned(L, cnt)
        pin_out, b = _pinned(L, cnt)
        a[:] = rng.random(cnt, dtype=np.float32)
        b[:] = -1
        _lib.check(L.mg_grid_upload_async(g._h, pin_in, 4 * cnt))
        _lib.check(L.mg_grid_download_async(g._h, pin_out, 4 * cnt))
        _lib.check(L.mg_solver_wait_copies(s._h))
        assert np.array_equal(a, b)
        want = a.reshape(n - 2, n + 3, n, comps) if comps == 3 else a.reshape(n - 2, n + 3, n)
        assert np.array_equal(g.numpy(), want)
        L.mg_host_free(pin_in)
        L.mg_host_free(pin_out)


def _scene(n):
    s = m.Solver(name="pipe", gridSize=m.vec3(n, n, n), dim=3)
    s.timestep = 1.0
    flags = s.create(m.FlagGrid)
    flags.initDomain(boundaryWidth=0)
    flags.fillGrid()
    m.setOpenBound(flags, 0, "Y", m.FlagOutflow | m.FlagEmpty)
    return s, flags, s.create(m.MACGrid), s.create(m.RealGrid), s.create(m.RealGrid), s.create(m.RealGrid)


def _step(flags, vel, dens, p, noise):
    dens.join(noise)
    m.advectSemiLagrange(flags=flags, vel=vel, grid=dens, order=2, clampMode=2)
    m.advectSemiLagrange(flags=flags, vel=vel, grid=vel, order=2, clampMode=2)
    m.setWallBcs(flags=flags, vel=vel)
    m.addBuoyancy(density=dens, vel=vel, gravity=m.vec3(0, -4e-3, 0), flags=flags)
    m.solvePressure(flags=flags, vel=vel, pressure=p, cgAccuracy=1e-3, preconditioner=m.PcMGStatic)


def test_async_pipeline_matches_sync():
    L = _lib.load()
    n, K = 32, 4
    cells = n ** 3
    rng = np.random.default_rng(11)
    src = np.zeros((n, n, n), np.float32)
    src[2:6, 12:20, 12:20] = 1
    noise = [(rng.random((n, n, n), dtype=np.float32) * src).astype(np.float32) for _ in range(K)]
    pin_in, ins = _pinned(L, cells * K)
    for t in range(K):
        ins[t * cells:(t + 1) * cells] = noise[t].ravel()
    results = {}
    for mode in ("sync", "async"):
        s, flags, vel, dens, p, ng = _scene(n)
        pin_out, outs = _pinned(L, 5 * cells * K)
        for t in range(K):
            src_ptr = C.c_void_p(pin_in.value + 4 * cells * t)
            base = pin_out.value + 4 * 5 * cells * t
            if mode == "sync":
                _lib.check(L.mg_grid_upload(ng._h, src_ptr, 4 * cells))
            else:
                _lib.check(L.mg_grid_upload_async(ng._h, src_ptr, 4 * cells))
            _step(flags, vel, dens, p, ng)
            fn = L.mg_grid_download if mode == "sync" else L.mg_grid_download_async
            _lib.check(fn(dens._h, C.c_void_p(base), 4 * cells))
            _lib.check(fn(p._h, C.c_void_p(base + 4 * cells), 4 * cells))
            _lib.check(fn(vel._h, C.c_void_p(base + 8 * cells), 12 * cells))
        _lib.check(L.mg_solver_wait_copies(s._h))
        results[mode] = outs.copy()
        L.mg_host_free(pin_out)
    L.mg_host_free(pin_in)
    assert np.array_equal(results["sync"], results["async"])
    # the per-step densities differ from step to step (the steps really ran)
    d0 = results["async"][:cells]
    d1 = results["async"][5 * cells:6 * cells]
    assert not np.array_equal(d0, d1)
