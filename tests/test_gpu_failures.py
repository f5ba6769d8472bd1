"""Failure paths, exercised without faulting or hanging the GPU.

* A MIC(0) wavefront wait that runs out: the solver is told to make its next
  solve's sweeps wait for tile words that no tile publishes; the bounded
  wait gives up, the solve returns MG_ERR_TIMEOUT with its message, and the
  next solve on the same solver (normal limit) matches the oracle.
* CG divergence: velocities of 1e37 drive the residual norm above 1e35 in
  the first iteration, which the reference reports with its errMsg text
  (conjugategrad.cpp:288-295).
* An allocation that fails on the host side: a solver memory cap below what
  advection's temporaries need; the call fails with the out-of-memory text
  and the solver stays usable once the cap is lifted.
* A served job larger than the memory budget is refused at submission and
  the server runs the other jobs.
"""
import numpy as np
import pytest

from oracle import oracle as og

pytestmark = pytest.mark.gpu

m = pytest.importorskip("mantaflow_gb300")


def _scene(n, seed):
    rng = np.random.default_rng(seed)
    f = np.zeros((n, n, n), np.int32)
    og.init_domain(f, 0)
    og.fill_grid(f)
    og.set_open_bound(f, 0, "Y")
    v = (rng.random((n, n, n, 3), dtype=np.float32) - 0.5).astype(np.float32)
    return f, v


def _solver(n):
    s = m.Solver(name="fail", gridSize=m.vec3(n, n, n), dim=3)
    s.timestep = 1.0
    return s


def test_mic_wait_timeout_then_recovers(monkeypatch):
    monkeypatch.setenv("MANTA_GB300_MIC", "flow")
    n = 40  # 27 tiles of 16^3: downstream tiles wait on upstream faces
    f, v = _scene(n, 3)
    s = _solver(n)
    flags = s.create(m.FlagGrid)
    m.copyArrayToGridReal(f, flags)
    vel = s.create(m.MACGrid)
    p = s.create(m.RealGrid)
    m.copyArrayToGridReal(v, vel)
    s.setWaitLimit(2_000_000, stallNextSolve=True)  # 2 ms, first wait runs out
    with pytest.raises(m.MantaError) as e:
        m.solvePressure(flags=flags, vel=vel, pressure=p, preconditioner=m.PcMIC)
    assert "exceeded its spin limit" in str(e.value)
    # the context is intact: a normal solve on the same solver is right
    s.setWaitLimit(0)
    m.copyArrayToGridReal(v, vel)
    p.setConst(0.0)
    m.solvePressure(flags=flags, vel=vel, pressure=p, preconditioner=m.PcMIC)
    it, _ = m.lastSolveStats()
    vo, po = v.copy(), np.zeros(f.shape, np.float32)
    it_ref, _, _ = og.solve_pressure(f, vo, po, preconditioner=og.PC_MIC)
    assert abs(it - it_ref) <= 1
    assert np.max(np.abs(p.numpy() - po)) <= 1e-4


def test_cg_divergence_reports_reference_text():
    n = 24
    f, v = _scene(n, 4)
    s = _solver(n)
    flags = s.create(m.FlagGrid)
    m.copyArrayToGridReal(f, flags)
    vel = s.create(m.MACGrid)
    p = s.create(m.RealGrid)
    m.copyArrayToGridReal((v * 2e37).astype(np.float32), vel)
    with pytest.raises(m.MantaError) as e:
        m.solvePressure(flags=flags, vel=vel, pressure=p, preconditioner=m.PcMIC)
    assert "The CG solver diverged, residual norm > 1e30, stopping." in str(e.value)
    # and the solver keeps working
    m.copyArrayToGridReal(v, vel)
    p.setConst(0.0)
    m.solvePressure(flags=flags, vel=vel, pressure=p, preconditioner=m.PcMIC)


def test_memory_cap_refuses_allocation_cleanly():
    n = 32
    f, v = _scene(n, 5)
    s = _solver(n)
    flags = s.create(m.FlagGrid)
    m.copyArrayToGridReal(f, flags)
    vel = s.create(m.MACGrid)
    m.copyArrayToGridReal(v, vel)
    dens = s.create(m.RealGrid)
    d0 = np.random.default_rng(6).random((n, n, n), dtype=np.float32)
    m.copyArrayToGridReal(d0, dens)
    held = s.memoryBytes()
    s.setMemoryLimit(held + 4 * n ** 3)  # room for one Real temporary, not the two MacCormack needs
    with pytest.raises(m.MantaError) as e:
        m.advectSemiLagrange(flags=flags, vel=vel, grid=dens, order=2, clampMode=2)
    assert "out of device memory" in str(e.value)
    with pytest.raises(m.MantaError):
        s.create(m.MACGrid)
    assert np.array_equal(dens.numpy(), d0)  # nothing was written
    s.setMemoryLimit(0)
    m.advectSemiLagrange(flags=flags, vel=vel, grid=dens, order=2, clampMode=2)
    do, vo = d0.copy(), v.copy()
    og.advect_semi_lagrange(f, vo, do, og.KIND_REAL, order=2, clampMode=2)
    assert np.array_equal(dens.numpy(), do)


def test_served_job_over_budget_is_refused():
    from mantaflow_gb300 import batch as mb
    small = (20, 20, 20)
    need = mb.PlumeServer.job_bytes(small)
    srv = mb.PlumeServer(budget_bytes=2 * need)
    with pytest.raises(m.MantaError) as e:
        srv.submit(size=(96, 96, 96), gravity=(0, -4e-3, 0), seed=1, steps=3)
    assert "exceeds the memory budget" in str(e.value)
    j = srv.submit(size=small, gravity=(0, -4e-3, 0), seed=2, steps=3)
    st = srv.run()
    assert st["jobs"] == 1 and srv.job(j)["steps"] == 3
    srv.close()
