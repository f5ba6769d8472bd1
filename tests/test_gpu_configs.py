"""GPU parity on the benchmark scenes at their own sizes.

* Dam break (free surface, ghost fluid): the composed step -- extrapolate
  MAC velocities 4 cells, advect phi (SL order 1), update the flags from phi,
  advect the velocity (SL order 1), gravity, walls, ghost-fluid pressure
  solve, walls -- replayed against the reference executable's per-step
  outputs (tests/golden/dam_24.npz), and at 128^3 against the oracle.
* Smoke plume at 256^3 (the headline scene) with PcMGStatic and PcMIC, and
  at 64^3 with PcMIC for 30 steps (the small-plume scene).

Lockstep comparisons start the oracle's step from the GPU's state at the
start of that step, so each step's error is measured on its own:
  - advected fields (density, velocity after MacCormack): within 1e-5
    relative to the field's magnitude, >= 99.9% of cells bit-identical;
  - CG iterations within +-1 of the oracle (reduction order differs);
  - pressure and projected velocity within 1e-4 (the reference's own float
    threshold, tools/tests/test_0100_psolve.py);
  - divergence left after projection no worse than the oracle's at the same
    cgAccuracy (5% slack, or below cgAccuracy).
The free-running 64^3 run compares the two independent trajectories at the
end with tools/tests/test_2010_plume3d.py's thresholds (density 1e-3,
velocity 5e-3, absolute).
"""
import os

import numpy as np
import pytest

from oracle import oracle as og
from tests.conftest import golden_path

pytestmark = pytest.mark.gpu

m = pytest.importorskip("mantaflow_gb300")


@pytest.fixture(scope="module", autouse=True)
def oracle_threads():
    og.set_num_threads(os.cpu_count() or 1)
    yield
    og.set_num_threads(1)


def divergence(flags, vel):
    """max |MakeRhs| over fluid cells (the oracle, on the CPU)"""
    rhs = np.zeros(flags.shape, np.float32)
    og.compute_pressure_rhs(rhs, vel.astype(np.float32).copy(), flags)
    fl = (flags & og.FLUID) != 0
    return float(np.max(np.abs(rhs[fl]))) if fl.any() else 0.0


def assert_advected(got, want, what, rel=1e-5, min_exact=0.999):
    scale = max(1.0, float(np.max(np.abs(want))))
    d = float(np.max(np.abs(got.astype(np.float64) - want)))
    assert d <= rel * scale, "%s: max diff %g (scale %g)" % (what, d, scale)
    exact = float(np.mean(got == want))
    assert exact >= min_exact, "%s: %.5f of cells bit-identical" % (what, exact)


def assert_projected(it, it_ref, p, p_ref, v, v_ref, flags, acc, what):
    assert abs(it - it_ref) <= 1, "%s: %d CG iterations vs oracle %d" % (what, it, it_ref)
    dp = float(np.max(np.abs(p - p_ref)))
    assert dp <= 1e-4 * max(1.0, float(np.max(np.abs(p_ref)))), "%s: pressure off by %g" % (what, dp)
    dv = float(np.max(np.abs(v - v_ref)))
    assert dv <= 1e-4, "%s: velocity off by %g" % (what, dv)
    d_gpu, d_ref = divergence(flags, v), divergence(flags, v_ref)
    assert d_gpu <= max(1.05 * d_ref, acc), "%s: divergence %g vs oracle %g" % (what, d_gpu, d_ref)


# ------------------------------------------------------------------ plume
class GpuPlume:
    def __init__(self, n, pc, dt=1.0):
        s = m.Solver(name="plume%d" % n, gridSize=m.vec3(n, n, n), dim=3)
        s.timestep = dt
        self.s, self.n, self.pc = s, n, pc
        self.flags = s.create(m.FlagGrid)
        self.flags.initDomain(boundaryWidth=0)
        self.flags.fillGrid()
        m.setOpenBound(self.flags, 0, "Y", m.FlagOutflow | m.FlagEmpty)
        self.vel = s.create(m.MACGrid)
        self.dens = s.create(m.RealGrid)
        self.pres = s.create(m.RealGrid)
        self.noise = s.create(m.RealGrid)
        gs = m.vec3(n, n, n)
        mask = s.create(m.RealGrid)
        src = s.create(m.Cylinder, center=gs * m.vec3(0.5, 0.1, 0.5), radius=n * 0.14, z=gs * m.vec3(0, 0.02, 0))
        src.applyToGrid(grid=mask, value=1.0)
        self.mask = mask.numpy()

    def step(self, a, record=False):
        m.copyArrayToGridReal(a, self.noise)
        self.dens.join(self.noise)
        m.advectSemiLagrange(flags=self.flags, vel=self.vel, grid=self.dens, order=2, clampMode=2)
        m.advectSemiLagrange(flags=self.flags, vel=self.vel, grid=self.vel, order=2, clampMode=2)
        adv = (self.dens.numpy(), self.vel.numpy()) if record else None
        m.setWallBcs(flags=self.flags, vel=self.vel)
        m.addBuoyancy(density=self.dens, vel=self.vel, gravity=m.vec3(0, -4e-3, 0), flags=self.flags)
        m.solvePressure(flags=self.flags, vel=self.vel, pressure=self.pres, cgAccuracy=1e-3, preconditioner=self.pc)
        self.s.step()
        return adv, m.lastSolveStats()[0]


def oracle_plume_step(f, dens, vel, a, pc, mg_cache, record=False):
    """one plume step of the oracle in place; returns (advected, iterations, pressure)"""
    og.join_real(dens, a)
    og.advect_semi_lagrange(f, vel, dens, og.KIND_REAL, order=2, clampMode=2)
    og.advect_semi_lagrange(f, vel, vel, og.KIND_MAC, order=2, clampMode=2)
    adv = (dens.copy(), vel.copy()) if record else None
    og.set_wall_bcs(f, vel)
    og.add_buoyancy(f, dens, vel, (0, -4e-3, 0))
    pres = np.zeros(f.shape, np.float32)
    it, _, _ = og.solve_pressure(f, vel, pres, cgAccuracy=1e-3, preconditioner=pc, mg_cache=mg_cache)
    return adv, it, pres


def _plume_lockstep(n, steps, pc_m, pc_o, seed):
    g = GpuPlume(n, pc_m)
    f = g.flags.numpy()
    rng = np.random.default_rng(seed)
    cache = og.MGCache() if pc_o == og.PC_MG_STATIC else None
    try:
        for t in range(steps):
            dens0, vel0 = g.dens.numpy(), g.vel.numpy()
            a = (rng.random((n, n, n), dtype=np.float32) * g.mask).astype(np.float32)
            adv, it = g.step(a, record=True)
            do, vo = dens0.copy(), vel0.copy()
            adv_ref, it_ref, p_ref = oracle_plume_step(f, do, vo, a, pc_o, cache, record=True)
            what = "%d^3 step %d" % (n, t)
            assert_advected(adv[0], adv_ref[0], what + " density")
            assert_advected(adv[1], adv_ref[1], what + " velocity")
            assert_projected(it, it_ref, g.pres.numpy(), p_ref, g.vel.numpy(), vo, f, 1e-3, what)
    finally:
        if cache is not None:
            cache.release()


@pytest.mark.parametrize("pc", ["mgstatic", "mic"])
def test_plume_256_lockstep_against_oracle(pc):
    """The headline scene at its size: 3 steps from rest (the static
    multigrid hierarchy is built in the first and reused)."""
    pc_m, pc_o = {"mgstatic": (m.PcMGStatic, og.PC_MG_STATIC), "mic": (m.PcMIC, og.PC_MIC)}[pc]
    _plume_lockstep(256, 3, pc_m, pc_o, seed=2024)


def test_plume_64_config_run():
    """The small-plume scene (64^3, PcMIC, cgAccuracy 1e-3): 30 steps in
    lockstep against the oracle, and the free-running trajectories at the
    end against tools/tests/test_2010_plume3d.py's thresholds."""
    n, steps = 64, 30
    _plume_lockstep(n, steps, m.PcMIC, og.PC_MIC, seed=64)
    g = GpuPlume(n, m.PcMIC)
    f = g.flags.numpy()
    dens = np.zeros((n, n, n), np.float32)
    vel = np.zeros((n, n, n, 3), np.float32)
    rng = np.random.default_rng(65)
    for t in range(steps):
        a = (rng.random((n, n, n), dtype=np.float32) * g.mask).astype(np.float32)
        g.step(a)
        oracle_plume_step(f, dens, vel, a, og.PC_MIC, None)
    dd = float(np.max(np.abs(g.dens.numpy() - dens)))
    dv = float(np.max(np.abs(g.vel.numpy() - vel)))
    assert dd <= 1e-3, "density after %d steps off by %g" % (steps, dd)
    assert dv <= 5e-3, "velocity after %d steps off by %g" % (steps, dv)


# -------------------------------------------------------------- dam break
class GpuDam:
    def __init__(self, flags0, phi0):
        n = flags0.shape[0]
        s = m.Solver(name="dam%d" % n, gridSize=m.vec3(n, n, n), dim=3)
        s.timestep = 1.0
        self.s = s
        self.flags = s.create(m.FlagGrid)
        m.copyArrayToGridReal(flags0, self.flags)
        self.phi = s.create(m.LevelsetGrid)
        m.copyArrayToGridReal(phi0, self.phi)
        self.vel = s.create(m.MACGrid)
        self.pres = s.create(m.RealGrid)

    def step(self):
        m.extrapolateMACSimple(flags=self.flags, vel=self.vel, distance=4)
        m.advectSemiLagrange(flags=self.flags, vel=self.vel, grid=self.phi, order=1)
        self.flags.updateFromLevelset(self.phi)
        m.advectSemiLagrange(flags=self.flags, vel=self.vel, grid=self.vel, order=1)
        m.addGravity(flags=self.flags, vel=self.vel, gravity=m.vec3(0, -1e-3, 0))
        m.setWallBcs(flags=self.flags, vel=self.vel)
        m.solvePressure(flags=self.flags, vel=self.vel, pressure=self.pres, phi=self.phi)
        m.setWallBcs(flags=self.flags, vel=self.vel)
        self.s.step()
        return m.lastSolveStats()[0]


def test_dam_break_steps_against_reference():
    """The composed dam-break step on the GPU against the reference
    executable's per-step flags, phi, velocity, pressure and iterations."""
    g = np.load(golden_path("dam_24"), allow_pickle=False)
    dam = GpuDam(g["flags0"], g["phi0"])
    for t in range(len(g["iters"])):
        it = dam.step()
        assert abs(it - int(g["iters"][t])) <= 1, "step %d: %d iterations vs %d" % (t, it, int(g["iters"][t]))
        assert np.array_equal(dam.flags.numpy(), g["flags"][t]), "step %d flags" % t
        assert float(np.max(np.abs(dam.phi.numpy() - g["phi"][t]))) <= 1e-4, "step %d phi" % t
        assert float(np.max(np.abs(dam.vel.numpy() - g["vel"][t]))) <= 1e-4, "step %d velocity" % t
        assert float(np.max(np.abs(dam.pres.numpy() - g["pressure"][t]))) <= 1e-4, "step %d pressure" % t


def test_dam_break_128_lockstep_against_oracle():
    """The dam-break scene at its size (128^3, box of liquid x < 0.4N,
    y < 0.6N): 4 steps, each started on the oracle from the GPU's state."""
    n = 128
    f0 = np.zeros((n, n, n), np.int32)
    og.init_domain(f0, 0)
    phi0 = np.zeros((n, n, n), np.float32)
    og.box_sdf(phi0, (0, 0, 0), (0.4 * n, 0.6 * n, n))
    og.update_from_levelset(f0, phi0)
    dam = GpuDam(f0, phi0)
    for t in range(4):
        f, phi, vel = dam.flags.numpy(), dam.phi.numpy(), dam.vel.numpy()
        it = dam.step()
        og.extrapolate_mac_simple(f, vel, 4)
        og.advect_semi_lagrange(f, vel, phi, og.KIND_REAL, order=1)
        og.update_from_levelset(f, phi)
        og.advect_semi_lagrange(f, vel, vel, og.KIND_MAC, order=1)
        og.add_gravity(f, vel, (0, -1e-3, 0))
        og.set_wall_bcs(f, vel)
        pres = np.zeros((n, n, n), np.float32)
        it_ref, _, _ = og.solve_pressure(f, vel, pres, phi=phi)
        og.set_wall_bcs(f, vel)
        what = "dam 128^3 step %d" % t
        assert np.array_equal(dam.flags.numpy(), f), what + " flags"
        assert_advected(dam.phi.numpy(), phi, what + " phi")
        assert_projected(it, it_ref, dam.pres.numpy(), pres, dam.vel.numpy(), vel, f, 1e-3, what)
