"""The helper entries of the drop-in boundary on the GPU against the oracle:
resetPhiInObs (advection.cpp:396-401), resetOutflow without particles
(extforces.cpp:133-160), addGravity with an exclude grid and
addGravityNoScale (extforces.cpp:45-69), and solvePressure's three parts
computePressureRhs / solvePressureSystem / correctVelocity
(pressure.cpp:277-476), which together must give solvePressure's result,
and extrapolateMACSimple with an obstacle levelset (fastmarch.cpp:316-375).
"""
import numpy as np
import pytest

from oracle import oracle as og

pytestmark = pytest.mark.gpu

m = pytest.importorskip("mantaflow_gb300")


def _solver(shape, dt=1.0):
    nz, ny, nx = shape
    s = m.Solver(name="entries", gridSize=m.vec3(nx, ny, nz), dim=3 if nz > 1 else 2)
    s.timestep = dt
    return s


def _flags(shape, seed, obstacles=True, open_top=True):
    rng = np.random.default_rng(seed)
    f = np.zeros(shape, np.int32)
    og.init_domain(f, 0)
    og.fill_grid(f)
    if open_top:
        og.set_open_bound(f, 0, "Y")
    if obstacles:
        inner = f[1:-1, 1:-1, 1:-1] if shape[0] > 1 else f[:, 1:-1, 1:-1]
        mask = rng.random(inner.shape) < 0.05
        inner[mask] = og.OBSTACLE
    return f


@pytest.mark.parametrize("shape", [(20, 22, 24), (1, 40, 36)])
def test_reset_phi_in_obs(shape):
    f = _flags(shape, 1)
    rng = np.random.default_rng(2)
    phi = (rng.random(shape, dtype=np.float32) - 0.5).astype(np.float32)
    s = _solver(shape)
    flags, g = s.create(m.FlagGrid), s.create(m.LevelsetGrid)
    m.copyArrayToGridReal(f, flags)
    m.copyArrayToGridReal(phi, g)
    m.resetPhiInObs(flags, g)
    want = phi.copy()
    og.reset_phi_in_obs(f, want)
    assert np.array_equal(g.numpy(), want)
    assert np.any(want != phi)


@pytest.mark.parametrize("shape", [(20, 22, 24), (1, 40, 36)])
def test_reset_outflow(shape):
    f = _flags(shape, 3)
    f[f == (og.OUTFLOW | og.EMPTY)] |= og.FLUID  # outflow cells that still carry the fluid bit
    rng = np.random.default_rng(4)
    phi = (rng.random(shape, dtype=np.float32) - 0.5).astype(np.float32)
    real = rng.random(shape, dtype=np.float32)
    s = _solver(shape)
    flags, gp, gr = s.create(m.FlagGrid), s.create(m.LevelsetGrid), s.create(m.RealGrid)
    m.copyArrayToGridReal(f, flags)
    m.copyArrayToGridReal(phi, gp)
    m.copyArrayToGridReal(real, gr)
    m.resetOutflow(flags, phi=gp, real=gr)
    fo, po, ro = f.copy(), phi.copy(), real.copy()
    og.reset_outflow(fo, po, ro)
    assert np.array_equal(flags.numpy(), fo)
    assert np.array_equal(gp.numpy(), po)
    assert np.array_equal(gr.numpy(), ro)
    assert np.any(fo != f)


@pytest.mark.parametrize("shape", [(18, 20, 22), (1, 30, 34)])
def test_add_gravity_exclude_and_no_scale(shape):
    dt = 0.7
    f = _flags(shape, 5)
    rng = np.random.default_rng(6)
    f[(rng.random(shape) < 0.2) & (f == og.FLUID)] = og.EMPTY
    v = (rng.random(shape + (3,), dtype=np.float32) - 0.5).astype(np.float32)
    ex = (rng.random(shape, dtype=np.float32) - 0.3).astype(np.float32)
    s = _solver(shape, dt)
    flags, vel, exg = s.create(m.FlagGrid), s.create(m.MACGrid), s.create(m.RealGrid)
    m.copyArrayToGridReal(f, flags)
    m.copyArrayToGridReal(ex, exg)
    grav = (0.01, -0.2, 0.03)
    m.copyArrayToGridReal(v, vel)
    m.addGravity(flags=flags, vel=vel, gravity=m.vec3(*grav), exclude=exg, scale=True)
    want = v.copy()
    og.add_gravity(f, want, grav, exclude=ex, scale=True, dt=dt)
    assert np.array_equal(vel.numpy(), want)
    m.copyArrayToGridReal(v, vel)
    m.addGravityNoScale(flags=flags, vel=vel, gravity=m.vec3(*grav))
    want = v.copy()
    og.add_gravity(f, want, grav, scale=False, dt=dt)
    assert np.array_equal(vel.numpy(), want)


@pytest.mark.parametrize("pc", ["mic", "mgdynamic"])
@pytest.mark.parametrize("gf", [False, True])
def test_split_solve_equals_solve_pressure(pc, gf):
    """computePressureRhs + solvePressureSystem + correctVelocity on one grid
    set, solvePressure on another: identical results; the right-hand side is
    the oracle's bit for bit and the pressure within its solver tolerance."""
    shape = (28, 30, 32)
    pcm = {"mic": m.PcMIC, "mgdynamic": m.PcMGDynamic}[pc]
    pco = {"mic": og.PC_MIC, "mgdynamic": og.PC_MG_DYNAMIC}[pc]
    f = _flags(shape, 7, open_top=not gf)
    rng = np.random.default_rng(8)
    v = (rng.random(shape + (3,), dtype=np.float32) - 0.5).astype(np.float32)
    phi = None
    if gf:
        z, y, x = np.mgrid[0:shape[0], 0:shape[1], 0:shape[2]].astype(np.float32) + 0.5
        phi = (y - 0.55 * shape[1] + 1.5 * np.sin(x / 4.0)).astype(np.float32)
        og.update_from_levelset(f, phi)
    s = _solver(shape)
    flags = s.create(m.FlagGrid)
    m.copyArrayToGridReal(f, flags)
    gphi = None
    if gf:
        gphi = s.create(m.LevelsetGrid)
        m.copyArrayToGridReal(phi, gphi)
    kw = dict(cgAccuracy=1e-4, preconditioner=pcm)
    # split
    vel, pres, rhs = s.create(m.MACGrid), s.create(m.RealGrid), s.create(m.RealGrid)
    m.copyArrayToGridReal(v, vel)
    m.computePressureRhs(rhs=rhs, vel=vel, pressure=pres, flags=flags, phi=gphi, **kw)
    rhs0 = rhs.numpy()
    m.solvePressureSystem(rhs=rhs, vel=vel, pressure=pres, flags=flags, phi=gphi, **kw)
    it_split = m.lastSolveStats()[0]
    m.correctVelocity(vel=vel, pressure=pres, flags=flags, phi=gphi, **kw)
    # whole
    vel2, pres2 = s.create(m.MACGrid), s.create(m.RealGrid)
    m.copyArrayToGridReal(v, vel2)
    m.solvePressure(vel=vel2, pressure=pres2, flags=flags, phi=gphi, **kw)
    it_whole = m.lastSolveStats()[0]
    assert it_split == it_whole
    assert np.array_equal(pres.numpy(), pres2.numpy())
    assert np.array_equal(vel.numpy(), vel2.numpy())
    # against the oracle
    r_ref = np.zeros(shape, np.float32)
    og.compute_pressure_rhs(r_ref, v.copy(), f, phi=phi)
    assert np.array_equal(rhs0, r_ref)
    vo, po = v.copy(), np.zeros(shape, np.float32)
    it_ref, _, _ = og.solve_pressure(f, vo, po, phi=phi, preconditioner=pco, cgAccuracy=1e-4)
    assert abs(it_whole - it_ref) <= 1
    assert float(np.max(np.abs(pres2.numpy() - po))) <= 1e-4 * max(1.0, float(np.max(np.abs(po))))
    assert float(np.max(np.abs(vel2.numpy() - vo))) <= 1e-4


@pytest.mark.parametrize("shape", [(24, 26, 28), (1, 44, 40)])
@pytest.mark.parametrize("intoObs", [False, True])
def test_extrapolate_mac_simple_with_phi_obs(shape, intoObs):
    """extrapolateMACSimple with an obstacle levelset (fastmarch.cpp:337-375,
    knUnprojectNormalComp :316-330): velocities inside the obstacle band
    lose their component against the obstacle normal.  Against the oracle's
    restatement (the golden set holds no phiObs case: oracle only)."""
    nz, ny, nx = shape
    f = np.zeros(shape, np.int32)
    og.init_domain(f, 0)
    og.fill_grid(f)
    z, y, x = np.mgrid[0:nz, 0:ny, 0:nx].astype(np.float32) + 0.5
    cz = nz / 2 if nz > 1 else 0.5
    obs = (np.sqrt((x - 0.6 * nx) ** 2 + (y - 0.45 * ny) ** 2 + (z - cz) ** 2) - 0.22 * min(nx, ny)).astype(np.float32)
    f[(obs < 0) & (f == og.FLUID)] = og.OBSTACLE
    rng = np.random.default_rng(9)
    f[(rng.random(shape) < 0.3) & (f == og.FLUID)] = og.EMPTY
    v = (rng.random(shape + (3,), dtype=np.float32) - 0.5).astype(np.float32)
    s = _solver(shape)
    flags, vel, phi = s.create(m.FlagGrid), s.create(m.MACGrid), s.create(m.LevelsetGrid)
    m.copyArrayToGridReal(f, flags)
    m.copyArrayToGridReal(v, vel)
    m.copyArrayToGridReal(obs, phi)
    m.extrapolateMACSimple(flags=flags, vel=vel, distance=3, phiObs=phi, intoObs=intoObs)
    want = v.copy()
    og.extrapolate_mac_simple(f, want, 3, intoObs=intoObs, phiObs=obs)
    assert np.array_equal(vel.numpy(), want)
    plain = v.copy()
    og.extrapolate_mac_simple(f, plain, 3, intoObs=intoObs)
    assert np.any(plain != want)  # the obstacle band changed something
