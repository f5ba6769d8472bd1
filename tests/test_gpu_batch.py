"""Batched form: many plume scenes in one launch per stage.

* Each scene of a mixed batch gives bit for bit the result it gives alone:
  per-scene CG scalars are reduced in a fixed tile order and a scene stops
  at its own convergence, so its neighbours in the batch cannot change it.
* Against the single-scene path fed the same inflow: both run the same
  algorithm (MIC(0)-preconditioned CG in 3D, unpreconditioned CG in 2D as
  the reference's GridCg), so fields agree to the pressure tolerance of the
  other parity tests (1e-4) and iteration counts within +-1.  With the
  batch's preconditioner switched off, 3D scenes are solved without one and
  agree with the single-scene MIC(0) path only to the reference's plume-test
  thresholds (density 1e-3, velocity 5e-3, tools/tests/test_2010_plume3d.py).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

m = pytest.importorskip("mantaflow_gb300")
from mantaflow_gb300 import batch as mb  # noqa: E402

SIZES = [(40, 40, 1), (64, 48, 1), (33, 70, 1), (24, 24, 24), (20, 28, 16)]
GRAV = [(0.0, -g, 0.0) for g in (4e-3, 2e-3, 7e-3, 4e-3, 1e-3)]
SEEDS = [11, 12, 13, 14, 15]
STEPS = 3


def _run_batch(idx, preconditioner=1):
    b = mb.BatchedPlumes([SIZES[i] for i in idx], [GRAV[i] for i in idx], [SEEDS[i] for i in idx],
                         preconditioner=preconditioner)
    graphs = 0
    for _ in range(STEPS):
        graphs += b.step()["graph_launches"]
    _run_batch.graphs = graphs
    out = [(b.download(q, mb.DENSITY), b.download(q, mb.VELOCITY), b.download(q, mb.PRESSURE)) for q in range(len(idx))]
    inflows = [[b.inflow(q, t) for t in range(STEPS)] for q in range(len(idx))]
    its = [b.iterations(q)[0] for q in range(len(idx))]
    b.close()
    return out, inflows, its


def test_batch_scene_alone_equals_in_mix():
    mix, _, its_mix = _run_batch(list(range(len(SIZES))))
    assert _run_batch.graphs > 0  # the sweeps ran as CUDA graphs after the tile tuning
    for q in (0, 3):
        alone, _, its_alone = _run_batch([q])
        assert its_alone[0] == its_mix[q]
        for a, b in zip(alone[0], mix[q]):
            assert np.array_equal(a, b), "scene %d differs alone vs in the batch" % q


@pytest.mark.parametrize("preconditioner", [1, 0])
def test_batch_against_single_scene_path(preconditioner):
    out, inflows, its = _run_batch(list(range(len(SIZES))), preconditioner)
    for q, (nx, ny, nz) in enumerate(SIZES):
        dim = 3 if nz > 1 else 2
        s = m.Solver(name="one", gridSize=m.vec3(nx, ny, nz), dim=dim)
        s.timestep = 1.0
        flags = s.create(m.FlagGrid)
        flags.initDomain(boundaryWidth=0)
        flags.fillGrid()
        m.setOpenBound(flags, 0, "Y", m.FlagOutflow | m.FlagEmpty)
        vel, dens, pres, src = s.create(m.MACGrid), s.create(m.RealGrid), s.create(m.RealGrid), s.create(m.RealGrid)
        gs = m.vec3(nx, ny, nz)
        mask = s.create(m.RealGrid)
        cyl = s.create(m.Cylinder, center=gs * m.vec3(0.5, 0.1, 0.5), radius=nx * 0.14, z=gs * m.vec3(0, 0.02, 0))
        cyl.applyToGrid(grid=mask, value=1.0)
        for t in range(STEPS):
            assert np.array_equal(inflows[q][t], (np.asarray(inflows[q][t] > 0) * inflows[q][t]))
            m.copyArrayToGridReal(inflows[q][t], src)
            dens.join(src)
            m.advectSemiLagrange(flags=flags, vel=vel, grid=dens, order=2, clampMode=2)
            m.advectSemiLagrange(flags=flags, vel=vel, grid=vel, order=2, clampMode=2)
            m.setWallBcs(flags=flags, vel=vel)
            m.addBuoyancy(density=dens, vel=vel, gravity=m.vec3(*GRAV[q]), flags=flags)
            m.solvePressure(flags=flags, vel=vel, pressure=pres, cgAccuracy=1e-3, preconditioner=m.PcMIC)
        d, v, p = out[q]
        if dim == 2 or preconditioner == 1:
            assert abs(its[q] - m.lastSolveStats()[0]) <= 1, (q, its[q], m.lastSolveStats()[0])
            assert np.max(np.abs(d - dens.numpy())) <= 1e-4, q
            assert np.max(np.abs(v - vel.numpy())) <= 1e-4, q
            assert np.max(np.abs(p - pres.numpy())) <= 1e-4 * max(1.0, float(np.max(np.abs(p)))), q
        else:
            assert np.max(np.abs(d - dens.numpy())) <= 1e-3, q
            assert np.max(np.abs(v - vel.numpy())) <= 5e-3, q


def test_batch_fp64_refined_against_single_scene_refined():
    """The batched precision form: every scene's FP32 solve refined in FP64
    to max|b - A p| < 1e-5, against the single-scene refined solve
    (solvePressureRefined) fed the same inflow: 1e-5 absolute in pressure and
    velocity (both are within 1e-5 of the exact solution's residual)."""
    sizes, grav, seeds = [(48, 40, 1), (24, 20, 22)], [(0.0, -4e-3, 0.0), (0.0, -6e-3, 0.0)], [21, 22]
    b = mb.BatchedPlumes(sizes, grav, seeds)
    b.set_refinement(1e-5)
    steps = 3
    for _ in range(steps):
        b.step()
    for q, (nx, ny, nz) in enumerate(sizes):
        s = m.Solver(name="ref", gridSize=m.vec3(nx, ny, nz), dim=3 if nz > 1 else 2)
        s.timestep = 1.0
        flags = s.create(m.FlagGrid)
        flags.initDomain(boundaryWidth=0)
        flags.fillGrid()
        m.setOpenBound(flags, 0, "Y", m.FlagOutflow | m.FlagEmpty)
        vel, dens, pres, src = s.create(m.MACGrid), s.create(m.RealGrid), s.create(m.RealGrid), s.create(m.RealGrid)
        for t in range(steps):
            m.copyArrayToGridReal(b.inflow(q, t), src)
            dens.join(src)
            m.advectSemiLagrange(flags=flags, vel=vel, grid=dens, order=2, clampMode=2)
            m.advectSemiLagrange(flags=flags, vel=vel, grid=vel, order=2, clampMode=2)
            m.setWallBcs(flags=flags, vel=vel)
            m.addBuoyancy(density=dens, vel=vel, gravity=m.vec3(*grav[q]), flags=flags)
            m.solvePressureRefined(flags=flags, vel=vel, pressure=pres, cgAccuracy=1e-3, refineAccuracy=1e-5,
                                   preconditioner=m.PcMIC)
        assert np.max(np.abs(b.download(q, mb.PRESSURE) - pres.numpy())) <= 1e-5, q
        assert np.max(np.abs(b.download(q, mb.VELOCITY) - vel.numpy())) <= 1e-5, q
        assert np.max(np.abs(b.download(q, mb.DENSITY) - dens.numpy())) <= 1e-5, q
    b.close()
