"""Served form: continuous batching of plume jobs under a memory budget.

* A job's result is bit for bit the same alone and in a mix of jobs that
  arrive before, with and after it, on a budget small enough that jobs wait
  for admission: its scene's arithmetic and reductions involve only its own
  data.
* Admission respects the budget and the arrival order, and every job runs
  exactly its steps.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

m = pytest.importorskip("mantaflow_gb300")
from mantaflow_gb300 import batch as mb  # noqa: E402

JOB = dict(size=(24, 28, 20), gravity=(0.0, -4e-3, 0.0), seed=77, steps=6)


def _result(srv, jid):
    return [srv.result(jid, w) for w in (mb.DENSITY, mb.VELOCITY, mb.PRESSURE)]


def test_job_alone_equals_in_mix():
    alone = mb.PlumeServer(budget_bytes=2 * 10 ** 9)
    a = alone.submit(keep=True, **JOB)
    alone.run()
    want = _result(alone, a)
    alone.close()

    others = [dict(size=(40, 40), gravity=(0.0, -2e-3, 0.0), seed=1, steps=9),
              dict(size=(20, 20, 20), gravity=(0.0, -6e-3, 0.0), seed=2, steps=4),
              dict(size=(64, 33), gravity=(0.0, -1e-3, 0.0), seed=3, steps=7),
              dict(size=(32, 24, 28), gravity=(0.0, -8e-3, 0.0), seed=4, steps=5)]
    need = max(mb.PlumeServer.job_bytes(o["size"]) for o in others + [JOB])
    mix = mb.PlumeServer(budget_bytes=2 * need + 1)  # at most two resident jobs
    ids = [mix.submit(arrival=0.0, **others[0]), mix.submit(arrival=0.0, **others[1])]
    j = mix.submit(arrival=0.02, keep=True, **JOB)
    ids += [mix.submit(arrival=0.03, **others[2]), mix.submit(arrival=0.05, **others[3])]
    st = mix.run()
    assert st["peak_bytes"] <= 2 * need + 1
    got = _result(mix, j)
    for w, g in zip(want, got):
        assert np.array_equal(w, g)
    infos = [mix.job(q) for q in ids + [j]]
    for q, info in zip(ids + [j], infos):
        assert info["admitted"] >= info["arrival"] - 1e-9
        assert info["finished"] > info["admitted"]
    assert [mix.job(q)["steps"] for q in ids] == [o["steps"] for o in others]
    ms, jobs = mix.ticks()
    assert max(jobs) <= 2 and len(ms) == st["ticks"]
    mix.close()


def _dam_single(size, steps):
    """the dam-break scene through the single-scene path (one solver)"""
    from oracle import oracle as og
    nx, ny, nz = size
    f0 = np.zeros((nz, ny, nx), np.int32)
    og.init_domain(f0, 0)
    phi0 = np.zeros((nz, ny, nx), np.float32)
    og.box_sdf(phi0, (0, 0, 0), (0.4 * nx, 0.6 * ny, nz))
    og.update_from_levelset(f0, phi0)
    s = m.Solver(name="dam", gridSize=m.vec3(nx, ny, nz), dim=3 if nz > 1 else 2)
    s.timestep = 1.0
    flags = s.create(m.FlagGrid)
    m.copyArrayToGridReal(f0, flags)
    phi = s.create(m.LevelsetGrid)
    m.copyArrayToGridReal(phi0, phi)
    vel, pres = s.create(m.MACGrid), s.create(m.RealGrid)
    for _ in range(steps):
        m.extrapolateMACSimple(flags=flags, vel=vel, distance=4)
        m.advectSemiLagrange(flags=flags, vel=vel, grid=phi, order=1)
        flags.updateFromLevelset(phi)
        m.advectSemiLagrange(flags=flags, vel=vel, grid=vel, order=1)
        m.addGravity(flags=flags, vel=vel, gravity=m.vec3(0, -1e-3, 0))
        m.setWallBcs(flags=flags, vel=vel)
        m.solvePressure(flags=flags, vel=vel, pressure=pres, phi=phi)
        m.setWallBcs(flags=flags, vel=vel)
    return phi.numpy(), vel.numpy(), pres.numpy()


DAM = dict(size=(28, 24, 20), gravity=(0.0, -1e-3, 0.0), seed=5, steps=6, kind=mb.DAM_BREAK)


def test_dam_break_job_alone_equals_in_mix_and_single_path():
    """A dam-break job (free-surface liquid, ghost-fluid MIC(0) solve) gives
    the same bits alone and among plume and dam-break jobs, and agrees with
    the single-scene path's composed dam-break step (reduction order differs:
    1e-4, the pressure tolerance of the other parity tests)."""
    alone = mb.PlumeServer(budget_bytes=2 * 10 ** 9)
    a = alone.submit(keep=True, **DAM)
    alone.run()
    want = _result(alone, a)
    alone.close()
    others = [dict(size=(24, 28, 20), gravity=(0.0, -4e-3, 0.0), seed=1, steps=5),
              dict(size=(40, 36, 1), gravity=(0.0, -1e-3, 0.0), seed=2, steps=7, kind=mb.DAM_BREAK),
              dict(size=(20, 24, 28), gravity=(0.0, -1e-3, 0.0), seed=3, steps=4, kind=mb.DAM_BREAK)]
    mix = mb.PlumeServer(budget_bytes=2 * 10 ** 9)
    ids = [mix.submit(arrival=0.0, **others[0]), mix.submit(arrival=0.0, **others[1])]
    j = mix.submit(arrival=0.01, keep=True, **DAM)
    ids.append(mix.submit(arrival=0.02, **others[2]))
    mix.run()
    got = _result(mix, j)
    for w, g in zip(want, got):
        assert np.array_equal(w, g)
    assert [mix.job(q)["steps"] for q in ids] == [o["steps"] for o in others]
    mix.close()
    phi, vel, pres = _dam_single(DAM["size"], DAM["steps"])
    assert np.max(np.abs(want[0] - phi)) <= 1e-4
    assert np.max(np.abs(want[1] - vel)) <= 1e-4
    assert np.max(np.abs(want[2] - pres)) <= 1e-4
    assert np.max(np.abs(vel)) > 1e-3  # the liquid moved


def test_jobs_of_different_sizes():
    """Small and large plume and dam-break jobs resident together: every
    job's result equals its result alone, and admission keeps the arrival
    order."""
    jobs = [dict(size=(24, 28, 20), gravity=(0.0, -4e-3, 0.0), seed=11, steps=5),
            dict(size=(70, 66, 72), gravity=(0.0, -3e-3, 0.0), seed=12, steps=3),
            dict(size=(100, 104, 100), gravity=(0.0, -2e-3, 0.0), seed=13, steps=2, kind=mb.DAM_BREAK),
            dict(size=(30, 30, 30), gravity=(0.0, -1e-3, 0.0), seed=14, steps=4, kind=mb.DAM_BREAK)]
    want = []
    for jb in jobs:
        alone = mb.PlumeServer(budget_bytes=20 * 10 ** 9)
        a = alone.submit(keep=True, **jb)
        alone.run()
        want.append(_result(alone, a))
        alone.close()
    mix = mb.PlumeServer(budget_bytes=20 * 10 ** 9)
    ids = [mix.submit(arrival=0.001 * q, keep=True, **jb) for q, jb in enumerate(jobs)]
    mix.run()
    for q, w in zip(ids, want):
        for a, b in zip(w, _result(mix, q)):
            assert np.array_equal(a, b)
    adm = [mix.job(q)["admitted"] for q in ids]
    assert adm == sorted(adm)
    assert [mix.job(q)["steps"] for q in ids] == [jb["steps"] for jb in jobs]
    mix.close()
