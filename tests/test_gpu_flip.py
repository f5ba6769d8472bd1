"""FLIP particle <-> grid transfers (plugin/flip.cpp:549-673) on the GPU
against the oracle, bit for bit.

The reference splats particles with single-threaded loops, so a face's sums
follow particle order; the GPU gathers per face from particles sorted by
stencil cell and merges them back into particle order, so every sum is the
same sequence of float additions.  The cases cover 2D and 3D, particles
outside the domain (border clamps), deleted particles, a type mask with
exclude, empty systems, one crowded cell, and a 64^3 system of 2M particles.
"""
import numpy as np
import pytest

from oracle import oracle as og

pytestmark = pytest.mark.gpu

m = pytest.importorskip("mantaflow_gb300")


def _scene(n, dim):
    nz = n if dim == 3 else 1
    s = m.Solver(name="flip", gridSize=m.vec3(n, n, nz), dim=dim)
    flags = s.create(m.FlagGrid)
    flags.initDomain(boundaryWidth=0)
    flags.fillGrid()
    return s, flags


def _particles(rng, n, dim, count, spread=1.0, deleted=0.05):
    lo, hi = -spread, n + spread
    pos = rng.uniform(lo, hi, size=(count, 3)).astype(np.float32)
    if dim == 2:
        pos[:, 2] = rng.uniform(0.0, 1.0, size=count).astype(np.float32)
    flag = np.zeros(count, np.int32)
    flag[rng.random(count) < deleted] = m.ParticleDelete
    return pos, flag


def _system(s, pos, flag):
    pp = s.create(m.BasicParticleSystem)
    pp.setPositions(pos, flag)
    return pp


def _oracle_flags(flags):
    return flags.numpy()


@pytest.mark.parametrize("dim,n,count", [(3, 20, 60000), (2, 40, 20000), (3, 17, 5000)])
def test_map_parts_to_mac_bitwise(dim, n, count):
    rng = np.random.default_rng(100 + dim * n)
    s, flags = _scene(n, dim)
    pos, flag = _particles(rng, n, dim, count)
    pv = rng.standard_normal((count, 3)).astype(np.float32)
    ptype = rng.integers(1, 5, size=count).astype(np.int32)
    pp = _system(s, pos, flag)
    pvel = pp.create(m.PdataVec3)
    m.copyArrayToPdataVec3(pv, pvel)
    pt = pp.create(m.PdataInt)
    m.copyArrayToPdataInt(ptype, pt)
    vel, velOld, weight = s.create(m.MACGrid), s.create(m.MACGrid), s.create(m.VecGrid)
    f = _oracle_flags(flags)
    for exclude, use_type in ((0, False), (2, True)):
        m.mapPartsToMAC(flags=flags, vel=vel, velOld=velOld, parts=pp, partVel=pvel, weight=weight,
                        ptype=pt if use_type else None, exclude=exclude)
        shape = f.shape + (3,)
        v_ref, vo_ref, w_ref = np.zeros(shape, np.float32), np.zeros(shape, np.float32), np.zeros(shape, np.float32)
        og.map_parts_to_mac(f, v_ref, vo_ref, pos, flag, pv, weight=w_ref, ptype=ptype if use_type else None,
                            exclude=exclude)
        assert np.array_equal(weight.numpy(), w_ref), "weights differ"
        got = vel.numpy()
        assert np.array_equal(got, v_ref), "velocity differs at %d faces" % int(np.sum(got != v_ref))
        assert np.array_equal(velOld.numpy(), vo_ref)


def test_map_parts_to_mac_64_two_million():
    n, ppc = 64, 8
    rng = np.random.default_rng(7)
    s, flags = _scene(n, 3)
    count = ppc * n ** 3
    pos, flag = _particles(rng, n, 3, count, spread=0.5, deleted=0.01)
    pv = rng.standard_normal((count, 3)).astype(np.float32)
    pp = _system(s, pos, flag)
    pvel = pp.create(m.PdataVec3)
    m.copyArrayToPdataVec3(pv, pvel)
    vel, velOld = s.create(m.MACGrid), s.create(m.MACGrid)
    m.mapPartsToMAC(flags=flags, vel=vel, velOld=velOld, parts=pp, partVel=pvel)
    f = _oracle_flags(flags)
    v_ref, vo_ref = np.zeros(f.shape + (3,), np.float32), np.zeros(f.shape + (3,), np.float32)
    og.map_parts_to_mac(f, v_ref, vo_ref, pos, flag, pv)
    assert np.array_equal(vel.numpy(), v_ref)


def test_map_parts_to_mac_crowded_cell_and_empty():
    n = 12
    rng = np.random.default_rng(9)
    s, flags = _scene(n, 3)
    f = _oracle_flags(flags)
    # 30000 particles inside one cell, a few elsewhere
    pos = (np.float32(5.0) + rng.random((30000, 3), dtype=np.float32)).astype(np.float32)
    pos[:50] = rng.uniform(0, n, size=(50, 3)).astype(np.float32)
    flag = np.zeros(len(pos), np.int32)
    pv = rng.standard_normal((len(pos), 3)).astype(np.float32)
    pp = _system(s, pos, flag)
    pvel = pp.create(m.PdataVec3)
    m.copyArrayToPdataVec3(pv, pvel)
    vel, velOld = s.create(m.MACGrid), s.create(m.MACGrid)
    m.mapPartsToMAC(flags=flags, vel=vel, velOld=velOld, parts=pp, partVel=pvel)
    v_ref, vo_ref = np.zeros(f.shape + (3,), np.float32), np.zeros(f.shape + (3,), np.float32)
    og.map_parts_to_mac(f, v_ref, vo_ref, pos, flag, pv)
    assert np.array_equal(vel.numpy(), v_ref)
    # every particle deleted: the grid is cleared
    flag[:] = m.ParticleDelete
    pp.setPositions(pos, flag)
    vel.setConst(m.vec3(1, 2, 3))
    m.mapPartsToMAC(flags=flags, vel=vel, velOld=velOld, parts=pp, partVel=pvel)
    assert not np.any(vel.numpy())
    # an empty system
    empty = s.create(m.BasicParticleSystem)
    ev = empty.create(m.PdataVec3)
    vel.setConst(m.vec3(1, 2, 3))
    m.mapPartsToMAC(flags=flags, vel=vel, velOld=velOld, parts=empty, partVel=ev)
    assert not np.any(vel.numpy())


@pytest.mark.parametrize("dim", [3, 2])
def test_mac_to_parts_and_flip_update_bitwise(dim):
    n, count = 24, 40000
    rng = np.random.default_rng(30 + dim)
    s, flags = _scene(n, dim)
    f = _oracle_flags(flags)
    pos, flag = _particles(rng, n, dim, count)
    pv0 = rng.standard_normal((count, 3)).astype(np.float32)
    ptype = rng.integers(1, 5, size=count).astype(np.int32)
    gv = rng.standard_normal(f.shape + (3,)).astype(np.float32)
    gvo = rng.standard_normal(f.shape + (3,)).astype(np.float32)
    vel, velOld = s.create(m.MACGrid), s.create(m.MACGrid)
    m.copyArrayToGridReal(gv, vel)
    m.copyArrayToGridReal(gvo, velOld)
    pp = _system(s, pos, flag)
    pvel = pp.create(m.PdataVec3)
    pt = pp.create(m.PdataInt)
    m.copyArrayToPdataInt(ptype, pt)
    # PIC
    m.copyArrayToPdataVec3(pv0, pvel)
    m.mapMACToParts(flags=flags, vel=vel, parts=pp, partVel=pvel, ptype=pt, exclude=1)
    ref = pv0.copy()
    og.map_mac_to_parts(f, gv, pos, flag, ref, ptype=ptype, exclude=1)
    assert np.array_equal(pvel.numpy(), ref)
    # FLIP
    for ratio in (0.95, 0.0, 1.0, 0.3):
        m.copyArrayToPdataVec3(pv0, pvel)
        m.flipVelocityUpdate(flags=flags, vel=vel, velOld=velOld, parts=pp, partVel=pvel, flipRatio=ratio)
        ref = pv0.copy()
        og.flip_velocity_update(f, gv, gvo, pos, flag, ref, float(ratio))
        assert np.array_equal(pvel.numpy(), ref), "flipRatio %g" % ratio


@pytest.mark.parametrize("dim", [3, 2])
def test_parts_to_grid_and_back_bitwise(dim):
    n, count = 22, 30000
    rng = np.random.default_rng(50 + dim)
    s, flags = _scene(n, dim)
    f = _oracle_flags(flags)
    pos, flag = _particles(rng, n, dim, count, spread=0.7)
    pp = _system(s, pos, flag)
    pr = pp.create(m.PdataReal)
    pv = pp.create(m.PdataVec3)
    sr = rng.standard_normal(count).astype(np.float32)
    sv = rng.standard_normal((count, 3)).astype(np.float32)
    m.copyArrayToPdataReal(sr, pr)
    m.copyArrayToPdataVec3(sv, pv)
    gr, gvec = s.create(m.RealGrid), s.create(m.VecGrid)
    m.mapPartsToGrid(flags=flags, target=gr, parts=pp, source=pr)
    m.mapPartsToGridVec3(flags=flags, target=gvec, parts=pp, source=pv)
    r_ref = np.zeros(f.shape, np.float32)
    v_ref = np.zeros(f.shape + (3,), np.float32)
    og.map_parts_to_grid(f, r_ref, pos, flag, sr)
    og.map_parts_to_grid(f, v_ref, pos, flag, sv)
    assert np.array_equal(gr.numpy(), r_ref)
    assert np.array_equal(gvec.numpy(), v_ref)
    # and back
    tr = pp.create(m.PdataReal)
    tv = pp.create(m.PdataVec3)
    m.mapGridToParts(source=gr, parts=pp, target=tr)
    m.mapGridToPartsVec3(source=gvec, parts=pp, target=tv)
    br = np.zeros(count, np.float32)
    bv = np.zeros((count, 3), np.float32)
    og.map_grid_to_parts(r_ref, pos, flag, br)
    og.map_grid_to_parts(v_ref, pos, flag, bv)
    assert np.array_equal(tr.numpy(), br)
    assert np.array_equal(tv.numpy(), bv)


def test_particle_system_records_and_errors():
    n = 10
    s, flags = _scene(n, 3)
    pp = s.create(m.BasicParticleSystem)
    for i in range(5):
        pp.addParticle(m.vec3(i + 0.5, 1.5, 2.5))
    d = pp.create(m.PdataReal)
    assert pp.pySize() == 5 and d.numpy().shape == (5,)
    m.copyArrayToPdataReal(np.arange(5, dtype=np.float32), d)
    pp.addParticle(m.vec3(9.5, 9.5, 9.5))  # data grows by a zero
    pos, fl = pp.positions()
    assert pos.shape == (6, 3) and np.array_equal(d.numpy(), np.array([0, 1, 2, 3, 4, 0], np.float32))
    pp.kill(2)
    assert pp.positions()[1][2] == m.ParticleDelete
    # a grid of another solver is refused
    s2, flags2 = _scene(n + 2, 3)
    v2 = s2.create(m.MACGrid)
    pv = pp.create(m.PdataVec3)
    with pytest.raises(m.MantaError):
        m.mapPartsToMAC(flags=flags2, vel=v2, velOld=v2, parts=pp, partVel=pv)
