"""Pin the CPU oracle against the reference's own outputs (tests/golden/).

The golden vectors come from the reference mantaflow float executable run
with one OpenMP thread (tests/golden/make_golden.py), so every reduction is
serial there and in the oracle: the comparisons below are bit-exact unless a
tolerance is written next to them.
"""
import numpy as np
import pytest

from oracle import oracle as og
from tests.conftest import golden_path


def load(name):
    return np.load(golden_path(name), allow_pickle=False)


def assert_same(got, want, what, atol=0.0):
    got = np.asarray(got)
    want = np.asarray(want)
    assert got.shape == want.shape, what
    if atol == 0.0:
        bad = np.count_nonzero(got != want)
        assert bad == 0, "%s: %d cells differ, max %g" % (what, bad, np.max(np.abs(got - want)))
    else:
        diff = np.max(np.abs(got.astype(np.float64) - want))
        assert diff <= atol, "%s: max diff %g > %g" % (what, diff, atol)


@pytest.mark.parametrize("tag", ["3d", "2d"])
def test_advection_bitexact(tag):
    g = load("advect_" + tag)
    flags, vel, dens, vec3, dt = g["flags"], g["vel"], g["dens"], g["vec3"], float(g["dt"])
    for name_kind, meta in zip(g["names"], g["meta"]):
        name, kind = str(name_kind).split(":")
        order, clamp, ospace, otrace, strength = meta
        v = vel.copy()
        if kind == "real":
            tgt, k = dens.copy(), og.KIND_REAL
        elif kind == "vec3":
            tgt, k = vec3.copy(), og.KIND_VEC3
        else:
            tgt, k = v, og.KIND_MAC
        og.advect_semi_lagrange(flags, v, tgt, k, order=int(order), strength=float(strength),
                                orderSpace=int(ospace), clampMode=int(clamp), orderTrace=int(otrace), dt=dt)
        assert_same(tgt, g[name], "advect %s %s" % (tag, name))


@pytest.mark.parametrize("tag", ["3d", "2d"])
def test_forces_bitexact(tag):
    g = load("forces_" + tag)
    flags, vel, obvel, dens, dt = g["flags"], g["vel"], g["obvel"], g["dens"], float(g["dt"])
    v = vel.copy(); og.set_wall_bcs(flags, v); assert_same(v, g["wall"], "setWallBcs")
    v = vel.copy(); og.set_wall_bcs(flags, v, obvel); assert_same(v, g["wall_obvel"], "setWallBcs obvel")
    v = vel.copy(); og.add_buoyancy(flags, dens, v, (0, -4e-3, 0), dt=dt); assert_same(v, g["buoy"], "addBuoyancy")
    v = vel.copy(); og.add_buoyancy(flags, dens, v, (1e-3, -6e-3, 2e-3), coefficient=0.7, scale=False, dt=dt)
    assert_same(v, g["buoy_noscale"], "addBuoyancy noscale")
    v = vel.copy(); og.add_gravity(flags, v, (0, -1e-3, 0), dt=dt); assert_same(v, g["grav"], "addGravity")
    v = vel.copy(); og.add_gravity(flags, v, (2e-3, -1e-3, 5e-4), scale=False, dt=dt)
    assert_same(v, g["grav_noscale"], "addGravity noscale")


PC = {"mic": og.PC_MIC, "mgdyn": og.PC_MG_DYNAMIC, "mgstat": og.PC_MG_STATIC}


def _pressure_kwargs(name):
    kw = {}
    base = name.replace("gf_", "")
    for key, pc in PC.items():
        if base.startswith(key):
            kw["preconditioner"] = pc
    if "acc1e5" in name:
        kw["cgAccuracy"] = 1e-5
    if "l2" in name:
        kw["useL2Norm"] = True
        kw["cgAccuracy"] = 1e-6
    if "compat" in name:
        kw["enforceCompatibility"] = True
    if "closed_fix" in name:
        kw["zeroPressureFixing"] = True
        kw["cgAccuracy"] = 1e-4
    if name == "mgstat_b":
        kw["cgAccuracy"] = 1e-4
    return kw


@pytest.mark.parametrize("tag", ["3d", "2d"])
def test_pressure_bitexact(tag):
    g = load("pressure_" + tag)
    names = [str(n) for n in g["names"]]
    cache = og.MGCache()
    for idx, name in enumerate(names):
        if name.startswith("gf_"):
            flags, phi = g["flags_liquid"], g["phi"]
            if name == "gf_mic":
                cache.release()  # releaseMG between the two blocks of the generator
        else:
            flags, phi = (g["flags_closed"] if "closed" in name else g["flags_smoke"]), None
        vel = g["vel"].copy()
        if name == "mgstat_b":
            vel = (g["vel"] * 0.5 + 0.1).astype(np.float32)
        p = np.zeros(flags.shape, np.float32)
        rhs = np.zeros(flags.shape, np.float32)
        it, res, _ = og.solve_pressure(flags, vel, p, phi=phi, mg_cache=cache, retRhs=rhs, **_pressure_kwargs(name))
        assert it == g["iters"][idx], "%s %s: iterations %d vs reference %d" % (tag, name, it, g["iters"][idx])
        assert_same(rhs, g["rhs_" + name], "%s rhs %s" % (tag, name))
        assert_same(p, g["p_" + name], "%s pressure %s" % (tag, name))
        assert_same(vel, g["v_" + name], "%s vel %s" % (tag, name))
    cache.release()
    # PcNone is rejected with the reference's own message
    with pytest.raises(RuntimeError) as e:
        og.solve_pressure(g["flags_smoke"], g["vel"].copy(), np.zeros(g["flags_smoke"].shape, np.float32),
                          preconditioner=og.PC_NONE)
    assert "Invalid method specified" in str(e.value)
    assert "Invalid method specified" in str(g["none_error"])


@pytest.mark.parametrize("tag", ["3d", "2d"])
def test_extrapolate_bitexact(tag):
    g = load("extrap_" + tag)
    v = g["vel"].copy(); og.extrapolate_mac_simple(g["flags"], v, 4); assert_same(v, g["ext4"], "extrap 4")
    v = g["vel"].copy(); og.extrapolate_mac_simple(g["flags"], v, 2, intoObs=True)
    assert_same(v, g["ext2_obs"], "extrap 2 intoObs")


def test_setup_bitexact():
    g = load("setup_3d")
    nx, ny, nz = [int(x) for x in g["size"]]
    f = np.zeros((nz, ny, nx), np.int32)
    og.init_domain(f, 0)
    assert_same(f, g["flags_init"], "initDomain")
    og.fill_grid(f)
    assert_same(f, g["flags_fill"], "fillGrid")
    og.set_open_bound(f, 0, "Y")
    assert_same(f, g["flags_open"], "setOpenBound")
    og.init_domain(f, 1, wall="xXyY", outflow="zZ")
    assert_same(f, g["flags_init_bw1"], "initDomain bw1")
    n = nx
    gs = np.array([nx, ny, nz], np.float32)
    mask = np.zeros((nz, ny, nx), np.float32)
    og.cylinder_apply(mask, gs * np.float32([0.5, 0.1, 0.5]), np.float32(n * 0.14), gs * np.float32([0, 0.02, 0]), 1.0)
    assert_same(mask, g["cyl_mask"], "cylinder mask")
    phi = np.zeros((nz, ny, nx), np.float32)
    og.box_sdf(phi, (0, 0, 0), (np.float32(n * 0.4), np.float32(ny * 0.6), np.float32(nz)))
    assert_same(phi, g["box_phi"], "box sdf")
    og.init_domain(f, 0)
    og.update_from_levelset(f, phi)
    assert_same(f, g["flags_lvl"], "updateFromLevelset")


def _plume_run(g, steps):
    flags = g["flags"]
    mask = g["mask"]
    n = flags.shape[0]
    pc = int(g["pc"])
    rng = np.random.default_rng(int(g["seed"]))
    dens = np.zeros((n, n, n), np.float32)
    vel = np.zeros((n, n, n, 3), np.float32)
    pres = np.zeros((n, n, n), np.float32)
    cache = og.MGCache()
    for t in range(steps):
        a = (rng.random((n, n, n), dtype=np.float32) * mask).astype(np.float32)
        og.join_real(dens, a)
        og.advect_semi_lagrange(flags, vel, dens, og.KIND_REAL, order=2, clampMode=2)
        og.advect_semi_lagrange(flags, vel, vel, og.KIND_MAC, order=2, clampMode=2)
        og.set_wall_bcs(flags, vel)
        og.add_buoyancy(flags, dens, vel, (0, -4e-3, 0))
        it, _, _ = og.solve_pressure(flags, vel, pres, cgAccuracy=1e-3, preconditioner=pc, mg_cache=cache)
        yield t, it, dens, vel, pres
    cache.release()


@pytest.mark.parametrize("case", ["plume_mic24", "plume_mgstat24"])
def test_plume_steps_bitexact(case):
    g = load(case)
    for t, it, dens, vel, pres in _plume_run(g, len(g["iters"])):
        assert it == g["iters"][t], "step %d iterations %d vs %d" % (t, it, g["iters"][t])
        assert_same(dens, g["density"][t], "%s step %d density" % (case, t))
        assert_same(vel, g["vel"][t], "%s step %d vel" % (case, t))
        assert_same(pres, g["pressure"][t], "%s step %d pressure" % (case, t))


def test_dam_steps_bitexact():
    g = load("dam_24")
    flags = g["flags0"].copy()
    phi = g["phi0"].copy()
    n = flags.shape[0]
    vel = np.zeros((n, n, n, 3), np.float32)
    pres = np.zeros((n, n, n), np.float32)
    for t in range(len(g["iters"])):
        og.extrapolate_mac_simple(flags, vel, 4)
        og.advect_semi_lagrange(flags, vel, phi, og.KIND_REAL, order=1)
        og.update_from_levelset(flags, phi)
        og.advect_semi_lagrange(flags, vel, vel, og.KIND_MAC, order=1)
        og.add_gravity(flags, vel, (0, -1e-3, 0))
        og.set_wall_bcs(flags, vel)
        it, _, _ = og.solve_pressure(flags, vel, pres, phi=phi)
        og.set_wall_bcs(flags, vel)
        assert it == g["iters"][t], "step %d iterations %d vs %d" % (t, it, g["iters"][t])
        assert_same(flags, g["flags"][t], "dam step %d flags" % t)
        assert_same(phi, g["phi"][t], "dam step %d phi" % t)
        assert_same(vel, g["vel"][t], "dam step %d vel" % t)
        assert_same(pres, g["pressure"][t], "dam step %d pressure" % t)
