"""The FP64 oracle (the restatement compiled as the reference's double
build, Real = double) against the reference's own float outputs
(tests/golden/): run on the same inputs widened to double, it must agree
with the float executable to within float rounding -- the same algorithm in
a wider type.  This cross-checks the FP64 oracle of the precision tests; it
does not pin it to the reference's double executable, whose outputs are not
among the goldens.  The tolerances are written beside each comparison.
"""
import numpy as np
import pytest

from oracle import oracle as og
from tests.conftest import golden_path
from tests.test_oracle_golden import _pressure_kwargs


def load(name):
    return np.load(golden_path(name), allow_pickle=False)


def f64(a):
    return np.asarray(a).astype(np.float64)


@pytest.mark.parametrize("tag", ["3d", "2d"])
def test_fp64_advection_within_float_rounding(tag):
    g = load("advect_" + tag)
    flags, vel, dens, vec3, dt = g["flags"], f64(g["vel"]), f64(g["dens"]), f64(g["vec3"]), float(g["dt"])
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
        want = f64(g[name])
        # float rounding of the reference's sweeps: a few units of 2^-24 relative
        rel = np.max(np.abs(tgt - want)) / max(np.max(np.abs(want)), 1e-30)
        assert rel <= 1e-5, "advect %s %s: relative difference %g" % (tag, name, rel)


@pytest.mark.parametrize("tag", ["3d", "2d"])
def test_fp64_forces_within_float_rounding(tag):
    g = load("forces_" + tag)
    flags, vel, obvel, dens, dt = g["flags"], f64(g["vel"]), f64(g["obvel"]), f64(g["dens"]), float(g["dt"])
    got = {}
    v = vel.copy(); og.set_wall_bcs(flags, v); got["wall"] = v
    v = vel.copy(); og.set_wall_bcs(flags, v, obvel); got["wall_obvel"] = v
    v = vel.copy(); og.add_buoyancy(flags, dens, v, (0, -4e-3, 0), dt=dt); got["buoy"] = v
    v = vel.copy(); og.add_buoyancy(flags, dens, v, (1e-3, -6e-3, 2e-3), coefficient=0.7, scale=False, dt=dt)
    got["buoy_noscale"] = v
    v = vel.copy(); og.add_gravity(flags, v, (0, -1e-3, 0), dt=dt); got["grav"] = v
    v = vel.copy(); og.add_gravity(flags, v, (2e-3, -1e-3, 5e-4), scale=False, dt=dt); got["grav_noscale"] = v
    for key, v in got.items():
        diff = np.max(np.abs(v - f64(g[key])))
        # one float rounding of velocities of order 1
        assert diff <= 1e-6, "%s %s: max difference %g" % (tag, key, diff)


@pytest.mark.parametrize("tag", ["3d", "2d"])
def test_fp64_pressure_within_solver_tolerance(tag):
    g = load("pressure_" + tag)
    names = [str(n) for n in g["names"]]
    cache = og.MGCache()
    for idx, name in enumerate(names):
        if name.startswith("gf_"):
            flags, phi = g["flags_liquid"], f64(g["phi"])
            if name == "gf_mic":
                cache.release()
        else:
            flags, phi = (g["flags_closed"] if "closed" in name else g["flags_smoke"]), None
        vel = f64(g["vel"])
        if name == "mgstat_b":
            vel = f64((g["vel"] * 0.5 + 0.1).astype(np.float32))
        p = np.zeros(flags.shape, np.float64)
        rhs = np.zeros(flags.shape, np.float64)
        it, _, _ = og.solve_pressure(flags, vel, p, phi=phi, mg_cache=cache, retRhs=rhs, **_pressure_kwargs(name))
        # the right-hand side is one divergence per cell: float rounding
        assert np.max(np.abs(rhs - f64(g["rhs_" + name]))) <= 1e-6, "%s rhs %s" % (tag, name)
        # the CG in double and in float stop within two iterations of each
        # other and at the same accuracy: pressure and corrected velocity
        # agree to 1e-3 of their magnitude
        assert abs(it - int(g["iters"][idx])) <= 2, "%s %s: iterations %d vs %d" % (tag, name, it, g["iters"][idx])
        for key, got in (("p_", p), ("v_", vel)):
            want = f64(g[key + name])
            diff = np.max(np.abs(got - want))
            assert diff <= 1e-3 * np.max(np.abs(want)) + 1e-6, "%s %s%s: max difference %g" % (tag, key, name, diff)
    cache.release()


@pytest.mark.parametrize("case", ["plume_mic24", "plume_mgstat24"])
def test_fp64_plume_steps_within_float_rounding(case):
    """Whole plume steps (inflow, MacCormack advection, walls, buoyancy,
    pressure) in double against the float executable's steps: the same CG
    iteration counts and fields within float rounding of their magnitude."""
    g = load(case)
    flags, mask = g["flags"], g["mask"]
    n = flags.shape[0]
    rng = np.random.default_rng(int(g["seed"]))
    dens = np.zeros((n, n, n))
    vel = np.zeros((n, n, n, 3))
    pres = np.zeros((n, n, n))
    cache = og.MGCache()
    for t in range(len(g["iters"])):
        a = f64((rng.random((n, n, n), dtype=np.float32) * mask).astype(np.float32))
        og.join_real(dens, a)
        og.advect_semi_lagrange(flags, vel, dens, og.KIND_REAL, order=2, clampMode=2)
        og.advect_semi_lagrange(flags, vel, vel, og.KIND_MAC, order=2, clampMode=2)
        og.set_wall_bcs(flags, vel)
        og.add_buoyancy(flags, dens, vel, (0, -4e-3, 0))
        it, _, _ = og.solve_pressure(flags, vel, pres, cgAccuracy=1e-3, preconditioner=int(g["pc"]), mg_cache=cache)
        assert it == int(g["iters"][t]), "%s step %d: iterations %d vs %d" % (case, t, it, g["iters"][t])
        for name, got in (("density", dens), ("vel", vel), ("pressure", pres)):
            want = f64(g[name][t])
            diff = np.max(np.abs(got - want))
            # float rounding accumulated over a few steps: 1e-5 of the magnitude
            assert diff <= 1e-5 * max(np.max(np.abs(want)), 1.0), "%s step %d %s: %g" % (case, t, name, diff)
    cache.release()


def test_fp64_dam_steps_within_float_rounding():
    """Dam-break steps (extrapolation, order-1 advection of phi and velocity,
    flags from the levelset, gravity, walls, ghost-fluid pressure) in double
    against the float executable's: the same flags and CG iteration counts,
    fields within float rounding."""
    g = load("dam_24")
    flags = g["flags0"].copy()
    phi = f64(g["phi0"])
    n = flags.shape[0]
    vel = np.zeros((n, n, n, 3))
    pres = np.zeros((n, n, n))
    for t in range(len(g["iters"])):
        og.extrapolate_mac_simple(flags, vel, 4)
        og.advect_semi_lagrange(flags, vel, phi, og.KIND_REAL, order=1)
        og.update_from_levelset(flags, phi)
        og.advect_semi_lagrange(flags, vel, vel, og.KIND_MAC, order=1)
        og.add_gravity(flags, vel, (0, -1e-3, 0))
        og.set_wall_bcs(flags, vel)
        it, _, _ = og.solve_pressure(flags, vel, pres, phi=phi)
        og.set_wall_bcs(flags, vel)
        assert it == int(g["iters"][t]), "dam step %d: iterations %d vs %d" % (t, it, g["iters"][t])
        assert np.array_equal(flags, g["flags"][t]), "dam step %d flags" % t
        for name, got in (("phi", phi), ("vel", vel), ("pressure", pres)):
            want = f64(g[name][t])
            diff = np.max(np.abs(got - want))
            assert diff <= 1e-5 * max(np.max(np.abs(want)), 1.0), "dam step %d %s: %g" % (t, name, diff)
