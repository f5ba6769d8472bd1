#
# Golden-vector generator: runs INSIDE the reference mantaflow executable.
#
#   OMP_NUM_THREADS=1 MANTA_DISABLE_UI=1 <manta> tests/golden/make_golden.py <outdir>
#
# (tests/golden/gen_golden.sh does exactly that.)  One OpenMP thread makes
# every reduction in the reference serial, so the CPU oracle in oracle/ must
# reproduce these outputs bit for bit.  Inputs are seeded numpy arrays in the
# reference layout ((nz, ny, nx[, 3]) float32 / int32); each case stores its
# inputs and the reference's outputs in one compressed .npz file.
#
import os
import re
import sys
import tempfile

import numpy as np
from manta import *

OUT = sys.argv[1] if len(sys.argv) > 1 else "."
os.makedirs(OUT, exist_ok=True)
setDebugLevel(0)

F_FLUID, F_OBS, F_EMPTY, F_OUT, F_STICK = 1, 2, 4, 16, 64


def solver(nx, ny, nz, dt):
    dim = 3 if nz > 1 else 2
    s = Solver(name="g%dx%dx%d" % (nx, ny, nz), gridSize=vec3(nx, ny, nz), dim=dim)
    s.timestep = dt
    return s


def arr_real(g):
    a = np.zeros((g.getSizeZ(), g.getSizeY(), g.getSizeX()), np.float32)
    copyGridToArrayReal(g, a)
    return a


def arr_mac(g):
    a = np.zeros((g.getSizeZ(), g.getSizeY(), g.getSizeX(), 3), np.float32)
    copyGridToArrayMAC(g, a)
    return a


def arr_vec3(g):
    a = np.zeros((g.getSizeZ(), g.getSizeY(), g.getSizeX(), 3), np.float32)
    copyGridToArrayVec3(g, a)
    return a


def arr_flags(g):
    a = np.zeros((g.getSizeZ(), g.getSizeY(), g.getSizeX()), np.int32)
    copyGridToArrayFlag(g, a)
    return a


def smoke_flags(nx, ny, nz, rng, obstacle=True, stick=False):
    """walls, open top (outflow|empty), an obstacle block, fluid elsewhere"""
    f = np.full((nz, ny, nx), F_FLUID, np.int32)
    f[:, :, 0] = f[:, :, -1] = F_OBS
    f[:, 0, :] = F_OBS
    f[:, -1, :] = F_OUT | F_EMPTY
    f[:, -1, 0] = f[:, -1, -1] = F_OBS
    if nz > 1:
        f[0, :, :] = f[-1, :, :] = F_OBS
        f[0, -1, :] = f[-1, -1, :] = F_OBS
    if obstacle:
        z0 = nz // 3 if nz > 1 else 0
        z1 = (2 * nz) // 3 if nz > 1 else 1
        f[z0:z1, ny // 3:ny // 2, nx // 3:nx // 2] = F_OBS
    if stick:
        f[z0:z1, ny // 3:ny // 2, nx // 2] = F_OBS | F_STICK
    return f


def liquid_flags(nx, ny, nz, level):
    """closed box, fluid below `level` rows, empty above"""
    f = np.full((nz, ny, nx), F_EMPTY, np.int32)
    f[:, :level, :] = F_FLUID
    f[:, :, 0] = f[:, :, -1] = F_OBS
    f[:, 0, :] = f[:, -1, :] = F_OBS
    if nz > 1:
        f[0] = f[-1] = F_OBS
    return f


class Capture:
    """capture the C++ std::cout of a plugin call (fd 1)"""

    def __enter__(self):
        sys.stdout.flush()
        self.tmp = tempfile.TemporaryFile(mode="w+b")
        self.saved = os.dup(1)
        os.dup2(self.tmp.fileno(), 1)
        return self

    def __exit__(self, *a):
        sys.stdout.flush()
        os.dup2(self.saved, 1)
        os.close(self.saved)
        self.tmp.seek(0)
        self.text = self.tmp.read().decode(errors="replace")
        self.tmp.close()


def cg_stats(text):
    m = re.findall(r"Iterations:(\d+), residual:([0-9eE.+\-naif]+)", text)
    if not m:
        return -1, float("nan")
    return int(m[-1][0]), float(m[-1][1])


def save(name, **kw):
    np.savez_compressed(os.path.join(OUT, name + ".npz"), **kw)
    print("wrote", name, flush=True)


# ---------------------------------------------------------------- advection
def advection_cases(nx, ny, nz, tag, seed):
    rng = np.random.default_rng(seed)
    dt = 1.2
    s = solver(nx, ny, nz, dt)
    flags = s.create(FlagGrid)
    vel = s.create(MACGrid)
    dens = s.create(RealGrid)
    v3g = s.create(VecGrid)
    f = smoke_flags(nx, ny, nz, rng)
    v = (rng.random((nz, ny, nx, 3), dtype=np.float32) * 3.0 - 1.5).astype(np.float32)
    if nz == 1:
        v[..., 2] = 0
    d = rng.random((nz, ny, nx), dtype=np.float32)
    w = (rng.random((nz, ny, nx, 3), dtype=np.float32) * 2.0 - 1.0).astype(np.float32)
    if nz == 1:
        w[..., 2] = 0
    copyArrayToGridFlag(f, flags)
    cases = [
        # (name, target, order, clampMode, orderSpace, orderTrace, strength)
        ("real_o1", "real", 1, 2, 1, 1, 1.0),
        ("real_o2c1", "real", 2, 1, 1, 1, 1.0),
        ("real_o2c2", "real", 2, 2, 1, 1, 1.0),
        ("real_o2c2_s07", "real", 2, 2, 1, 1, 0.7),
        ("real_o1_trace2", "real", 1, 2, 1, 2, 1.0),
        ("real_o2_trace2", "real", 2, 2, 1, 2, 1.0),
        ("real_o1_cubic", "real", 1, 2, 2, 1, 1.0),
        ("vec3_o2c2", "vec3", 2, 2, 1, 1, 1.0),
        ("vec3_o2c1", "vec3", 2, 1, 1, 1, 1.0),
        ("mac_o1", "mac", 1, 2, 1, 1, 1.0),
        ("mac_o2c1", "mac", 2, 1, 1, 1, 1.0),
        ("mac_o2c2", "mac", 2, 2, 1, 1, 1.0),
        ("mac_o2_trace2", "mac", 2, 2, 1, 2, 1.0),
    ]
    out = {}
    for (name, tgt, order, cm, osp, otr, stren) in cases:
        copyArrayToGridMAC(v, vel)
        copyArrayToGridReal(d, dens)
        copyArrayToGridVec3(w, v3g)
        if tgt == "real":
            advectSemiLagrange(flags=flags, vel=vel, grid=dens, order=order, clampMode=cm, orderSpace=osp,
                               orderTrace=otr, strength=stren)
            out[name] = arr_real(dens)
        elif tgt == "vec3":
            advectSemiLagrange(flags=flags, vel=vel, grid=v3g, order=order, clampMode=cm, orderSpace=osp,
                               orderTrace=otr, strength=stren)
            out[name] = arr_vec3(v3g)
        else:
            advectSemiLagrange(flags=flags, vel=vel, grid=vel, order=order, clampMode=cm, orderSpace=osp,
                               orderTrace=otr, strength=stren)
            out[name] = arr_mac(vel)
    meta = np.array([[c[2], c[3], c[4], c[5], c[6]] for c in cases], np.float32)
    names = np.array([c[0] + ":" + c[1] for c in cases])
    save("advect_" + tag, flags=f, vel=v, dens=d, vec3=w, dt=np.float32(dt), meta=meta, names=names, **out)


# ------------------------------------------------------- forces and walls
def force_cases(nx, ny, nz, tag, seed):
    rng = np.random.default_rng(seed)
    dt = 0.8
    s = solver(nx, ny, nz, dt)
    flags = s.create(FlagGrid)
    vel = s.create(MACGrid)
    obv = s.create(MACGrid)
    dens = s.create(RealGrid)
    f = smoke_flags(nx, ny, nz, rng, stick=True)
    # a few empty cells inside the fluid region for the gravity face rules
    f[(rng.random(f.shape) < 0.05) & (f == F_FLUID)] = F_EMPTY
    v = (rng.random((nz, ny, nx, 3), dtype=np.float32) * 2.0 - 1.0).astype(np.float32)
    ov = (rng.random((nz, ny, nx, 3), dtype=np.float32) * 0.2 - 0.1).astype(np.float32)
    d = rng.random((nz, ny, nx), dtype=np.float32)
    copyArrayToGridFlag(f, flags)
    copyArrayToGridReal(d, dens)
    out = {}
    copyArrayToGridMAC(v, vel)
    setWallBcs(flags=flags, vel=vel)
    out["wall"] = arr_mac(vel)
    copyArrayToGridMAC(v, vel)
    copyArrayToGridMAC(ov, obv)
    setWallBcs(flags=flags, vel=vel, obvel=obv)
    out["wall_obvel"] = arr_mac(vel)
    copyArrayToGridMAC(v, vel)
    addBuoyancy(flags=flags, density=dens, vel=vel, gravity=vec3(0, -4e-3, 0))
    out["buoy"] = arr_mac(vel)
    copyArrayToGridMAC(v, vel)
    addBuoyancy(flags=flags, density=dens, vel=vel, gravity=vec3(1e-3, -6e-3, 2e-3), coefficient=0.7, scale=False)
    out["buoy_noscale"] = arr_mac(vel)
    copyArrayToGridMAC(v, vel)
    addGravity(flags=flags, vel=vel, gravity=vec3(0, -1e-3, 0))
    out["grav"] = arr_mac(vel)
    copyArrayToGridMAC(v, vel)
    addGravity(flags=flags, vel=vel, gravity=vec3(2e-3, -1e-3, 5e-4), scale=False)
    out["grav_noscale"] = arr_mac(vel)
    save("forces_" + tag, flags=f, vel=v, obvel=ov, dens=d, dt=np.float32(dt), **out)


# ------------------------------------------------------------- pressure
def pressure_cases(nx, ny, nz, tag, seed):
    rng = np.random.default_rng(seed)
    s = solver(nx, ny, nz, 1.0)
    flags = s.create(FlagGrid)
    vel = s.create(MACGrid)
    pres = s.create(RealGrid)
    rhs = s.create(RealGrid)
    phi = s.create(LevelsetGrid)
    f_smoke = smoke_flags(nx, ny, nz, rng)
    f_closed = smoke_flags(nx, ny, nz, rng)
    f_closed[f_closed == (F_OUT | F_EMPTY)] = F_OBS
    v = (rng.random((nz, ny, nx, 3), dtype=np.float32) * 2.0 - 1.0).astype(np.float32)
    if nz == 1:
        v[..., 2] = 0
    out = {}
    stats = []
    runs = [
        # name, flags, kwargs
        ("mic", f_smoke, dict(preconditioner=PcMIC)),
        ("mic_acc1e5", f_smoke, dict(preconditioner=PcMIC, cgAccuracy=1e-5)),
        ("mic_l2", f_smoke, dict(preconditioner=PcMIC, useL2Norm=True, cgAccuracy=1e-6)),
        ("mic_compat", f_smoke, dict(preconditioner=PcMIC, enforceCompatibility=True)),
        ("mgdyn", f_smoke, dict(preconditioner=PcMGDynamic)),
        ("mgdyn_closed_fix", f_closed, dict(preconditioner=PcMGDynamic, zeroPressureFixing=True, cgAccuracy=1e-4)),
        ("mic_closed_fix", f_closed, dict(preconditioner=PcMIC, zeroPressureFixing=True, cgAccuracy=1e-4)),
        ("mgstat_a", f_smoke, dict(preconditioner=PcMGStatic)),
        ("mgstat_b", f_smoke, dict(preconditioner=PcMGStatic, cgAccuracy=1e-4)),
    ]
    for (name, fl, kw) in runs:
        copyArrayToGridFlag(fl, flags)
        copyArrayToGridMAC(v, vel)
        if name == "mgstat_b":
            copyArrayToGridMAC((v * 0.5 + 0.1).astype(np.float32), vel)
        pres.setConst(0.)
        setDebugLevel(2)
        with Capture() as c:
            solvePressure(flags=flags, vel=vel, pressure=pres, retRhs=rhs, **kw)
        setDebugLevel(0)
        it, res = cg_stats(c.text)
        stats.append((it, res))
        out["p_" + name] = arr_real(pres)
        out["v_" + name] = arr_mac(vel)
        out["rhs_" + name] = arr_real(rhs)
    releaseMG(s)
    # ghost fluid: liquid below 60% height, phi from a box levelset
    fl = liquid_flags(nx, ny, nz, int(ny * 0.6))
    box = Box(parent=s, p0=vec3(0, 0, 0), p1=vec3(nx, ny * 0.6 - 0.3, nz))
    phiv = box.computeLevelset()
    phi.copyFrom(phiv)
    ph = arr_real(phi)
    for (name, kw) in [("gf_mic", dict(preconditioner=PcMIC)), ("gf_mgdyn", dict(preconditioner=PcMGDynamic))]:
        copyArrayToGridFlag(fl, flags)
        copyArrayToGridMAC(v, vel)
        pres.setConst(0.)
        setDebugLevel(2)
        with Capture() as c:
            solvePressure(flags=flags, vel=vel, pressure=pres, phi=phi, retRhs=rhs, **kw)
        setDebugLevel(0)
        it, res = cg_stats(c.text)
        stats.append((it, res))
        out["p_" + name] = arr_real(pres)
        out["v_" + name] = arr_mac(vel)
        out["rhs_" + name] = arr_real(rhs)
        runs.append((name, fl, kw))
    releaseMG(s)
    # PcNone is rejected by the reference (GridCg::setICPreconditioner asserts)
    copyArrayToGridFlag(f_smoke, flags)
    try:
        solvePressure(flags=flags, vel=vel, pressure=pres, preconditioner=PcNone)
        none_error = ""
    except RuntimeError as e:
        none_error = str(e).splitlines()[0]
    names = np.array([r[0] for r in runs])
    save("pressure_" + tag, flags_smoke=f_smoke, flags_closed=f_closed, flags_liquid=fl, phi=ph, vel=v,
         names=names, none_error=np.array(none_error), iters=np.array([a for a, b in stats], np.int32),
         resnorm=np.array([b for a, b in stats], np.float64), **out)


# --------------------------------------------------- extrapolateMACSimple
def extrap_cases(nx, ny, nz, tag, seed):
    rng = np.random.default_rng(seed)
    s = solver(nx, ny, nz, 1.0)
    flags = s.create(FlagGrid)
    vel = s.create(MACGrid)
    fl = liquid_flags(nx, ny, nz, int(ny * 0.45))
    v = (rng.random((nz, ny, nx, 3), dtype=np.float32) * 2.0 - 1.0).astype(np.float32)
    if nz == 1:
        v[..., 2] = 0
    copyArrayToGridFlag(fl, flags)
    out = {}
    copyArrayToGridMAC(v, vel)
    extrapolateMACSimple(flags=flags, vel=vel, distance=4)
    out["ext4"] = arr_mac(vel)
    copyArrayToGridMAC(v, vel)
    extrapolateMACSimple(flags=flags, vel=vel, distance=2, intoObs=True)
    out["ext2_obs"] = arr_mac(vel)
    save("extrap_" + tag, flags=fl, vel=v, **out)


# ------------------------------------------------------------ scene setup
def setup_cases(n, tag):
    s = solver(n, n + 4, n - 2, 1.0)
    gs = vec3(n, n + 4, n - 2)
    flags = s.create(FlagGrid)
    mask = s.create(RealGrid)
    phi = s.create(LevelsetGrid)
    out = {}
    flags.initDomain(boundaryWidth=0)
    out["flags_init"] = arr_flags(flags)
    flags.fillGrid()
    out["flags_fill"] = arr_flags(flags)
    setOpenBound(flags, 0, 'Y', FlagOutflow | FlagEmpty)
    out["flags_open"] = arr_flags(flags)
    flags.initDomain(boundaryWidth=1, wall="xXyY", outflow="zZ")
    out["flags_init_bw1"] = arr_flags(flags)
    src = s.create(Cylinder, center=gs * vec3(0.5, 0.1, 0.5), radius=n * 0.14, z=gs * vec3(0, 0.02, 0))
    src.applyToGrid(grid=mask, value=1.0)
    out["cyl_mask"] = arr_real(mask)
    box = s.create(Box, p0=vec3(0, 0, 0), p1=vec3(n * 0.4, (n + 4) * 0.6, n - 2))
    phi.copyFrom(box.computeLevelset())
    out["box_phi"] = arr_real(phi)
    flags.initDomain(boundaryWidth=0)
    flags.updateFromLevelset(phi)
    out["flags_lvl"] = arr_flags(flags)
    save("setup_" + tag, size=np.array([n, n + 4, n - 2], np.int32), **out)


# ------------------------------------------------------ full plume steps
def plume_steps(n, steps, tag, pc, seed):
    gs = vec3(n, n, n)
    s = Solver(name="plume%d" % n, gridSize=gs, dim=3)
    s.timestep = 1.0
    flags = s.create(FlagGrid)
    vel = s.create(MACGrid)
    density = s.create(RealGrid)
    pressure = s.create(RealGrid)
    noise = s.create(RealGrid)
    mask = s.create(RealGrid)
    flags.initDomain(boundaryWidth=0)
    flags.fillGrid()
    setOpenBound(flags, 0, 'Y', FlagOutflow | FlagEmpty)
    src = s.create(Cylinder, center=gs * vec3(0.5, 0.1, 0.5), radius=n * 0.14, z=gs * vec3(0, 0.02, 0))
    src.applyToGrid(grid=mask, value=1.0)
    m = arr_real(mask)
    rng = np.random.default_rng(seed)
    dens_h, vel_h, pres_h, its = [], [], [], []
    for t in range(steps):
        a = (rng.random((n, n, n), dtype=np.float32) * m).astype(np.float32)
        copyArrayToGridReal(a, noise)
        density.join(noise)
        advectSemiLagrange(flags=flags, vel=vel, grid=density, order=2, clampMode=2)
        advectSemiLagrange(flags=flags, vel=vel, grid=vel, order=2, clampMode=2)
        setWallBcs(flags=flags, vel=vel)
        addBuoyancy(density=density, vel=vel, gravity=vec3(0, -4e-3, 0), flags=flags)
        setDebugLevel(2)
        with Capture() as c:
            solvePressure(flags=flags, vel=vel, pressure=pressure, cgAccuracy=1e-3, preconditioner=pc)
        setDebugLevel(0)
        its.append(cg_stats(c.text)[0])
        dens_h.append(arr_real(density))
        vel_h.append(arr_mac(vel))
        pres_h.append(arr_real(pressure))
        s.step()
    releaseMG(s)
    save("plume_" + tag, flags=arr_flags(flags), mask=m, seed=np.int64(seed), density=np.stack(dens_h),
         vel=np.stack(vel_h), pressure=np.stack(pres_h), iters=np.array(its, np.int32), pc=np.int32(pc))


# -------------------------------------------------------- dam break steps
def dam_steps(n, steps, tag):
    gs = vec3(n, n, n)
    s = Solver(name="dam%d" % n, gridSize=gs, dim=3)
    s.timestep = 1.0
    flags = s.create(FlagGrid)
    vel = s.create(MACGrid)
    pressure = s.create(RealGrid)
    phi = s.create(LevelsetGrid)
    flags.initDomain(boundaryWidth=0)
    box = s.create(Box, p0=vec3(0, 0, 0), p1=vec3(0.4 * n, 0.6 * n, n))
    phi.copyFrom(box.computeLevelset())
    flags.updateFromLevelset(phi)
    phi0 = arr_real(phi)
    flags0 = arr_flags(flags)
    phi_h, vel_h, pres_h, fl_h, its = [], [], [], [], []
    for t in range(steps):
        extrapolateMACSimple(flags=flags, vel=vel, distance=4)
        advectSemiLagrange(flags=flags, vel=vel, grid=phi, order=1)
        flags.updateFromLevelset(phi)
        advectSemiLagrange(flags=flags, vel=vel, grid=vel, order=1)
        addGravity(flags=flags, vel=vel, gravity=vec3(0, -1e-3, 0))
        setWallBcs(flags=flags, vel=vel)
        setDebugLevel(2)
        with Capture() as c:
            solvePressure(flags=flags, vel=vel, pressure=pressure, phi=phi)
        setDebugLevel(0)
        its.append(cg_stats(c.text)[0])
        setWallBcs(flags=flags, vel=vel)
        phi_h.append(arr_real(phi))
        vel_h.append(arr_mac(vel))
        pres_h.append(arr_real(pressure))
        fl_h.append(arr_flags(flags))
        s.step()
    save("dam_" + tag, flags0=flags0, phi0=phi0, phi=np.stack(phi_h), vel=np.stack(vel_h),
         pressure=np.stack(pres_h), flags=np.stack(fl_h), iters=np.array(its, np.int32))


advection_cases(20, 18, 16, "3d", 11)
advection_cases(26, 21, 1, "2d", 12)
force_cases(18, 16, 14, "3d", 21)
force_cases(22, 19, 1, "2d", 22)
pressure_cases(24, 20, 18, "3d", 31)
pressure_cases(30, 26, 1, "2d", 32)
extrap_cases(18, 16, 14, "3d", 41)
extrap_cases(22, 19, 1, "2d", 42)
setup_cases(20, "3d")
plume_steps(24, 8, "mic24", 1, 1234)
plume_steps(24, 4, "mgstat24", 3, 99)
dam_steps(24, 6, "24")
print("golden done", flush=True)
