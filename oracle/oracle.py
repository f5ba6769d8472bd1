"""ctypes front end of the CPU oracle (oracle/manta_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU legs as the parity checker / CPU baseline, never by the
product package.

Arrays use the reference's memory layout (source/grid.h:70): Real grids are
float32 arrays of shape (nz, ny, nx), Vec3/MAC grids (nz, ny, nx, 3), flag
grids int32 (nz, ny, nx).  All calls modify their outputs in place.
"""
import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libmantaoracle.so")

FLUID, OBSTACLE, EMPTY, INFLOW, OUTFLOW, OPEN, STICK = 1, 2, 4, 8, 16, 32, 64
KIND_REAL, KIND_VEC3, KIND_MAC = 0, 1, 2
PC_NONE, PC_MIC, PC_MG_DYNAMIC, PC_MG_STATIC = 0, 1, 2, 3


class Dims(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("is3d", C.c_int)]


class NoiseParams(C.Structure):
    _fields_ = [("gsInv", C.c_float * 3), ("seedOffset", C.c_float * 3), ("timeOffset", C.c_float),
                ("posScale", C.c_float * 3), ("posOffset", C.c_float * 3), ("valOffset", C.c_float),
                ("valScale", C.c_float), ("clampNeg", C.c_float), ("clampPos", C.c_float), ("clamp", C.c_int)]


def _structs(R):
    class PressureParams(C.Structure):
        _fields_ = [("cgAccuracy", R), ("gfClamp", R), ("cgMaxIterFac", R),
                    ("preconditioner", C.c_int), ("enforceCompatibility", C.c_int), ("useL2Norm", C.c_int),
                    ("zeroPressureFixing", C.c_int), ("surfTens", R)]

    class PressureResult(C.Structure):
        _fields_ = [("iterations", C.c_int), ("resNorm", R), ("fixPidx", C.c_int)]

    return PressureParams, PressureResult


# float build (the reference's float executable, pinned by the goldens) and
# double build (the reference's -DDOUBLEPRECISION=ON executable)
_PREC = {np.float32: ("libmantaoracle.so", C.c_float), np.float64: ("libmantaoracle64.so", C.c_double)}
_STRUCTS = {t: _structs(r) for t, (_, r) in _PREC.items()}
PressureParams, PressureResult = _STRUCTS[np.float32]


def build(force=False):
    """Compile the oracle with its Makefile (gcc/g++ only)."""
    src = os.path.getmtime(os.path.join(_HERE, "manta_oracle.cpp"))
    paths = [os.path.join(_HERE, "_build", f) for f, _ in _PREC.values()]
    if force or any(not os.path.exists(p) or os.path.getmtime(p) < src for p in paths):
        subprocess.run(["make", "-C", _HERE, "-s"], check=True)
    return _LIB_PATH


_libs = {}


def _prec(dtype):
    t = np.dtype(dtype).type
    if t not in _PREC:
        raise TypeError("oracle grids are float32 or float64, not %s" % np.dtype(dtype))
    return t


def lib(dtype=np.float32):
    t = _prec(dtype)
    if t not in _libs:
        build()
        L = C.CDLL(os.path.join(_HERE, "_build", _PREC[t][0]))
        fp = np.ctypeslib.ndpointer(dtype=t, flags="C_CONTIGUOUS")
        ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
        F = _PREC[t][1]
        I = C.c_int
        PP, PR = _STRUCTS[t]
        L.og_advect_semi_lagrange.argtypes = [Dims, ip, fp, I, fp, I, F, I, I, I, F]
        L.og_advect_semi_lagrange.restype = I
        L.og_set_wall_bcs.argtypes = [Dims, ip, fp, C.c_void_p]
        L.og_add_buoyancy.argtypes = [Dims, ip, fp, fp, F, F, F, F, I, F]
        L.og_add_gravity.argtypes = [Dims, ip, fp, F, F, F, C.c_void_p, I, F]
        L.og_extrapolate_mac_simple.argtypes = [Dims, ip, fp, I, C.c_void_p, I]
        L.og_extrapolate_ls_simple.argtypes = [Dims, fp, I, I]
        L.og_mg_create.argtypes = [Dims]
        L.og_mg_create.restype = C.c_void_p
        L.og_mg_destroy.argtypes = [C.c_void_p]
        L.og_compute_pressure_rhs.argtypes = [Dims, fp, fp, ip, C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(PP)]
        L.og_solve_pressure.argtypes = [Dims, fp, fp, ip, C.c_void_p, C.c_void_p, C.c_void_p,
                                        C.POINTER(PP), C.POINTER(C.c_void_p), C.POINTER(PR), C.c_void_p]
        L.og_solve_pressure.restype = I
        L.og_make_laplace_matrix.argtypes = [Dims, ip, fp, fp, fp, fp]
        L.og_apply_ghost_fluid_diagonal.argtypes = [Dims, fp, ip, fp, F]
        L.og_mic_init.argtypes = [Dims, ip, fp, fp, fp, fp, fp]
        L.og_mic_apply.argtypes = [Dims, fp, fp, ip, fp, fp, fp, fp]
        L.og_apply_matrix.argtypes = [Dims, ip, fp, fp, fp, fp, fp, fp]
        L.og_mg_vcycle.argtypes = [C.c_void_p, fp, fp, fp, fp, fp, fp, F]
        L.og_mg_num_levels.argtypes = [C.c_void_p]
        L.og_mg_num_levels.restype = I
        L.og_mg_level_size.argtypes = [C.c_void_p, I, C.POINTER(C.c_int * 3)]
        L.og_mg_level_types.argtypes = [C.c_void_p, I]
        L.og_mg_level_types.restype = C.POINTER(C.c_int8)
        L.og_mg_level_matrix.argtypes = [C.c_void_p, I]
        L.og_mg_level_matrix.restype = C.POINTER(F)
        L.og_init_domain.argtypes = [Dims, ip, I, C.c_char_p, C.c_char_p, C.c_char_p, C.c_char_p]
        L.og_fill_grid.argtypes = [Dims, ip, I]
        L.og_set_open_bound.argtypes = [Dims, ip, I, C.c_char_p, I]
        L.og_update_from_levelset.argtypes = [Dims, ip, fp]
        L.og_box_sdf.argtypes = [Dims, fp, F, F, F, F, F, F]
        L.og_cylinder_apply.argtypes = [Dims, fp, F, F, F, F, F, F, F, F, C.c_void_p]
        L.og_box_apply.argtypes = [Dims, fp, F, F, F, F, F, F, F, C.c_void_p]
        L.og_join_real.argtypes = [C.c_longlong, fp, fp, I]
        L.og_get_max_abs.argtypes = [C.c_longlong, fp]
        L.og_get_max_abs.restype = F
        if t is np.float32:
            f32 = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
            L.og_noise_tile.argtypes = [f32]
            L.og_noise_seed_offset.argtypes = [I, f32]
            L.og_noise_evaluate.argtypes = [C.POINTER(NoiseParams), f32, C.c_float, C.c_float, C.c_float]
            L.og_noise_evaluate.restype = C.c_float
            L.og_cylinder_sdf.argtypes = [Dims, f32, f32, C.c_float, f32, C.c_float]
            L.og_density_inflow.argtypes = [Dims, ip, f32, f32, C.POINTER(NoiseParams), f32, C.c_float, C.c_float]
        LL = C.c_longlong
        L.og_map_parts_to_mac.argtypes = [Dims, fp, fp, C.c_void_p, LL, fp, ip, fp, C.c_void_p, I]
        L.og_map_parts_to_grid.argtypes = [Dims, fp, I, LL, fp, ip, fp]
        L.og_map_mac_to_parts.argtypes = [Dims, fp, C.c_void_p, F, LL, fp, ip, fp, C.c_void_p, I]
        L.og_map_grid_to_parts.argtypes = [Dims, fp, I, LL, fp, ip, fp]
        L.og_reset_outflow.argtypes = [Dims, ip, C.c_void_p, C.c_void_p]
        L.og_reset_phi_in_obs.argtypes = [Dims, ip, fp]
        L.og_set_fractions.argtypes = [C.c_void_p, C.c_void_p]
        L.og_set_num_threads.argtypes = [I]
        L.og_get_num_threads.restype = I
        _libs[t] = L
    return _libs[t]


def dims(shape):
    """Dims from a (nz, ny, nx[, 3]) array shape."""
    nz, ny, nx = shape[:3]
    return Dims(nx, ny, nz, 1 if nz > 1 else 0)


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def set_num_threads(n):
    for t in _PREC:
        lib(t).og_set_num_threads(int(n))


def advect_semi_lagrange(flags, vel, grid, kind, order=1, strength=1.0, orderSpace=1, clampMode=2,
                         orderTrace=1, dt=1.0):
    st = lib(vel.dtype).og_advect_semi_lagrange(dims(flags.shape), flags, vel, kind, grid, order, strength, orderSpace,
                                       clampMode, orderTrace, dt)
    if st != 0:
        raise RuntimeError("AdvectSemiLagrange: Only order 1 (regular SL) and 2 (MacCormack) supported")


def set_wall_bcs(flags, vel, obvel=None):
    lib(vel.dtype).og_set_wall_bcs(dims(flags.shape), flags, vel, _ptr(obvel))


def add_buoyancy(flags, density, vel, gravity, coefficient=1.0, scale=True, dt=1.0):
    lib(vel.dtype).og_add_buoyancy(dims(flags.shape), flags, density, vel, *map(float, gravity), coefficient, int(scale), dt)


def add_gravity(flags, vel, gravity, exclude=None, scale=True, dt=1.0):
    lib(vel.dtype).og_add_gravity(dims(flags.shape), flags, vel, *map(float, gravity), _ptr(exclude), int(scale), dt)


def extrapolate_mac_simple(flags, vel, distance=4, intoObs=False, phiObs=None):
    lib(vel.dtype).og_extrapolate_mac_simple(dims(flags.shape), flags, vel, distance, _ptr(phiObs), int(intoObs))


def reset_outflow(flags, phi=None, real=None, dtype=np.float32):
    """resetOutflow (extforces.cpp:133-160) without particles, in place"""
    lib(phi.dtype if phi is not None else (real.dtype if real is not None else dtype)).og_reset_outflow(
        dims(flags.shape), flags, _ptr(phi), _ptr(real))


def reset_phi_in_obs(flags, sdf):
    """resetPhiInObs (advection.cpp:396-401), in place"""
    lib(sdf.dtype).og_reset_phi_in_obs(dims(flags.shape), flags, sdf)


def extrapolate_ls_simple(phi, distance=4, inside=False):
    lib(phi.dtype).og_extrapolate_ls_simple(dims(phi.shape), phi, int(distance), int(bool(inside)))


# -------------------------------------------------- FLIP transfers
# particles: pos (np, 3) and flag (np,) int32 -- BasicParticleData; ptype an
# int32 (np,) array or None; Vec3 particle data (np, 3); grids as elsewhere


def map_parts_to_mac(flags, vel, velOld, pos, pflag, pvel, weight=None, ptype=None, exclude=0):
    """mapPartsToMAC (flip.cpp:573-595): vel, velOld (and weight) in place"""
    lib(vel.dtype).og_map_parts_to_mac(dims(flags.shape), vel, velOld, _ptr(weight), len(pflag), pos, pflag, pvel,
                                       _ptr(ptype), int(exclude))


def map_parts_to_grid(flags, target, pos, pflag, src):
    """mapPartsToGrid / mapPartsToGridVec3 (flip.cpp:599-622)"""
    comps = 3 if target.ndim == 4 else 1
    lib(target.dtype).og_map_parts_to_grid(dims(flags.shape), target, comps, len(pflag), pos, pflag, src)


def map_mac_to_parts(flags, vel, pos, pflag, pvel, ptype=None, exclude=0):
    """mapMACToParts (flip.cpp:651-655): pvel in place"""
    lib(vel.dtype).og_map_mac_to_parts(dims(flags.shape), vel, None, 0.0, len(pflag), pos, pflag, pvel, _ptr(ptype),
                                       int(exclude))


def flip_velocity_update(flags, vel, velOld, pos, pflag, pvel, flipRatio, ptype=None, exclude=0):
    """flipVelocityUpdate (flip.cpp:669-673): pvel in place"""
    lib(vel.dtype).og_map_mac_to_parts(dims(flags.shape), vel, _ptr(velOld), flipRatio, len(pflag), pos, pflag, pvel,
                                       _ptr(ptype), int(exclude))


def map_grid_to_parts(grid, pos, pflag, target):
    """mapGridToParts / mapGridToPartsVec3 (flip.cpp:625-638): target in place"""
    comps = 3 if grid.ndim == 4 else 1
    lib(grid.dtype).og_map_grid_to_parts(dims(grid.shape), grid, comps, len(pflag), pos, pflag, target)


_TILE = None


def noise_tile():
    """WaveletNoiseField's 3 x 128^3 tile (generated once per process)"""
    global _TILE
    if _TILE is None:
        t = np.zeros(3 * 128 ** 3, np.float32)
        lib().og_noise_tile(t)
        _TILE = t
    return _TILE


def noise_params(shape, fixedSeed=-1, time=0.0, posScale=(1, 1, 1), posOffset=(0, 0, 0), valOffset=0.0,
                 valScale=1.0, clamp=False, clampNeg=0.0, clampPos=1.0, timeAnim=0.0):
    """the evaluate() parameters of a NoiseField on a grid of shape (nz, ny, nx)"""
    nz, ny, nx = shape[:3]
    q = NoiseParams()
    scale = np.float32(1.0 / max(nx, ny, nz))
    q.gsInv[:] = [scale, scale, scale if nz > 1 else np.float32(1.0)]
    so = np.zeros(3, np.float32)
    lib().og_noise_seed_offset(int(fixedSeed), so)
    q.seedOffset[:] = list(so)
    dx = np.float32(1.0 / max(nx, ny, nz))
    q.timeOffset = float(np.float32(np.float32(time) * dx) * np.float32(timeAnim))
    q.posScale[:] = [float(np.float32(v)) for v in posScale]
    q.posOffset[:] = [float(np.float32(v)) for v in posOffset]
    q.valOffset, q.valScale = float(valOffset), float(valScale)
    q.clamp, q.clampNeg, q.clampPos = int(bool(clamp)), float(clampNeg), float(clampPos)
    return q


def cylinder_sdf(phi, center, radius, zaxis, maxz):
    lib().og_cylinder_sdf(dims(phi.shape), phi, np.asarray(center, np.float32), float(radius),
                          np.asarray(zaxis, np.float32), float(maxz))


def density_inflow(flags, density, sdf, q, scale=1.0, sigma=0.0):
    lib().og_density_inflow(dims(flags.shape), flags, density, sdf, C.byref(q), noise_tile(), float(scale), float(sigma))


def params(cgAccuracy=1e-3, gfClamp=1e-4, cgMaxIterFac=1.5, preconditioner=PC_MIC, enforceCompatibility=False,
           useL2Norm=False, zeroPressureFixing=False, surfTens=0.0, dtype=np.float32):
    PP = _STRUCTS[_prec(dtype)][0]
    return PP(cgAccuracy, gfClamp, cgMaxIterFac, preconditioner, int(enforceCompatibility),
              int(useL2Norm), int(zeroPressureFixing), surfTens)


class MGCache:
    """The per-solver static multigrid slot (plugin/pressure.cpp:250)."""

    def __init__(self):
        self.ptr = C.c_void_p(None)
        self.dtype = np.float32

    def release(self):
        if self.ptr.value:
            lib(self.dtype).og_mg_destroy(self.ptr)
            self.ptr = C.c_void_p(None)

    def __del__(self):
        try:
            self.release()
        except Exception:
            pass


def compute_pressure_rhs(rhs, vel, flags, phi=None, perCellCorr=None, curv=None, **kw):
    p = params(dtype=vel.dtype, **kw)
    lib(vel.dtype).og_compute_pressure_rhs(dims(flags.shape), rhs, vel, flags, _ptr(phi), _ptr(perCellCorr), _ptr(curv),
                                  C.byref(p))


def solve_pressure(flags, vel, pressure, phi=None, perCellCorr=None, curv=None, mg_cache=None, retRhs=None,
                   fractions=None, obvel=None, **kw):
    """solvePressure; returns (iterations, resNorm, fixPidx)."""
    t = _prec(vel.dtype)
    lib(t).og_set_fractions(_ptr(fractions), _ptr(obvel))
    try:
        return _solve_pressure(t, flags, vel, pressure, phi, perCellCorr, curv, mg_cache, retRhs, **kw)
    finally:
        lib(t).og_set_fractions(None, None)


def _solve_pressure(t, flags, vel, pressure, phi, perCellCorr, curv, mg_cache, retRhs, **kw):
    p = params(dtype=t, **kw)
    res = _STRUCTS[t][1]()
    cache = mg_cache if mg_cache is not None else MGCache()
    if cache.ptr.value and cache.dtype is not t:
        raise ValueError("a multigrid cache serves one precision")
    cache.dtype = t
    st = lib(t).og_solve_pressure(dims(flags.shape), vel, pressure, flags, _ptr(phi), _ptr(perCellCorr), _ptr(curv),
                                 C.byref(p), C.byref(cache.ptr), C.byref(res), _ptr(retRhs))
    if st == -4:
        raise RuntimeError("GridCg::iterate: The CG solver diverged, residual norm > 1e30, stopping.")
    if st == -5:
        raise RuntimeError("GridCg<APPLYMAT>::setICPreconditioner: Invalid method specified.")
    if st != 0:
        raise RuntimeError("solvePressure failed (%d)" % st)
    return res.iterations, res.resNorm, res.fixPidx


def make_laplace_matrix(flags, dtype=np.float32):
    A = [np.zeros(flags.shape, dtype) for _ in range(4)]
    lib(dtype).og_make_laplace_matrix(dims(flags.shape), flags, *A)
    return A


def apply_ghost_fluid_diagonal(A0, flags, phi, gfClamp=1e-4):
    lib(A0.dtype).og_apply_ghost_fluid_diagonal(dims(flags.shape), A0, flags, phi, gfClamp)


def mic_init(flags, A0, Ai, Aj, Ak):
    P = np.zeros(flags.shape, A0.dtype)
    lib(A0.dtype).og_mic_init(dims(flags.shape), flags, P, A0, Ai, Aj, Ak)
    return P


def mic_apply(dst, src, flags, P, Ai, Aj, Ak):
    lib(dst.dtype).og_mic_apply(dims(flags.shape), dst, src, flags, P, Ai, Aj, Ak)


def apply_matrix(flags, dst, src, A0, Ai, Aj, Ak):
    lib(dst.dtype).og_apply_matrix(dims(flags.shape), flags, dst, src, A0, Ai, Aj, Ak)


def init_domain(flags, boundaryWidth=0, wall="xXyYzZ", open="      ", inflow="      ", outflow="      "):
    lib().og_init_domain(dims(flags.shape), flags, boundaryWidth, wall.encode(), open.encode(), inflow.encode(),
                         outflow.encode())


def fill_grid(flags, type=FLUID):
    lib().og_fill_grid(dims(flags.shape), flags, type)


def set_open_bound(flags, bWidth, openBound="", type=OUTFLOW | EMPTY):
    lib().og_set_open_bound(dims(flags.shape), flags, bWidth, openBound.encode(), type)


def update_from_levelset(flags, phi):
    lib(phi.dtype).og_update_from_levelset(dims(flags.shape), flags, phi)


def box_sdf(phi, p0, p1):
    lib(phi.dtype).og_box_sdf(dims(phi.shape), phi, *map(float, p0), *map(float, p1))


def cylinder_apply(grid, center, radius, z, value, respectFlags=None):
    lib(grid.dtype).og_cylinder_apply(dims(grid.shape), grid, *map(float, center), float(radius), *map(float, z), float(value),
                            _ptr(respectFlags))


def box_apply(grid, p0, p1, value, respectFlags=None):
    lib(grid.dtype).og_box_apply(dims(grid.shape), grid, *map(float, p0), *map(float, p1), float(value), _ptr(respectFlags))


def join_real(a, b, keepMax=True):
    lib(a.dtype).og_join_real(a.size, a, b, int(keepMax))


def get_max_abs(a):
    return lib(a.dtype).og_get_max_abs(a.size, a)
