"""Scene-script API of mantaflow's grid-step hot path, backed by libmantagpu.

Names, argument names, defaults and enum values follow the reference's
Python bindings (the PYTHON() declarations in source/plugin/advection.cpp,
pressure.cpp, extforces.cpp, fastmarch.cpp, source/grid.h, source/shapes.h
and source/python/defines.py), so a scene written as

    from manta import *
    s = Solver(name='main', gridSize=vec3(64,64,64), dim=3)
    flags = s.create(FlagGrid); vel = s.create(MACGrid)
    ...
    advectSemiLagrange(flags=flags, vel=vel, grid=density, order=2)
    solvePressure(flags=flags, vel=vel, pressure=pressure)

runs unchanged with `from mantaflow_gb300 import *`.  Grids are device
resident; copyArrayToGrid* / copyGridToArray* (plugin/numpyconvert.cpp) move
them between numpy arrays in the reference layout and the GPU.
"""
import ctypes as C

import numpy as np

from . import _lib
from ._lib import MantaError, PressureParams, PressureResult, check, ensure_init, fptr

# ----------------------------------------------------------------- constants
# source/python/defines.py
Real = float
false = False
true = True
FlagFluid, FlagObstacle, FlagEmpty, FlagInflow, FlagOutflow, FlagOpen, FlagStick = 1, 2, 4, 8, 16, 32, 64
FlagReserved = 256
TypeFluid, TypeObstacle, TypeEmpty, TypeInflow, TypeOutflow, TypeOpen, TypeStick = 1, 2, 4, 8, 16, 32, 64
TypeReserved = 256
PcNone, PcMIC, PcMGDynamic, PcMGStatic = 0, 1, 2, 3
CUDA = True  # the reference exposes CUDA=False (pwrapper/registry.cpp:419-420)

_KIND_REAL, _KIND_INT, _KIND_VEC3, _KIND_MAC, _KIND_FLAGS, _KIND_LEVELSET = 0, 1, 2, 3, 4, 5


class vec3:
    """Float32 3-vector with the reference's component-wise arithmetic
    (pwrapper/pvec3.cpp: PbVec3 holds float data[3])."""

    __slots__ = ("v",)

    def __init__(self, x=None, y=None, z=None):
        if x is None:
            self.v = np.zeros(3, np.float32)
        elif y is None and z is None:
            if isinstance(x, (vec3, tuple, list, np.ndarray)):
                self.v = np.asarray(x.v if isinstance(x, vec3) else x, np.float32).copy()
            else:
                self.v = np.full(3, x, np.float32)
        else:
            self.v = np.array([x, y, z], np.float32)

    @staticmethod
    def _o(o):
        return o.v if isinstance(o, vec3) else np.float32(o)

    def __add__(self, o): return vec3(self.v + self._o(o))
    __radd__ = __add__
    def __sub__(self, o): return vec3(self.v - self._o(o))
    def __rsub__(self, o): return vec3(self._o(o) - self.v)
    def __mul__(self, o): return vec3(self.v * self._o(o))
    __rmul__ = __mul__
    def __truediv__(self, o): return vec3(self.v / self._o(o))
    def __neg__(self): return vec3(-self.v)
    def __getitem__(self, i): return float(self.v[i])
    def __iter__(self): return iter(float(a) for a in self.v)
    def __repr__(self): return "[%+4.6f,%+4.6f,%+4.6f]" % tuple(float(a) for a in self.v)

    @property
    def x(self): return float(self.v[0])

    @property
    def y(self): return float(self.v[1])

    @property
    def z(self): return float(self.v[2])


Vec3 = vec3


def _vec(v):
    if isinstance(v, vec3):
        return v.v
    if np.isscalar(v):
        return np.full(3, v, np.float32)
    return np.asarray(v, np.float32)


# -------------------------------------------------------------------- solver
class Solver:
    """FluidSolver (source/fluidsolver.h): grid size, timestep, grid storage."""

    def __init__(self, name="solver", gridSize=None, dim=3, fourthDim=0):
        L = ensure_init()
        gs = _vec(gridSize if gridSize is not None else vec3(100, 100, 100))
        nx, ny, nz = int(gs[0]), int(gs[1]), int(gs[2])
        if dim == 2:
            nz = 1
        self.name = name
        self.dim = dim
        self._size = (nx, ny, nz)
        h = C.c_void_p()
        check(L.mg_solver_create(nx, ny, nz, dim, C.byref(h)))
        self._h = h
        self.frame = 0
        self.timeTotal = 0.0
        self._grids = []

    # FluidSolver properties
    @property
    def timestep(self):
        v = C.c_float()
        check(_lib.load().mg_solver_get_dt(self._h, C.byref(v)))
        return float(v.value)

    @timestep.setter
    def timestep(self, dt):
        check(_lib.load().mg_solver_set_dt(self._h, float(dt)))

    def getDt(self):
        return self.timestep

    def getGridSize(self):
        return vec3(*self._size)

    def is2D(self):
        return self.dim == 2

    def is3D(self):
        return self.dim == 3

    def create(self, cls, **kwargs):
        """FluidSolver::create: grids and shapes bound to this solver."""
        obj = cls(self, **kwargs)
        return obj

    def step(self):
        """FluidSolver::step (fluidsolver.cpp:142-158): frame bookkeeping."""
        self.sync()
        self.timeTotal += self.timestep
        self.frame += 1

    def sync(self):
        check(_lib.load().mg_solver_sync(self._h))

    def memoryBytes(self):
        v = C.c_size_t()
        check(_lib.load().mg_solver_memory(self._h, C.byref(v)))
        return int(v.value)

    def setMemoryLimit(self, nbytes):
        """Cap the device memory this solver may hold (0: no cap)."""
        check(_lib.load().mg_solver_set_memory_limit(self._h, int(nbytes)))

    def setWaitLimit(self, ns, stallNextSolve=False):
        """Limit of each device-side MIC(0) wavefront wait in nanoseconds (0:
        the default 200 ms).  stallNextSolve makes the next MIC(0) solve's
        waits run out, to exercise the timeout path."""
        check(_lib.load().mg_solver_set_wait_limit(self._h, int(ns), 1 if stallNextSolve else 0))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and _lib._lib is not None:
            try:
                for g in self._grids:
                    g._h = None
                for ps in getattr(self, "_particles", []):
                    ps._h = None
                    for d in ps._data:
                        d._h = None
                _lib._lib.mg_solver_destroy(h)
            except Exception:
                pass


# --------------------------------------------------------------------- grids
class GridBase:
    _kind = None

    def __init__(self, parent, show=True, name=None):
        self._parent = parent
        self.name = name
        h = C.c_void_p()
        check(_lib.load().mg_grid_create(parent._h, self._kind, C.byref(h)))
        self._h = h
        parent._grids.append(self)

    def getParent(self):
        return self._parent

    def getSizeX(self):
        return self._parent._size[0]

    def getSizeY(self):
        return self._parent._size[1]

    def getSizeZ(self):
        return self._parent._size[2]

    def getSize(self):
        return vec3(*self._parent._size)

    def is3D(self):
        return self._parent.dim == 3

    def _shape(self):
        nx, ny, nz = self._parent._size
        return (nz, ny, nx, 3) if self._kind in (_KIND_VEC3, _KIND_MAC) else (nz, ny, nx)

    def _dtype(self):
        return np.int32 if self._kind in (_KIND_INT, _KIND_FLAGS) else np.float32

    def _upload(self, a):
        a = np.ascontiguousarray(a, dtype=self._dtype()).reshape(self._shape())
        check(_lib.load().mg_grid_upload(self._h, a.ctypes.data_as(C.c_void_p), a.nbytes))

    def _download(self):
        a = np.empty(self._shape(), self._dtype())
        check(_lib.load().mg_grid_download(self._h, a.ctypes.data_as(C.c_void_p), a.nbytes))
        return a

    def numpy(self):
        """Download the grid as a numpy array in the reference layout."""
        return self._download()

    def save(self, name):
        """Grid<T>::save (grid.cpp:135-156): .uni, .raw or .npz, written from
        the device mirror."""
        check(_lib.load().mg_grid_save(self._h, str(name).encode()))
        return 1

    def copyFrom(self, other, copyType=True):
        check(_lib.load().mg_grid_copy(self._h, other._h))
        return self

    def swap(self, other):
        check(_lib.load().mg_grid_swap(self._h, other._h))

    def clear(self):
        check(_lib.load().mg_grid_set_const(self._h, 0.0, 0.0, 0.0))

    def setConst(self, s):
        v = _vec(s)
        check(_lib.load().mg_grid_set_const(self._h, float(v[0]), float(v[1]), float(v[2])))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and _lib._lib is not None:
            try:
                _lib._lib.mg_grid_destroy(h)
            except Exception:
                pass


class RealGrid(GridBase):
    """Grid<Real>"""
    _kind = _KIND_REAL

    def getMaxAbs(self):
        v = C.c_float()
        check(_lib.load().mg_grid_get_max_abs(self._h, C.byref(v)))
        return float(v.value)

    def getMax(self):
        return float(self._download().max())

    def getMin(self):
        return float(self._download().min())

    def join(self, a, keepMax=True):
        check(_lib.load().mg_grid_join(self._h, a._h, int(keepMax)))


class LevelsetGrid(RealGrid):
    """LevelsetGrid (source/levelset.h)"""
    _kind = _KIND_LEVELSET


class IntGrid(GridBase):
    _kind = _KIND_INT


class VecGrid(GridBase):
    """Grid<Vec3>"""
    _kind = _KIND_VEC3


Vec3Grid = VecGrid


class MACGrid(GridBase):
    _kind = _KIND_MAC


class FlagGrid(GridBase):
    """FlagGrid (source/grid.h:283-341)"""
    _kind = _KIND_FLAGS

    def __init__(self, parent, dim=3, show=True, name=None):
        super().__init__(parent, show, name)

    def initDomain(self, boundaryWidth=0, wall="xXyYzZ", open="      ", inflow="      ", outflow="      ",
                   phiWalls=None):
        check(_lib.load().mg_flags_init_domain(self._h, int(boundaryWidth), wall.encode(), open.encode(),
                                               inflow.encode(), outflow.encode(),
                                               phiWalls._h if phiWalls is not None else None))

    def fillGrid(self, type=TypeFluid):
        check(_lib.load().mg_flags_fill_grid(self._h, int(type)))

    def updateFromLevelset(self, levelset):
        check(_lib.load().mg_flags_update_from_levelset(self._h, levelset._h))

    def countCells(self, flag, bnd=0, mask=None):
        f = self._download()
        if bnd > 0:
            if f.shape[0] > 1:
                f = f[bnd:-bnd, bnd:-bnd, bnd:-bnd]
            else:
                f = f[:, bnd:-bnd, bnd:-bnd]
        return int(np.count_nonzero(f & int(flag)))


def _h(g):
    return None if g is None else g._h


# -------------------------------------------------------------------- shapes
class Shape:
    def __init__(self, parent):
        self._parent = parent


class Box(Shape):
    """Box (source/shapes.h:69-88): center+size or p0+p1."""

    def __init__(self, parent, center=None, p0=None, p1=None, size=None):
        super().__init__(parent)
        if center is not None and size is not None:
            c, s = _vec(center), _vec(size)
            self.p0, self.p1 = c - s, c + s
        elif p0 is not None and p1 is not None:
            self.p0, self.p1 = _vec(p0).copy(), _vec(p1).copy()
        else:
            raise MantaError("Box: specify either p0,p1 or size,center")

    def applyToGrid(self, grid, value=None, respectFlags=None):
        v = _vec(value if value is not None else 0.0)
        iv = int(v[0])
        check(_lib.load().mg_shape_box_apply(grid._h, fptr(self.p0), fptr(self.p1), fptr(v), iv, _h(respectFlags)))

    def computeLevelset(self):
        phi = LevelsetGrid(self._parent)
        check(_lib.load().mg_shape_box_levelset(phi._h, fptr(self.p0), fptr(self.p1)))
        return phi


class Cylinder(Shape):
    """Cylinder (source/shapes.h:106-126)."""

    def __init__(self, parent, center=None, radius=1.0, z=None):
        super().__init__(parent)
        self.center = _vec(center if center is not None else vec3(0, 0, 0)).copy()
        self.radius = np.float32(radius)
        self.z = _vec(z if z is not None else vec3(0, 0, 1)).copy()

    def applyToGrid(self, grid, value=None, respectFlags=None):
        v = _vec(value if value is not None else 0.0)
        iv = int(v[0])
        check(_lib.load().mg_shape_cylinder_apply(grid._h, fptr(self.center), float(self.radius), fptr(self.z),
                                                  fptr(v), iv, _h(respectFlags)))

    def computeLevelset(self):
        phi = LevelsetGrid(self._parent)
        check(_lib.load().mg_shape_cylinder_levelset(phi._h, fptr(self.center), float(self.radius), fptr(self.z)))
        return phi


# -------------------------------------------------------------- noise field
class NoiseField:
    """WaveletNoiseField (source/noisefield.h:27-98), Python name NoiseField:
    the shared 128^3 wavelet noise tile (generated on first use, kept on the
    device) sampled with the properties below."""

    def __init__(self, parent, fixedSeed=-1, loadFromFile=False):
        self._parent = parent
        h = C.c_void_p()
        check(_lib.load().mg_noise_create(parent._h, int(fixedSeed), C.byref(h)))
        self._h = h
        self.posOffset = vec3(0.0)
        self.posScale = vec3(1.0)
        self.valOffset = 0.0
        self.valScale = 1.0
        self.clamp = False
        self.clampNeg = 0.0
        self.clampPos = 1.0
        self.timeAnim = 0.0

    def _sync(self):
        p = _lib.NoiseParams()
        p.posOffset[:] = [float(x) for x in _vec(self.posOffset)]
        p.posScale[:] = [float(x) for x in _vec(self.posScale)]
        p.valOffset, p.valScale = float(self.valOffset), float(self.valScale)
        p.clamp, p.clampNeg, p.clampPos = int(bool(self.clamp)), float(self.clampNeg), float(self.clampPos)
        p.timeAnim = float(self.timeAnim)
        check(_lib.load().mg_noise_set_params(self._h, C.byref(p)))

    def seedOffset(self):
        out = (C.c_float * 3)()
        check(_lib.load().mg_noise_seed_offset(self._h, out))
        return vec3(out[0], out[1], out[2])

    def evaluateGrid(self, grid):
        """grid(i,j,k) = evaluate(Vec3(i,j,k)) at the solver's time"""
        self._sync()
        check(_lib.load().mg_noise_evaluate_grid(self._h, grid._h, float(self._parent.timeTotal)))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and _lib._lib is not None:
            try:
                _lib._lib.mg_noise_destroy(h)
            except Exception:
                pass


WaveletNoiseField = NoiseField


# ------------------------------------------------------------- numpy bridge
# plugin/numpyconvert.cpp:145-182
def copyArrayToGridReal(source, target):
    target._upload(source)


def copyGridToArrayReal(source, target):
    target[...] = source._download().reshape(target.shape)


copyArrayToGridLevelset = copyArrayToGridReal
copyGridToArrayLevelset = copyGridToArrayReal
copyArrayToGridFlag = copyArrayToGridReal
copyGridToArrayFlag = copyGridToArrayReal
copyArrayToGridVec3 = copyArrayToGridReal
copyGridToArrayVec3 = copyGridToArrayReal
copyArrayToGridMAC = copyArrayToGridReal
copyGridToArrayMAC = copyGridToArrayReal


# ------------------------------------------------------------------- plugins
def advectSemiLagrange(flags, vel, grid, order=1, strength=1.0, orderSpace=1, openBounds=False, boundaryWidth=-1,
                       clampMode=2, orderTrace=1):
    """plugin/advection.cpp:442-460"""
    if boundaryWidth != -1 or openBounds:
        print("Warning: boundaryWidth and openBounds parameters in AdvectSemiLagrange plugin are deprecated "
              "(and have no more effect), please remove.")
    check(_lib.load().mg_advect_semi_lagrange(flags._h, vel._h, grid._h, int(order), float(strength),
                                              int(orderSpace), int(openBounds), int(boundaryWidth), int(clampMode),
                                              int(orderTrace)))


def resetPhiInObs(flags, sdf):
    """plugin/advection.cpp:401"""
    check(_lib.load().mg_reset_phi_in_obs(flags._h, sdf._h))


def setWallBcs(flags, vel, obvel=None, fractions=None, phiObs=None, boundaryWidth=0):
    """plugin/extforces.cpp:307-315"""
    check(_lib.load().mg_set_wall_bcs(flags._h, vel._h, _h(obvel), _h(fractions), _h(phiObs), int(boundaryWidth)))


def addBuoyancy(flags, density, vel, gravity, coefficient=1.0, scale=True):
    """plugin/extforces.cpp:83-87"""
    g = _vec(gravity)
    check(_lib.load().mg_add_buoyancy(flags._h, density._h, vel._h, float(g[0]), float(g[1]), float(g[2]),
                                      float(coefficient), int(bool(scale))))


def addGravity(flags, vel, gravity, exclude=None, scale=True):
    """plugin/extforces.cpp:61-65"""
    g = _vec(gravity)
    check(_lib.load().mg_add_gravity(flags._h, vel._h, float(g[0]), float(g[1]), float(g[2]), _h(exclude),
                                     int(bool(scale))))


def addGravityNoScale(flags, vel, gravity, exclude=None):
    """plugin/extforces.cpp:67-69"""
    addGravity(flags, vel, gravity, exclude, scale=False)


def setOpenBound(flags, bWidth, openBound="", type=TypeOutflow | TypeEmpty):
    """plugin/extforces.cpp:105-130"""
    check(_lib.load().mg_set_open_bound(flags._h, int(bWidth), openBound.encode(), int(type)))


def resetOutflow(flags, phi=None, parts=None, real=None, index=None, indexSys=None):
    """plugin/extforces.cpp:133-160 (grid part)"""
    if parts is not None:
        raise MantaError("resetOutflow: particle systems are not part of the GPU grid path")
    check(_lib.load().mg_reset_outflow(flags._h, _h(phi), _h(real)))


def extrapolateMACSimple(flags, vel, distance=4, phiObs=None, intoObs=False):
    """fastmarch.cpp:337-375"""
    check(_lib.load().mg_extrapolate_mac_simple(flags._h, vel._h, int(distance), _h(phiObs), int(bool(intoObs))))


def densityInflow(flags, density, noise, shape, scale=1.0, sigma=0.0):
    """plugin/initplugins.cpp:38-43"""
    sdf = shape.computeLevelset()
    noise._sync()
    check(_lib.load().mg_density_inflow(flags._h, density._h, noise._h, sdf._h, float(scale), float(sigma),
                                        float(noise._parent.timeTotal)))


def extrapolateLsSimple(phi, distance=4, inside=False):
    """fastmarch.cpp:470-507"""
    check(_lib.load().mg_extrapolate_ls_simple(phi._h, int(distance), int(bool(inside))))


def _params(cgAccuracy, gfClamp, cgMaxIterFac, precondition, preconditioner, enforceCompatibility, useL2Norm,
            zeroPressureFixing, surfTens):
    return PressureParams(float(cgAccuracy), float(gfClamp), float(cgMaxIterFac), int(bool(precondition)),
                          int(preconditioner), int(bool(enforceCompatibility)), int(bool(useL2Norm)),
                          int(bool(zeroPressureFixing)), float(surfTens))


_last_cg = {"iterations": 0, "resNorm": 0.0}


def solvePressure(vel, pressure, flags, cgAccuracy=1e-3, phi=None, perCellCorr=None, fractions=None, obvel=None,
                  gfClamp=1e-04, cgMaxIterFac=1.5, precondition=True, preconditioner=PcMIC,
                  enforceCompatibility=False, useL2Norm=False, zeroPressureFixing=False, curv=None, surfTens=0.,
                  retRhs=None):
    """plugin/pressure.cpp:480-521.  Returns nothing, like the reference;
    the CG statistics are available from lastSolveStats()."""
    p = _params(cgAccuracy, gfClamp, cgMaxIterFac, precondition, preconditioner, enforceCompatibility, useL2Norm,
                zeroPressureFixing, surfTens)
    res = PressureResult()
    check(_lib.load().mg_solve_pressure(vel._h, pressure._h, flags._h, C.byref(p), _h(phi), _h(perCellCorr),
                                        _h(fractions), _h(obvel), _h(curv), _h(retRhs), C.byref(res)))
    _last_cg["iterations"] = res.iterations
    _last_cg["resNorm"] = res.resNorm


def solvePressureRefined(vel, pressure, flags, cgAccuracy=1e-3, refineAccuracy=1e-5, innerAccuracy=1e-2,
                         maxRefine=10, phi=None, gfClamp=1e-04, cgMaxIterFac=1.5, preconditioner=PcMIC,
                         useL2Norm=False, zeroPressureFixing=False):
    """Precision form of solvePressure: FP32 PCG inner solves with the
    pressure accumulated in double and the residual recomputed in double
    after each, until max|b - A p| < refineAccuracy.  The first inner solve
    runs at cgAccuracy, later ones at innerAccuracy * max|r|.  Returns
    (inner solves, total CG iterations, final double residual)."""
    from ._lib import RefineParams, RefineResult
    p = _params(cgAccuracy, gfClamp, cgMaxIterFac, True, preconditioner, False, useL2Norm, zeroPressureFixing, 0.)
    rp = RefineParams(float(refineAccuracy), float(innerAccuracy), int(maxRefine))
    res = RefineResult()
    check(_lib.load().mg_solve_pressure_refined(vel._h, pressure._h, flags._h, C.byref(p), _h(phi), C.byref(rp),
                                                C.byref(res)))
    _last_cg["iterations"] = res.iterations
    _last_cg["resNorm"] = res.resNorm
    return res.refinements, res.iterations, res.resNorm


def lastSolveStats():
    """(iterations, residual norm) of the last pressure solve of this process."""
    return _last_cg["iterations"], _last_cg["resNorm"]


def computePressureRhs(rhs, vel, pressure, flags, cgAccuracy=1e-3, phi=None, perCellCorr=None, fractions=None,
                       obvel=None, gfClamp=1e-04, cgMaxIterFac=1.5, precondition=True, preconditioner=PcMIC,
                       enforceCompatibility=False, useL2Norm=False, zeroPressureFixing=False, curv=None, surfTens=0.):
    """plugin/pressure.cpp:277-299"""
    p = _params(cgAccuracy, gfClamp, cgMaxIterFac, precondition, preconditioner, enforceCompatibility, useL2Norm,
                zeroPressureFixing, surfTens)
    check(_lib.load().mg_compute_pressure_rhs(rhs._h, vel._h, pressure._h, flags._h, C.byref(p), _h(phi),
                                              _h(perCellCorr), _h(fractions), _h(obvel), _h(curv)))


def solvePressureSystem(rhs, vel, pressure, flags, cgAccuracy=1e-3, phi=None, perCellCorr=None, fractions=None,
                        gfClamp=1e-04, cgMaxIterFac=1.5, precondition=True, preconditioner=PcMIC,
                        enforceCompatibility=False, useL2Norm=False, zeroPressureFixing=False, curv=None,
                        surfTens=0.):
    """plugin/pressure.cpp:312-452"""
    p = _params(cgAccuracy, gfClamp, cgMaxIterFac, precondition, preconditioner, enforceCompatibility, useL2Norm,
                zeroPressureFixing, surfTens)
    res = PressureResult()
    check(_lib.load().mg_solve_pressure_system(rhs._h, vel._h, pressure._h, flags._h, C.byref(p), _h(phi),
                                               _h(perCellCorr), _h(fractions), _h(curv), C.byref(res)))
    _last_cg["iterations"] = res.iterations
    _last_cg["resNorm"] = res.resNorm


def correctVelocity(vel, pressure, flags, cgAccuracy=1e-3, phi=None, perCellCorr=None, fractions=None,
                    gfClamp=1e-04, cgMaxIterFac=1.5, precondition=True, preconditioner=PcMIC,
                    enforceCompatibility=False, useL2Norm=False, zeroPressureFixing=False, curv=None, surfTens=0.):
    """plugin/pressure.cpp:455-476"""
    p = _params(cgAccuracy, gfClamp, cgMaxIterFac, precondition, preconditioner, enforceCompatibility, useL2Norm,
                zeroPressureFixing, surfTens)
    check(_lib.load().mg_correct_velocity(vel._h, pressure._h, flags._h, C.byref(p), _h(phi), _h(perCellCorr),
                                          _h(fractions), _h(curv)))


def releaseMG(solver=None):
    """plugin/pressure.cpp:252-266"""
    check(_lib.load().mg_release_mg(solver._h if solver is not None else None))


def setDebugLevel(level=1):
    """fluidsolver.cpp:213-215 (messages of the GPU path are not printed)"""
    return None



# ----------------------------------------------------------------- particles
ParticleDelete = 1 << 10  # ParticleBase::PDELETE (source/particle.h:41)


class BasicParticleSystem:
    """BasicParticleSystem (source/particle.h:193-230): particle positions and
    status flags in device memory.  addParticle collects particles on the
    host; they reach the device (and every particle data of the system grows
    by zeros, as ParticleDataImpl does) before the next transfer."""

    def __init__(self, parent, show=True, name=None):
        self._parent = parent
        self.name = name
        self._h = None
        self._cap = 0
        self._n = 0
        self._pending = []
        self._data = []
        parent._particles = getattr(parent, "_particles", [])
        parent._particles.append(self)

    def create(self, cls, **kwargs):
        """ParticleBase::create: particle data of this system"""
        d = cls(self, **kwargs)
        return d

    def addParticle(self, pos):
        self._pending.append([float(x) for x in _vec(pos)])

    def pySize(self):
        return self._n + len(self._pending)

    def size(self):
        return self.pySize()

    def _records(self):
        rec = np.zeros(self._n, dtype=[("pos", np.float32, 3), ("flag", np.int32)])
        if self._n:
            check(_lib.load().mg_particles_download(self._h, rec.ctypes.data_as(C.c_void_p), self._n))
        return rec

    def _set_records(self, rec):
        """replace every particle (positions and flags); data keeps its values
        for the first min(old, new) particles and is zero beyond"""
        L = _lib.load()
        n = len(rec)
        saved = [(d, d._download()) for d in self._data]
        if self._h is None or n > self._cap:
            cap = max(1024, n, 2 * self._cap)
            if self._h is not None:
                for d in self._data:
                    d._h = None  # destroyed with the system
                check(L.mg_particles_destroy(self._h))
                self._h = None
            h = C.c_void_p()
            check(L.mg_particles_create(self._parent._h, cap, C.byref(h)))
            self._h, self._cap = h, cap
            for d in self._data:
                d._alloc()
        rec = np.ascontiguousarray(rec)
        check(L.mg_particles_upload(self._h, rec.ctypes.data_as(C.c_void_p), n))
        self._n = n
        for d, old in saved:
            new = np.zeros((n,) + old.shape[1:], old.dtype)
            m = min(n, len(old))
            new[:m] = old[:m]
            d._upload(new)

    def _flush(self):
        if not self._pending and self._h is not None:
            return
        rec = self._records()
        add = np.zeros(len(self._pending), dtype=rec.dtype)
        if self._pending:
            add["pos"] = np.asarray(self._pending, np.float32)
        self._pending = []
        self._set_records(np.concatenate([rec, add]))

    def setPositions(self, pos, flags=None):
        """all particles at once from an (n, 3) array (flags: (n,) int32, 0 if
        omitted); a bulk form of addParticle"""
        pos = np.asarray(pos, np.float32).reshape(-1, 3)
        rec = np.zeros(len(pos), dtype=[("pos", np.float32, 3), ("flag", np.int32)])
        rec["pos"] = pos
        if flags is not None:
            rec["flag"] = np.asarray(flags, np.int32)
        self._pending = []
        self._set_records(rec)

    def positions(self):
        """(positions (n, 3), flags (n,)) from the device"""
        self._flush()
        rec = self._records()
        return np.ascontiguousarray(rec["pos"]), np.ascontiguousarray(rec["flag"])

    def getPosPdata(self, target):
        target._upload(self.positions()[0])

    def setPosPdata(self, source):
        self._flush()
        rec = self._records()
        rec["pos"] = source._download()
        self._set_records(rec)

    def kill(self, idx):
        """ParticleBase::kill: mark particle idx deleted"""
        self._flush()
        rec = self._records()
        rec["flag"][idx] |= ParticleDelete
        self._set_records(rec)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and _lib._lib is not None:
            try:
                _lib._lib.mg_particles_destroy(h)
            except Exception:
                pass


class _Pdata:
    """ParticleDataImpl<T> (source/particle.h:306-360) of one particle system"""
    _kind = None
    _comps = 1
    _dtype = np.float32

    def __init__(self, parts, show=True, name=None):
        self._parts = parts
        self.name = name
        self._h = None
        parts._data.append(self)
        parts._flush()  # creates the device system (and this data) if needed
        if self._h is None:
            self._alloc()

    def _alloc(self):
        h = C.c_void_p()
        check(_lib.load().mg_pdata_create(self._parts._h, self._kind, C.byref(h)))
        self._h = h

    def _shape(self):
        n = self._parts._n
        return (n, 3) if self._comps == 3 else (n,)

    def _upload(self, a):
        self._parts._flush()
        a = np.ascontiguousarray(a, dtype=self._dtype).reshape(self._shape())
        check(_lib.load().mg_pdata_upload(self._h, a.ctypes.data_as(C.c_void_p), self._parts._n))

    def _download(self):
        a = np.zeros(self._shape(), self._dtype)
        if self._parts._n:
            check(_lib.load().mg_pdata_download(self._h, a.ctypes.data_as(C.c_void_p), self._parts._n))
        return a

    def numpy(self):
        self._parts._flush()
        return self._download()

    def setConst(self, s):
        v = np.broadcast_to(np.asarray(_vec(s) if self._comps == 3 else s, self._dtype), self._shape())
        self._upload(v)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and _lib._lib is not None:
            try:
                _lib._lib.mg_pdata_destroy(h)
            except Exception:
                pass


class PdataReal(_Pdata):
    _kind = _KIND_REAL


class PdataVec3(_Pdata):
    _kind = _KIND_VEC3
    _comps = 3


class PdataInt(_Pdata):
    _kind = _KIND_INT
    _dtype = np.int32


# plugin/numpyconvert.cpp:202-223
def copyArrayToPdataInt(source, target):
    target._upload(source)


def copyPdataToArrayInt(source, target):
    target[...] = source.numpy().reshape(target.shape)


def copyArrayToPdataReal(source, target):
    target._upload(source)


def copyPdataToArrayReal(source, target):
    target[...] = source.numpy().reshape(target.shape)


def copyArrayToPdataVec3(source, target):
    target._upload(source)


def copyPdataToArrayVec3(source, target):
    target[...] = source.numpy().reshape(target.shape)


def mapPartsToMAC(flags, vel, velOld, parts, partVel, weight=None, ptype=None, exclude=0):
    """plugin/flip.cpp:573-595"""
    parts._flush()
    check(_lib.load().mg_map_parts_to_mac(flags._h, vel._h, velOld._h, parts._h, partVel._h, _h(weight), _h(ptype),
                                          int(exclude)))


def mapMACToParts(flags, vel, parts, partVel, ptype=None, exclude=0):
    """plugin/flip.cpp:651-655"""
    parts._flush()
    check(_lib.load().mg_map_mac_to_parts(flags._h, vel._h, parts._h, partVel._h, _h(ptype), int(exclude)))


def flipVelocityUpdate(flags, vel, velOld, parts, partVel, flipRatio, ptype=None, exclude=0):
    """plugin/flip.cpp:669-673"""
    parts._flush()
    check(_lib.load().mg_flip_velocity_update(flags._h, vel._h, velOld._h, parts._h, partVel._h, float(flipRatio),
                                              _h(ptype), int(exclude)))


def mapPartsToGrid(flags, target, parts, source):
    """plugin/flip.cpp:617-619"""
    parts._flush()
    check(_lib.load().mg_map_parts_to_grid(flags._h, target._h, parts._h, source._h))


def mapPartsToGridVec3(flags, target, parts, source):
    """plugin/flip.cpp:620-622"""
    mapPartsToGrid(flags, target, parts, source)


def mapGridToParts(source, parts, target):
    """plugin/flip.cpp:633-635"""
    parts._flush()
    check(_lib.load().mg_map_grid_to_parts(source._h, parts._h, target._h))


def mapGridToPartsVec3(source, parts, target):
    """plugin/flip.cpp:636-638"""
    mapGridToParts(source, parts, target)

__all__ = [n for n in dir() if not n.startswith("_") and n not in ("C", "np")]
