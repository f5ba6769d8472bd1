"""mantaflow_gb300: mantaflow's Eulerian grid-step hot path on one GB300.

`from mantaflow_gb300 import *` gives the reference's scene-script names
(Solver, FlagGrid, MACGrid, RealGrid, advectSemiLagrange, solvePressure,
setWallBcs, addBuoyancy, ...) backed by hand-written sm_103a CUDA kernels in
libmantagpu.so (C ABI: include/mantagpu.h).
"""
from .manta import *  # noqa: F401,F403
from .manta import __all__  # noqa: F401
