"""ctypes binding of libmantagpu (include/mantagpu.h).

There is no CPU fallback: if the CUDA library cannot be built or loaded, or no
CUDA device is present, the calls raise.
"""
import ctypes as C
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libmantagpu.so")

_lib = None
_lock = threading.Lock()


class PressureParams(C.Structure):
    _fields_ = [("cgAccuracy", C.c_float), ("gfClamp", C.c_float), ("cgMaxIterFac", C.c_float),
                ("precondition", C.c_int), ("preconditioner", C.c_int), ("enforceCompatibility", C.c_int),
                ("useL2Norm", C.c_int), ("zeroPressureFixing", C.c_int), ("surfTens", C.c_float)]


class PressureResult(C.Structure):
    _fields_ = [("iterations", C.c_int), ("resNorm", C.c_float)]


class BatchStats(C.Structure):
    _fields_ = [("sweeps", C.c_int), ("maxIterations", C.c_int), ("totalIterations", C.c_longlong),
                ("diverged", C.c_int), ("graphLaunches", C.c_longlong)]


class ServeStats(C.Structure):
    _fields_ = [("jobs", C.c_int), ("ticks", C.c_longlong), ("wallSeconds", C.c_double), ("cellSteps", C.c_longlong),
                ("peakBytes", C.c_size_t)]


class ServeJob(C.Structure):
    _fields_ = [("arrival", C.c_double), ("admitted", C.c_double), ("finished", C.c_double), ("steps", C.c_int),
                ("meanStepMs", C.c_double)]


class NoiseParams(C.Structure):
    _fields_ = [("posOffset", C.c_float * 3), ("posScale", C.c_float * 3), ("valOffset", C.c_float),
                ("valScale", C.c_float), ("clamp", C.c_int), ("clampNeg", C.c_float), ("clampPos", C.c_float),
                ("timeAnim", C.c_float)]


class RefineParams(C.Structure):
    _fields_ = [("refineAccuracy", C.c_double), ("innerAccuracy", C.c_double), ("maxRefine", C.c_int)]


class RefineResult(C.Structure):
    _fields_ = [("refinements", C.c_int), ("iterations", C.c_int), ("resNorm", C.c_double)]


class MultigridLayout(C.Structure):
    _fields_ = [("levels", C.c_int), ("tailFirst", C.c_int), ("tailCtas", C.c_int),
                ("size", (C.c_int * 3) * 32), ("dictStencils", C.c_int * 32)]


# (name, restype, argtypes) of every exported entry point
_P = C.c_void_p
_I = C.c_int
_F = C.c_float
_FP = C.POINTER(C.c_float)
SIGNATURES = [
    ("mg_init", _I, [_I]),
    ("mg_shutdown", _I, []),
    ("mg_last_error", C.c_char_p, []),
    ("mg_version", _I, []),
    ("mg_device_count", _I, [C.POINTER(_I)]),
    ("mg_solver_create", _I, [_I, _I, _I, _I, C.POINTER(_P)]),
    ("mg_solver_destroy", _I, [_P]),
    ("mg_solver_set_dt", _I, [_P, _F]),
    ("mg_solver_get_dt", _I, [_P, _FP]),
    ("mg_solver_sync", _I, [_P]),
    ("mg_solver_memory", _I, [_P, C.POINTER(C.c_size_t)]),
    ("mg_solver_set_memory_limit", _I, [_P, C.c_size_t]),
    ("mg_solver_set_wait_limit", _I, [_P, C.c_longlong, _I]),
    ("mg_grid_create", _I, [_P, _I, C.POINTER(_P)]),
    ("mg_grid_destroy", _I, [_P]),
    ("mg_grid_upload", _I, [_P, _P, C.c_size_t]),
    ("mg_grid_download", _I, [_P, _P, C.c_size_t]),
    ("mg_grid_upload_async", _I, [_P, _P, C.c_size_t]),
    ("mg_grid_download_async", _I, [_P, _P, C.c_size_t]),
    ("mg_solver_wait_copies", _I, [_P]),
    ("mg_solver_size", _I, [_P, C.POINTER(_I), C.POINTER(_I), C.POINTER(_I)]),
    ("mg_grid_device", _I, [_P, C.POINTER(_P), C.POINTER(_P)]),
    ("mg_grid_get_info", _I, [_P, C.POINTER(_I), C.POINTER(_I), C.POINTER(_I), C.POINTER(_I)]),
    ("mg_grid_save", _I, [_P, C.c_char_p]),
    ("mg_grid_swap", _I, [_P, _P]),
    ("mg_grid_copy", _I, [_P, _P]),
    ("mg_grid_set_const", _I, [_P, _F, _F, _F]),
    ("mg_grid_join", _I, [_P, _P, _I]),
    ("mg_grid_get_max_abs", _I, [_P, _FP]),
    ("mg_host_alloc", _I, [C.c_size_t, C.POINTER(_P)]),
    ("mg_host_free", _I, [_P]),
    ("mg_advect_semi_lagrange", _I, [_P, _P, _P, _I, _F, _I, _I, _I, _I, _I]),
    ("mg_advect_semi_lagrange_noalloc", _I, [_P, _P, _P, _I, _F, _I, _I, _I, _I, _I]),
    ("mg_reset_phi_in_obs", _I, [_P, _P]),
    ("mg_set_wall_bcs", _I, [_P, _P, _P, _P, _P, _I]),
    ("mg_add_buoyancy", _I, [_P, _P, _P, _F, _F, _F, _F, _I]),
    ("mg_add_gravity", _I, [_P, _P, _F, _F, _F, _P, _I]),
    ("mg_add_gravity_no_scale", _I, [_P, _P, _F, _F, _F, _P]),
    ("mg_set_open_bound", _I, [_P, _I, C.c_char_p, _I]),
    ("mg_reset_outflow", _I, [_P, _P, _P]),
    ("mg_extrapolate_mac_simple", _I, [_P, _P, _I, _P, _I]),
    ("mg_extrapolate_ls_simple", _I, [_P, _I, _I]),
    ("mg_noise_params_default", None, [C.POINTER(NoiseParams)]),
    ("mg_noise_create", _I, [_P, _I, C.POINTER(_P)]),
    ("mg_noise_destroy", _I, [_P]),
    ("mg_noise_set_params", _I, [_P, C.POINTER(NoiseParams)]),
    ("mg_noise_seed_offset", _I, [_P, _FP]),
    ("mg_noise_evaluate_grid", _I, [_P, _P, _F]),
    ("mg_density_inflow", _I, [_P, _P, _P, _P, _F, _F, _F]),
    ("mg_shape_cylinder_levelset", _I, [_P, _FP, _F, _FP]),
    ("mg_particles_create", _I, [_P, C.c_longlong, C.POINTER(_P)]),
    ("mg_particles_destroy", _I, [_P]),
    ("mg_particles_upload", _I, [_P, _P, C.c_longlong]),
    ("mg_particles_download", _I, [_P, _P, C.c_longlong]),
    ("mg_particles_size", _I, [_P, C.POINTER(C.c_longlong)]),
    ("mg_pdata_create", _I, [_P, _I, C.POINTER(_P)]),
    ("mg_pdata_destroy", _I, [_P]),
    ("mg_pdata_upload", _I, [_P, _P, C.c_longlong]),
    ("mg_pdata_download", _I, [_P, _P, C.c_longlong]),
    ("mg_map_parts_to_mac", _I, [_P, _P, _P, _P, _P, _P, _P, _I]),
    ("mg_map_mac_to_parts", _I, [_P, _P, _P, _P, _P, _I]),
    ("mg_flip_velocity_update", _I, [_P, _P, _P, _P, _P, _F, _P, _I]),
    ("mg_map_parts_to_grid", _I, [_P, _P, _P, _P]),
    ("mg_map_grid_to_parts", _I, [_P, _P, _P]),
    ("mg_pressure_params_default", None, [C.POINTER(PressureParams)]),
    ("mg_solve_pressure", _I, [_P, _P, _P, C.POINTER(PressureParams), _P, _P, _P, _P, _P, _P,
                               C.POINTER(PressureResult)]),
    ("mg_refine_params_default", None, [C.POINTER(RefineParams)]),
    ("mg_solve_pressure_refined", _I, [_P, _P, _P, C.POINTER(PressureParams), _P, C.POINTER(RefineParams),
                                       C.POINTER(RefineResult)]),
    ("mg_batch_create", _I, [_I, C.POINTER(_I), _FP, C.POINTER(C.c_ulonglong), _F, C.POINTER(_P)]),
    ("mg_batch_destroy", _I, [_P]),
    ("mg_batch_set_solver", _I, [_P, _F, _F]),
    ("mg_batch_set_refinement", _I, [_P, C.c_double, C.c_double, _I]),
    ("mg_batch_set_preconditioner", _I, [_P, _I]),
    ("mg_batch_step", _I, [_P, C.POINTER(BatchStats)]),
    ("mg_batch_scene_iterations", _I, [_P, _I, C.POINTER(_I), _FP]),
    ("mg_batch_download", _I, [_P, _I, _I, _P, C.c_size_t]),
    ("mg_batch_noise", _I, [C.c_ulonglong, _I, C.c_longlong, _FP]),
    ("mg_batch_info", _I, [_P, C.POINTER(_I), C.POINTER(C.c_longlong), C.POINTER(C.c_longlong),
                           C.POINTER(C.c_size_t)]),
    ("mg_batch_sync", _I, [_P]),
    ("mg_batch_tuning", _I, [_P, C.POINTER(_I), _FP]),
    ("mg_serve_create", _I, [C.c_size_t, _F, C.POINTER(_P)]),
    ("mg_serve_destroy", _I, [_P]),
    ("mg_serve_set_solver", _I, [_P, _F, _F]),
    ("mg_serve_job_bytes", C.c_size_t, [_I, _I, _I]),
    ("mg_serve_submit", _I, [_P, _I, _I, _I, _FP, C.c_ulonglong, _I, C.c_double, _I, C.POINTER(_I)]),
    ("mg_serve_submit_kind", _I, [_P, _I, _I, _I, _I, C.POINTER(C.c_float), C.c_ulonglong, _I, C.c_double, _I, C.POINTER(_I)]),
    ("mg_serve_job_bytes_kind", C.c_size_t, [_I, _I, _I, _I]),
    ("mg_serve_run", _I, [_P, C.POINTER(ServeStats)]),
    ("mg_serve_job_info", _I, [_P, _I, C.POINTER(ServeJob)]),
    ("mg_serve_job_result", _I, [_P, _I, _I, _P, C.c_size_t]),
    ("mg_serve_ticks", _I, [_P, C.POINTER(_I), _FP, C.POINTER(_I)]),
    ("mg_compute_pressure_rhs", _I, [_P, _P, _P, _P, C.POINTER(PressureParams), _P, _P, _P, _P, _P]),
    ("mg_solve_pressure_system", _I, [_P, _P, _P, _P, C.POINTER(PressureParams), _P, _P, _P, _P,
                                      C.POINTER(PressureResult)]),
    ("mg_correct_velocity", _I, [_P, _P, _P, C.POINTER(PressureParams), _P, _P, _P, _P]),
    ("mg_release_mg", _I, [_P]),
    ("mg_multigrid_vcycle", _I, [_P, _P, _P, _P, _F, _F]),
    ("mg_multigrid_describe", _I, [_P, _P]),
    ("mg_flags_init_domain", _I, [_P, _I, C.c_char_p, C.c_char_p, C.c_char_p, C.c_char_p, _P]),
    ("mg_flags_fill_grid", _I, [_P, _I]),
    ("mg_flags_update_from_levelset", _I, [_P, _P]),
    ("mg_shape_box_apply", _I, [_P, _FP, _FP, _FP, _I, _P]),
    ("mg_shape_cylinder_apply", _I, [_P, _FP, _F, _FP, _FP, _I, _P]),
    ("mg_shape_box_levelset", _I, [_P, _FP, _FP]),
    ("mg_profile_enable", _I, [_P, _I]),
    ("mg_profile_read", _I, [_P, C.POINTER(_I), C.POINTER(C.c_char_p), C.POINTER(C.c_double),
                             C.POINTER(C.c_longlong)]),
    ("mg_profile_reset", _I, [_P]),
    ("mg_mark", _I, [_P, _I]),
    ("mg_elapsed", _I, [_P, _I, _I, _FP]),
    ("mg_launch_count", _I, [C.POINTER(C.c_longlong)]),
]


def load(path=LIB_PATH, build_if_missing=True):
    """Load (building first if needed) libmantagpu and declare its ABI."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(path) and build_if_missing:
            from . import build as _build
            _build.build()
        if not os.path.exists(path):
            raise ImportError("libmantagpu.so is missing: run `python -m mantaflow_gb300.build` "
                              "(needs nvcc for sm_103a)")
        L = C.CDLL(path)
        for name, res, args in SIGNATURES:
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
        return L


class MantaError(RuntimeError):
    """Raised where the reference raises Manta::Error (a RuntimeError in Python)."""


def check(status):
    if status != 0:
        msg = load().mg_last_error()
        raise MantaError(msg.decode() if msg else "libmantagpu error %d" % status)
    return status


_init_device = None


def ensure_init(device=None):
    """Initialise the library on `device` (default: $MANTA_GB300_DEVICE or 0)."""
    global _init_device
    L = load()
    if _init_device is None:
        dev = int(os.environ.get("MANTA_GB300_DEVICE", "0")) if device is None else int(device)
        check(L.mg_init(dev))
        _init_device = dev
    return L


def fptr(vals):
    arr = (C.c_float * len(vals))(*[float(v) for v in vals])
    return arr
