"""Batched form: many independent smoke-plume scenes stepped together on
one GPU (mg_batch_* of include/mantagpu.h).

Every scene is the reference's plume (walls, open top, cylinder source with
seeded uniform inflow noise, buoyancy, MacCormack advection, setWallBcs,
addBuoyancy, solvePressure), with its own size, gravity and noise seed.
Each stage of a step is one launch over the tiles of all scenes; the
pressure solve iterates until every scene has converged.
"""
import ctypes as C

import numpy as np

from . import _lib
from ._lib import check, ensure_init

DENSITY, VELOCITY, PRESSURE, FLAGS, SOURCE = 0, 1, 2, 3, 4


class BatchedPlumes:
    def __init__(self, sizes, gravity, seeds, dt=1.0, cgAccuracy=1e-3, cgMaxIterFac=1.5, preconditioner=1):
        """preconditioner: 1 (PcMIC, the default: MIC(0) for the 3D scenes, none
        in 2D as the reference's GridCg) or 0 (no scene preconditioned)"""
        ensure_init()
        self._L = _lib.load()
        sizes = [tuple(int(v) for v in s) + ((1,) if len(s) == 2 else ()) for s in sizes]
        self.sizes = [s[:3] for s in sizes]
        n = len(self.sizes)
        sz = (C.c_int * (3 * n))(*[v for s in self.sizes for v in s])
        gr = (C.c_float * (3 * n))(*[float(v) for g in gravity for v in g])
        sd = (C.c_ulonglong * n)(*[int(x) for x in seeds])
        self.seeds = [int(x) for x in seeds]
        h = C.c_void_p()
        check(self._L.mg_batch_create(n, sz, gr, sd, float(dt), C.byref(h)))
        self._h = h
        check(self._L.mg_batch_set_solver(h, float(cgAccuracy), float(cgMaxIterFac)))
        check(self._L.mg_batch_set_preconditioner(h, int(preconditioner)))
        self.steps = 0

    def set_refinement(self, refineAccuracy=1e-5, innerAccuracy=1e-2, maxRefine=10):
        """FP64 residual refinement of every scene's pressure solve
        (refineAccuracy 0: off)"""
        check(self._L.mg_batch_set_refinement(self._h, float(refineAccuracy), float(innerAccuracy), int(maxRefine)))

    def __len__(self):
        return len(self.sizes)

    def step(self):
        st = _lib.BatchStats()
        check(self._L.mg_batch_step(self._h, C.byref(st)))
        self.steps += 1
        return {"sweeps": st.sweeps, "max_iterations": st.maxIterations, "total_iterations": st.totalIterations,
                "graph_launches": st.graphLaunches}

    def iterations(self, scene):
        it = C.c_int()
        res = C.c_float()
        check(self._L.mg_batch_scene_iterations(self._h, int(scene), C.byref(it), C.byref(res)))
        return it.value, res.value

    def _shape(self, scene):
        nx, ny, nz = self.sizes[scene]
        return (nz, ny, nx)

    def download(self, scene, what):
        shape = self._shape(scene)
        if what == VELOCITY:
            a = np.empty(shape + (3,), np.float32)
        elif what == FLAGS:
            a = np.empty(shape, np.int32)
        else:
            a = np.empty(shape, np.float32)
        check(self._L.mg_batch_download(self._h, int(scene), int(what), a.ctypes.data_as(C.c_void_p), a.nbytes))
        return a

    def inflow(self, scene, step):
        """density source the batch joins into scene `scene` at `step`:
        U[0,1) noise times the cylinder mask"""
        shape = self._shape(scene)
        u = np.empty(shape, np.float32)
        check(self._L.mg_batch_noise(C.c_ulonglong(self.seeds[scene]), int(step), u.size,
                                     u.ctypes.data_as(C.POINTER(C.c_float))))
        return (u * self.download(scene, SOURCE)).astype(np.float32)

    def info(self):
        c = C.c_int()
        cells = C.c_longlong()
        tiles = C.c_longlong()
        nbytes = C.c_size_t()
        check(self._L.mg_batch_info(self._h, C.byref(c), C.byref(cells), C.byref(tiles), C.byref(nbytes)))
        return {"scenes": c.value, "cells": cells.value, "tiles": tiles.value, "bytes": nbytes.value}

    def tuning(self):
        """(CG sweep tile height chosen by the autotuner, timings per candidate)"""
        rows = C.c_int()
        ms = (C.c_float * 4)()
        check(self._L.mg_batch_tuning(self._h, C.byref(rows), ms))
        return rows.value, list(ms)

    def sync(self):
        check(self._L.mg_batch_sync(self._h))

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self._L.mg_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


PLUME, DAM_BREAK = 0, 1


class PlumeServer:
    """Served form: a request loop for plume and dam-break jobs with
    device-memory admission and continuous batching (mg_serve_* of
    include/mantagpu.h)."""

    def __init__(self, budget_bytes=150 * 10 ** 9, dt=1.0, cgAccuracy=1e-3, cgMaxIterFac=1.5):
        ensure_init()
        self._L = _lib.load()
        h = C.c_void_p()
        check(self._L.mg_serve_create(int(budget_bytes), float(dt), C.byref(h)))
        self._h = h
        check(self._L.mg_serve_set_solver(h, float(cgAccuracy), float(cgMaxIterFac)))
        self.shapes = []

    @staticmethod
    def job_bytes(size, kind=PLUME):
        nx, ny, nz = (tuple(size) + (1,))[:3]
        return int(_lib.load().mg_serve_job_bytes_kind(int(kind), nx, ny, nz))

    def submit(self, size, gravity, seed, steps, arrival=0.0, keep=False, kind=PLUME):
        """kind PLUME (0) or DAM_BREAK (1); a dam-break job's DENSITY result is
        its levelset phi"""
        nx, ny, nz = (tuple(int(v) for v in size) + (1,))[:3]
        g = (C.c_float * 3)(*[float(v) for v in gravity])
        jid = C.c_int()
        check(self._L.mg_serve_submit_kind(self._h, int(kind), nx, ny, nz, g, C.c_ulonglong(int(seed)), int(steps),
                                           float(arrival), int(bool(keep)), C.byref(jid)))
        self.shapes.append((nz, ny, nx))
        return jid.value

    def run(self):
        st = _lib.ServeStats()
        check(self._L.mg_serve_run(self._h, C.byref(st)))
        return {"jobs": st.jobs, "ticks": st.ticks, "wall_s": st.wallSeconds, "cell_steps": st.cellSteps,
                "peak_bytes": st.peakBytes}

    def job(self, jid):
        j = _lib.ServeJob()
        check(self._L.mg_serve_job_info(self._h, int(jid), C.byref(j)))
        return {"arrival": j.arrival, "admitted": j.admitted, "finished": j.finished, "steps": j.steps,
                "mean_step_ms": j.meanStepMs}

    def result(self, jid, what):
        shape = self.shapes[jid] + ((3,) if what == VELOCITY else ())
        a = np.empty(shape, np.float32)
        check(self._L.mg_serve_job_result(self._h, int(jid), int(what), a.ctypes.data_as(C.c_void_p), a.nbytes))
        return a

    def ticks(self):
        n = C.c_int(0)
        check(self._L.mg_serve_ticks(self._h, C.byref(n), None, None))
        ms = (C.c_float * max(1, n.value))()
        jobs = (C.c_int * max(1, n.value))()
        cap = C.c_int(n.value)
        check(self._L.mg_serve_ticks(self._h, C.byref(cap), ms, jobs))
        return list(ms)[: n.value], list(jobs)[: n.value]

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self._L.mg_serve_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
