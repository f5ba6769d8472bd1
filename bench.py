"""Throughput of the grid-step hot path on GB300.

Workload: the 3D smoke plume at 256^3 (float32 MAC grid, walls with an open
top, cylinder source with seeded uniform inflow noise, buoyancy (0,-4e-3,0),
dt = 1, MacCormack advection of density and velocity with clampMode 2,
setWallBcs, addBuoyancy, solvePressure at cgAccuracy 1e-3 with the static
multigrid preconditioner -- the reference's fastest solver for this scene;
--pc mic selects MIC(0), which is also measured and reported beside the
headline).  One step is that full sequence; the metric is cells / step time.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Multi-GPU runs (torchrun) are independent replicas, one scene per GPU:
value = all ranks' cells / the slowest rank's time ("scaling": "weak").
Prints one JSON line (rank 0).
"""
import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "cell-updates/s per full step at 256³; batched sims/h + p99 latency vs plain"

# Algorithmic bytes per cell of each kernel family, in the formulation the
# kernel implements (inputs read once, outputs written once; gathered
# neighbours count once; matrix-free Poisson stencil codes of 2 B per cell).
BYTES_PER_CELL = {
    "mic_forward": 4 + 4 + 2 + 4,           # r, P, code -> z
    "mic_backward": 4 + 4 + 2 + 4 + 4,      # z, P, code, r (fused dot) -> z
    "mic_init": 4 + 2 + 4,                  # A0/code (+GF diag) -> P
    "pcg_spmv": 4 + 2 + 4,                  # search, code -> tmp (+dot)
    "pcg_axpy": 4 + 4 + 4 + 4 + 4 + 4,      # p, s, r, tmp -> p, r (+max-abs)
    "pcg_update": 4 + 4 + 4,                # tmp, s -> s
    "pcg_init": 4 + 4 + 4 + 4,              # rhs -> p, r, tmp
    "pcg_set_search": 4 + 4 + 4,            # tmp, r -> search (+dot)
    "advect_real_fwd": 12 + 4 + 4,          # vel, src -> fwd
    "advect_real_maccormack": 12 + 4 + 4 + 4 + 4,  # vel, fwd, orig, flags -> new
    "advect_mac_fwd": 12 + 12,              # vel (= src) -> fwd
    "advect_mac_maccormack": 12 + 12 + 4 + 12,     # vel (= orig), fwd, flags -> new
    "advect_outflow": 4,                    # flags (outflow cells only do work)
    "set_wall_bcs": 4 + 12 + 12,
    "add_buoyancy": 4 + 4 + 12 + 12,
    "make_rhs": 4 + 12 + 4,
    "make_codes": 4 + 2 + 2 + 2,
    "correct_velocity": 4 + 4 + 12 + 12,
    "join": 4 + 4 + 4,
    # multigrid V-cycle, level 0 (bytes per fine cell; the level-1 vectors
    # are 1/8 of the cells)
    "mg_down_l0": 2 + 4 + 4 + 4,            # code, residual -> x (pre-smoothed), r
    "mg_up_l0": 2 + 4 + 4 + 0.5 + 4,        # code, residual, x, level-1 x -> x (+dot)
    "mg_restrict_l0": 4 + 0.5,              # r -> level-1 b
    "mg_dot": 4 + 4,                        # z, residual (+dot)
}


# the advection and SpMV families, each reported against its own roofline
ROOFLINE_FAMILIES = ("advect_mac_fwd", "advect_mac_maccormack", "advect_real_fwd", "advect_real_maccormack",
                     "pcg_spmv", "mg_up_l0", "mg_down_l0")


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = max(smax, float(parts[2]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


class Plume:
    """The plume scene on the GPU through the scene-script API."""

    def __init__(self, m, n, pc, seed, nsteps_noise):
        self.m, self.n, self.pc = m, n, pc
        s = m.Solver(name="plume%d" % n, gridSize=m.vec3(n, n, n), dim=3)
        s.timestep = 1.0
        self.s = s
        gs = m.vec3(n, n, n)
        self.flags = s.create(m.FlagGrid)
        self.flags.initDomain(boundaryWidth=0)
        self.flags.fillGrid()
        m.setOpenBound(self.flags, 0, "Y", m.FlagOutflow | m.FlagEmpty)
        self.vel = s.create(m.MACGrid)
        self.density = s.create(m.RealGrid)
        self.pressure = s.create(m.RealGrid)
        mask = s.create(m.RealGrid)
        src = s.create(m.Cylinder, center=gs * m.vec3(0.5, 0.1, 0.5), radius=n * 0.14, z=gs * m.vec3(0, 0.02, 0))
        src.applyToGrid(grid=mask, value=1.0)
        self.mask = mask.numpy()
        self.rng = np.random.default_rng(seed)
        self.iters = []
        self.refined = False
        self.refine_stats = []

    def noise(self):
        n = self.n
        return (self.rng.random((n, n, n), dtype=np.float32) * self.mask).astype(np.float32)

    def step(self, noise_grid):
        m = self.m
        self.density.join(noise_grid)
        m.advectSemiLagrange(flags=self.flags, vel=self.vel, grid=self.density, order=2, clampMode=2)
        m.advectSemiLagrange(flags=self.flags, vel=self.vel, grid=self.vel, order=2, clampMode=2)
        m.setWallBcs(flags=self.flags, vel=self.vel)
        m.addBuoyancy(density=self.density, vel=self.vel, gravity=m.vec3(0, -4e-3, 0), flags=self.flags)
        if self.refined:
            self.refine_stats.append(m.solvePressureRefined(flags=self.flags, vel=self.vel, pressure=self.pressure,
                                                            cgAccuracy=1e-3, refineAccuracy=1e-5,
                                                            preconditioner=self.pc)[:2])
        else:
            m.solvePressure(flags=self.flags, vel=self.vel, pressure=self.pressure, cgAccuracy=1e-3,
                            preconditioner=self.pc)
        self.iters.append(m.lastSolveStats()[0])


PC_NAMES = {"mic": "MIC(0)-PCG (PcMIC)", "mgstatic": "multigrid-PCG (PcMGStatic)",
            "mgdynamic": "multigrid-PCG (PcMGDynamic)"}


def workload(n, pcname):
    return "3D smoke plume %d^3, MacCormack advection + %s, cgAccuracy 1e-3" % (n, PC_NAMES[pcname])


def cpu_plume_steps(n, steps, warm, threads, seed, state=None, pc=1):
    """The same plume step with the CPU oracle (OpenMP sweeps, serial MIC as
    in the reference).  Returns (seconds per timed step list, iterations)."""
    from oracle import oracle as og
    og.set_num_threads(threads)
    f = np.zeros((n, n, n), np.int32)
    og.init_domain(f, 0)
    og.fill_grid(f)
    og.set_open_bound(f, 0, "Y")
    mask = np.zeros((n, n, n), np.float32)
    gs = np.float32([n, n, n])
    og.cylinder_apply(mask, gs * np.float32([0.5, 0.1, 0.5]), np.float32(n * 0.14), gs * np.float32([0, 0.02, 0]), 1.0)
    if state is None:
        dens = np.zeros((n, n, n), np.float32)
        vel = np.zeros((n, n, n, 3), np.float32)
    else:
        dens, vel = state
    pres = np.zeros((n, n, n), np.float32)
    rng = np.random.default_rng(seed)
    times, iters = [], []
    for t in range(warm + steps):
        a = (rng.random((n, n, n), dtype=np.float32) * mask).astype(np.float32)
        t0 = time.perf_counter()
        og.join_real(dens, a)
        og.advect_semi_lagrange(f, vel, dens, og.KIND_REAL, order=2, clampMode=2)
        og.advect_semi_lagrange(f, vel, vel, og.KIND_MAC, order=2, clampMode=2)
        og.set_wall_bcs(f, vel)
        og.add_buoyancy(f, dens, vel, (0, -4e-3, 0))
        it, _, _ = og.solve_pressure(f, vel, pres, cgAccuracy=1e-3, preconditioner=pc)
        dt = time.perf_counter() - t0
        if t >= warm:
            times.append(dt)
            iters.append(it)
    og.set_num_threads(1)
    return times, iters


def precision_form(m, n, steps, seed):
    """Config-2 precision form on a bounded sample: the plume for `steps`
    steps at n^3 through the plain FP32 path (cgAccuracy 1e-3, PcMIC and
    PcMGStatic) and through the FP64-refined solve (target 1e-5), each
    against the FP64 oracle (the reference's double build restated, PcMIC
    at cgAccuracy 1e-5).  Per field: max-abs error and relative L2 error."""
    from oracle import oracle as og
    og.set_num_threads(os.cpu_count() or 1)
    f = np.zeros((n, n, n), np.int32)
    og.init_domain(f, 0)
    og.fill_grid(f)
    og.set_open_bound(f, 0, "Y")
    mask = np.zeros((n, n, n), np.float32)
    gs = np.float32([n, n, n])
    og.cylinder_apply(mask, gs * np.float32([0.5, 0.1, 0.5]), np.float32(n * 0.14), gs * np.float32([0, 0.02, 0]), 1.0)
    rng = np.random.default_rng(seed)
    noise = [(rng.random(f.shape, dtype=np.float32) * mask).astype(np.float32) for _ in range(steps)]

    def divergence(vel):
        rhs = np.zeros(f.shape, np.float64)
        og.compute_pressure_rhs(rhs, vel.astype(np.float64), f)
        return rhs

    d64 = np.zeros(f.shape, np.float64)
    v64 = np.zeros(f.shape + (3,), np.float64)
    p64 = np.zeros(f.shape, np.float64)
    for t in range(steps):
        og.join_real(d64, noise[t].astype(np.float64))
        og.advect_semi_lagrange(f, v64, d64, og.KIND_REAL, order=2, clampMode=2)
        og.advect_semi_lagrange(f, v64, v64, og.KIND_MAC, order=2, clampMode=2)
        og.set_wall_bcs(f, v64)
        og.add_buoyancy(f, d64, v64, (0, -4e-3, 0))
        og.solve_pressure(f, v64, p64, cgAccuracy=1e-5, preconditioner=og.PC_MIC)
    div64 = divergence(v64)
    og.set_num_threads(1)

    def err(a, b):
        a = np.asarray(a, np.float64)
        return {"max_abs": float(np.max(np.abs(a - b))),
                "rel_l2": float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))}

    out = {"workload": "3D smoke plume %d^3, %d steps, MacCormack + walls + buoyancy + pressure" % (n, steps),
           "fp64_oracle": "oracle restatement compiled as the reference's double build, PcMIC, cgAccuracy 1e-5"}
    for name, pc, refined in (("fp32_pcmic_acc1e-3", m.PcMIC, False), ("fp32_pcmgstatic_acc1e-3", m.PcMGStatic, False),
                              ("fp32_refined_fp64_to_1e-5", m.PcMGStatic, True)):
        s = m.Solver(name="prec", gridSize=m.vec3(n, n, n), dim=3)
        flags = s.create(m.FlagGrid)
        m.copyArrayToGridReal(f, flags)
        vel, dens, pres, src = s.create(m.MACGrid), s.create(m.RealGrid), s.create(m.RealGrid), s.create(m.RealGrid)
        for t in range(steps):
            m.copyArrayToGridReal(noise[t], src)
            dens.join(src)
            m.advectSemiLagrange(flags=flags, vel=vel, grid=dens, order=2, clampMode=2)
            m.advectSemiLagrange(flags=flags, vel=vel, grid=vel, order=2, clampMode=2)
            m.setWallBcs(flags=flags, vel=vel)
            m.addBuoyancy(density=dens, vel=vel, gravity=m.vec3(0, -4e-3, 0), flags=flags)
            if refined:
                m.solvePressureRefined(flags=flags, vel=vel, pressure=pres, refineAccuracy=1e-5, preconditioner=pc)
            else:
                m.solvePressure(flags=flags, vel=vel, pressure=pres, cgAccuracy=1e-3, preconditioner=pc)
        v = vel.numpy()
        out[name] = {"density": err(dens.numpy(), d64), "velocity": err(v, v64), "pressure": err(pres.numpy(), p64),
                     "divergence": err(divergence(v), div64)}
        del s
    return out


def batch_config(seed, n2=512, n3=64):
    """Config 4: 512 2D scenes with sides round(exp(U[ln 64, ln 512])) and 64
    3D scenes with sides U{32..96}; buoyancy magnitudes U[1e-3, 8e-3]."""
    rng = np.random.default_rng(seed)
    sizes = [(int(round(np.exp(rng.uniform(np.log(64), np.log(512))))),) * 2 + (1,) for _ in range(n2)]
    sizes += [(int(rng.integers(32, 97)),) * 3 for _ in range(n3)]
    grav = [(0.0, -float(g), 0.0) for g in rng.uniform(1e-3, 8e-3, len(sizes))]
    seeds = [int(x) for x in rng.integers(1, 2 ** 62, len(sizes))]
    return sizes, grav, seeds


def _plain_plume(m, size, grav):
    """one plume scene on the plain per-scene path"""
    nx, ny, nz = size
    s = m.Solver(name="plain", gridSize=m.vec3(nx, ny, nz), dim=3 if nz > 1 else 2)
    flags = s.create(m.FlagGrid)
    flags.initDomain(boundaryWidth=0)
    flags.fillGrid()
    m.setOpenBound(flags, 0, "Y", m.FlagOutflow | m.FlagEmpty)
    g = {"s": s, "flags": flags, "vel": s.create(m.MACGrid), "dens": s.create(m.RealGrid),
         "pres": s.create(m.RealGrid), "src": s.create(m.RealGrid), "grav": m.vec3(*grav)}
    gs = m.vec3(nx, ny, nz)
    mask = s.create(m.RealGrid)
    s.create(m.Cylinder, center=gs * m.vec3(0.5, 0.1, 0.5), radius=nx * 0.14,
             z=gs * m.vec3(0, 0.02, 0)).applyToGrid(grid=mask, value=1.0)
    g["mask"] = mask.numpy()
    return g


def _plain_step(m, g, inflow):
    m.copyArrayToGridReal(inflow, g["src"])
    g["dens"].join(g["src"])
    m.advectSemiLagrange(flags=g["flags"], vel=g["vel"], grid=g["dens"], order=2, clampMode=2)
    m.advectSemiLagrange(flags=g["flags"], vel=g["vel"], grid=g["vel"], order=2, clampMode=2)
    m.setWallBcs(flags=g["flags"], vel=g["vel"])
    m.addBuoyancy(density=g["dens"], vel=g["vel"], gravity=g["grav"], flags=g["flags"])
    m.solvePressure(flags=g["flags"], vel=g["vel"], pressure=g["pres"], cgAccuracy=1e-3, preconditioner=m.PcMIC)


def batch_accuracy(m, sizes, grav, seeds, pick, steps):
    """Batched and plain results of a few scenes after `steps` steps from
    rest (same inflow), each against the FP64 oracle (the reference's double
    build restated, cgAccuracy 1e-5): per-field relative L2 errors."""
    from mantaflow_gb300 import batch as mb
    from oracle import oracle as og
    og.set_num_threads(os.cpu_count() or 1)
    b = mb.BatchedPlumes([sizes[i] for i in pick], [grav[i] for i in pick], [seeds[i] for i in pick])
    for _ in range(steps):
        b.step()
    rows = []
    for q, i in enumerate(pick):
        nx, ny, nz = sizes[i]
        inflow = [b.inflow(q, t) for t in range(steps)]
        g = _plain_plume(m, sizes[i], grav[i])
        for t in range(steps):
            _plain_step(m, g, inflow[t])
        f = g["flags"].numpy()
        d64 = np.zeros(f.shape, np.float64)
        v64 = np.zeros(f.shape + (3,), np.float64)
        p64 = np.zeros(f.shape, np.float64)
        for t in range(steps):
            og.join_real(d64, inflow[t].astype(np.float64))
            og.advect_semi_lagrange(f, v64, d64, og.KIND_REAL, order=2, clampMode=2)
            og.advect_semi_lagrange(f, v64, v64, og.KIND_MAC, order=2, clampMode=2)
            og.set_wall_bcs(f, v64)
            og.add_buoyancy(f, d64, v64, grav[i])
            og.solve_pressure(f, v64, p64, cgAccuracy=1e-5, preconditioner=og.PC_MIC)

        def rel(a, ref):
            a = np.asarray(a, np.float64)
            return float(np.linalg.norm(a - ref) / max(np.linalg.norm(ref), 1e-30))

        rows.append({"size": [nx, ny, nz],
                     "batched_rel_l2": {"density": rel(b.download(q, mb.DENSITY), d64),
                                        "velocity": rel(b.download(q, mb.VELOCITY), v64),
                                        "pressure": rel(b.download(q, mb.PRESSURE), p64)},
                     "plain_rel_l2": {"density": rel(g["dens"].numpy(), d64), "velocity": rel(g["vel"].numpy(), v64),
                                      "pressure": rel(g["pres"].numpy(), p64)}})
        del g
    b.close()
    og.set_num_threads(1)
    return {"steps": steps, "fp64_oracle": "oracle restatement compiled as the reference's double build, PcMIC, "
                                           "cgAccuracy 1e-5", "scenes": rows}


def batched_form(m, steps, seed, plain_steps, acc_steps, sim_steps=100):
    """Config 4, batched against plain: the whole batch for `steps` steps,
    and the plain per-scene path (one solver per scene, scenes one after
    another) on every scene of the batch with the same solver (PcMIC in 3D,
    no preconditioner in 2D as GridCg); sims/hour for `sim_steps`-step
    simulations, per-step latency percentiles, and the accuracy of both
    paths against the FP64 oracle on a few scenes."""
    from mantaflow_gb300 import batch as mb
    sizes, grav, seeds = batch_config(seed)
    b = mb.BatchedPlumes(sizes, grav, seeds)
    info = b.info()
    b.step()  # untimed first step
    b.sync()
    lat, sweeps = [], []
    for _ in range(steps):
        t0 = time.perf_counter()
        st = b.step()
        lat.append(time.perf_counter() - t0)
        sweeps.append(st["sweeps"])
    tune = b.tuning()
    b.close()
    per_step = statistics.mean(lat)
    batched = {"sims_per_hour": len(sizes) * 3600.0 / (per_step * sim_steps), "step_ms_mean": 1e3 * per_step,
               "step_ms_p50": 1e3 * float(np.percentile(lat, 50)), "step_ms_p99": 1e3 * float(np.percentile(lat, 99)),
               "cells_per_s": info["cells"] / per_step, "cg_sweeps_per_step": sweeps, "steps_timed": steps,
               "preconditioner": "MIC(0) in 3D scenes (one dataflow launch over all 3D scenes), none in 2D",
               "autotuned_sweep_tile": {"rows": tune[0], "ms_per_8_sweeps_for_8_16_32_64_rows": tune[1]}}
    # plain: every scene, one after another
    per_scene, plain_lat = [], []
    for i in range(len(sizes)):
        g = _plain_plume(m, sizes[i], grav[i])
        rng = np.random.default_rng(seeds[i] % (2 ** 32))
        nx, ny, nz = sizes[i]
        ts = []
        for t in range(plain_steps + 1):
            a = (rng.random((nz, ny, nx), dtype=np.float32) * g["mask"]).astype(np.float32)
            g["s"].sync()
            t0 = time.perf_counter()
            _plain_step(m, g, a)
            g["s"].sync()
            if t > 0:
                ts.append(time.perf_counter() - t0)
        per_scene.append(statistics.mean(ts))
        plain_lat += ts
        del g
    est = sum(per_scene)  # seconds per step of all scenes, one after another
    plain = {"sims_per_hour": len(sizes) * 3600.0 / (est * sim_steps), "step_ms_p50": 1e3 * float(np.percentile(plain_lat, 50)),
             "step_ms_p99": 1e3 * float(np.percentile(plain_lat, 99)), "all_scenes_step_s": est,
             "sample": "every scene, %d timed steps each after one untimed (seeded uniform inflow noise in the "
                       "cylinder source; solver identical to the batch's)" % plain_steps}
    order2 = sorted(range(512), key=lambda i: sizes[i][0])
    order3 = sorted(range(512, len(sizes)), key=lambda i: sizes[i][0])
    pick = [order2[len(order2) // 4], order2[len(order2) // 2], order3[len(order3) // 4], order3[len(order3) // 2]]
    acc = batch_accuracy(m, sizes, grav, seeds, pick, acc_steps) if acc_steps > 0 else None
    return {"workload": "config 4: %d 2D plume scenes (sides log-uniform in [64,512]) + %d 3D (sides U{32..96}), "
                        "buoyancy U[1e-3,8e-3], cgAccuracy 1e-3; %d-step simulations" % (512, len(sizes) - 512, sim_steps),
            "scenes": len(sizes), "cells": info["cells"], "tiles": info["tiles"], "device_bytes": info["bytes"],
            "batched": batched, "plain_per_scene": plain, "speedup_sims_per_hour":
                batched["sims_per_hour"] / plain["sims_per_hour"], "accuracy_vs_fp64": acc}


def _plain_dam(m, n):
    """the dam-break scene (config 3's setup) on the plain per-scene path"""
    s = m.Solver(name="dam", gridSize=m.vec3(n, n, n), dim=3)
    s.timestep = 1.0
    flags = s.create(m.FlagGrid)
    flags.initDomain(boundaryWidth=0)
    box = s.create(m.Box, p0=m.vec3(0, 0, 0), p1=m.vec3(n * 0.4, n * 0.6, n))
    phi = box.computeLevelset()
    flags.updateFromLevelset(phi)
    return {"s": s, "flags": flags, "phi": phi, "vel": s.create(m.MACGrid), "pres": s.create(m.RealGrid)}


def _plain_dam_step(m, g):
    m.extrapolateMACSimple(flags=g["flags"], vel=g["vel"], distance=4)
    m.advectSemiLagrange(flags=g["flags"], vel=g["vel"], grid=g["phi"], order=1)
    g["flags"].updateFromLevelset(g["phi"])
    m.advectSemiLagrange(flags=g["flags"], vel=g["vel"], grid=g["vel"], order=1)
    m.addGravity(flags=g["flags"], vel=g["vel"], gravity=m.vec3(0, -1e-3, 0))
    m.setWallBcs(flags=g["flags"], vel=g["vel"])
    m.solvePressure(flags=g["flags"], vel=g["vel"], pressure=g["pres"], phi=g["phi"])
    m.setWallBcs(flags=g["flags"], vel=g["vel"])


def served_form(m, seed, njobs, plain_sample, rate=20.0, budget=150 * 10 ** 9):
    """Config 5: a Poisson stream (rate jobs/s) of 3D jobs, half smoke plume
    and half dam break, sides U{32..128}, steps U{100..400}, per-job seeds;
    served (continuous batching under the HBM budget) against the plain
    sequential path (each job alone through the scene API, first come first
    served).  The plain path's time per job is its measured step time
    (`plain_sample` steps after one untimed) times the job's steps; its job
    latencies follow from the arrivals in first-come order."""
    from mantaflow_gb300 import batch as mb
    rng = np.random.default_rng(seed)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, njobs))
    sides = rng.integers(32, 129, njobs)
    steps = rng.integers(100, 401, njobs)
    kinds = rng.integers(0, 2, njobs)
    grav = rng.uniform(1e-3, 8e-3, njobs)
    seeds = rng.integers(1, 2 ** 62, njobs)
    srv = mb.PlumeServer(budget_bytes=budget)
    ids = [srv.submit((int(n),) * 3, (0.0, -(float(g) if kd == 0 else 1e-3), 0.0), int(sd), int(k), float(a),
                      kind=int(kd))
           for n, g, sd, k, a, kd in zip(sides, grav, seeds, steps, arrivals, kinds)]
    st = srv.run()
    infos = [srv.job(q) for q in ids]
    tick_ms, tick_jobs = srv.ticks()
    srv.close()
    step_lat = np.repeat(tick_ms, tick_jobs)  # every resident job's step took the tick
    job_lat = np.array([i["finished"] - i["arrival"] for i in infos])
    served = {"cells_per_s": st["cell_steps"] / st["wall_s"], "wall_s": st["wall_s"], "ticks": st["ticks"],
              "step_ms_p50": float(np.percentile(step_lat, 50)), "step_ms_p99": float(np.percentile(step_lat, 99)),
              "job_s_p50": float(np.percentile(job_lat, 50)), "job_s_p99": float(np.percentile(job_lat, 99)),
              "peak_device_bytes": st["peak_bytes"], "max_resident_jobs": int(max(tick_jobs))}
    # plain sequential path: each job's step time measured, one job at a time
    job_time, plain_steps, cell_steps = [], [], 0
    for n, g, sd, k, kd in zip(sides, grav, seeds, steps, kinds):
        n = int(n)
        ts = []
        if kd == 0:
            pg = _plain_plume(m, (n, n, n), (0.0, -float(g), 0.0))
            r = np.random.default_rng(int(sd) % (2 ** 32))
        else:
            pg = _plain_dam(m, n)
        for t in range(plain_sample + 1):
            if kd == 0:
                a = (r.random((n, n, n), dtype=np.float32) * pg["mask"]).astype(np.float32)
            pg["s"].sync()
            t0 = time.perf_counter()
            if kd == 0:
                _plain_step(m, pg, a)
            else:
                _plain_dam_step(m, pg)
            pg["s"].sync()
            if t > 0:
                ts.append(time.perf_counter() - t0)
        plain_steps += ts
        job_time.append(statistics.mean(ts) * int(k))
        cell_steps += n ** 3 * int(k)
        del pg
    end, plain_lat = 0.0, []
    for a, jt in zip(arrivals, job_time):
        end = max(end, float(a)) + jt
        plain_lat.append(end - float(a))
    plain = {"cells_per_s": cell_steps / end, "wall_s": end,
             "step_ms_p50": 1e3 * float(np.percentile(plain_steps, 50)),
             "step_ms_p99": 1e3 * float(np.percentile(plain_steps, 99)),
             "job_s_p50": float(np.percentile(plain_lat, 50)), "job_s_p99": float(np.percentile(plain_lat, 99)),
             "sample": "each job's step time measured over %d steps after one untimed, times its steps; "
                       "first-come-first-served schedule from the arrivals" % plain_sample}
    return {"workload": "config 5: %d 3D jobs (%d plume, %d dam break), Poisson arrivals %.0f/s, sides U{32..128}, "
                        "steps U{100..400}, HBM budget %.0f GB" % (njobs, int((kinds == 0).sum()),
                                                                    int((kinds == 1).sum()), rate, budget / 1e9),
            "served": served, "plain_sequential": plain,
            "throughput_ratio": served["cells_per_s"] / plain["cells_per_s"]}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    return world, rank, local, dist


def allmax(dist, x):
    if dist is None:
        return x
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_reference(args, world, rank, dist):
    """--impl reference: the CPU path of the reference restated by the
    oracle (the reference itself needs its own code generator and CMake
    build, which this project does not run), all host threads."""
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    # the same steps as the GPU arm: W untimed steps from rest, then K timed
    # (about 1.7 s per 256^3 step on 16 host cores with PcMGStatic)
    warm = max(3, args.warmup)
    steps = args.steps
    pc = {"mic": 1, "mgdynamic": 2, "mgstatic": 3}[args.pc]
    times, iters = cpu_plume_steps(args.size, steps, warm, threads, args.seed, pc=pc)
    t = statistics.median(times)
    value = args.size ** 3 / t
    sample = ("%d^3 plume steps %d..%d from rest (first %d untimed%s), full CG to cgAccuracy 1e-3 with %s; "
              "CG iterations %s" % (args.size, warm + 1, warm + steps, warm,
                                    ", it builds the static multigrid hierarchy" if args.pc == "mgstatic" else "",
                                    PC_NAMES[args.pc], iters))
    out = {"metric": METRIC, "value": value, "unit": "cells/s", "n_gpus": world, "steps": steps, "warmup": warm,
           "ms_per_step": 1e3 * t, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "f32", "data": "synthetic",
           "config": {"workload": workload(args.size, args.pc),
                      "global_batch": 1, "seq_len": args.size ** 3, "parallelism": "cpu-openmp"},
           "impl": "reference",
           "cpu_baseline": {"value": value, "unit": "cells/s", "cores": threads, "kind": "port", "sample": sample},
           "e2e": {"value": value, "unit": "cells/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def _events_ms(L, h, a, b):
    import ctypes as C
    from mantaflow_gb300 import _lib
    ms = C.c_float()
    _lib.check(L.mg_elapsed(h, a, b, C.byref(ms)))
    return float(ms.value)


def config_runs(m, seed, cpu_steps):
    """Configs 1 and 3 at their own sizes and step counts on the plain path:
    the 64^3 plume with PcMIC for 100 steps and the 128^3 dam break for 150
    steps, device time per step from CUDA events on the solver's stream (the
    plume's inflow noise uploaded before the timed steps), with the CG
    iterations.  Beside them, the oracle on the host cores over the first
    `cpu_steps` steps of the same scenes from rest, with the GPU's time for
    the same first steps (a from-rest sample: fewer CG iterations than the
    run's average)."""
    from mantaflow_gb300 import _lib
    from oracle import oracle as og
    L = _lib.load()
    threads = os.cpu_count() or 1
    out = {}
    # config 1: 64^3 plume, MacCormack, PcMIC, 100 steps
    n, K = 64, 100
    sim = Plume(m, n, m.PcMIC, seed, K)
    noise = []
    for _ in range(K):
        g = sim.s.create(m.RealGrid)
        m.copyArrayToGridReal(sim.noise(), g)
        noise.append(g)
    sim.s.sync()
    _lib.check(L.mg_mark(sim.s._h, 0))
    for t in range(K):
        sim.step(noise[t])
        if t + 1 == cpu_steps:
            _lib.check(L.mg_mark(sim.s._h, 1))
    _lib.check(L.mg_mark(sim.s._h, 2))
    sim.s.sync()
    tot = _events_ms(L, sim.s._h, 0, 2)
    first = _events_ms(L, sim.s._h, 0, 1) if 0 < cpu_steps <= K else 0.0
    c1 = {"workload": "config 1: 3D smoke plume 64^3, MacCormack advection, MIC(0)-PCG (PcMIC), cgAccuracy 1e-3, "
                      "100 steps from rest", "cells_per_s": n ** 3 * K / (tot / 1e3), "ms_per_step": tot / K,
          "cg_iterations_mean": float(np.mean(sim.iters)), "gpu_ms_first_steps": first / max(1, cpu_steps)}
    del noise, sim
    # config 3: 128^3 dam break, 150 steps
    n3, K3 = 128, 150
    g = _plain_dam(m, n3)
    g["s"].sync()
    its = []
    _lib.check(L.mg_mark(g["s"]._h, 0))
    for t in range(K3):
        _plain_dam_step(m, g)
        its.append(m.lastSolveStats()[0])
        if t + 1 == cpu_steps:
            _lib.check(L.mg_mark(g["s"]._h, 1))
    _lib.check(L.mg_mark(g["s"]._h, 2))
    g["s"].sync()
    tot3 = _events_ms(L, g["s"]._h, 0, 2)
    first3 = _events_ms(L, g["s"]._h, 0, 1) if 0 < cpu_steps <= K3 else 0.0
    c3 = {"workload": "config 3: free-surface dam break 128^3, SL order 1, ghost-fluid MIC(0)-PCG, "
                      "extrapolateMACSimple 4, 150 steps from rest", "cells_per_s": n3 ** 3 * K3 / (tot3 / 1e3),
          "ms_per_step": tot3 / K3, "cg_iterations_mean": float(np.mean(its)),
          "gpu_ms_first_steps": first3 / max(1, cpu_steps)}
    del g
    if cpu_steps > 0:
        t1, it1 = cpu_plume_steps(64, cpu_steps, 0, threads, seed, pc=1)
        c1["cpu_oracle"] = {"ms_per_step": 1e3 * float(np.mean(t1)), "cores": threads, "kind": "port",
                            "sample": "steps 1..%d from rest, CG iterations %s" % (cpu_steps, it1)}
        og.set_num_threads(threads)
        f = np.zeros((n3, n3, n3), np.int32)
        og.init_domain(f, 0)
        phi = np.zeros((n3, n3, n3), np.float32)
        og.box_sdf(phi, (0, 0, 0), (0.4 * n3, 0.6 * n3, n3))
        og.update_from_levelset(f, phi)
        vel = np.zeros((n3, n3, n3, 3), np.float32)
        pres = np.zeros((n3, n3, n3), np.float32)
        t3, it3 = [], []
        for t in range(cpu_steps):
            t0 = time.perf_counter()
            og.extrapolate_mac_simple(f, vel, 4)
            og.advect_semi_lagrange(f, vel, phi, og.KIND_REAL, order=1)
            og.update_from_levelset(f, phi)
            og.advect_semi_lagrange(f, vel, vel, og.KIND_MAC, order=1)
            og.add_gravity(f, vel, (0, -1e-3, 0))
            og.set_wall_bcs(f, vel)
            it_o, _, _ = og.solve_pressure(f, vel, pres, phi=phi)
            og.set_wall_bcs(f, vel)
            t3.append(time.perf_counter() - t0)
            it3.append(it_o)
        og.set_num_threads(1)
        c3["cpu_oracle"] = {"ms_per_step": 1e3 * float(np.mean(t3)), "cores": threads, "kind": "port",
                            "sample": "steps 1..%d from rest, CG iterations %s" % (cpu_steps, it3)}
    return {"config1_plume64_mic": c1, "config3_dam_break128": c3}


def flip_form(m, n, ppc, reps, seed):
    """The FLIP transfers (plugin/flip.cpp:573-673) at n^3 with ppc particles
    per cell, seeded cell by cell with jitter as a fresh FLIP scene seeds
    them: device time per call of mapPartsToMAC, mapMACToParts and
    flipVelocityUpdate (CUDA events on the solver's stream), against the
    oracle's serial loops (the reference's single-threaded splat) on the
    same particles."""
    from mantaflow_gb300 import _lib
    from oracle import oracle as og
    L = _lib.load()
    s = m.Solver(name="flip", gridSize=m.vec3(n, n, n), dim=3)
    flags = s.create(m.FlagGrid)
    flags.initDomain(boundaryWidth=0)
    flags.fillGrid()
    rng = np.random.default_rng(seed)
    cells = np.stack(np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")[::-1], -1).reshape(-1, 3)
    pos = (np.repeat(cells, ppc, axis=0) + rng.random((n ** 3 * ppc, 3))).astype(np.float32)
    count = len(pos)
    pv = rng.standard_normal((count, 3)).astype(np.float32)
    pp = s.create(m.BasicParticleSystem)
    pp.setPositions(pos)
    pvel = pp.create(m.PdataVec3)
    m.copyArrayToPdataVec3(pv, pvel)
    vel, velOld = s.create(m.MACGrid), s.create(m.MACGrid)
    out = {"workload": "%d^3 grid, %d particles per cell (%d particles) seeded cell by cell with jitter" % (n, ppc, count),
           "particles": count}

    def timed(fn):
        fn()
        s.sync()
        _lib.check(L.mg_mark(s._h, 0))
        for _ in range(reps):
            fn()
        _lib.check(L.mg_mark(s._h, 1))
        ms = C.c_float()
        _lib.check(L.mg_elapsed(s._h, 0, 1, C.byref(ms)))
        return ms.value / reps

    t_p2g = timed(lambda: m.mapPartsToMAC(flags=flags, vel=vel, velOld=velOld, parts=pp, partVel=pvel))
    t_g2p = timed(lambda: m.mapMACToParts(flags=flags, vel=vel, parts=pp, partVel=pvel))
    t_flip = timed(lambda: m.flipVelocityUpdate(flags=flags, vel=vel, velOld=velOld, parts=pp, partVel=pvel,
                                                flipRatio=0.95))
    # the same particles in a random order, as a long-running scene leaves
    # them (particles move between cells; the reference never re-sorts them)
    perm = rng.permutation(count)
    pp.setPositions(pos[perm])
    m.copyArrayToPdataVec3(pv[perm], pvel)
    t_p2g_shuf = timed(lambda: m.mapPartsToMAC(flags=flags, vel=vel, velOld=velOld, parts=pp, partVel=pvel))
    t_g2p_shuf = timed(lambda: m.mapMACToParts(flags=flags, vel=vel, parts=pp, partVel=pvel))
    del perm
    f = flags.numpy()
    pflag = np.zeros(count, np.int32)
    v0, v1 = np.zeros(f.shape + (3,), np.float32), np.zeros(f.shape + (3,), np.float32)
    t0 = time.perf_counter()
    og.map_parts_to_mac(f, v0, v1, pos, pflag, pv)
    c_p2g = 1e3 * (time.perf_counter() - t0)
    t0 = time.perf_counter()
    og.map_mac_to_parts(f, v0, pos, pflag, pv)
    c_g2p = 1e3 * (time.perf_counter() - t0)
    out.update({"map_parts_to_mac_ms": t_p2g, "map_mac_to_parts_ms": t_g2p, "flip_velocity_update_ms": t_flip,
                "shuffled_order": {"map_parts_to_mac_ms": t_p2g_shuf, "map_mac_to_parts_ms": t_g2p_shuf},
                "map_parts_to_mac_particles_per_s": count / (t_p2g / 1e3),
                "cpu_oracle": {"map_parts_to_mac_ms": c_p2g, "map_mac_to_parts_ms": c_g2p, "cores": 1,
                               "kind": "port", "sample": "one call each on the same particles, serial as the reference"},
                "speedup_map_parts_to_mac": c_p2g / t_p2g, "reps": reps})
    del pp, pvel, vel, velOld, flags, s
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--size", type=int, default=256)
    ap.add_argument("--pc", default="mgstatic", choices=["mic", "mgstatic", "mgdynamic"])
    ap.add_argument("--mic-steps", type=int, default=10, help="timed PcMIC steps reported beside the headline (0: skip)")
    ap.add_argument("--seed", type=int, default=1234)
    ap.add_argument("--cpu-steps", type=int, default=1, help="timed oracle steps for cpu_baseline (0: skip)")
    ap.add_argument("--no-profile", action="store_true")
    ap.add_argument("--precision-size", type=int, default=64, help="grid side of the precision-form sample (0: skip)")
    ap.add_argument("--precision-steps", type=int, default=10)
    ap.add_argument("--batched-steps", type=int, default=10, help="timed steps of the config-4 batch (0: skip)")
    ap.add_argument("--plain-steps", type=int, default=2, help="timed steps per scene of the plain path")
    ap.add_argument("--accuracy-steps", type=int, default=5,
                    help="steps of the batched/plain accuracy sample against the FP64 oracle (0: skip)")
    ap.add_argument("--served-jobs", type=int, default=32, help="jobs of the config-5 served run (0: skip)")
    ap.add_argument("--served-plain-sample", type=int, default=3,
                    help="timed steps per job measuring the plain sequential path")
    ap.add_argument("--flip-size", type=int, default=128, help="grid side of the FLIP transfer measurement (0: skip)")
    ap.add_argument("--config-runs", type=int, default=1,
                    help="run configs 1 (64^3 plume, PcMIC, 100 steps) and 3 (128^3 dam break, 150 steps) (0: skip)")
    ap.add_argument("--config-cpu-steps", type=int, default=3, help="oracle steps beside each config run (0: skip)")
    ap.add_argument("--refined-steps", type=int, default=5,
                    help="timed 256^3 steps of the FP64-refined form reported beside the headline (0: skip)")
    args = ap.parse_args()
    world, rank, local, dist = dist_setup()
    if args.impl == "reference":
        run_reference(args, world, rank, dist)
        return
    os.environ["MANTA_GB300_DEVICE"] = str(local)
    import mantaflow_gb300 as m
    from mantaflow_gb300 import _lib
    pc = {"mic": m.PcMIC, "mgstatic": m.PcMGStatic, "mgdynamic": m.PcMGDynamic}[args.pc]
    n = args.size
    K, W = args.steps, max(3, args.warmup)
    sim = Plume(m, n, pc, args.seed + rank, W + 2 * K + 4)
    L = _lib.load()

    # inflow noise for every step, generated up front (host) and uploaded
    # before the device-resident timed region
    noise_dev = []
    for _ in range(W + K):
        g = sim.s.create(m.RealGrid)
        m.copyArrayToGridReal(sim.noise(), g)
        noise_dev.append(g)
    for t in range(W):
        sim.step(noise_dev[t])
    sim.s.sync()
    if dist is not None:
        dist.barrier()

    # ---- device-resident throughput (value)
    cnt0 = C.c_longlong()
    _lib.check(L.mg_launch_count(C.byref(cnt0)))
    clocks = ClockSampler(local)
    clocks.start()
    _lib.check(L.mg_mark(sim.s._h, 0))
    it0 = len(sim.iters)
    for t in range(K):
        sim.step(noise_dev[W + t])
    _lib.check(L.mg_mark(sim.s._h, 1))
    ms = C.c_float()
    _lib.check(L.mg_elapsed(sim.s._h, 0, 1, C.byref(ms)))
    clk = clocks.stop()
    cnt1 = C.c_longlong()
    _lib.check(L.mg_launch_count(C.byref(cnt1)))
    elapsed = allmax(dist, ms.value / 1e3)
    timed_iters = sim.iters[it0:]
    value = world * n ** 3 * K / elapsed
    for g in noise_dev:
        del g
    noise_dev = None

    # ---- end to end through the API with host buffers: every step uploads
    # its inflow noise from pinned host memory and downloads the new state.
    # The transfers are the asynchronous entries: step t's results stream
    # out on the copy stream while step t+1 computes.
    nb = n ** 3 * 4
    pin = C.c_void_p()
    _lib.check(L.mg_host_alloc(nb * 6, C.byref(pin)))
    hbuf = np.ctypeslib.as_array((C.c_float * (n ** 3 * 6)).from_address(pin.value))
    h_noise = hbuf[: n ** 3].reshape(n, n, n)
    pin_in = C.c_void_p()
    _lib.check(L.mg_host_alloc(nb * K, C.byref(pin_in)))
    in_all = np.ctypeslib.as_array((C.c_float * (n ** 3 * K)).from_address(pin_in.value)).reshape(K, n, n, n)
    for t in range(K):
        in_all[t] = sim.noise()
    noise_g = sim.s.create(m.RealGrid)
    sim.s.sync()
    if dist is not None:
        dist.barrier()
    t0 = time.perf_counter()
    for t in range(K):
        _lib.check(L.mg_grid_upload_async(noise_g._h, C.c_void_p(pin_in.value + t * nb), nb))
        sim.step(noise_g)
        _lib.check(L.mg_grid_download_async(sim.density._h, C.c_void_p(pin.value + nb), nb))
        _lib.check(L.mg_grid_download_async(sim.pressure._h, C.c_void_p(pin.value + 2 * nb), nb))
        _lib.check(L.mg_grid_download_async(sim.vel._h, C.c_void_p(pin.value + 3 * nb), 3 * nb))
    _lib.check(L.mg_solver_wait_copies(sim.s._h))
    e2e_t = allmax(dist, time.perf_counter() - t0)
    L.mg_host_free(pin_in)
    e2e = {"value": world * n ** 3 * K / e2e_t, "unit": "cells/s", "h2d_bytes_per_step": nb,
           "d2h_bytes_per_step": 5 * nb,
           "transfers": "pinned host buffers; asynchronous upload/download entries, overlapped with the next step"}

    # ---- per-kernel device time (separate pass, events around each family)
    roofline = None
    rooflines = {}
    kernels = {}
    if not args.no_profile:
        _lib.check(L.mg_profile_reset(sim.s._h))
        _lib.check(L.mg_profile_enable(sim.s._h, 1))
        for t in range(2):
            h_noise[...] = sim.noise()
            _lib.check(L.mg_grid_upload(noise_g._h, pin, nb))
            sim.step(noise_g)
        _lib.check(L.mg_profile_enable(sim.s._h, 0))
        cap = C.c_int(64)
        names = (C.c_char_p * 64)()
        tms = (C.c_double * 64)()
        lns = (C.c_longlong * 64)()
        _lib.check(L.mg_profile_read(sim.s._h, C.byref(cap), names, tms, lns))
        for i in range(cap.value):
            kernels[names[i].decode()] = (tms[i], lns[i])
        hbm, src = load_peaks()
        traffic_tab = {}
        tp = os.path.join(ROOT, "profiles", "ncu_traffic.json")
        if os.path.exists(tp):
            with open(tp) as f:
                traffic_tab = json.load(f)
        total_ms = sum(v[0] for v in kernels.values())

        def family_roofline(fam):
            tot_ms, launches = kernels[fam]
            per = tot_ms / 1e3 / launches
            achieved = BYTES_PER_CELL[fam] * n ** 3 / per / 1e9
            tr = traffic_tab.get(fam)
            return {"bound": "hbm", "kernel": fam, "achieved": achieved, "peak": hbm, "unit": "GB/s",
                    "frac": achieved / hbm, "peak_source": src,
                    "traffic": tr["bytes_per_cell"] * n ** 3 if tr else None,
                    "bytes_per_cell": BYTES_PER_CELL[fam], "launches": launches, "avg_launch_ms": 1e3 * per,
                    "share_of_step": tot_ms / total_ms}

        # every profiled launch did work: the solver polls convergence after
        # each residual update while profiling and leaves out the launches a
        # converged iteration would make
        cand = {k: v for k, v in kernels.items() if k in BYTES_PER_CELL}
        if cand:
            top = max(cand, key=lambda k: cand[k][0])
            roofline = family_roofline(top)
        for fam in ROOFLINE_FAMILIES:
            if fam in kernels:
                rooflines[fam] = family_roofline(fam)
    L.mg_host_free(pin)

    # ---- the same scene with PcMIC, reported beside the headline
    alt = None
    if args.mic_steps > 0 and pc != m.PcMIC:
        KM = args.mic_steps
        mic = Plume(m, n, m.PcMIC, args.seed + 7 + rank, 0)
        ng = mic.s.create(m.RealGrid)
        for t in range(3):
            m.copyArrayToGridReal(mic.noise(), ng)
            mic.step(ng)
        noise_m = [mic.s.create(m.RealGrid) for _ in range(KM)]
        for g in noise_m:
            m.copyArrayToGridReal(mic.noise(), g)
        mic.s.sync()
        _lib.check(L.mg_mark(mic.s._h, 0))
        i0 = len(mic.iters)
        for t in range(KM):
            mic.step(noise_m[t])
        _lib.check(L.mg_mark(mic.s._h, 1))
        msm = C.c_float()
        _lib.check(L.mg_elapsed(mic.s._h, 0, 1, C.byref(msm)))
        alt = {"workload": workload(n, "mic"), "value": n ** 3 * KM / (msm.value / 1e3), "unit": "cells/s",
               "ms_per_step": msm.value / KM, "steps": KM, "warmup": 3, "cg_iterations": mic.iters[i0:]}
        del noise_m, ng, mic

    # ---- precision form: the refined solve's throughput on the headline
    # scene, and per-field errors against the FP64 oracle on a bounded sample
    refined = None
    if args.refined_steps > 0 and rank == 0:
        KR = args.refined_steps
        rp = Plume(m, n, m.PcMGStatic, args.seed + 11, 0)
        rp.refined = True
        ng = rp.s.create(m.RealGrid)
        for t in range(3):
            m.copyArrayToGridReal(rp.noise(), ng)
            rp.step(ng)
        noise_r = [rp.s.create(m.RealGrid) for _ in range(KR)]
        for g in noise_r:
            m.copyArrayToGridReal(rp.noise(), g)
        rp.s.sync()
        _lib.check(L.mg_mark(rp.s._h, 0))
        for t in range(KR):
            rp.step(noise_r[t])
        _lib.check(L.mg_mark(rp.s._h, 1))
        msr = C.c_float()
        _lib.check(L.mg_elapsed(rp.s._h, 0, 1, C.byref(msr)))
        refined = {"workload": "3D smoke plume %d^3, MacCormack advection + FP32 multigrid-PCG inner solves with "
                               "FP64 residual refinement to max|b - Ap| < 1e-5" % n,
                   "value": n ** 3 * KR / (msr.value / 1e3), "unit": "cells/s", "ms_per_step": msr.value / KR,
                   "steps": KR, "warmup": 3, "refine_stats": rp.refine_stats[-KR:]}
        del noise_r, ng, rp
    batched = None
    if args.batched_steps > 0 and rank == 0:
        batched = batched_form(m, args.batched_steps, args.seed + 13, args.plain_steps, args.accuracy_steps)
    served = None
    if args.served_jobs > 0 and rank == 0:
        served = served_form(m, args.seed + 17, args.served_jobs, args.served_plain_sample)
    flip = None
    if args.flip_size > 0 and rank == 0:
        flip = flip_form(m, args.flip_size, 8, 10, args.seed + 23)
    configs = None
    if args.config_runs > 0 and rank == 0:
        configs = config_runs(m, args.seed + 29, args.config_cpu_steps)
    precision = None
    if args.precision_size > 0 and rank == 0 and world == 1:
        precision = precision_form(m, args.precision_size, args.precision_steps, args.seed + 5)

    # ---- CPU baseline on a bounded sample (rank 0, one GPU)
    cpu = None
    if rank == 0 and world == 1 and args.cpu_steps > 0:
        state = (sim.density.numpy(), sim.vel.numpy())
        threads = os.cpu_count() or 1
        warm = 1 if pc == m.PcMGStatic else 0  # the static hierarchy is built in an untimed step
        times, iters = cpu_plume_steps(n, args.cpu_steps, warm, threads, args.seed + 99, state=state, pc=pc)
        tc = statistics.median(times)
        cpu = {"value": n ** 3 / tc, "unit": "cells/s", "cores": threads, "kind": "port",
               "sample": "%d step(s) of the %d^3 plume continued from the GPU run's state%s on %d host threads "
                         "(the oracle: OpenMP sweeps; serial MIC(0) and serial coarse-grid selection as in the "
                         "reference), %s; CG iterations %s" %
                         (args.cpu_steps, n, " after one untimed step that builds the hierarchy" if warm else "",
                          threads, PC_NAMES[args.pc], iters)}

    if rank == 0:
        out = {"metric": METRIC, "value": value, "unit": "cells/s", "n_gpus": world, "steps": K, "warmup": W,
               "ms_per_step": 1e3 * elapsed / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
               "dtype": "f32", "data": "synthetic",
               "config": {"workload": workload(n, args.pc),
                          "global_batch": world, "seq_len": n ** 3, "parallelism": "replicas x%d" % world,
                          "l2": "inputs larger than L2 (working set > 1 GB per step)",
                          "cg_iterations": timed_iters},
               "gpu_launches": int(cnt1.value - cnt0.value),
               "clocks": clk, "e2e": e2e, "roofline": roofline, "rooflines": rooflines, "cpu_baseline": cpu,
               "kernels_ms": {k: round(v[0], 4) for k, v in sorted(kernels.items(), key=lambda kv: -kv[1][0])},
               "same_scene_pc_mic": alt, "precision_form": {"refined_256": refined, "errors_vs_fp64": precision},
               "batched_form": batched, "served_form": served, "flip_transfers": flip, "config_runs": configs}
        print(json.dumps(out), flush=True)
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
