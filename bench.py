#!/usr/bin/env python
"""Benchmark of the plain (bit-exact) stable-fluids frame step on GB300.

Workload (one scene, fits one GPU): N = 1024 interior cells per side
(size 1026 with the ghost frame), dt = 0.05, diffusion = viscosity = 1e-5,
20 Gauss-Seidel sweeps per lin_solve, four seeded rectangle obstacles of 2-8 %
of the area each, eight seeded source cells injecting density U[0, 50] and
velocity N(0, 3^2) every frame. A step is one frame: that frame's sources, then
Fluid::step. The metric counts interior cells advanced one full step.

  value  device-resident: sources pre-staged on the GPU, per-step CUDA events
         on the scene's stream, L2 flushed (256 MiB write) between timed steps.
  e2e    through the C ABI with host buffers: per step the sources go
         host->device from pinned memory, the step runs, and the three pub
         fields (density, velocities_x, velocities_y) come back device->host,
         as a drop-in Fluid keeps its Vec<f32> fields current after step().

`--impl reference` times the reference's algorithm on the host CPU instead:
the C++ restatement in oracle/ (the Rust reference cannot be built here), one
thread, as the reference runs step() on one thread.

Multi-GPU (torchrun, N > 1): the plain single grid does not shard; every rank
runs an independent replica (weak scaling) and `value` sums the replicas.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

SIZE, DT, DIFF, VISC, ITERS, NSRC, SEED = 1026, 0.05, 1e-5, 1e-5, 20, 8, 2
N = SIZE - 2
BYTES_PER_CELL_LINSOLVE = 13  # read x0, read x, write x (f32) + mask byte, per S^2 cell
BYTES_PER_CELL_FRAME = 164    # fused-phase compulsory traffic per S^2 cell per frame
BYTES_PER_CELL_FRAME_HALF = 86  # the same with FP16 / BF16 fields: (164 - 8) / 2 + 8


def baseline_metric():
    try:
        with open(os.path.join(ROOT, "BASELINE.json")) as f:
            return json.load(f)["metric"]
    except Exception:
        return "cell-steps/s on 1 GB300"


def scene(seed=SEED, nframes=1):
    """Seeded obstacles (valid Rectangle inputs) and per-frame sources."""
    rng = np.random.default_rng(seed)
    rects = []
    while len(rects) < 4:
        frac = rng.uniform(0.02, 0.08)
        aspect = rng.uniform(0.5, 2.0)
        w = int(round(math.sqrt(frac * N * N * aspect)))
        h = int(round(frac * N * N / max(w, 1)))
        if w < 2 or h < 2 or w > N - 2 or h > N - 2:
            continue
        x0 = int(rng.integers(1, SIZE - 1 - w))
        y0 = int(rng.integers(1, SIZE - 1 - h))
        rects.append((x0, y0, x0 + w, y0 + h))
    cells = rng.integers(1, SIZE - 1, size=(NSRC, 2))
    # Box-Muller on the same stream for the velocity impulses
    u1 = rng.uniform(size=(nframes, NSRC, 2))
    u2 = rng.uniform(size=(nframes, NSRC, 2))
    gauss = np.sqrt(-2.0 * np.log(np.maximum(u1, 1e-12))) * np.cos(2 * np.pi * u2) * 3.0
    dens = rng.uniform(0.0, 50.0, size=(nframes, NSRC))
    sx = np.broadcast_to(cells[:, 0], (nframes, NSRC)).astype(np.uint32).copy()
    sy = np.broadcast_to(cells[:, 1], (nframes, NSRC)).astype(np.uint32).copy()
    return (rects, sx, sy, dens.astype(np.float32), gauss[..., 0].astype(np.float32),
            gauss[..., 1].astype(np.float32))


# ---- the batched form's workload: many independent scenes of uneven size
BATCH_SCENES, BATCH_SEED = 4096, 3


def batch_workload(n=BATCH_SCENES, seed=BATCH_SEED, nmin=32, nmax=512):
    """n scenes, N log-uniform in [nmin, nmax] (size N+2), diffusion and viscosity
    log-uniform in [1e-6, 1e-3], dt uniform in [0.02, 0.2], 20 sweeps, 0-8 seeded
    rectangles of up to N/4 x N/4 each."""
    rng = np.random.default_rng(seed)
    cfgs, rects = [], []
    for _ in range(n):
        n_in = int(round(nmin * (nmax / nmin) ** rng.uniform()))
        size = n_in + 2
        cfgs.append((size, float(rng.uniform(0.02, 0.2)), 20, float(10 ** rng.uniform(-6, -3)),
                     float(10 ** rng.uniform(-6, -3))))
        rr = []
        for _ in range(int(rng.integers(0, 9))):
            w = int(rng.integers(1, max(2, n_in // 4)))
            h = int(rng.integers(1, max(2, n_in // 4)))
            x0 = int(rng.integers(1, size - 1 - w))
            y0 = int(rng.integers(1, size - 1 - h))
            rr.append((x0, y0, x0 + w, y0 + h))
        rects.append(rr)
    return cfgs, rects


def run_batched_form(local_rank: int, frames: int, plain_sample: int = 12, storage: str = "f32",
                     autotune: bool = True, err_sample: int = 0):
    """The batched form on the many-scene workload: one persistent launch per
    frame (graph-replayed), autotuned; timed with CUDA events on the batch's
    stream (inputs ~4.6 GB, far larger than L2). Also the plain kernels looped
    scene by scene over a sample of the same scenes, for comparison."""
    import torch
    from equilibrium_gb300 import _lib
    from equilibrium_gb300.batch import Batch, SceneConfig
    from equilibrium_gb300.simulation import Fluid, FluidConfigs, SimulationConfigs
    L = _lib.load()
    cfgs, rects = batch_workload()
    b = Batch([SceneConfig(*c) for c in cfgs], device=local_rank, storage=storage)
    for sidx, rr in enumerate(rects):
        for r in rr:
            b.fill_obstacle(sidx, *r)
    cells = b.cell_count()
    tune_ms = b.autotune(trial_frames=1) if autotune else None
    nw, bps = b.tuning()
    sp = ctypes.c_void_p()
    _lib.check(L.eq_batch_get_stream(b.handle, ctypes.byref(sp)))
    stream = torch.cuda.ExternalStream(sp.value)
    b.step(1)  # captures the one-frame graph, first touch
    b.synchronize()
    c0 = b.launch_count()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(frames)]
    for a, e in ev:
        a.record(stream)
        b.step(1)
        e.record(stream)
    b.synchronize()
    torch.cuda.synchronize()
    launches = b.launch_count() - c0
    ms = statistics.mean(a.elapsed_time(e) for a, e in ev)
    value = cells / (ms / 1e3)
    out = {"value": cells / (ms / 1e3), "unit": "cell-steps/s", "ms_per_frame": ms,
           "frames_timed": frames, "scenes": len(cfgs), "interior_cells": cells,
           "dtype": "f32" if storage == "f32" else f"{storage} storage, f32 arithmetic",
           "workload": f"{len(cfgs)} scenes, N log-uniform in [32, 512], dt U[0.02, 0.2], "
                       "diffusion and viscosity log-uniform [1e-6, 1e-3], 20 sweeps, 0-8 "
                       "seeded rectangles each, no sources (seed 3)",
           "tuning": {"sweeps_per_pass": nw, "blocks_per_sm": bps,
                      "autotune_ms_per_frame": tune_ms},
           "gpu_launches": int(launches),
           "roofline": {"bound": "hbm",
                        "achieved": (BYTES_PER_CELL_FRAME if storage == "f32" else
                                     BYTES_PER_CELL_FRAME_HALF) * cells / (ms / 1e3) / 1e9,
                        "unit": "GB/s",
                        "bytes_per_cell_frame": (BYTES_PER_CELL_FRAME if storage == "f32"
                                                 else BYTES_PER_CELL_FRAME_HALF)}}
    if storage == "f32":
        # end to end: one frame through the C ABI, then every scene's three pub
        # fields read back to host memory
        t0 = time.perf_counter()
        b.step(1)
        d2h = 0
        for sidx, c in enumerate(cfgs):
            for f in (_lib.FIELD_DENSITY, _lib.FIELD_VX, _lib.FIELD_VY):
                d2h += b.read_field(sidx, f).nbytes
        e2e_s = time.perf_counter() - t0
        out["e2e"] = {"value": cells / e2e_s, "unit": "cell-steps/s", "h2d_bytes_per_step": 0,
                      "d2h_bytes_per_step": d2h, "ms_per_step": e2e_s * 1e3}
        out["bit_exact"] = "per scene, vs the reference step (tests/test_gpu_batch.py)"
    b.close()
    if err_sample:
        out["density_rel_l2_vs_f64"] = batch_half_errors(storage, err_sample, local_rank)
    if plain_sample:
        # the plain (eq_fluid) kernels looped over a sample of the same scenes
        rng = np.random.default_rng(7)
        pick = rng.choice(len(cfgs), size=plain_sample, replace=False)
        pcells, pms = 0, 0.0
        for q in pick:
            size, dt, k, dif, vis = cfgs[q]
            g = Fluid(FluidConfigs(dif, vis, False), SimulationConfigs(dt, k, size),
                      device=local_rank)
            for r in rects[q]:
                _lib.check(L.eq_fluid_fill_obstacle(g.handle, *r))
            g.step()
            g.synchronize()
            t = time.perf_counter()
            g.step()
            g.step()
            g.synchronize()
            pms += (time.perf_counter() - t) / 2 * 1e3
            pcells += (size - 2) ** 2
            g.close()
        out["plain_looped"] = {"value": pcells / (pms / 1e3), "unit": "cell-steps/s",
                               "sample": f"{plain_sample} scenes of the workload stepped one by "
                                         "one through eq_fluid (host clock, 2 frames each)"}
    return out


def batch_half_errors(storage: str, nsample: int, local_rank: int, frames=(1, 3)):
    """Relative L2 density error of half-storage batch scenes against the f64
    reference step (the oracle built with f64), for a seeded sample of the
    workload's scenes: the median and maximum over the sample per frame."""
    import oracle
    from equilibrium_gb300.batch import Batch, SceneConfig
    from equilibrium_gb300.precision import rel_l2
    cfgs, rects = batch_workload()
    rng = np.random.default_rng(11)
    pick = [int(q) for q in rng.choice(len(cfgs), size=nsample, replace=False)
            if cfgs[int(q)][0] <= 258][:nsample]
    b = Batch([SceneConfig(*cfgs[q]) for q in pick], device=local_rank, storage=storage)
    refs = []
    for k, q in enumerate(pick):
        size, dt, K, dif, vis = cfgs[q]
        r = oracle.OracleFluid(size, dt, K, dif, vis, dtype=np.float64)
        for rc in rects[q]:
            r.fill_obstacle(*rc)
            b.fill_obstacle(k, *rc)
        refs.append(r)
    res, done = {}, 0
    for fr in frames:
        b.step(fr - done)
        for r in refs:
            for _ in range(fr - done):
                r.step()
        done = fr
        errs = [rel_l2(b.read_field(k, _lib_field_density()), r.fields[1])
                for k, r in enumerate(refs)]
        res[f"frame_{fr}"] = {"median": float(np.median(errs)), "max": float(np.max(errs))}
    b.close()
    res["scenes"] = f"{len(pick)} seeded scenes of the workload with size <= 258"
    return res


def _lib_field_density():
    from equilibrium_gb300 import _lib
    return _lib.FIELD_DENSITY


# ---- the precision form's workload: one N = 2048 scene in half storage
PREC_SIZE, PREC_DT, PREC_DIFF, PREC_VISC, PREC_RTOL = 2050, 0.05, 1e-5, 1e-5, 1e-5


def precision_scene(size, seed=4, nframes=1):
    """Obstacles and sources seeded as the N = 1024 plain workload, scaled to
    `size` (4 rectangles of 2-8 % of the area, 8 source cells per frame)."""
    n = size - 2
    rng = np.random.default_rng(seed)
    rects = []
    while len(rects) < 4:
        frac = rng.uniform(0.02, 0.08)
        aspect = rng.uniform(0.5, 2.0)
        w = int(round(math.sqrt(frac * n * n * aspect)))
        h = int(round(frac * n * n / max(w, 1)))
        if w < 2 or h < 2 or w > n - 2 or h > n - 2:
            continue
        x0 = int(rng.integers(1, size - 1 - w))
        y0 = int(rng.integers(1, size - 1 - h))
        rects.append((x0, y0, x0 + w, y0 + h))
    cells = rng.integers(1, size - 1, size=(NSRC, 2))
    u1 = rng.uniform(size=(nframes, NSRC, 2))
    u2 = rng.uniform(size=(nframes, NSRC, 2))
    gauss = np.sqrt(-2.0 * np.log(np.maximum(u1, 1e-12))) * np.cos(2 * np.pi * u2) * 3.0
    dens = rng.uniform(0.0, 50.0, size=(nframes, NSRC))
    return (rects, cells[:, 0].astype(np.uint32), cells[:, 1].astype(np.uint32),
            dens.astype(np.float32), gauss[..., 0].astype(np.float32),
            gauss[..., 1].astype(np.float32))


def run_precision_form(local_rank: int, frames: int, size: int = PREC_SIZE,
                       err_frames=(1,), storages=("f16", "bf16")):
    """The precision form on one scene: throughput of `frames` timed frames per
    storage format, its refinement statistics, and at `err_frames` the relative
    L2 density error, max-abs velocity error and post-projection divergence
    against two f64 references run on the host: the reference step itself and
    the same step with both pressure solves converged exactly."""
    import torch
    import oracle
    from equilibrium_gb300.precision import HalfFluid, max_abs, rel_l2
    nmax = max(err_frames) if err_frames else 0
    total = max(frames + 1, nmax)
    rects, sx, sy, sd, su, sv = precision_scene(size, nframes=total)
    refs = {}
    if err_frames:
        for kind in ("f64_reference", "f64_converged_pressure"):
            r = oracle.OracleFluid(size, PREC_DT, ITERS, PREC_DIFF, PREC_VISC, dtype=np.float64)
            for rc in rects:
                r.fill_obstacle(*rc)
            refs[kind] = (r, {})
        for fr in range(nmax):
            for kind, (r, snaps) in refs.items():
                oracle.add_sources(r, sx, sy, sd[fr], su[fr], sv[fr])
                if kind == "f64_reference":
                    r.step()
                else:
                    oracle.converged_step_f64(r)
                if fr + 1 in err_frames:
                    snaps[fr + 1] = (r.fields[1].copy(), r.fields[2].copy(), r.fields[3].copy())
    out = {"workload": f"one scene, N = {size - 2} interior, dt {PREC_DT}, diffusion = viscosity "
                       f"= {PREC_DIFF}, 20 sweeps per diffusion solve, pressure refined to a "
                       f"relative residual of {PREC_RTOL}, 4 seeded rectangles, {NSRC} seeded "
                       "sources per frame"}
    for storage in storages:
        g = HalfFluid(size, PREC_DT, ITERS, PREC_DIFF, PREC_VISC, storage, PREC_RTOL, 30,
                      device=local_rank)
        for rc in rects:
            g.fill_obstacle(*rc)
        errs = {}
        ms, launches = [], []
        for fr in range(max(total, frames + 1)):
            g.add_sources(sx, sy, sd[fr % total], su[fr % total], sv[fr % total])
            torch.cuda.synchronize()
            c0 = g.launch_count()
            t0 = time.perf_counter()
            g.step()
            ms.append((time.perf_counter() - t0) * 1e3)
            launches.append(g.launch_count() - c0)
            if fr + 1 in err_frames:
                de, vx, vy = g.read_field(1), g.read_field(2), g.read_field(3)
                st = g.stats()
                errs[f"frame_{fr + 1}"] = {
                    kind: {"density_rel_l2": rel_l2(de, snaps[fr + 1][0]),
                           "velocity_max_abs": max(max_abs(vx, snaps[fr + 1][1]),
                                                   max_abs(vy, snaps[fr + 1][2]))}
                    for kind, (_, snaps) in refs.items()}
                errs[f"frame_{fr + 1}"]["post_projection_divergence_l2"] = st["div_norm"]
        timed = ms[1:frames + 1]
        t = statistics.mean(timed)
        out[storage] = {"value": (size - 2) ** 2 / (t / 1e3), "unit": "cell-steps/s",
                        "ms_per_frame": t, "frames_timed": len(timed),
                        "clock": "host, per frame (the refinement loop reads its norms)",
                        "stats_last_frame": g.stats(), "errors": errs,
                        "gpu_launches_per_frame": statistics.mean(launches[1:frames + 1])}
        g.close()
    return out


def run_case(case: str):
    """Small, self-contained runs of one form, for kernel profiles."""
    import torch
    from equilibrium_gb300 import build as eqbuild
    eqbuild.build()
    torch.cuda.set_device(0)
    if case.startswith("batch256"):
        from equilibrium_gb300.batch import Batch, SceneConfig
        cfgs, rects = batch_workload(n=256)
        b = Batch([SceneConfig(*c) for c in cfgs], storage="f16" if case.endswith("f16") else "f32")
        for sidx, rr in enumerate(rects):
            for r in rr:
                b.fill_obstacle(sidx, *r)
        b.step(1, graph=False)
        b.synchronize()
        t = time.perf_counter()
        b.step(1, graph=False)
        b.synchronize()
        print(json.dumps({"case": case, "ms": (time.perf_counter() - t) * 1e3,
                          "cells": b.cell_count()}))
        b.close()
    else:
        from equilibrium_gb300.precision import HalfFluid
        size = 1026
        rects, sx, sy, sd, su, sv = precision_scene(size, nframes=2)
        g = HalfFluid(size, PREC_DT, ITERS, PREC_DIFF, PREC_VISC, "f16", PREC_RTOL, 30)
        for r in rects:
            g.fill_obstacle(*r)
        for fr in range(2):
            g.add_sources(sx, sy, sd[fr], su[fr], sv[fr])
            g.step()
        print(json.dumps({"case": case, "stats": g.stats()}))
        g.close()


def replicas_value(local_seconds: float, steps: int, world: int, reduce_max=None):
    """Whole-job cell-steps/s of `world` independent replicas: every rank ran
    `steps` frames; the job time is the slowest rank's (max over ranks)."""
    t = reduce_max(local_seconds) if (reduce_max and world > 1) else local_seconds
    return world * N * N * steps / t, t


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("LOCAL_RANK", 0)), int(
        os.environ.get("WORLD_SIZE", 1))


class ClockSampler:
    """nvidia-smi clock / throttle sampling while the timed region runs."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu, self.proc, self.lines = gpu, None, []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}", "--format=csv,noheader",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.t.join(timeout=2)

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1].split()[0]))
                mx.append(float(p[2].split()[0]))
            except ValueError:
                continue
            for name, val in zip(names, p[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx),
                "reasons": sorted(reasons), "samples": len(sm)}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profile_traffic():
    """Per-launch DRAM traffic of the lin_solve wavefront from the committed ncu summary."""
    try:
        with open(os.path.join(ROOT, "profiles", "lin_solve_traffic.json")) as f:
            d = json.load(f)
        return d.get("dram_bytes_per_launch"), d.get("source")
    except Exception:
        return None, None


def cpu_baseline_run(nframes: int):
    """The oracle port (single thread) on the same workload from its initial state."""
    import oracle
    rects, sx, sy, sd, su, sv = scene(SEED, nframes)
    f = oracle.OracleFluid(SIZE, DT, ITERS, DIFF, VISC)
    for r in rects:
        f.fill_obstacle(*r)
    secs = f.run(nframes, sx, sy, sd, su, sv, timed=True)
    return {"value": N * N * nframes / secs, "unit": "cell-steps/s", "cores": 1, "kind": "port",
            "sample": f"{nframes} frames of the N=1024 workload from its initial state "
                      f"({secs:.1f} s, oracle/ C++ restatement, -O3 -ffp-contract=off)"}


def config_dict():
    return {"workload": "plain frame step, N=1024 (size 1026), 20 GS sweeps, dt=0.05, "
                        "diff=visc=1e-5, 4 seeded rectangles, 8 seeded sources/frame",
            "size": SIZE, "interior_n": N, "gs_iterations": ITERS, "delta_t": DT,
            "diffusion": DIFF, "viscosity": VISC, "obstacles": 4, "sources_per_frame": NSRC,
            "seed": SEED, "l2": "flushed between timed steps (256 MiB write, untimed)",
            "form": "plain, bit-exact vs the reference step"}


def run_reference(args):
    rank, _, world = dist_env()
    if rank != 0:
        return
    import oracle
    oracle.build()
    # Each step is one CPU frame (~1 s at N=1024): time at most 30 of them so
    # the run stays within a few minutes whatever --steps is.
    warm = min(args.warmup, 3)
    timed = min(args.steps, 30)
    rects, sx, sy, sd, su, sv = scene(SEED, warm + timed)
    f = oracle.OracleFluid(SIZE, DT, ITERS, DIFF, VISC)
    for r in rects:
        f.fill_obstacle(*r)
    for w in range(warm):
        f.run(1, sx[w:w + 1], sy[w:w + 1], sd[w:w + 1], su[w:w + 1], sv[w:w + 1])
    times = []
    for s in range(timed):
        q = warm + s
        times.append(f.run(1, sx[q:q + 1], sy[q:q + 1], sd[q:q + 1], su[q:q + 1], sv[q:q + 1],
                           timed=True))
    t = statistics.mean(times)
    value = N * N / t
    line = {"impl": "reference", "metric": baseline_metric(), "value": value,
            "unit": "cell-steps/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": t * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": config_dict(),
            "cpu_baseline": {"value": value, "unit": "cell-steps/s", "cores": 1, "kind": "port",
                             "sample": f"{timed} frames (one per step, after {warm} warm-up "
                                       "frames) of the workload on the host CPU: the oracle/ C++ "
                                       "restatement of the reference step, one thread like the "
                                       "reference"},
            "e2e": {"value": value, "unit": "cell-steps/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args):
    import torch
    from equilibrium_gb300 import build as eqbuild
    from equilibrium_gb300 import _lib
    from equilibrium_gb300.simulation import Fluid, FluidConfigs, SimulationConfigs

    rank, local_rank, world = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local_rank)
    eqbuild.build()
    L = _lib.load()

    total = args.warmup + args.steps
    rects, sx, sy, sd, su, sv = scene(SEED + rank, 2 * total)
    fl = Fluid(FluidConfigs(DIFF, VISC, False), SimulationConfigs(DT, ITERS, SIZE), device=local_rank)
    for r in rects:
        _lib.check(L.eq_fluid_fill_obstacle(fl.handle, *r))
    stream_ptr = ctypes.c_void_p()
    _lib.check(L.eq_fluid_get_stream(fl.handle, ctypes.byref(stream_ptr)))
    stream = torch.cuda.ExternalStream(stream_ptr.value)
    dev = torch.device("cuda", local_rank)
    d_sx = torch.from_numpy(sx.astype(np.int32)).to(dev)
    d_sy = torch.from_numpy(sy.astype(np.int32)).to(dev)
    d_sd, d_su, d_sv = (torch.from_numpy(a).to(dev) for a in (sd, su, sv))
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    torch.cuda.synchronize()

    def frame(q):
        o = q * NSRC * 4
        _lib.check(L.eq_fluid_run_device_sources(
            fl.handle, 1, NSRC, d_sx.data_ptr() + o, d_sy.data_ptr() + o, d_sd.data_ptr() + o,
            d_su.data_ptr() + o, d_sv.data_ptr() + o))

    for w in range(args.warmup):
        frame(w)
    fl.synchronize()

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    # ---- device-resident timed region
    count0 = ctypes.c_uint64()
    _lib.check(L.eq_fluid_launch_count(fl.handle, ctypes.byref(count0)))
    _lib.check(L.eq_fluid_set_profiling(fl.handle, 1))
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    barrier()
    torch.cuda.synchronize()
    wall0 = time.perf_counter()
    with ClockSampler(local_rank) as clk:
        for s in range(args.steps):
            with torch.cuda.stream(stream):
                flush.fill_(float(s))
                starts[s].record(stream)
            frame(args.warmup + s)
            ends[s].record(stream)
        fl.synchronize()
        torch.cuda.synchronize()
    wall = time.perf_counter() - wall0
    barrier()
    count1 = ctypes.c_uint64()
    _lib.check(L.eq_fluid_launch_count(fl.handle, ctypes.byref(count1)))
    ls_ms, ls_n = ctypes.c_double(), ctypes.c_uint64()
    _lib.check(L.eq_fluid_kernel_stats(fl.handle, 0, ctypes.byref(ls_ms), ctypes.byref(ls_n)))
    _lib.check(L.eq_fluid_set_profiling(fl.handle, 0))
    step_ms = [a.elapsed_time(b) for a, b in zip(starts, ends)]
    def reduce_max(x):
        import torch.distributed as dist
        t = torch.tensor([x], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    value, dev_s = replicas_value(sum(step_ms) / 1e3, args.steps, world, reduce_max)
    ms_per_step = dev_s / args.steps * 1e3

    # ---- end to end through the C ABI with host buffers
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory()
    h_sx, h_sy, h_sd, h_su, h_sv = (pin(a) for a in (sx, sy, sd, su, sv))
    outs = [torch.empty(SIZE * SIZE, dtype=torch.float32).pin_memory() for _ in range(3)]
    e2e_times = []
    base = total
    barrier()
    for s in range(args.steps):
        with torch.cuda.stream(stream):
            flush.fill_(float(s))
        torch.cuda.synchronize()
        fl.synchronize()
        t0 = time.perf_counter()
        q = (base + s) % (2 * total)
        o = q * NSRC
        _lib.check(L.eq_fluid_add_sources(
            fl.handle, NSRC, h_sx.data_ptr() + 4 * o, h_sy.data_ptr() + 4 * o,
            h_sd.data_ptr() + 4 * o, h_su.data_ptr() + 4 * o, h_sv.data_ptr() + 4 * o))
        _lib.check(L.eq_fluid_step(fl.handle))
        for f_idx, buf in zip((_lib.FIELD_DENSITY, _lib.FIELD_VX, _lib.FIELD_VY), outs):
            _lib.check(L.eq_fluid_read_field(fl.handle, f_idx, buf.data_ptr(), SIZE * SIZE))
        e2e_times.append(time.perf_counter() - t0)
    e2e_value, e2e_s = replicas_value(sum(e2e_times), args.steps, world, reduce_max)
    assert np.isfinite(outs[0].numpy()).all()

    if rank != 0:
        return
    hbm, peak_kind = peaks()
    avg_ls = ls_ms.value / max(ls_n.value, 1) / 1e3
    achieved = BYTES_PER_CELL_LINSOLVE * SIZE * SIZE / avg_ls / 1e9 if avg_ls > 0 else None
    traffic, traffic_src = profile_traffic()
    roofline = {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                "frac": (achieved / hbm) if achieved else None, "traffic": traffic,
                "kernel": "k_lin_solve (persistent temporal-wavefront Gauss-Seidel)",
                "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)",
                "algorithmic_bytes_per_launch": BYTES_PER_CELL_LINSOLVE * SIZE * SIZE,
                "launches_timed": int(ls_n.value), "avg_launch_ms": avg_ls * 1e3,
                "share_of_step": (ls_ms.value / (dev_s / world * 1e3)) if dev_s else None,
                "frame_roofline_frac": (BYTES_PER_CELL_FRAME * SIZE * SIZE /
                                        (ms_per_step / 1e3) / 1e9 / hbm),
                "traffic_source": traffic_src}
    try:
        cpu = cpu_baseline_run(args.cpu_frames)
    except Exception as e:  # the oracle is only the reported baseline
        cpu = {"value": None, "unit": "cell-steps/s", "cores": 1, "kind": "port",
               "sample": f"failed: {e}"}
    forms = {}
    if args.forms:
        def form(name, fn):
            try:
                r = fn()
                if "roofline" in r:
                    r["roofline"]["peak"] = hbm
                    r["roofline"]["frac"] = r["roofline"]["achieved"] / hbm
                if "value" in r:
                    r["vs_plain"] = r["value"] / value
            except Exception as e:  # reported, never silently replaced
                r = {"error": f"{type(e).__name__}: {e}"}
            forms[name] = r

        form("batched", lambda: run_batched_form(local_rank, args.batch_frames))
        form("batched_f16", lambda: run_batched_form(local_rank, args.batch_frames, 0, "f16",
                                                     autotune=False, err_sample=24))
        form("precision", lambda: run_precision_form(local_rank, args.precision_frames))
        for k in ("f16", "bf16"):
            if "precision" in forms and k in forms["precision"]:
                forms["precision"][k]["vs_plain"] = forms["precision"][k]["value"] / value
    line = {"metric": baseline_metric(), "value": value, "unit": "cell-steps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded obstacles and sources; no dataset)",
            "config": config_dict(), "roofline": roofline, "cpu_baseline": cpu,
            "e2e": {"value": e2e_value, "unit": "cell-steps/s",
                    "h2d_bytes_per_step": NSRC * 20,
                    "d2h_bytes_per_step": 3 * SIZE * SIZE * 4,
                    "ms_per_step": e2e_s / args.steps * 1e3},
            "gpu_launches": int(count1.value - count0.value), "clocks": clk.summary(),
            "wall_s_timed_region": wall}
    if forms:
        line["forms"] = forms
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-frames", type=int, default=12)
    ap.add_argument("--batch-frames", type=int, default=5)
    ap.add_argument("--precision-frames", type=int, default=4)
    ap.add_argument("--case", default=None,
                    choices=["batch256", "batch256_f16", "precision1024"],
                    help="one small run for profiling: 'batch256' = one frame of 256 scenes of "
                         "the batched workload (after one warm-up frame), 'precision1024' = two "
                         "frames of the precision form at N = 1024 (FP16)")
    ap.add_argument("--precision-study", action="store_true",
                    help="only the precision form's error study: N=512, errors at frames 1, "
                         "50 and 200 against both f64 references")
    ap.add_argument("--no-forms", dest="forms", action="store_false",
                    help="skip the batched / half-storage forms")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.case:
        run_case(args.case)
    elif args.precision_study:
        import torch
        from equilibrium_gb300 import build as eqbuild
        eqbuild.build()
        torch.cuda.set_device(0)
        print(json.dumps({"precision_study": run_precision_form(
            0, 3, size=514, err_frames=(1, 50, 200))}), flush=True)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
