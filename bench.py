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
BYTES_PER_CELL_FRAME_F16_SCALARS = 150  # density and scratch FP16, velocities FP32
BYTES_BY_STORAGE = {"f32": BYTES_PER_CELL_FRAME, "f16": BYTES_PER_CELL_FRAME_HALF,
                    "bf16": BYTES_PER_CELL_FRAME_HALF,
                    "f16_scalars": BYTES_PER_CELL_FRAME_F16_SCALARS}


METRIC = "cell-steps/s on 1 GB300: plain vs batched/half-storage, % HBM peak, err vs FP64"


def baseline_metric():
    return METRIC


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


def cells_total(cfgs):
    """size * size summed over a batch's scenes (ghost cells included)."""
    return sum(int(c[0]) ** 2 for c in cfgs)


def run_batched_form(local_rank: int, frames: int, plain_sample: int = 12, storage: str = "f32",
                     autotune: bool = True, err_sample: int = 0, rank: int = 0, world: int = 1,
                     reduce_max=None, reduce_sum=None):
    """The batched form on the many-scene workload: one persistent launch per
    frame (graph-replayed), autotuned; timed with CUDA events on the batch's
    stream (inputs ~4.6 GB, far larger than L2). Also the plain kernels looped
    scene by scene over a sample of the same scenes, for comparison.

    With world > 1 ranks (one GPU each) the scenes are split by
    batch.partition_scenes (no data shared, no collective on the data path):
    each rank builds and steps only its own scenes, and the value is all
    ranks' cells over the slowest rank's frame time (weak in the scenes per
    rank). Only rank 0 runs the end-to-end, looped-plain and CPU legs."""
    import torch
    from equilibrium_gb300 import _lib
    from equilibrium_gb300.batch import Batch, SceneConfig, partition_scenes
    from equilibrium_gb300.simulation import Fluid, FluidConfigs, SimulationConfigs
    L = _lib.load()
    all_cfgs, all_rects = batch_workload()
    parts, loads = partition_scenes(all_cfgs, world)
    mine = parts[rank]
    cfgs = [all_cfgs[q] for q in mine]
    rects = [all_rects[q] for q in mine]
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
    local_cells = cells
    if world > 1:  # all ranks' cells over the slowest rank's frame time
        ms = reduce_max(ms)
        cells = int(round(reduce_sum(float(cells))))
    value = cells / (ms / 1e3)
    out = {"value": cells / (ms / 1e3), "unit": "cell-steps/s", "ms_per_frame": ms,
           "frames_timed": frames, "scenes": len(all_cfgs), "interior_cells": cells,
           "ranks": world, "scenes_per_rank": [len(p) for p in parts],
           "work_imbalance": max(loads) / (sum(loads) / world) - 1.0,
           "dtype": "f32" if storage == "f32" else f"{storage} storage, f32 arithmetic",
           "workload": f"{len(cfgs)} scenes, N log-uniform in [32, 512], dt U[0.02, 0.2], "
                       "diffusion and viscosity log-uniform [1e-6, 1e-3], 20 sweeps, 0-8 "
                       "seeded rectangles each, no sources (seed 3)",
           "tuning": {"sweeps_per_pass": nw, "blocks_per_sm": bps,
                      "autotune_ms_per_frame": tune_ms},
           "gpu_launches": int(launches),
           "roofline": {"bound": "hbm",
                        "achieved": BYTES_BY_STORAGE[storage] * cells / (ms / 1e3) / 1e9,
                        "unit": "GB/s",
                        "bytes_per_cell_frame": BYTES_BY_STORAGE[storage]}}
    if rank != 0:
        b.close()
        return out
    if storage == "f32":
        # end to end: one frame through the C ABI, then every scene's three pub
        # fields read back to (pinned) host memory, one field of all scenes per
        # call
        host = [torch.empty(cells_total(cfgs), dtype=torch.float32).pin_memory().numpy()
                for _ in range(3)]
        # (rank 0's own scenes: the e2e number is rank 0's cells over its time)
        b.read_fields(_lib.FIELD_DENSITY, host[0])  # first use allocates its device staging
        b.synchronize()
        t0 = time.perf_counter()
        b.step(1)
        d2h = 0
        for f, buf in zip((_lib.FIELD_DENSITY, _lib.FIELD_VX, _lib.FIELD_VY), host):
            d2h += b.read_fields(f, buf).nbytes
        e2e_s = time.perf_counter() - t0
        out["e2e"] = {"value": local_cells / e2e_s, "unit": "cell-steps/s", "h2d_bytes_per_step": 0,
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
    out["cpu_baseline"] = batch_cpu_baseline(cfgs, rects)
    return out


def batch_cpu_baseline(cfgs, rects, nsample: int = 24, seed: int = 7):
    """The reference's step on one host core (the oracle, f32) over a seeded
    sample of the batch workload's scenes, one frame each: cell-steps/s of
    the sample (the workload's sizes are log-uniform, so a uniform sample of
    scenes is a fair sample of its cost per cell)."""
    import oracle
    rng = np.random.default_rng(seed)
    pick = rng.choice(len(cfgs), size=nsample, replace=False)
    cells, secs = 0, 0.0
    for q in pick:
        size, dt, k, dif, vis = cfgs[q]
        r = oracle.OracleFluid(size, dt, k, dif, vis)
        for rc in rects[q]:
            r.fill_obstacle(*rc)
        t = time.perf_counter()
        r.step()
        secs += time.perf_counter() - t
        cells += (size - 2) ** 2
    return {"value": cells / secs, "unit": "cell-steps/s", "cores": 1, "kind": "port",
            "sample": f"{nsample} seeded scenes of the workload, one frame each, the oracle's "
                      f"f32 step ({secs:.1f} s)"}


def _half_ref_task(task):
    """The reference step of one batch scene on the host, in f32 and f64:
    density at each checkpoint frame (a worker of batch_half_errors)."""
    import oracle
    (size, dt, K, dif, vis), rects, frames = task
    out = {}
    for dtype in (np.float32, np.float64):
        r = oracle.OracleFluid(size, dt, K, dif, vis, dtype=dtype)
        for rc in rects:
            r.fill_obstacle(*rc)
        done, dens = 0, []
        for fr in frames:
            for _ in range(fr - done):
                r.step()
            done = fr
            dens.append(np.array(r.fields[1], dtype=np.float64))
        out[np.dtype(dtype).name] = dens
    return out


def batch_half_errors(storage: str, nsample: int, local_rank: int, frames=(1, 50, 200)):
    """Relative L2 density error of half-storage batch scenes against the f64
    reference step (the oracle built with f64), for a seeded sample of the
    workload's scenes, at frames 1, 50 and 200: the median and maximum over
    the sample per frame, beside the reference's own f32 step's distance to
    the f64 step on the same scenes (the flow's sensitivity, which any
    rounding grows, separated from the storage error)."""
    import multiprocessing as mp
    from equilibrium_gb300.batch import Batch, SceneConfig
    from equilibrium_gb300.precision import rel_l2
    cfgs, rects = batch_workload()
    rng = np.random.default_rng(11)
    pick = [int(q) for q in rng.choice(len(cfgs), size=nsample, replace=False)
            if cfgs[int(q)][0] <= 258][:nsample]
    tasks = [(cfgs[q], rects[q], tuple(frames)) for q in pick]
    with mp.get_context("spawn").Pool(min(len(tasks), os.cpu_count() or 1)) as pool:
        refs = pool.map(_half_ref_task, tasks)
    b = Batch([SceneConfig(*cfgs[q]) for q in pick], device=local_rank, storage=storage)
    for k, q in enumerate(pick):
        for rc in rects[q]:
            b.fill_obstacle(k, *rc)
    res, done = {}, 0
    for n, fr in enumerate(frames):
        b.step(fr - done)
        done = fr
        errs = [rel_l2(b.read_field(k, _lib_field_density()), refs[k]["float64"][n])
                for k in range(len(pick))]
        drift = [rel_l2(refs[k]["float32"][n], refs[k]["float64"][n]) for k in range(len(pick))]
        res[f"frame_{fr}"] = {"median": float(np.median(errs)), "max": float(np.max(errs)),
                              "f32_step_median": float(np.median(drift)),
                              "f32_step_max": float(np.max(drift))}
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


def _precision_reference(task):
    """One f64 host reference of the precision workload (spawned worker, the
    oracle only): 'f64_reference' = the reference step, 'f64_converged_pressure'
    = the same step with both pressure solves converged; returns the density
    and velocities after each frame in err_frames."""
    import oracle
    kind, size, err_frames, ndraw = task
    nmax = max(err_frames)
    # the same draw as the GPU run's (the per-frame sources depend on its length)
    rects, sx, sy, sd, su, sv = precision_scene(size, nframes=ndraw)
    r = oracle.OracleFluid(size, PREC_DT, ITERS, PREC_DIFF, PREC_VISC, dtype=np.float64)
    for rc in rects:
        r.fill_obstacle(*rc)
    snaps = {}
    for fr in range(nmax):
        oracle.add_sources(r, sx, sy, sd[fr], su[fr], sv[fr])
        if kind == "f64_reference":
            r.step()
        else:
            oracle.converged_step_f64(r)
        if fr + 1 in err_frames:
            snaps[fr + 1] = (r.fields[1].copy(), r.fields[2].copy(), r.fields[3].copy())
    return kind, snaps


def run_precision_form(local_rank: int, frames: int, size: int = PREC_SIZE,
                       err_frames=(1,), storages=("f16", "bf16", "f16_scalars")):
    """The precision form on one scene: throughput of `frames` timed frames per
    storage format, its refinement statistics, and at `err_frames` the relative
    L2 density error, max-abs velocity error and post-projection divergence
    against two f64 references run on the host (in two spawned processes,
    after the timed frames: the frames are host-clocked and launch-bound, so
    they must not share the host with the references): the reference step
    itself and the same step with both pressure solves converged exactly."""
    import concurrent.futures as cf
    import multiprocessing as mp
    import torch
    from equilibrium_gb300.precision import HalfFluid, max_abs, rel_l2
    nmax = max(err_frames) if err_frames else 0
    total = max(frames + 1, nmax)
    rects, sx, sy, sd, su, sv = precision_scene(size, nframes=total)
    pool, futs, refs = None, [], {}
    out = {"workload": f"one scene, N = {size - 2} interior, dt {PREC_DT}, diffusion = viscosity "
                       f"= {PREC_DIFF}, 20 sweeps per diffusion solve, pressure refined to a "
                       f"relative residual of {PREC_RTOL}, 4 seeded rectangles, {NSRC} seeded "
                       "sources per frame"}
    gpu_snaps = {}
    for storage in storages:
        g = HalfFluid(size, PREC_DT, ITERS, PREC_DIFF, PREC_VISC, storage, PREC_RTOL, 30,
                      device=local_rank)
        for rc in rects:
            g.fill_obstacle(*rc)
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
                gpu_snaps[(storage, fr + 1)] = (g.read_field(1), g.read_field(2),
                                                g.read_field(3), g.stats()["div_norm"])
        timed = ms[1:frames + 1]
        t = statistics.mean(timed)
        hbm, _ = peaks()
        ach = BYTES_PER_CELL_FRAME_HALF * size * size / (t / 1e3) / 1e9
        out[storage] = {"value": (size - 2) ** 2 / (t / 1e3), "unit": "cell-steps/s",
                        "roofline": {"bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s",
                                     "frac": ach / hbm,
                                     "bytes_per_cell_frame": BYTES_PER_CELL_FRAME_HALF,
                                     "note": "the fused-phase bytes of a frame with half fields; "
                                             "the refinement rounds' own traffic is not counted"},
                        "ms_per_frame": t, "frames_timed": len(timed),
                        "clock": "host, per frame (the refinement loop reads its norms)",
                        "stats_last_frame": g.stats(),
                        "gpu_launches_per_frame": statistics.mean(launches[1:frames + 1])}
        g.close()
    # the reference's step on one host core at this size (the oracle, f32), one frame
    import oracle
    r = oracle.OracleFluid(size, PREC_DT, ITERS, PREC_DIFF, PREC_VISC)
    for rc in rects:
        r.fill_obstacle(*rc)
    oracle.add_sources(r, sx, sy, sd[0], su[0], sv[0])
    t0 = time.perf_counter()
    r.step()
    tc = time.perf_counter() - t0
    out["cpu_baseline"] = {"value": (size - 2) ** 2 / tc, "unit": "cell-steps/s", "cores": 1,
                           "kind": "port",
                           "sample": f"one frame of this workload, the oracle's f32 step "
                                     f"({tc:.1f} s)"}
    if err_frames:
        t0 = time.perf_counter()
        pool = cf.ProcessPoolExecutor(2, mp_context=mp.get_context("spawn"))
        futs = [pool.submit(_precision_reference, (kind, size, tuple(err_frames), total))
                for kind in ("f64_reference", "f64_converged_pressure")]
        for f in futs:
            kind, snaps = f.result()
            refs[kind] = snaps
        pool.shutdown()
        for storage in storages:
            errs = {}
            for fr in err_frames:
                de, vx, vy, div = gpu_snaps[(storage, fr)]
                errs[f"frame_{fr}"] = {
                    kind: {"density_rel_l2": rel_l2(de, snaps[fr][0]),
                           "velocity_max_abs": max(max_abs(vx, snaps[fr][1]),
                                                   max_abs(vy, snaps[fr][2]))}
                    for kind, snaps in refs.items()}
                errs[f"frame_{fr}"]["post_projection_divergence_l2"] = div
            out[storage]["errors"] = errs
        out["f64_references_wait_s"] = time.perf_counter() - t0
    return out


# ---- the differentiation form ------------------------------------------------
DIFF_SIZE, DIFF_FRAMES, DIFF_EVERY, DIFF_SEED = 258, 64, 8, 11
DIFF_DT, DIFF_NU = 0.1, 1e-4


def diff_problem(size=DIFF_SIZE, frames=DIFF_FRAMES, seed=DIFF_SEED):
    """The differentiable workload: Fluid::new's density (the 0.9 block),
    an initial velocity that is divergence-free and smooth (the curl of a
    stream function of four seeded Gaussian vortices, sigma U[10, 30] cells,
    scaled to max |v| = 0.3, i.e. backtraces of up to 7.7 cells a frame), two
    seeded rectangle obstacles, per-frame density source fields (three
    Gaussian puffs a frame, amplitude U[0, 2], sigma U[3, 10] cells) and a
    target density of six Gaussian blobs (sigma U[8, 24] cells). Returns
    (rects, cells, init (6 f32 arrays), src (frames, n) f32, target f32)."""
    import oracle
    rng = np.random.default_rng(seed)
    n = size * size
    rects = []
    while len(rects) < 2:
        w, h = (int(v) for v in rng.integers(size // 10, size // 5, 2))
        x0, y0 = (int(v) for v in rng.integers(2, size - 2 - max(w, h), 2))
        rects.append((x0, y0, x0 + w, y0 + h))
    of = oracle.OracleFluid(size, DIFF_DT, ITERS, DIFF_NU, DIFF_NU)
    for r in rects:
        of.fill_obstacle(*r)
    init = [f.copy() for f in of.fields]
    y, x = np.mgrid[0:size, 0:size].astype(np.float64)
    psi = np.zeros((size, size))
    for _ in range(4):
        cx, cy = rng.uniform(size * 0.2, size * 0.8, 2)
        sg, sgn = rng.uniform(10, 30), rng.choice([-1.0, 1.0])
        psi += sgn * sg * np.exp(-((x - cx) ** 2 + (y - cy) ** 2) / (2 * sg * sg))
    vx, vy = np.gradient(psi, axis=0), -np.gradient(psi, axis=1)
    vmax = max(np.abs(vx).max(), np.abs(vy).max())
    init[2] = (vx * (0.3 / vmax)).reshape(-1).astype(np.float32)
    init[3] = (vy * (0.3 / vmax)).reshape(-1).astype(np.float32)
    init[4] = np.zeros(n, np.float32)
    init[5] = np.zeros(n, np.float32)
    src = np.zeros((frames, size, size))
    for fr in range(frames):
        for _ in range(3):
            cx, cy = rng.uniform(size * 0.2, size * 0.8, 2)
            sg, amp = rng.uniform(3, 10), rng.uniform(0, 2)
            src[fr] += amp * np.exp(-((x - cx) ** 2 + (y - cy) ** 2) / (2 * sg * sg))
    target = oracle.gaussian_target(size, 6, (8.0, 24.0), seed=seed + 1)
    return (rects, of.cells.copy(), init, src.reshape(frames, n).astype(np.float32),
            target.astype(np.float32))


_FD_CACHE = {}


def _fd_direction(k, n, nsrc):
    d = np.random.default_rng(1000 + k).standard_normal(2 * n + nsrc)
    return d / np.linalg.norm(d)


def _fd_task(task):
    """Central differences of the f64 forward of the differentiable workload
    along seeded random unit direction k: plain runs, or runs that replay the
    unperturbed run's advect choices (frozen). Runs in a spawned worker (the
    oracle only)."""
    import oracle
    k, hs, frozen, size, frames = task
    key = (size, frames)
    if key not in _FD_CACHE:
        _, cells, init, src, target = diff_problem(size, frames)
        _FD_CACHE[key] = (cells, [a.astype(np.float64) for a in init], src.astype(np.float64),
                          target.astype(np.float64))
    cells, init, src, target = _FD_CACHE[key]
    d = _fd_direction(k, size * size, src.size)
    return oracle.fd_direction_f64(cells, size, DIFF_DT, ITERS, DIFF_NU, DIFF_NU, init, src,
                                   target, d, hs, frozen=frozen)


def fd_check(grads, size, frames, ndirs=32, h=1e-3, workers=None):
    """Central differences of the f64 forward (step h) along `ndirs` seeded
    random unit directions over (initial vx, vy, every source field) against
    each gradient's directional derivative (grads: name -> flat gradient).
    'plain': ordinary runs; the forward is only piecewise smooth (advect's
    cell choice, clamps and row breaks), so a direction whose runs cross a
    bilinear cell boundary differs by the kink. 'frozen_path': the perturbed
    runs replay the unperturbed run's choices, the derivative the adjoint
    computes (O(h^2) agreement)."""
    import concurrent.futures as cf
    import multiprocessing as mp
    n = size * size
    tasks = [(k, (h,), frozen, size, frames) for k in range(ndirs) for frozen in (False, True)]
    workers = workers or max(1, min(len(tasks), os.cpu_count() or 1))
    t0 = time.perf_counter()
    with cf.ProcessPoolExecutor(workers, mp_context=mp.get_context("spawn")) as ex:
        res = list(ex.map(_fd_task, tasks))
    out = {"directions": ndirs, "h": h, "workers": workers,
           "seconds": time.perf_counter() - t0,
           "metric": "per direction d: |fd - g.d| / rms, rms = |g|_2 / sqrt(dim) (the typical "
                     "size of g.d over random unit d); 'rel_to_fd' = |fd - g.d| / |fd|"}
    nsrc = frames * n
    for name, gv in grads.items():
        gv = gv.astype(np.float64)
        rms = np.linalg.norm(gv) / np.sqrt(gv.size)
        for kind, fz in (("plain", False), ("frozen_path", True)):
            e_rms, e_fd = [], []
            for k in range(ndirs):
                (lp, lm), = res[2 * k + (1 if fz else 0)]
                fd = (lp - lm) / (2 * h)
                diff = abs(fd - gv @ _fd_direction(k, n, nsrc))
                e_rms.append(diff / rms)
                e_fd.append(diff / max(abs(fd), 1e-300))
            out[f"{name}_vs_{kind}"] = {"median": float(np.median(e_rms)),
                                        "max": float(np.max(e_rms)),
                                        "rel_to_fd_median": float(np.median(e_fd))}
    return out


def concurrent_gradients(local_rank: int, size: int, frames: int, nscenes: int):
    """nscenes independent gradients of the differentiation workload (seeds
    11, 12, ...), each on its own handle and stream, driven from one host
    thread each: one gradient's solves occupy a cluster of 8 SMs, so several
    run side by side. Aggregate cell-steps/s over the wall time of all."""
    import threading
    import torch
    from equilibrium_gb300 import _lib
    from equilibrium_gb300.adjoint import Recorder
    from equilibrium_gb300.simulation import Fluid, FluidConfigs, SimulationConfigs
    L = _lib.load()
    dev = torch.device("cuda", local_rank)
    jobs = []
    for q in range(nscenes):
        rects, cells, init, src, target = diff_problem(size, frames, DIFF_SEED + q)
        f = Fluid(FluidConfigs(DIFF_NU, DIFF_NU, False), SimulationConfigs(DIFF_DT, ITERS, size),
                  device=local_rank)
        for r in rects:
            _lib.check(L.eq_fluid_fill_obstacle(f.handle, *r))
        g = Recorder(f, frames, DIFF_EVERY)
        n = size * size
        jobs.append((f, g, init, torch.from_numpy(src).to(dev), target,
                     torch.empty(6 * n, dtype=torch.float32, device=dev),
                     torch.empty(frames * n, dtype=torch.float32, device=dev)))
    errs = []

    def one(job):
        f, g, init, d_src, target, d_gi, d_gs = job
        try:
            _lib.check(L.eq_grad_forward_device(g.handle, frames, d_src.data_ptr()))
            g.nframes = frames
            g.l2_loss(target)
            _lib.check(L.eq_grad_backward_device(g.handle, None, d_gi.data_ptr(), d_gs.data_ptr()))
        except Exception as e:  # reported below
            errs.append(repr(e))

    def reset():
        for f, g, init, *_ in jobs:
            for k in range(6):
                f.write_field(k, init[k])
        torch.cuda.synchronize()

    reset()
    for job in jobs:  # warm-up, one at a time
        one(job)
    reset()
    t0 = time.perf_counter()
    th = [threading.Thread(target=one, args=(job,)) for job in jobs]
    for t in th:
        t.start()
    for t in th:
        t.join()
    wall = time.perf_counter() - t0
    for f, g, *_ in jobs:
        g.close()
        f.close()
    if errs:
        return {"error": errs[0]}
    return {"what": f"{nscenes} independent gradients (seeds {DIFF_SEED}..{DIFF_SEED + nscenes - 1}) "
                    "on their own handles and streams, one host thread each",
            "value": nscenes * (size - 2) ** 2 * frames / wall, "unit": "cell-steps/s",
            "wall_s": wall, "clock": "host, all gradients (each ends with a synchronisation)"}


def run_diff_form(local_rank: int, reps: int = 2, fd_dirs: int = 32, size: int = DIFF_SIZE,
                  frames: int = DIFF_FRAMES):
    """The differentiation form: one gradient evaluation = `frames` recorded
    frames + the L2 loss + backward() (checkpoints every 8 frames, the
    segment recomputed, the adjoint kernels); cell-steps/s counts the
    differentiated frames' interior cells. Checked against the f32 and f64
    tape adjoints and by central differences of the f64 forward."""
    import torch
    import oracle
    from equilibrium_gb300 import _lib
    from equilibrium_gb300.adjoint import Recorder
    from equilibrium_gb300.simulation import Fluid, FluidConfigs, SimulationConfigs
    L = _lib.load()
    rects, cells, init, src, target = diff_problem(size, frames)
    n = size * size
    f = Fluid(FluidConfigs(DIFF_NU, DIFF_NU, False), SimulationConfigs(DIFF_DT, ITERS, size),
              device=local_rank)
    for r in rects:
        _lib.check(L.eq_fluid_fill_obstacle(f.handle, *r))
    g = Recorder(f, frames, DIFF_EVERY)
    sp = ctypes.c_void_p()
    _lib.check(L.eq_fluid_get_stream(f.handle, ctypes.byref(sp)))
    stream = torch.cuda.ExternalStream(sp.value)
    dev = torch.device("cuda", local_rank)
    d_src = torch.from_numpy(src).to(dev)
    d_gi = torch.empty(6 * n, dtype=torch.float32, device=dev)
    d_gs = torch.empty(frames * n, dtype=torch.float32, device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def reset():
        for k in range(6):
            f.write_field(k, init[k])

    # device-resident: sources and gradients stay on the GPU
    dev_ms, fwd_ms, bwd_ms, launches = [], [], [], []
    gs_ms, gs_n = ctypes.c_double(), ctypes.c_uint64()
    for rep in range(reps + 1):
        reset()
        with torch.cuda.stream(stream):
            flush.fill_(float(rep))
        torch.cuda.synchronize()
        if rep == reps:
            _lib.check(L.eq_grad_set_profiling(g.handle, 1))
        c0 = g.launch_count()
        e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        e[0].record(stream)
        _lib.check(L.eq_grad_forward_device(g.handle, frames, d_src.data_ptr()))
        g.nframes = frames
        e[1].record(stream)
        g.l2_loss(target)
        _lib.check(L.eq_grad_backward_device(g.handle, None, d_gi.data_ptr(), d_gs.data_ptr()))
        e[2].record(stream)
        torch.cuda.synchronize()
        if rep > 0:
            dev_ms.append(e[0].elapsed_time(e[2]))
            fwd_ms.append(e[0].elapsed_time(e[1]))
            bwd_ms.append(e[1].elapsed_time(e[2]))
            launches.append(g.launch_count() - c0)
    _lib.check(L.eq_grad_kernel_stats(g.handle, ctypes.byref(gs_ms), ctypes.byref(gs_n)))
    _lib.check(L.eq_grad_set_profiling(g.handle, 0))
    gi = d_gi.view(6, n).cpu().numpy()
    gsrc = d_gs.view(frames, n).cpu().numpy()
    concurrent = concurrent_gradients(local_rank, size, frames, 16)
    # variant: one segment (the forward keeps the whole tape, no recompute)
    gf = Recorder(f, frames, frames)
    full_ms = []
    for rep in range(reps + 1):
        reset()
        torch.cuda.synchronize()
        e = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        e[0].record(stream)
        _lib.check(L.eq_grad_forward_device(gf.handle, frames, d_src.data_ptr()))
        gf.nframes = frames
        gf.l2_loss(target)
        _lib.check(L.eq_grad_backward_device(gf.handle, None, d_gi.data_ptr(), d_gs.data_ptr()))
        e[1].record(stream)
        torch.cuda.synchronize()
        if rep > 0:
            full_ms.append(e[0].elapsed_time(e[1]))
    full_diff = float(np.linalg.norm(d_gs.view(frames, n).cpu().numpy() - gsrc) /
                      np.linalg.norm(gsrc))
    gf.close()
    # end to end through the C ABI with host buffers
    e2e_ms = []
    for rep in range(reps):
        reset()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        g.forward(src)
        loss = g.l2_loss(target)
        h_gi, h_gs = g.backward()
        e2e_ms.append((time.perf_counter() - t0) * 1e3)
    # advect^T scatters with float atomics: runs agree to rounding, not bit for bit
    rerun = max(float(np.linalg.norm(h_gi - gi) / np.linalg.norm(gi)),
                float(np.linalg.norm(h_gs - gsrc) / np.linalg.norm(gsrc)))
    assert rerun < 1e-4, rerun
    t = statistics.mean(dev_ms)
    cells_steps = (size - 2) ** 2 * frames
    out = {"workload": f"one scene, N = {size - 2} interior, dt {DIFF_DT}, diffusion = viscosity "
                       f"= {DIFF_NU}, 20 sweeps, {frames} frames, 2 seeded rectangles, a seeded "
                       "density source field per frame, loss = 0.5 * L2^2 to a 6-blob Gaussian "
                       f"target; gradient w.r.t. the initial velocity and every source field, "
                       f"checkpoints every {DIFF_EVERY} frames",
           "value": cells_steps / (t / 1e3), "unit": "cell-steps/s (differentiated frames)",
           "ms_per_gradient": t, "ms_forward": statistics.mean(fwd_ms),
           "ms_loss_and_backward": statistics.mean(bwd_ms), "reps_timed": len(dev_ms),
           "gpu_launches_per_gradient": statistics.mean(launches),
           "clock": "CUDA events on the scene's stream, L2 flushed before each gradient",
           "e2e": {"value": cells_steps / (statistics.mean(e2e_ms) / 1e3),
                   "unit": "cell-steps/s", "ms_per_gradient": statistics.mean(e2e_ms),
                   "h2d_bytes_per_gradient": frames * n * 4 + n * 4,
                   "d2h_bytes_per_gradient": (6 + frames) * n * 4 + 8},
           "loss": loss, "rerun_rel_diff": rerun,
           "variant_concurrent": concurrent,
           "variant_full_tape": {
               "what": "checkpoint_every = frames: the forward keeps every frame's tape "
                       f"({frames * 5 * size * ((size + 31) // 32 * 32) * 4 / 1e6:.0f} MB), "
                       "backward recomputes nothing",
               "value": cells_steps / (statistics.mean(full_ms) / 1e3),
               "ms_per_gradient": statistics.mean(full_ms),
               "g_src_rel_diff_to_checkpointed": full_diff}}
    avg_gs = gs_ms.value / max(gs_n.value, 1)
    store, blocks = g.wavefront_storage()
    # the adjoint wavefront: per cell and sweep it reads 2 + 2 (+ sum) values
    # and writes 2 on chip; its DRAM traffic is the incoming adjoint, the
    # codes and the outputs (13 B per cell), so it is bound by the SM, not HBM
    out["roofline"] = {"bound": "hbm", "kernel": ("k_gs_adj_cl (transposed Gauss-Seidel "
                       f"wavefront over a cluster of {blocks} blocks, distributed shared memory)"
                       if store == 3 else f"k_gs_adj (transposed Gauss-Seidel wavefront, one "
                       f"block, storage form {store})"),
                       "achieved": 13 * size * size / (avg_gs / 1e3) / 1e9 if avg_gs > 0 else None,
                       "unit": "GB/s", "avg_launch_ms": avg_gs, "launches": int(gs_n.value),
                       "share_of_gradient": gs_ms.value / statistics.mean(dev_ms[-1:]),
                       "cell_sweeps_per_s": size * size * ITERS / (avg_gs / 1e3) if avg_gs else None,
                       "traffic": None}
    # accuracy against the tape adjoints (host, 1 core) and finite differences
    t0 = time.perf_counter()
    l32, s32, vx32, vy32, src32 = oracle.adjoint_problem_f32(
        cells, size, DIFF_DT, ITERS, DIFF_NU, DIFF_NU, init, src, target)
    t32 = time.perf_counter() - t0
    t0 = time.perf_counter()
    l64, s64, vx64, vy64, src64 = oracle.adjoint_problem_f64(
        cells, size, DIFF_DT, ITERS, DIFF_NU, DIFF_NU, [a.astype(np.float64) for a in init],
        src.astype(np.float64), target.astype(np.float64))
    t64 = time.perf_counter() - t0

    def rel(a, b):
        return float(np.linalg.norm(a.astype(np.float64) - b) / np.linalg.norm(b))
    out["errors"] = {
        "vs_f32_tape": {"g_vx": rel(gi[2], vx32), "g_vy": rel(gi[3], vy32),
                        "g_src": rel(gsrc, src32), "loss_rel": abs(loss - l32) / abs(l32)},
        "vs_f64_tape": {"g_vx": rel(gi[2], vx64), "g_vy": rel(gi[3], vy64),
                        "g_src": rel(gsrc, src64), "same_discrete_path": s32 == s64},
        "f32_tape_vs_f64_tape": {"g_vx": rel(vx32, vx64), "g_vy": rel(vy32, vy64),
                                 "g_src": rel(src32, src64)},
        "metric": "relative L2 norm of the difference"}
    out["cpu_baseline"] = {"value": cells_steps / t64, "unit": "cell-steps/s", "cores": 1,
                           "kind": "port",
                           "sample": f"the f64 tape adjoint of the oracle, forward + backward, "
                                     f"the full workload ({t64:.1f} s); the f32 tape: "
                                     f"{cells_steps / t32:.3g} cell-steps/s"}
    if fd_dirs:
        try:
            flat = lambda a, b, c: np.concatenate([a.reshape(-1), b.reshape(-1), c.reshape(-1)])
            out["finite_differences"] = fd_check(
                {"gpu": flat(gi[2], gi[3], gsrc), "f64_tape": flat(vx64, vy64, src64)},
                size, frames, fd_dirs)
        except Exception as e:  # reported, never silently replaced
            out["finite_differences"] = {"error": f"{type(e).__name__}: {e}"}
    g.close()
    f.close()
    return out


def run_fma_form(local_rank: int, steps: int = 20, warmup: int = 5):
    """The plain step of the headline workload built with FMA contraction
    (libeqfluid_fma.so): device time per step as in the timed region (L2
    flushed between steps), and its distance after one frame to the
    bit-exact library's state from the same start (rel. L2 per field)."""
    import torch
    from equilibrium_gb300 import _lib
    from equilibrium_gb300.simulation import Fluid, FluidConfigs, SimulationConfigs
    F = _lib.load_fma()
    L = _lib.load()
    rects, sx, sy, sd, su, sv = scene(SEED, warmup + steps)
    dev = torch.device("cuda", local_rank)

    def make(lib):
        f = Fluid(FluidConfigs(DIFF, VISC, False), SimulationConfigs(DT, ITERS, SIZE),
                  device=local_rank, lib=lib)
        for r in rects:
            _lib.check(lib.eq_fluid_fill_obstacle(f.handle, *r), lib)
        return f

    f = make(F)
    sp = ctypes.c_void_p()
    _lib.check(F.eq_fluid_get_stream(f.handle, ctypes.byref(sp)), F)
    stream = torch.cuda.ExternalStream(sp.value)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    for q in range(warmup):
        f.add_sources(sx[q], sy[q], sd[q], su[q], sv[q])
        f.step()
    f.synchronize()
    ms = []
    for q in range(warmup, warmup + steps):
        f.add_sources(sx[q], sy[q], sd[q], su[q], sv[q])  # host sources staged before timing
        with torch.cuda.stream(stream):
            flush.fill_(float(q))
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
        f.step()
        b.record(stream)
        f.synchronize()
        ms.append(a.elapsed_time(b))
    f.close()
    # one frame from the same start in both builds
    f, g = make(F), make(L)
    for h in (f, g):
        h.add_sources(sx[0], sy[0], sd[0], su[0], sv[0])
        h.step()
        h.synchronize()
    errs = {}
    for k, name in ((1, "density"), (2, "vx"), (3, "vy")):
        x, y = f.read_field(k).astype(np.float64), g.read_field(k).astype(np.float64)
        errs[name] = float(np.linalg.norm(x - y) / max(np.linalg.norm(y), 1e-300))
    f.close()
    g.close()
    step_ms = float(np.mean(ms))
    return {"value": N * N / (step_ms / 1e3), "unit": "cell-steps/s", "ms_per_step": step_ms,
            "build": "libeqfluid_fma.so: --fmad=true, x0 + a*sum and the advect / project "
                     "arithmetic contracted (backtrace position unfused)",
            "rel_l2_vs_bit_exact_frame_1": errs,
            "tolerance": "1e-6 per phase (tests/test_gpu_fma.py)"}


def solve_alone_ms(L, fl, reps: int = 10):
    """One Passive lin_solve of the headline grid with nothing beside it (the
    pressure solves' situation): the library's per-launch CUDA-event time."""
    a = np.float32(1.0)
    c = np.float32(4.0)
    for _ in range(3):
        _lib_check(L, L.eq_fluid_lin_solve(fl.handle, 2, 4, 5, a, c))
    fl.synchronize()
    _lib_check(L, L.eq_fluid_set_profiling(fl.handle, 1))
    for _ in range(reps):
        _lib_check(L, L.eq_fluid_lin_solve(fl.handle, 2, 4, 5, a, c))
    fl.synchronize()
    ms, n = ctypes.c_double(), ctypes.c_uint64()
    _lib_check(L, L.eq_fluid_kernel_stats(fl.handle, 0, ctypes.byref(ms), ctypes.byref(n)))
    _lib_check(L, L.eq_fluid_set_profiling(fl.handle, 0))
    return ms.value / max(n.value, 1)


def _lib_check(L, rc):
    from equilibrium_gb300 import _lib
    _lib.check(rc, L)


def latency_bound_ms(sm_mhz: float, strips: int, groups: int, handoff_us: float = 1.5,
                     op_cycles: int = 4):
    """The lin_solve dependency-chain bound: 2 S + 3 K cell updates in sequence
    (lexicographic Gauss-Seidel on the critical path), 6 dependent f32
    operations each at op_cycles per operation, plus one L2 hand-off for each
    block-to-block boundary on that path (strips - 1 strip edges, groups - 1
    sweep-group edges; hand-offs inside a block go through shared memory)."""
    chain_ms = (2 * SIZE + 3 * ITERS) * 6 * op_cycles / (sm_mhz * 1e3)
    hand_ms = (strips - 1 + groups - 1) * handoff_us / 1e3
    return {"latency_bound_ms": chain_ms + hand_ms, "chain_ms": chain_ms,
            "handoff_ms": hand_ms, "sm_mhz": sm_mhz, "dependent_op_cycles": op_cycles,
            "handoff_us": handoff_us, "strips": strips, "sweep_groups": groups}


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
    elif case in ("lscs1024", "lssw1024"):
        from equilibrium_gb300 import _lib
        from equilibrium_gb300.simulation import Fluid, FluidConfigs, SimulationConfigs
        L = _lib.load()
        f = Fluid(FluidConfigs(DIFF, VISC, False), SimulationConfigs(DT, ITERS, SIZE))
        _lib.check(L.eq_fluid_fill_obstacle(f.handle, SIZE // 4, SIZE // 4, SIZE // 3,
                                            SIZE // 3))
        # every solve by the streamed cluster form (2) or the strip wavefront (3)
        _lib.check(L.eq_fluid_set_solver(f.handle, 2 if case == "lscs1024" else 3))
        ms = []
        for _ in range(2):
            t = time.perf_counter()
            _lib.check(L.eq_fluid_lin_solve(f.handle, _lib.MODE_PASSIVE, 2, 4, 0.37, 2.48))
            f.synchronize()
            ms.append((time.perf_counter() - t) * 1e3)
        print(json.dumps({"case": case, "ms": ms}))
        f.close()
    elif case == "diff256":
        from equilibrium_gb300 import _lib
        from equilibrium_gb300.adjoint import Recorder
        from equilibrium_gb300.simulation import Fluid, FluidConfigs, SimulationConfigs
        frames = 4
        rects, cells, init, src, target = diff_problem(DIFF_SIZE, frames)
        f = Fluid(FluidConfigs(DIFF_NU, DIFF_NU, False),
                  SimulationConfigs(DIFF_DT, ITERS, DIFF_SIZE))
        for r in rects:
            _lib.check(_lib.load().eq_fluid_fill_obstacle(f.handle, *r))
        for k in range(6):
            f.write_field(k, init[k])
        g = Recorder(f, frames, frames)
        t = time.perf_counter()
        g.forward(src)
        loss = g.l2_loss(target)
        gi, gs = g.backward()
        print(json.dumps({"case": case, "ms": (time.perf_counter() - t) * 1e3, "loss": loss,
                          "launches": g.launch_count()}))
        g.close()
        f.close()
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


def parity_check(local_rank: int, frames=(1, 10, 100)):
    """The headline workload's state after 1, 10 and 100 frames (a fresh
    handle, the step() the timed region runs, sources of the 1000-frame draw)
    against the oracle's hashes in tests/golden/long_horizon_hashes.json:
    all six fields with ghost cells, bit for bit."""
    from equilibrium_gb300 import _lib
    from equilibrium_gb300.simulation import Fluid, FluidConfigs, SimulationConfigs
    from tests.util import state_hashes
    L = _lib.load()
    with open(os.path.join(ROOT, "tests", "golden", "long_horizon_hashes.json")) as fh:
        c = json.load(fh)["n1024"]
    rects, sx, sy, sd, su, sv = scene(SEED, c["frames"])
    f = Fluid(FluidConfigs(DIFF, VISC, False), SimulationConfigs(DT, ITERS, SIZE),
              device=local_rank)
    for r in rects:
        _lib.check(L.eq_fluid_fill_obstacle(f.handle, *r))
    done, bad = 0, []
    for fr in frames:
        for q in range(done, fr):
            f.add_sources(sx[q], sy[q], sd[q], su[q], sv[q])
            f.step()
        done = fr
        f.synchronize()
        got = state_hashes([f.read_field(k) for k in range(6)])
        if got != c["checkpoints"][str(fr)]:
            bad.append(fr)
    f.close()
    return {"status": "bit-exact" if not bad else f"differs at frames {bad}",
            "frames_checked": list(frames), "fields": "all six, ghost cells included",
            "reference": "oracle state hashes, tests/golden/long_horizon_hashes.json "
                         "(the 1000-frame hash is checked by tests/test_gpu_long_horizon.py)"}


def summarize(line):
    """A compact per-form digest, last in the JSON line: value (cell-steps/s),
    ratio to the plain form, fraction of the HBM roofline, accuracy."""
    def g(d, *ks):
        for k in ks:
            if not isinstance(d, dict) or k not in d:
                return None
            d = d[k]
        return d

    def r3(x):
        return float(f"{x:.3g}") if isinstance(x, (int, float)) else x

    out = {"plain": {"value": r3(line["value"]), "e2e": r3(g(line, "e2e", "value")),
                     "frame_frac": r3(g(line, "roofline", "frame_roofline_frac")),
                     "parity": g(line, "parity", "status")}}
    forms = line.get("forms", {})
    for name in ("batched", "batched_f16", "batched_f16_scalars", "batched_bf16"):
        fm = forms.get(name)
        if fm:
            out[name] = {"value": r3(fm.get("value")), "vs_plain": r3(fm.get("vs_plain")),
                         "frac": r3(g(fm, "roofline", "frac")),
                         "err": g(fm, "density_rel_l2_vs_f64"), "error": fm.get("error")}
    pr = forms.get("precision")
    if pr:
        for k in ("f16", "bf16", "f16_scalars"):
            if k in pr:
                fe = g(pr[k], "errors", "frame_1", "f64_converged_pressure", "density_rel_l2")
                out[f"precision_{k}"] = {"value": r3(pr[k].get("value")),
                                         "vs_plain": r3(pr[k].get("vs_plain")),
                                         "density_err_frame_1": r3(fe)}
    df = forms.get("differentiation")
    if df:
        out["differentiation"] = {"value": r3(df.get("value")), "error": df.get("error")}
    fm = forms.get("fma")
    if fm:
        errs = fm.get("rel_l2_vs_bit_exact_frame_1") or {}
        out["fma"] = {"value": r3(fm.get("value")), "vs_plain": r3(fm.get("vs_plain")),
                      "err": r3(max(errs.values())) if errs else None, "error": fm.get("error")}
    out["plain"]["solve_alone_ms"] = r3(g(line, "roofline", "alone_ms"))
    out["plain"]["latency_bound_ms"] = r3(g(line, "roofline", "latency_bound_ms"))
    return out


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
        fl.read_fields((_lib.FIELD_DENSITY, _lib.FIELD_VX, _lib.FIELD_VY), outs)
        e2e_times.append(time.perf_counter() - t0)
    e2e_value, e2e_s = replicas_value(sum(e2e_times), args.steps, world, reduce_max)
    assert np.isfinite(outs[0].numpy()).all()
    alone_ms = solve_alone_ms(L, fl)  # after the timed regions (it changes vx0 / vy0)

    # the batched form shards by scene: every rank steps its own part
    sharded = None
    if args.forms and world > 1:
        def reduce_sum(x):
            import torch.distributed as dist
            t = torch.tensor([x], device=dev, dtype=torch.float64)
            dist.all_reduce(t, op=dist.ReduceOp.SUM)
            return float(t.item())
        try:
            sharded = run_batched_form(local_rank, args.batch_frames, rank=rank, world=world,
                                       reduce_max=reduce_max, reduce_sum=reduce_sum)
        except Exception as e:  # reported by rank 0, never silently replaced
            sharded = {"error": f"{type(e).__name__}: {e}"}

    if rank != 0:
        return
    hbm, peak_kind = peaks()
    avg_ls = ls_ms.value / max(ls_n.value, 1) / 1e3
    achieved = BYTES_PER_CELL_LINSOLVE * SIZE * SIZE / avg_ls / 1e9 if avg_ls > 0 else None
    traffic, traffic_src = profile_traffic()
    clocks = clk.summary()
    sm_mhz = float(clocks.get("sm_mhz") or 2070.0)
    strips = (SIZE + 2 * (ITERS - 1) + 31) // 32
    groups_alone = max(2, min(5, 152 // strips))
    roofline = {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                "frac": (achieved / hbm) if achieved else None, "traffic": traffic,
                "kernel": ("lin_solve: k_ls_sw (strip wavefront), every solve of step(): "
                           "the three diffusions side by side, then the two pressure solves"),
                "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)",
                "alone_ms": alone_ms,
                "alone_achieved": BYTES_PER_CELL_LINSOLVE * SIZE * SIZE / (alone_ms / 1e3) / 1e9,
                **latency_bound_ms(sm_mhz, strips, groups_alone),
                "algorithmic_bytes_per_launch": BYTES_PER_CELL_LINSOLVE * SIZE * SIZE,
                "launches_timed": int(ls_n.value), "avg_launch_ms": avg_ls * 1e3,
                "share_of_step": (ls_ms.value / (dev_s / world * 1e3)) if dev_s else None,
                "overlap": ("step() runs the vy and the density diffusions on two side "
                            "streams, so up to three solves overlap: each launch's event "
                            "time includes the others' contention and share_of_step sums "
                            "overlapping intervals"),
                # every solve's algorithmic bytes of one step over the step time
                "aggregate_achieved": (BYTES_PER_CELL_LINSOLVE * SIZE * SIZE
                                       * (ls_n.value / max(args.steps, 1))
                                       / (ms_per_step / 1e3) / 1e9),
                "frame_roofline_frac": (BYTES_PER_CELL_FRAME * SIZE * SIZE /
                                        (ms_per_step / 1e3) / 1e9 / hbm),
                "traffic_source": traffic_src}
    try:
        cpu = cpu_baseline_run(args.cpu_frames)
    except Exception as e:  # the oracle is only the reported baseline
        cpu = {"value": None, "unit": "cell-steps/s", "cores": 1, "kind": "port",
               "sample": f"failed: {e}"}
    try:
        parity = parity_check(local_rank)
    except Exception as e:
        parity = {"status": f"not checked: {type(e).__name__}: {e}"}
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

        form("batched", lambda: sharded if sharded is not None
             else run_batched_form(local_rank, args.batch_frames))
        form("batched_f16", lambda: run_batched_form(local_rank, args.batch_frames, 0, "f16",
                                                     autotune=False, err_sample=24))
        form("batched_f16_scalars", lambda: run_batched_form(
            local_rank, args.batch_frames, 0, "f16_scalars", autotune=False, err_sample=24))
        form("batched_bf16", lambda: run_batched_form(local_rank, args.batch_frames, 0, "bf16",
                                                      autotune=False, err_sample=24))
        form("precision", lambda: run_precision_form(local_rank, args.precision_frames))
        form("differentiation", lambda: run_diff_form(local_rank, fd_dirs=args.fd_dirs))
        form("fma", lambda: run_fma_form(local_rank))
        for k in ("f16", "bf16", "f16_scalars"):
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
            "gpu_launches": int(count1.value - count0.value), "clocks": clocks,
            "parity": parity,
            "wall_s_timed_region": wall}
    if forms:
        line["forms"] = forms
    line["summary"] = summarize(line)
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
    ap.add_argument("--fd-dirs", type=int, default=32,
                    help="random directions of the differentiation form's finite-difference check")
    ap.add_argument("--diff-only", action="store_true",
                    help="only the differentiation form (N=256, 64 frames)")
    ap.add_argument("--case", default=None,
                    choices=["batch256", "batch256_f16", "precision1024", "diff256",
                             "lscs1024", "lssw1024"],
                    help="one small run for profiling: 'batch256' = one frame of 256 scenes of "
                         "the batched workload (after one warm-up frame), 'precision1024' = two "
                         "frames of the precision form at N = 1024 (FP16), 'diff256' = one "
                         "gradient of the differentiation workload at N = 256 over 4 frames, "
                         "'lscs1024' = two Passive lin_solves at N = 1024 by the streamed "
                         "cluster wavefront, 'lssw1024' = the same by the strip wavefront")
    ap.add_argument("--study-size", type=int, default=514,
                    help="size (N + 2) of --precision-study")
    ap.add_argument("--precision-study", action="store_true",
                    help="only the precision form's error study: N = study-size - 2, errors "
                         "at frames 1, 50 and 200 against both f64 references")
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
            0, 3, size=args.study_size, err_frames=(1, 50, 200))}), flush=True)
    elif args.diff_only:
        import torch
        from equilibrium_gb300 import build as eqbuild
        eqbuild.build()
        torch.cuda.set_device(0)
        print(json.dumps({"differentiation": run_diff_form(0, fd_dirs=args.fd_dirs)}), flush=True)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
