#!/usr/bin/env python
"""Benchmark of the SPH grid step on one GB300: particle-steps/s.

    python bench.py [--steps K] [--warmup W] [--gpus 1] [--form plain|f64] [--impl ours|reference]

Workload: the 1,000,000-particle dam break (100^3 lattice at 0.5 h spacing, +-1% seeded
jitter, anchored at the min corner of a 5 x 5 x 2.5 m box -- the 20^3 / 1 x 1 x 0.5 m
scene scaled x5 to keep its fill), gravity -9.81, the reference's constants. A step is
one pass of the whole step (grid build, density, forces + walls + integration) over all
particles, launched through the C ABI. By default the timed region is the configuration's
whole 500-step run after the warm-up steps: the column collapses under gravity and
densities (and neighbour counts) rise during the run, so a shorter --steps measures only
its early part.

value : particle-steps/s with the state resident in HBM; L2 is flushed (a 512 MiB write)
        before every timed step, and the step is timed with CUDA events on the
        library's own stream.
e2e   : the same metric through the public C ABI with pinned host buffers: every step
        uploads positions and velocities, steps once, and downloads them.
mixed : the mixed-precision form on the same workload and steps, timed the same way, with
        mixed / plain and its own one-step error against FP64 (--no-mixed skips it).
roofline: algorithmic bytes of the dominant kernel / its event-timed duration, against
        the measured HBM copy bandwidth.
cpu_baseline: the oracle (restatement of the reference's serial CPU step) on 1 host core
        for a bounded sample of the same workload.
--impl reference: the same restatement on all host cores (OpenMP over particles, the
        grid re-binning serial as in the reference), the same workload and metric.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "gmu-water-simulation_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

METRIC = "particle-steps/s, mixed vs plain FP32 on GB300 at stated FP64 error; % HBM peak"
UNIT = "particle-steps/s"
BOX = (5.0, 5.0, 2.5)
DIMS = (100, 100, 100)
GRAVITY = (0.0, -9.81, 0.0)
SEED = 1
H32 = np.float32(0.0457)
KERNELS_PER_STEP = 6  # scan reduce and apply, slot, rank+permute, density, forces


def workload_desc(form):
    return {
        "workload": "dam break, 1,000,000 particles (100^3 lattice, 0.5h spacing, +-1% jitter), "
                    "box 5 x 5 x 2.5 m, 110 x 110 x 55 cells",
        "form": form,
        "particles": 1_000_000,
        "cells": 665_500,
        "steps_from": "initial lattice, after one autotune step and the warm-up steps",
        "l2": "flushed before every timed step (512 MiB write)",
        "parallelism": "single GPU",
    }


def grid_cells(box):
    return int(np.prod([int(np.ceil(np.float32(b) / H32)) for b in box]))


def alg_bytes(N, C, rs=4, forces_variant=4):
    """Compulsory DRAM bytes of each kernel of one step: every array it must touch,
    read or written once (neighbour re-reads are cache hits). rs = bytes per real.
    Force variants 7 and up also have the density pass read velocities and write the packed force
    records, which the force pass then reads."""
    r4 = 4 * rs
    rec = 3 * r4 * N if forces_variant >= 7 else 0  # velocity read + 2 x r4 record written
    return {
        # counts read twice, starts/cursors written, counts zeroed
        "scan": 20 * C,
        # (cell, id) read, id scattered, cursor read-modify-write
        "slot": 12 * N + 8 * C,
        # (cell, id) + the cell's ids read, state read and written in sorted order, starts
        "rank_permute": 8 * N + 4 * N + 4 * r4 * N + 4 * C,
        # sorted positions read, (rho, p, p/rho^2, 1/rho) written, row starts; the mask form
        # also writes the neighbour masks (one word per row at rest density: 36 B)
        "density": r4 * N + r4 * N + 4 * C + MASK_BYTES * N + rec,
        # own position, velocity, aux read; new position, velocity, (cell, id) written;
        # row starts read; counts read-modify-write; the mask form reads the masks
        "forces": 3 * r4 * N + 2 * r4 * N + 8 * N + 12 * C + MASK_BYTES * N + (2 * rec) // 3,
    }


MASK_BYTES = 36  # 9 rows x one 32-bit mask word per particle (rest density)

# DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum) of the dominant kernels
# per force variant, from one ncu capture of an early step of this workload (L2 flushed before
# each replay); profiles/step_kernels_dam_break_1m.md (variant 4) and
# profiles/k_density_mask_k_forces_mask2_records_dam_break_1m.md (variants 7 to 11)
TRAFFIC = {("k_forces", 4): 102.44e6, ("k_density", 4): 21.43e6,
           ("k_forces", 7): 133.90e6, ("k_density", 7): 58.08e6,
           ("k_forces", 8): 133.22e6, ("k_density", 8): 58.17e6,
           ("k_forces", 9): 135.43e6, ("k_density", 9): 58.08e6,
           ("k_forces", 10): 135.40e6, ("k_density", 10): 58.26e6,
           ("k_forces", 11): 133.28e6, ("k_density", 11): 57.91e6}


def load_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region (read-only queries)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0, path=None):
        self.device = device
        self.proc = None
        # the raw samples: a caller-chosen file (--clocks-log), else a temporary one
        self.path = path or os.path.join(tempfile.gettempdir(), f"sph_bench_clocks_{os.getpid()}.csv")

    def start(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_baseline(pos, steps_budget_s=12.0, threads=1):
    """The oracle on `threads` host cores: steps of the same scene until the budget is used."""
    from oracle import oracle as O

    o = O.Oracle(BOX, O.REF, threads=threads, gravity=GRAVITY)
    o.add(pos)
    t0 = time.perf_counter()
    n = 0
    while True:
        o.step(1)
        n += 1
        el = time.perf_counter() - t0
        if el >= steps_budget_s or n >= 20:
            break
    o.close()
    return pos.shape[0] * n / el, n, el


def fp64_error(sphcuda, ctx, form, N):
    """Max relative error against FP64 of one step from the timed run's final state: the state
    (hi + lo positions in double for the mixed form) is uploaded into a fresh context of the
    measured form and into an FP64 context, each steps once, and density, acceleration and
    position are compared (acceleration against the largest FP64 acceleration, position in m)."""
    import ctypes

    L = sphcuda.load()
    x64 = np.zeros((N, 3))
    v32 = ctx.download()["vel"]
    if form == sphcuda.SPH_PLAIN_F32:
        x64 = ctx.download()["pos"].astype(np.float64)
    else:
        L.sph_download_f64(ctx.h, ctypes.c_void_p(x64.ctypes.data), None, None, None, None)
    x32 = x64.astype(np.float32)
    out = {}
    for name, prec in (("form", form), ("f64", sphcuda.SPH_F64)):
        c = sphcuda.SphContext(BOX, N, precision=prec, gravity=GRAVITY, flags=sphcuda.SPH_FLAG_RECORD_ACC)
        c.upload(x32, v32)
        c.step(1)
        out[name] = c.download(acc=True)
        if prec != sphcuda.SPH_PLAIN_F32:
            xx = np.zeros((N, 3))
            L.sph_download_f64(c.h, ctypes.c_void_p(xx.ctypes.data), None, None, None, None)
            out[name]["pos"] = xx
        c.close()
    a, b = out["form"], out["f64"]
    amax = float(np.max(np.linalg.norm(b["acc"], axis=1)))
    return {"after": "one step from the timed run's final state",
            "rho_max_rel": float(np.max(np.abs(a["rho"] - b["rho"]) / np.abs(b["rho"]))),
            "acc_max_err_over_max_acc": float(np.max(np.linalg.norm(a["acc"] - b["acc"], axis=1)) / amax),
            "pos_max_abs_m": float(np.max(np.abs(np.asarray(a["pos"], np.float64) - b["pos"])))}


def mixed_leg(sphcuda, torch, pos, vel0, steps, warmup, flush, dev):
    """The mixed-precision form on the same workload and the same number of steps, timed as the
    plain run (per step: L2 flush, then the three passes between CUDA events on the library's
    stream), with its own one-step FP64 check from its final state."""
    N = pos.shape[0]
    ctx = sphcuda.SphContext(BOX, N, precision=sphcuda.SPH_MIXED, gravity=GRAVITY)
    ctx.upload(pos, vel0)
    ctx.step(1)
    ext = torch.cuda.ExternalStream(ctx.stream, device=dev)

    def one(ev=None):
        with torch.cuda.stream(ext):
            flush.zero_()
        if ev is not None:
            ev[0].record(ext)
        ctx.pass_grid()
        ctx.pass_density()
        ctx.pass_forces()
        if ev is not None:
            ev[1].record(ext)

    for _ in range(warmup):
        one()
    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(2)] for _ in range(steps)]
    torch.cuda.synchronize()
    for k in range(steps):
        one(evs[k])
    torch.cuda.synchronize()
    total_ms = sum(e[0].elapsed_time(e[1]) for e in evs)
    check = fp64_error(sphcuda, ctx, sphcuda.SPH_MIXED, N)
    ctx.close()
    return N * steps / (total_ms / 1000.0), total_ms / steps, check


def run_reference(args):
    """--impl reference: the oracle restatement of the reference's CPU step on all cores."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    import sphcuda
    from oracle import oracle as O

    O.build()
    threads = args.threads or os.cpu_count() or 1
    if args.config == "dam1m":
        box, pos, obstacles, desc, emit = BOX, sphcuda.dam_break_scene(DIMS, BOX, SEED), None, None, None
    else:
        boxes, pos, counts, caps, obs, emit, desc = build_config(sphcuda, args.config)
        if len(boxes) != 1:
            print(json.dumps({"impl": "reference", "unavailable": f"config {args.config}: the oracle runs one "
                              "scene"}))
            return 0
        box, obstacles = boxes[0], (obs[0] if obs else None)
    o = O.Oracle(box, O.REF, threads=threads, gravity=GRAVITY, obstacles=obstacles)
    if pos.shape[0]:
        o.add(pos)
    emitted = [0]

    def one_step():
        # the emitter (host generator, the same particles as the device emitter) is the
        # step's first phase, as generateParticles is in the reference
        if emit is not None and o.n + emit["per_step"] <= emit["cap"]:
            xyz, vel = sphcuda.fountain_emit(7, emitted[0], emit["per_step"], emit["center"], emit["radius"],
                                             emit["speed"], emit["sigma"])
            o.add(xyz, vel)
        emitted[0] += 1
        o.step(1)
        return o.n

    warm = min(args.warmup, 3)
    for _ in range(warm):
        one_step()
    # each timed step is one full step of the scene; stop at K steps or the time budget
    t0 = time.perf_counter()
    done = 0
    work = 0
    while done < args.steps:
        work += one_step()
        done += 1
        if time.perf_counter() - t0 > args.ref_budget:
            break
    el = time.perf_counter() - t0
    value = work / el
    if desc is not None:
        print(json.dumps({"impl": "reference", "config": {"workload": desc}, "value": value, "unit": UNIT,
                          "steps": done, "cores": threads, "ms_per_step": 1000 * el / done}), flush=True)
        return 0
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": done,
        "warmup": warm, "ms_per_step": 1000 * el / done, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": workload_desc("reference CPU step (oracle restatement), float/double as the reference"),
        "impl": "reference",
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{done} of {args.steps} requested steps (time budget {args.ref_budget:.0f} s) of "
                                   f"the 1,000,000-particle dam break after {warm} warm-up steps; density/force "
                                   f"passes on {threads} threads (bit-identical to 1 thread), grid re-binning "
                                   "serial"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def build_config(sphcuda, name, seed=0):
    """Scenes of the other benchmark configurations: (boxes, positions, counts, capacities,
    obstacles, emitter or None, description)."""
    if name == "dam8k":
        box = (1.0, 1.0, 0.5)
        pos = sphcuda.dam_break_scene((20, 20, 20), box, seed)
        return [box], pos, [pos.shape[0]], [pos.shape[0]], None, None, (
            "dam break, 8,000 particles (20^3 lattice), box 1 x 1 x 0.5 m")
    if name == "batch256":
        dims, boxes = sphcuda.batch_plan(256, seed=3)
        parts = [sphcuda.dam_break_scene(tuple(int(x) for x in d), tuple(float(x) for x in b), s)
                 for s, (d, b) in enumerate(zip(dims, boxes))]
        counts = [p.shape[0] for p in parts]
        return list(map(tuple, boxes)), np.concatenate(parts), counts, counts, None, None, (
            f"256 dam-break scenes, {sum(counts):,} particles, counts log-uniform in [2000, 64000], "
            "aspect per axis uniform in [0.5, 2], one launch per pass over all scenes")
    if name == "fountain":
        box = (2.0, 2.0, 2.0)
        emit = {"per_step": 2000, "cap": 2_000_000, "center": (0.0, -1.0 + 0.0229, 0.0), "radius": 0.05,
                "speed": 5.0, "sigma": 0.2}
        return [box], np.zeros((0, 3), np.float32), [0], [emit["cap"]], None, emit, (
            "fountain, 2 x 2 x 2 m box, disc emitter r = 0.05 m at the floor centre, 2,000 particles per step at "
            "5 m/s + N(0, 0.2^2) per component, up to 2,000,000")
    if name == "dam16m":
        s_ = 4.57  # box scale: the 400 x 200 x 200 lattice at 0.5h spans 9.14 x 4.57 x 4.57 m
        box = (4 * s_, s_, s_)
        pos = sphcuda.dam_break_scene((400, 200, 200), box, seed)
        rng = np.random.default_rng(seed + 44)
        obs = []
        for _ in range(8):
            size = rng.uniform(0.05, 0.2, 3) * s_
            c = np.array([rng.uniform(0.05, 0.95) * box[0] / 2, rng.uniform(-0.5, 0.0) * box[1] / 2,
                          rng.uniform(-0.9, 0.9) * box[2] / 2])
            obs += list(c - size / 2) + list(c + size / 2)
        return [box], pos, [pos.shape[0]], [pos.shape[0]], [np.array(obs, np.float32)], None, (
            "dam break, 16,000,000 particles (400 x 200 x 200 lattice), box 18.28 x 4.57 x 4.57 m (the 4 x 1 x 1 m "
            "box scaled x4.57 so the lattice fits; it fills the upstream half), 8 seeded box obstacles of "
            "0.23-0.91 m in the downstream half")
    raise ValueError(name)


def run_config(args):
    """The other benchmark configurations, timed as replayed whole steps (CUDA graphs) with
    events on the context's stream; an emitter step times the device emitter and the step."""
    import torch

    import sphcuda

    sphcuda.load()
    form = {"plain": sphcuda.SPH_PLAIN_F32, "f64": sphcuda.SPH_F64, "mixed": sphcuda.SPH_MIXED}[args.form]
    boxes, pos, counts, caps, obstacles, emit, desc = build_config(sphcuda, args.config)
    ctx = sphcuda.SphContext(boxes, caps, precision=form, gravity=GRAVITY, obstacles=obstacles)
    ctx.upload(pos, None, counts)
    ext = torch.cuda.ExternalStream(ctx.stream, device=torch.device("cuda:0"))
    steps_done = [0]

    def advance(k, timed_ms):
        if emit is None:
            ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            ev0.record(ext)
            ctx.step(k)
            ev1.record(ext)
            ev1.synchronize()
            timed_ms.append(ev0.elapsed_time(ev1))
            return ctx.n * k
        work = 0
        for _ in range(k):
            # the emitter is the step's first phase (generateParticles), generated on the device
            ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            ev0.record(ext)
            if ctx.n + emit["per_step"] <= emit["cap"]:
                ctx.emit_fountain(0, 7, steps_done[0], emit["per_step"], emit["center"], emit["radius"],
                                  emit["speed"], emit["sigma"])
            ctx.step(1)
            ev1.record(ext)
            ev1.synchronize()
            timed_ms.append(ev0.elapsed_time(ev1))
            work += ctx.n
            steps_done[0] += 1
        return work

    if args.variant:
        ctx.set_variant(*[int(v) for v in args.variant.split(",")])
        variant = ctx.variant()
    else:
        variant = ctx.autotune(reps=2) if ctx.n else (0, 3)
        if args.form != "mixed":
            ctx.set_online_tuning(50)
    warm = []
    advance(max(args.warmup, 3), warm)
    ms = []
    work = advance(args.steps, ms)
    st = ctx.stats(0)
    finite = bool(np.isfinite(st["rho_mean"]))
    line = {"metric": METRIC, "value": work / (sum(ms) / 1000.0), "unit": UNIT, "config": {"workload": desc,
            "form": args.form, "particles_final": ctx.n, "scenes": len(boxes)}, "steps": args.steps,
            "warmup": max(args.warmup, 3), "ms_per_step": sum(ms) / args.steps, "launch_variant": list(variant),
            "finite": finite, "rho_mean_scene0": st["rho_mean"], "l2": "not flushed (replayed steps)"}
    ctx.close()
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=500)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--form", default="plain", choices=["plain", "f64", "mixed"])
    ap.add_argument("--e2e-steps", type=int, default=10,
                    help="accepted and ignored: the end-to-end leg always runs the timed run's own steps, "
                         "so that its final state can be compared with the resident run's")
    ap.add_argument("--cpu-budget", type=float, default=12.0)
    ap.add_argument("--ref-budget", type=float, default=90.0)
    ap.add_argument("--threads", type=int, default=0, help="host threads of the reference arm (0 = all)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--variant", default=None, help="pin launch variants 'density,forces' instead of autotuning")
    ap.add_argument("--no-mixed", action="store_true",
                    help="skip the mixed-precision leg of the plain run (mixed over plain on the same steps)")
    ap.add_argument("--clocks-log", default=None,
                    help="file for the raw nvidia-smi clock samples of the timed region (default: a temporary file)")
    ap.add_argument("--save-state", default=None,
                    help="write the final positions and velocities of the timed run (npz)")
    ap.add_argument("--init-state", default=None,
                    help="start from a state written by --save-state (the same 1M dam break, later in its "
                         "run) instead of the initial lattice, e.g. to profile the compressed column")
    ap.add_argument("--config", default="dam1m", choices=["dam1m", "dam8k", "batch256", "fountain", "dam16m"],
                    help="dam1m is the benchmark line; the others are measured separately")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.config != "dam1m":
        return run_config(args)
    if args.gpus != 1 or int(os.environ.get("WORLD_SIZE", "1")) != 1:
        print(json.dumps({"error": "this benchmark runs on one GPU (single-scene path; no multi-GPU path)"}))
        return 2
    args.warmup = max(args.warmup, 3)

    import torch

    import sphcuda

    sphcuda.load()
    form = {"plain": sphcuda.SPH_PLAIN_F32, "f64": sphcuda.SPH_F64, "mixed": sphcuda.SPH_MIXED}[args.form]
    rs = 8 if args.form == "f64" else 4
    pos = sphcuda.dam_break_scene(DIMS, BOX, SEED)
    vel0 = np.zeros_like(pos)
    if args.init_state:
        st = np.load(args.init_state)
        assert st["pos"].shape == pos.shape, "the state must be one of this workload"
        pos, vel0 = np.ascontiguousarray(st["pos"], np.float32), np.ascontiguousarray(st["vel"], np.float32)
    N = pos.shape[0]
    C = grid_cells(BOX)
    dev = torch.device("cuda:0")
    torch.cuda.init()

    ctx = sphcuda.SphContext(BOX, N, precision=form, gravity=GRAVITY)
    ctx.upload(pos, vel0)
    # one untimed step picks the launch variants (all variants compute the same bits)
    if args.variant:
        ctx.set_variant(*[int(v) for v in args.variant.split(",")])
        ctx.step(1)
        variant = ctx.variant()
    else:
        variant = ctx.autotune(reps=3)
        # the state changes over the run (the column compresses): re-time the mask-driven force
        # variants every 50 steps on real steps (all give the same bits)
        if args.form != "mixed":
            ctx.set_online_tuning(50)
    ext = torch.cuda.ExternalStream(ctx.stream, device=dev)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    used = []  # force variant of each timed step (online tuning may change it)

    def one_step(evs=None):
        if evs is not None:
            evs[0].record(ext)
        ctx.pass_grid()
        if evs is not None:
            used.append(ctx.variant()[1])
            evs[1].record(ext)
        ctx.pass_density()
        if evs is not None:
            evs[2].record(ext)
        ctx.pass_forces()
        if evs is not None:
            evs[3].record(ext)

    for _ in range(args.warmup):
        with torch.cuda.stream(ext):
            flush.zero_()
        one_step()
    torch.cuda.synchronize()

    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(4)] for _ in range(args.steps)]
    clocks = ClockSampler(0, args.clocks_log)
    clocks.start()
    time.sleep(0.3)
    torch.cuda.synchronize()
    t_wall0 = time.perf_counter()
    for k in range(args.steps):
        with torch.cuda.stream(ext):
            flush.zero_()
        one_step(evs[k])
    torch.cuda.synchronize()
    t_wall = time.perf_counter() - t_wall0
    clk = clocks.stop()
    grid_ms = [e[0].elapsed_time(e[1]) for e in evs]
    dens_ms = [e[1].elapsed_time(e[2]) for e in evs]
    forc_ms = [e[2].elapsed_time(e[3]) for e in evs]
    step_ms = [e[0].elapsed_time(e[3]) for e in evs]
    total_ms = sum(step_ms)
    value = N * args.steps / (total_ms / 1000.0)
    stats = ctx.stats()
    assert stats["count"] == N and np.isfinite(stats["rho_mean"])
    resident_final = ctx.download()
    if args.save_state:
        np.savez(args.save_state, pos=resident_final["pos"], vel=resident_final["vel"])
    fp64_check = fp64_error(sphcuda, ctx, form, N)

    # bytes of each timed step by the variant it ran, against the summed event times
    ab_steps = [alg_bytes(N, C, rs, v) for v in used]
    ab = {k: sum(a[k] for a in ab_steps) / len(ab_steps) for k in ab_steps[0]}
    main_v = max(set(used), key=used.count)
    peak, peak_src = load_peak()
    mean = lambda xs: sum(xs) / len(xs)
    dom = "forces" if mean(forc_ms) >= mean(dens_ms) else "density"
    dom_ms = mean(forc_ms) if dom == "forces" else mean(dens_ms)
    achieved = ab[dom] / (dom_ms / 1000.0) / 1e9
    traffic = TRAFFIC.get((f"k_{dom}", main_v)) if args.form == "plain" else None
    step_bytes = sum(ab.values())

    # ---- end to end through the C ABI with pinned host buffers, the same state sequence:
    # from the initial upload, one untimed step, W warm-up steps, then K timed steps, each
    # uploading positions and velocities, stepping once and downloading them
    bufs = [(torch.from_numpy(pos.copy()).pin_memory(), torch.from_numpy(vel0.copy()).pin_memory()),
            (torch.empty((N, 3), dtype=torch.float32).pin_memory(),
             torch.empty((N, 3), dtype=torch.float32).pin_memory())]
    counts = np.array([N], np.uint32)

    def e2e_step(k):
        src, dst = bufs[k % 2], bufs[(k + 1) % 2]
        ctx.upload_raw(src[0].data_ptr(), src[1].data_ptr(), counts)
        ctx.step(1)
        ctx.download_raw(dst[0].data_ptr(), dst[1].data_ptr())

    for k in range(1 + args.warmup):
        e2e_step(k)
    t0 = time.perf_counter()
    for k in range(1 + args.warmup, 1 + args.warmup + args.steps):
        e2e_step(k)
    e2e_s = time.perf_counter() - t0
    last = bufs[(1 + args.warmup + args.steps) % 2]
    same = bool(np.array_equal(last[0].numpy(), resident_final["pos"]))
    e2e = {"value": N * args.steps / e2e_s, "unit": UNIT, "h2d_bytes_per_step": 24 * N,
           "d2h_bytes_per_step": 24 * N,
           "path": "sph_upload (pinned xyz+vel) -> sph_step(1) -> sph_download (pinned xyz+vel), host timer",
           "same_final_state_as_resident_run": same}
    ctx.close()

    mixed = None
    if args.form == "plain" and not args.no_mixed:
        mv, mms, mcheck = mixed_leg(sphcuda, torch, pos, vel0, args.steps, args.warmup, flush, dev)
        mixed = {"value": mv, "unit": UNIT, "ms_per_step": mms, "mixed_over_plain": mv / value,
                 "steps": args.steps, "fp64_check": mcheck,
                 "form": "16-bit cell-relative neighbour positions, FP16 neighbour velocities, compensated "
                         "density sums, hi/lo positions"}

    cpu = None
    if not args.no_cpu_baseline:
        try:
            v, n, el = cpu_baseline(pos, args.cpu_budget, threads=1)
            cpu = {"value": v, "unit": UNIT, "cores": 1, "kind": "port",
                   "sample": f"first {n} steps of the same 1,000,000-particle dam break, oracle restatement of "
                             f"the reference's serial CPU step, 1 thread, {el:.1f} s"}
        except Exception as exc:  # report, never drop the line
            cpu = {"value": None, "unit": UNIT, "cores": 1, "kind": "port", "error": repr(exc)}

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if args.form == "f64" else "f32", "data": "synthetic (seeded lattice, no dataset)",
        "config": dict(workload_desc({"plain": "plain FP32", "f64": "FP64", "mixed": "mixed precision"}[args.form]),
                       **({"initial_state": args.init_state} if args.init_state else {})),
        "fp64_check": fp64_check,
        "roofline": {"bound": "hbm", "kernel": f"k_{dom}", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_source": peak_src, "traffic": traffic,
                     "alg_bytes_per_launch": ab[dom], "launch_ms": dom_ms},
        "step_roofline": {"alg_bytes_per_step": step_bytes, "achieved_gbs": step_bytes / (total_ms / args.steps / 1000) / 1e9,
                          "frac": step_bytes / (total_ms / args.steps / 1000) / 1e9 / peak},
        "passes_ms": {"grid": mean(grid_ms), "density": mean(dens_ms), "forces": mean(forc_ms)},
        "e2e": e2e,
        "mixed": mixed,
        "cpu_baseline": cpu,
        "gpu_launches": KERNELS_PER_STEP * args.steps,
        "launch_variant": {"density": variant[0], "forces": main_v,
                           "forces_steps": {str(v): used.count(v) for v in sorted(set(used))},
                           "picked_by": "--variant" if args.variant else
                           "sph_autotune, then online tuning every 50 steps"},
        "clocks": clk,
        "wall_s_timed_region": t_wall,
    }
    print(json.dumps(line), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
