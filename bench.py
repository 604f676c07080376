#!/usr/bin/env python
"""Benchmark of the SPH grid step on one GB300: particle-steps/s.

    python bench.py [--steps K] [--warmup W] [--gpus 1] [--form plain|f64] [--impl ours|reference]

Workload: the 1,000,000-particle dam break (100^3 lattice at 0.5 h spacing, +-1% seeded
jitter, anchored at the min corner of a 5 x 5 x 2.5 m box -- the 20^3 / 1 x 1 x 0.5 m
scene scaled x5 to keep its fill), gravity -9.81, the reference's constants, 500 steps. A
step is one pass of the whole step (grid build, density, forces + walls + integration) over
all particles, launched through the C ABI. The column collapses under gravity and densities
(and neighbour counts) rise during the run, so the K timed steps are spread evenly over the
configuration's whole 500-step run (every 500/K-th step; all of them for K >= 500); the steps
between them run untimed.

value : particle-steps/s with the state resident in HBM; L2 is flushed (a 512 MiB write)
        before every timed step, and the step is timed with CUDA events on the
        library's own stream.
e2e   : the same metric through the public C ABI with pinned host buffers: every step
        uploads positions and velocities, steps once, and downloads them.
mixed : the mixed-precision form on the same workload and steps, timed the same way, with
        mixed / plain and its own one-step error against FP64 (--no-mixed skips it).
batch : the 256-scene batch (particle counts log-uniform in [2000, 64000]), plain and mixed,
        K timed steps spread over its 1,000-step run, with mixed / plain and the error of
        one step against FP64 (--no-batch skips it).
roofline: compulsory bytes of the dominant kernel (each array it must touch read or written
        once) / its event-timed duration, against the measured HBM copy bandwidth; beside it
        the same with the implementation's own bytes (masks, force records) and an issue
        roofline from the kernel's measured instruction count.
cpu_baseline: the oracle (restatement of the reference's serial CPU step) on 1 host core
        for a bounded sample of the same workload.
--impl reference: the same restatement on all host cores (OpenMP over particles, the
        grid re-binning serial as in the reference), the same workload and metric; its
        inputs come from the oracle's own scene restatement, not from the product library.
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
KERNELS_PER_STEP = 6  # scan, slot, crowded-cell sort, rank+permute, density, forces
RUN_STEPS = 500        # the configuration's run
BATCH_RUN_STEPS = 1000  # the 256-scene batch's run
SM_COUNT = 152
ISSUE_PER_SM_CLK = 4   # warp instructions issued per SM and clock (four schedulers)


def workload_desc(form, steps=None):
    k = steps or RUN_STEPS
    run = max(k, RUN_STEPS)
    return {
        "workload": "dam break, 1,000,000 particles (100^3 lattice, 0.5h spacing, +-1% jitter), "
                    "box 5 x 5 x 2.5 m, 110 x 110 x 55 cells, 500-step run",
        "form": form,
        "particles": 1_000_000,
        "cells": 665_500,
        "steps_from": f"{k} timed steps spread evenly over a {run}-step run (every {run / k:g}-th step) that "
                      "starts from the initial lattice after one autotune step and the warm-up steps",
        "l2": "flushed before every timed step (512 MiB write)",
        "parallelism": "single GPU",
    }


def timed_steps(k, run):
    """Indices of the k timed steps, spread evenly over a run of `run` steps (run >= k)."""
    return sorted({(i * run) // k for i in range(k)})


def rehash_steps(sched):
    """Rehash launches inside each step, from the cell multiple of every step: online tuning
    switches into the other multiple at the start of its trial step and back, if the trial lost,
    at the end of that same step; other switches happen at the start of the step that follows."""
    inside = [0] * len(sched)
    for j in range(len(sched) - 1):
        if sched[j + 1] != sched[j]:
            inside[j if j > 0 and sched[j] != sched[j - 1] else j + 1] += 1
    return inside


def grid_cells(box):
    return int(np.prod([int(np.ceil(np.float32(b) / H32)) for b in box]))


def compulsory_bytes(N, C, form="plain"):
    """Algorithmic (compulsory) DRAM bytes of the step's passes: the state each pass must read
    and write once, nothing of the implementation's own intermediates. Plain FP32 per particle:
    density reads the position (16) and writes rho, p (8): 24; forces + walls + integration read
    position, velocity (16 each) and rho, p (8) and write position and velocity (16 each): 72;
    the whole step 196 B per particle plus 12 B per cell for the scan. The mixed form gathers
    8-byte codes and FP16 velocities: density 8 + 8 = 16, forces 32 read + 32 written = 64, the
    step about 115 B per particle. FP64 doubles the plain figures."""
    if form == "mixed":
        return {"density": 16 * N, "forces": 64 * N, "step": 115 * N + 12 * C}
    k = 2 if form == "f64" else 1
    return {"density": 24 * k * N, "forces": 72 * k * N, "step": 196 * k * N + 12 * C}


def alg_bytes(N, C, rs=4, forces_variant=4):
    """The implementation's own DRAM bytes of each kernel of one step: every array it touches,
    read or written once (neighbour re-reads are cache hits), including its intermediates (the
    neighbour masks, the packed force records). rs = bytes per real. Force variants 7 and up
    also have the density pass read velocities and write the packed force records, which the
    force pass then reads."""
    r4 = 4 * rs
    rec = 3 * r4 * N if forces_variant >= 7 else 0  # velocity read + 2 x r4 record written
    return {
        # counts read, starts written (the tile offsets come from the per-group counts)
        "scan": 8 * C,
        # (cell, id) read, id scattered, cell start read, count read-modify-write (back to 0)
        "slot": 12 * N + 12 * C,
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

# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) and warp instructions
# (smsp__inst_executed.sum) per launch of the dominant kernels in the compressed column (step ~254
# of this workload, where most of the run is spent): one `ncu --set full` capture of each kernel
# alone (one launch, cold L2) with force variant 10, keyed by (kernel, cell multiple)
TRAFFIC = {("k_forces", 1): 195.87e6, ("k_density", 1): 91.85e6,
           ("k_forces", 2): 210.64e6, ("k_density", 2): 108.91e6}
ISSUE = {("k_forces", 1): 395.07e6, ("k_density", 1): 311.76e6,
         ("k_forces", 2): 300.89e6, ("k_density", 2): 261.09e6}
TRAFFIC_SOURCE = ("ncu --set full, one launch of the kernel alone at step ~254 (the compressed column, restarted "
                  "with --init-state), force variant 10, on the run's main cell multiple, cold L2")
ISSUE_SOURCE = TRAFFIC_SOURCE


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
        if prec != sphcuda.SPH_F64:  # the measured run's grid
            c.set_cell_multiple(ctx.cell_multiple())
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


def timed_run(ctx, torch, ext, flush, warmup, k, run, on_step=None):
    """Steps a context through `warmup` untimed steps and then a `run`-step run of which the k
    steps of timed_steps(k, run) are timed: per timed step, L2 flushed, then the three passes
    between CUDA events on the library's stream. Returns the per-step event times
    [(grid, density, forces), ...], the (force variant, cell multiple) of each timed step and
    the cell multiple of every step, warm-up included (read after the step's grid pass: online
    tuning may change both between steps)."""
    chosen = []
    sched = []

    def passes(evs=None):
        if evs is not None:
            evs[0].record(ext)
        ctx.pass_grid()
        sched.append(ctx.cell_multiple())
        if evs is not None:
            chosen.append((ctx.variant()[1], sched[-1]))
            evs[1].record(ext)
        ctx.pass_density()
        if evs is not None:
            evs[2].record(ext)
        ctx.pass_forces()
        if evs is not None:
            evs[3].record(ext)

    for _ in range(warmup):
        with torch.cuda.stream(ext):
            flush.zero_()
        passes()
    torch.cuda.synchronize()
    want = set(timed_steps(k, run))
    evs, used = [], []
    if on_step:
        on_step("start")
    for q in range(run):
        if q in want:
            with torch.cuda.stream(ext):
                flush.zero_()
            e = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
            passes(e)
            evs.append(e)
            used.append(chosen[-1])
        else:
            passes()
    torch.cuda.synchronize()
    if on_step:
        on_step("stop")
    times = [(e[0].elapsed_time(e[1]), e[1].elapsed_time(e[2]), e[2].elapsed_time(e[3])) for e in evs]
    return times, used, sched


def mixed_leg(sphcuda, torch, pos, vel0, steps, warmup, flush, dev, run=RUN_STEPS):
    """The mixed-precision form on the same workload, the same warm-up and the same timed steps
    of the same run, timed as the plain run, with its own one-step FP64 check from its final
    state."""
    N = pos.shape[0]
    ctx = sphcuda.SphContext(BOX, N, precision=sphcuda.SPH_MIXED, gravity=GRAVITY)
    ctx.upload(pos, vel0)
    # one autotune step (the plain run's first step), then online tuning of the mixed form's
    # force launch forms, as the plain run does with its own
    ctx.autotune(reps=3)
    ctx.set_online_tuning(50)
    ext = torch.cuda.ExternalStream(ctx.stream, device=dev)
    times, used, _ = timed_run(ctx, torch, ext, flush, warmup, steps, max(steps, run))
    total_ms = sum(sum(t) for t in times)
    check = fp64_error(sphcuda, ctx, sphcuda.SPH_MIXED, N)
    check["cell_multiple_steps"] = {str(m): sum(1 for u in used if u[1] == m) for m in (1, 2)}
    check["passes_ms"] = {k: sum(t[q] for t in times) / len(times) for q, k in enumerate(("grid", "density", "forces"))}
    ctx.close()
    return N * len(times) / (total_ms / 1000.0), total_ms / len(times), check


def batch_scenes(sphcuda, seed=3):
    """The 256 dam-break scenes of the batch configuration: (boxes, positions, counts)."""
    dims, boxes = sphcuda.batch_plan(256, seed=seed)
    parts = [sphcuda.dam_break_scene(tuple(int(x) for x in d), tuple(float(x) for x in b), s)
             for s, (d, b) in enumerate(zip(dims, boxes))]
    return [tuple(float(x) for x in b) for b in boxes], np.concatenate(parts), [p.shape[0] for p in parts]


def batch_fp64_error(sphcuda, ctx, form, boxes, counts):
    """Max relative density error over all particles of all scenes, one step from the batch's
    final state, against an FP64 context of the same scenes."""
    st = ctx.download()
    out = {}
    for name, prec in (("form", form), ("f64", sphcuda.SPH_F64)):
        c = sphcuda.SphContext(boxes, counts, precision=prec, gravity=GRAVITY)
        if prec != sphcuda.SPH_F64:  # the measured run's grid
            c.set_cell_multiple(ctx.cell_multiple())
        c.upload(st["pos"], st["vel"], counts)
        c.step(1)
        out[name] = c.download()["rho"].astype(np.float64)
        c.close()
    return float(np.max(np.abs(out["form"] - out["f64"]) / np.abs(out["f64"])))


def batch_leg(sphcuda, torch, steps, warmup, flush, dev):
    """The 256-scene batch, plain FP32 and mixed: one launch per pass over all scenes, the same
    per-step timing as the headline (L2 flushed before every timed step), k timed steps spread
    over the 1,000-step run, launch variants picked by sph_autotune (and online tuning where the
    form has force variants)."""
    boxes, pos, counts = batch_scenes(sphcuda)
    N = int(sum(counts))
    res = {"workload": f"256 dam-break scenes, {N:,} particles, counts log-uniform in [2000, 64000], aspect "
                       "per axis uniform in [0.5, 2] (seed 3), 1,000-step run",
           "particles": N, "steps": steps, "run": max(steps, BATCH_RUN_STEPS)}
    for name, prec in (("plain", sphcuda.SPH_PLAIN_F32), ("mixed", sphcuda.SPH_MIXED)):
        ctx = sphcuda.SphContext(boxes, counts, precision=prec, gravity=GRAVITY)
        ctx.upload(pos, None, counts)
        ctx.autotune(reps=2)
        ctx.set_online_tuning(50)
        ext = torch.cuda.ExternalStream(ctx.stream, device=dev)
        times, used, _ = timed_run(ctx, torch, ext, flush, warmup, steps, max(steps, BATCH_RUN_STEPS))
        total_ms = sum(sum(t) for t in times)
        res[name] = {"value": N * len(times) / (total_ms / 1000.0), "ms_per_step": total_ms / len(times),
                     "cell_multiple_steps": {str(m): sum(1 for u in used if u[1] == m) for m in (1, 2)},
                     "forces_variants": sorted({u[0] for u in used}),
                     "passes_ms": {k: sum(t[q] for t in times) / len(times)
                                   for q, k in enumerate(("grid", "density", "forces"))},
                     "rho_max_rel_vs_fp64": batch_fp64_error(sphcuda, ctx, prec, boxes, counts)}
        ctx.close()
    res["mixed_over_plain"] = res["mixed"]["value"] / res["plain"]["value"]
    return res


def run_reference(args):
    """--impl reference: the oracle restatement of the reference's CPU step on all cores."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    from oracle import oracle as O
    from oracle import scenes as OS

    O.build()
    threads = args.threads or os.cpu_count() or 1
    if args.config == "dam1m":
        # the scene from the oracle's own restatement of the lattice: this arm loads no product code
        box, pos, obstacles, desc, emit = BOX, OS.dam_break(DIMS, BOX, SEED), None, None, None
    elif args.config == "dam8k":
        box, obstacles, emit = (1.0, 1.0, 0.5), None, None
        pos = OS.dam_break((20, 20, 20), box, 0)
        desc = "dam break, 8,000 particles (20^3 lattice), box 1 x 1 x 0.5 m"
    else:
        import sphcuda  # the other configurations' generators (batch plan, emitter, obstacles)

        boxes, pos, counts, caps, obs, emit, desc = build_config(sphcuda, args.config)
        if len(boxes) != 1:
            return run_reference_batch(args, O, boxes, pos, counts, desc, threads)
        box, obstacles = boxes[0], (obs[0] if obs else None)
    o = O.Oracle(box, O.REF, threads=threads, gravity=GRAVITY, obstacles=obstacles)
    if pos.shape[0]:
        o.add(pos)
    emitted = [0]

    def one_step():
        # the emitter (host generator, the same particles as the device emitter) is the
        # step's first phase, as generateParticles is in the reference
        if emit is not None and o.n + emit["per_step"] <= emit["cap"]:
            import sphcuda

            xyz, vel = sphcuda.fountain_emit(7, emitted[0], emit["per_step"], emit["center"], emit["radius"],
                                             emit["speed"], emit["sigma"])
            o.add(xyz, vel)
        emitted[0] += 1
        o.step(1)
        return o.n

    warm = args.warmup
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
        "config": dict(workload_desc("reference CPU step (oracle restatement), float/double as the reference"),
                       steps_from=f"the first {done} steps after {warm} warm-up steps from the initial lattice "
                                  "(a bounded sample of the run)"),
        "impl": "reference",
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{done} of {args.steps} requested steps (time budget {args.ref_budget:.0f} s) of "
                                   f"the 1,000,000-particle dam break after {warm} warm-up steps; density/force "
                                   f"passes on {threads} threads (bit-identical to 1 thread), grid re-binning "
                                   "serial; scene from the oracle's lattice restatement"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_reference_batch(args, O, boxes, pos, counts, desc, threads):
    """The reference's CPU step on a batch of scenes: one oracle per scene, every scene
    stepped once per step (the reference simulates one scene at a time)."""
    off = np.concatenate([[0], np.cumsum(counts)])
    sims = []
    for s_, box in enumerate(boxes):
        o = O.Oracle(box, O.REF, threads=threads, gravity=GRAVITY)
        o.add(pos[off[s_]:off[s_ + 1]])
        sims.append(o)
    for _ in range(args.warmup):
        for o in sims:
            o.step(1)
    t0 = time.perf_counter()
    done = 0
    while done < args.steps:
        for o in sims:
            o.step(1)
        done += 1
        if time.perf_counter() - t0 > args.ref_budget:
            break
    el = time.perf_counter() - t0
    value = int(off[-1]) * done / el
    print(json.dumps({"impl": "reference", "config": {"workload": desc}, "value": value, "unit": UNIT, "steps": done,
                      "warmup": args.warmup, "cores": threads, "ms_per_step": 1000 * el / done,
                      "sample": f"{done} whole steps of all {len(boxes)} scenes after {args.warmup} warm-up steps, "
                                f"one oracle per scene, density/force passes on {threads} threads"}), flush=True)
    for o in sims:
        o.close()
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


def config_fp64_error(sphcuda, ctx, form, boxes, obstacles, sample=1_000_000):
    """Max relative density error and acceleration error (of the largest FP64 acceleration) of
    one step from the run's final state against an FP64 context of the same scenes, over a seeded
    sample of at most `sample` particles."""
    counts = list(ctx.counts())
    st = ctx.download()
    out = {}
    for name, prec in (("form", form), ("f64", sphcuda.SPH_F64)):
        c = sphcuda.SphContext(boxes, counts, precision=prec, gravity=GRAVITY, obstacles=obstacles,
                               flags=sphcuda.SPH_FLAG_RECORD_ACC)
        if prec != sphcuda.SPH_F64:
            c.set_cell_multiple(ctx.cell_multiple())
        c.upload(st["pos"], st["vel"], counts)
        c.step(1)
        d = c.download(acc=True)
        out[name] = {"rho": d["rho"].astype(np.float64), "acc": d["acc"].astype(np.float64)}
        c.close()
    n = out["f64"]["rho"].shape[0]
    sub = np.random.default_rng(5).choice(n, min(n, sample), replace=False)
    a, b = out["form"], out["f64"]
    amax = float(np.max(np.linalg.norm(b["acc"][sub], axis=1)))
    return {"after": "one step from the run's final state", "particles_compared": int(sub.size),
            "rho_max_rel": float(np.max(np.abs(a["rho"][sub] - b["rho"][sub]) / b["rho"][sub])),
            "acc_max_err_over_max_acc": float(np.max(np.linalg.norm(a["acc"][sub] - b["acc"][sub], axis=1)) / amax)}


def run_config(args):
    """The other benchmark configurations, timed as replayed whole steps (CUDA graphs) with
    events on the context's stream; an emitter step times the device emitter and the step."""
    import torch

    import sphcuda

    sphcuda.load()
    form = {"plain": sphcuda.SPH_PLAIN_F32, "f64": sphcuda.SPH_F64, "mixed": sphcuda.SPH_MIXED}[args.form]
    boxes, pos, counts, caps, obstacles, emit, desc = build_config(sphcuda, args.config)
    ctx = sphcuda.SphContext(boxes, caps, precision=form, gravity=GRAVITY, obstacles=obstacles)
    if args.cell_multiple or args.variant:  # pinned choices (else the autotuner's)
        ctx.set_cell_multiple(args.cell_multiple or 1)
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
        ctx.set_online_tuning(50)
    warm = []
    advance(max(args.warmup, 3), warm)
    ms = []
    work = advance(args.steps, ms)
    # five more steps from the final state (the run's largest particle count), each pass between
    # its own events; the grid pass is the scan, slot, crowded-cell sort, rank and permute
    fin = []
    for _ in range(5):
        e = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
        for q, p in enumerate((ctx.pass_grid, ctx.pass_density, ctx.pass_forces)):
            e[q].record(ext)
            p()
        e[3].record(ext)
        fin.append(e)
    torch.cuda.synchronize()
    final_passes = {k: sum(e[q].elapsed_time(e[q + 1]) for e in fin) / len(fin)
                    for q, k in enumerate(("grid", "density", "forces"))}
    st = ctx.stats(0)
    finite = bool(np.isfinite(st["rho_mean"]))
    check = config_fp64_error(sphcuda, ctx, form, boxes, obstacles) if args.fp64_check else None
    line = {"metric": METRIC, "value": work / (sum(ms) / 1000.0), "unit": UNIT, "config": {"workload": desc,
            "form": args.form, "particles_final": ctx.n, "scenes": len(boxes)}, "steps": args.steps,
            "warmup": max(args.warmup, 3), "ms_per_step": sum(ms) / args.steps,
            "launch_variant": list(ctx.variant()), "cell_multiple": ctx.cell_multiple(),
            "finite": finite, "rho_mean_scene0": st["rho_mean"], "l2": "not flushed (replayed steps)",
            "final_passes_ms": final_passes, "fp64_check": check}
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
    ap.add_argument("--run", type=int, default=RUN_STEPS,
                    help="steps of the run over which the timed steps are spread (default: the configuration's "
                         "500; e.g. a few steps to profile a state given by --init-state)")
    ap.add_argument("--no-batch", action="store_true", help="skip the 256-scene batch leg")
    ap.add_argument("--fp64-check", action="store_true",
                    help="other configurations: one step from the final state against FP64 (density, acceleration)")
    ap.add_argument("--cell-multiple", type=int, default=0,
                    help="pin the step grid's cell multiple (1: cells of h, 2: cells of h/2) instead of autotuning it")
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
    if args.cell_multiple or args.variant:  # pinned choices (else the autotuner's)
        ctx.set_cell_multiple(args.cell_multiple or 1)
    if args.variant:
        ctx.set_variant(*[int(v) for v in args.variant.split(",")])
        ctx.step(1)
        variant = ctx.variant()
    else:
        variant = ctx.autotune(reps=3)
        # the state changes over the run (the column compresses): re-time the force variants
        # every 50 steps on real steps (all give the same bits)
        ctx.set_online_tuning(50)
    cell_mult = ctx.cell_multiple()
    ext = torch.cuda.ExternalStream(ctx.stream, device=dev)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    run = max(args.steps, args.run)
    clocks = ClockSampler(0, args.clocks_log)
    t_wall = [0.0]

    def on_step(what):
        if what == "start":
            clocks.start()
            time.sleep(0.3)
            torch.cuda.synchronize()
            t_wall[0] = time.perf_counter()
        else:
            t_wall[0] = time.perf_counter() - t_wall[0]

    times, used, sched = timed_run(ctx, torch, ext, flush, args.warmup, args.steps, run, on_step)
    # kernels launched in the timed steps: the step's own, plus a rehash for each switch of the
    # cell multiple that online tuning makes inside a timed step
    rehashes = rehash_steps(sched)
    timed_rehash = sum(rehashes[args.warmup + q] for q in timed_steps(args.steps, run))
    clk = clocks.stop()
    K = len(times)
    grid_ms = [t[0] for t in times]
    dens_ms = [t[1] for t in times]
    forc_ms = [t[2] for t in times]
    total_ms = sum(sum(t) for t in times)
    value = N * K / (total_ms / 1000.0)
    stats = ctx.stats()
    assert stats["count"] == N and np.isfinite(stats["rho_mean"])
    resident_final = ctx.download()
    if args.save_state:
        np.savez(args.save_state, pos=resident_final["pos"], vel=resident_final["vel"])
    fp64_check = fp64_error(sphcuda, ctx, form, N)

    peak, peak_src = load_peak()
    mean = lambda xs: sum(xs) / len(xs)
    dom = "forces" if mean(forc_ms) >= mean(dens_ms) else "density"
    dom_ms = mean(forc_ms) if dom == "forces" else mean(dens_ms)
    vs = [u[0] for u in used]
    main_v = max(set(vs), key=vs.count)
    # compulsory bytes (the roofline) and the implementation's own bytes, by the variant each
    # timed step ran
    comp = compulsory_bytes(N, C, args.form)
    ab_steps = [alg_bytes(N, C, rs, v) for v, _ in used]
    ab = {k: sum(a[k] for a in ab_steps) / len(ab_steps) for k in ab_steps[0]}
    achieved = comp[dom] / (dom_ms / 1000.0) / 1e9
    impl_achieved = ab[dom] / (dom_ms / 1000.0) / 1e9
    ms_ = [u[1] for u in used]
    main_m = max(set(ms_), key=ms_.count)  # the cell multiple most timed steps ran on
    traffic = TRAFFIC.get((f"k_{dom}", main_m)) if args.form == "plain" else None
    inst = ISSUE.get((f"k_{dom}", main_m)) if args.form == "plain" else None
    sm_mhz = clk.get("sm_mhz") or 2070.0
    issue = None
    if inst:
        issue_peak = SM_COUNT * ISSUE_PER_SM_CLK * sm_mhz * 1e6
        issue = {"warp_inst_per_launch": inst, "achieved": inst / (dom_ms / 1000.0), "peak": issue_peak,
                 "unit": "warp instructions/s", "frac": inst / (dom_ms / 1000.0) / issue_peak,
                 "source": ISSUE_SOURCE}
    step_ms = total_ms / K

    # ---- end to end through the C ABI with pinned host buffers, the same state sequence:
    # from the initial upload, one untimed step, W warm-up steps, then the run, every step
    # uploading positions and velocities, stepping once and downloading them; the run's sampled
    # steps are timed on the host
    bufs = [(torch.from_numpy(pos.copy()).pin_memory(), torch.from_numpy(vel0.copy()).pin_memory()),
            (torch.empty((N, 3), dtype=torch.float32).pin_memory(),
             torch.empty((N, 3), dtype=torch.float32).pin_memory())]
    counts = np.array([N], np.uint32)

    # the resident run's cell multiple of every step (its first, untimed step included), replayed:
    # the multiple sets the order of each particle's sums, so the same schedule gives the same
    # bits, while the force variants, re-timed online, do not change them
    sched = [cell_mult] + sched

    def e2e_step(k):
        src, dst = bufs[k % 2], bufs[(k + 1) % 2]
        ctx.upload_raw(src[0].data_ptr(), src[1].data_ptr(), counts)
        if ctx.cell_multiple() != sched[k]:
            ctx.set_cell_multiple(sched[k])
        ctx.step(1)
        ctx.download_raw(dst[0].data_ptr(), dst[1].data_ptr())

    for k in range(1 + args.warmup):
        e2e_step(k)
    want = set(timed_steps(args.steps, run))
    e2e_s = 0.0
    for q in range(run):
        k = 1 + args.warmup + q
        if q in want:
            t0 = time.perf_counter()
            e2e_step(k)
            e2e_s += time.perf_counter() - t0
        else:
            e2e_step(k)
    last = bufs[(1 + args.warmup + run) % 2]
    same = bool(np.array_equal(last[0].numpy(), resident_final["pos"]))
    e2e = {"value": N * K / e2e_s, "unit": UNIT, "h2d_bytes_per_step": 24 * N,
           "d2h_bytes_per_step": 24 * N,
           "path": "sph_upload (pinned xyz+vel) -> sph_step(1) -> sph_download (pinned xyz+vel), host timer, "
                   "the same sampled steps of the same run",
           "same_final_state_as_resident_run": same}
    ctx.close()

    mixed = None
    if args.form == "plain" and not args.no_mixed:
        mv, mms, mcheck = mixed_leg(sphcuda, torch, pos, vel0, args.steps, args.warmup, flush, dev, run)
        mixed = {"value": mv, "unit": UNIT, "ms_per_step": mms, "mixed_over_plain": mv / value,
                 "steps": K, "fp64_check": mcheck,
                 "form": "16-bit cell-relative neighbour positions, FP16 neighbour velocities, compensated "
                         "density sums, hi/lo positions"}

    batch = None
    if args.form == "plain" and not args.no_batch and not args.init_state:
        batch = batch_leg(sphcuda, torch, args.steps, args.warmup, flush, dev)

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
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1, "steps": K, "warmup": args.warmup,
        "ms_per_step": step_ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if args.form == "f64" else "f32", "data": "synthetic (seeded lattice, no dataset)",
        "config": dict(workload_desc({"plain": "plain FP32", "f64": "FP64", "mixed": "mixed precision"}[args.form],
                                     K),
                       **({"initial_state": args.init_state, "run": run} if args.init_state else {})),
        "fp64_check": fp64_check,
        "roofline": {"bound": "hbm", "kernel": f"k_{dom}", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_source": peak_src,
                     "bytes": "compulsory: each array the pass must touch read or written once",
                     "alg_bytes_per_launch": comp[dom], "launch_ms": dom_ms,
                     "traffic": traffic, "traffic_source": TRAFFIC_SOURCE if traffic else None,
                     "impl_bytes_per_launch": ab[dom], "frac_impl_bytes": impl_achieved / peak,
                     "issue": issue},
        "step_roofline": {"alg_bytes_per_step": comp["step"], "achieved_gbs": comp["step"] / (step_ms / 1000) / 1e9,
                          "frac": comp["step"] / (step_ms / 1000) / 1e9 / peak,
                          "impl_bytes_per_step": sum(ab.values()),
                          "frac_impl_bytes": sum(ab.values()) / (step_ms / 1000) / 1e9 / peak},
        "passes_ms": {"grid": mean(grid_ms), "density": mean(dens_ms), "forces": mean(forc_ms)},
        "e2e": e2e,
        "mixed": mixed,
        "batch": batch,
        "cpu_baseline": cpu,
        "gpu_launches": KERNELS_PER_STEP * K + timed_rehash,
        "launch_variant": {"density": variant[0], "forces": main_v, "cell_multiple_at_start": cell_mult,
                           "forces_steps": {str(v): vs.count(v) for v in sorted(set(vs))},
                           "cell_multiple_steps": {str(m): sum(1 for u in used if u[1] == m) for m in (1, 2)},
                           "picked_by": "--variant" if args.variant else
                           "sph_autotune (cell multiple and variants), then online tuning every 50 steps"},
        "clocks": clk,
        "wall_s_timed_region": t_wall[0],
    }
    print(json.dumps(line), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
