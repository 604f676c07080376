"""Parity at the benchmark configurations' own sizes.

One step from an identical state must match the reference's CPU method within 1e-5 (plain
FP32, per particle, against the oracle) and the FP64 GPU run; the mixed form must stay within
1e-3 relative density error of the FP64 run. Long runs are chaotic, so their aggregates are
compared with bands taken from the chaotic spread of the FP64 method itself: three FP64 runs
whose inputs differ from the reference FP64 run by one float ulp per particle (random signs). The
band at a snapshot is K_BAND times the running maximum of their deviation from the reference FP64
run up to that snapshot, plus a floor of the form's one-step error; the measured form must stay
inside it.

Configurations (sizes as the benchmark states them):
  1M dam break   100^3 lattice, 5 x 5 x 2.5 m, plain FP32: per particle against the oracle,
                 from the initial lattice and from the compressed column after 250 steps
  256 scenes     counts log-uniform in [2000, 64000]: every scene against its own FP64
                 context (plain and mixed), 8 seeded scenes per particle against the oracle
  16M dam break  400 x 200 x 200 lattice with 8 obstacles, mixed: one step against FP64 on a
                 seeded 1M subsample
  fountain       2,000 particles per step into a 2 m box, mixed and plain: aggregates every
                 100 steps to step 1,000 within bands of the FP64 run
Reference method: src/CCPUParticleSimulator.cpp:93-229 (restated in oracle/sph_oracle.c).
"""
import ctypes
import os

import numpy as np
import pytest

from helpers import assert_within, rel_errors

pytestmark = pytest.mark.gpu

G981 = (0.0, -9.81, 0.0)
K_BAND = 3.0  # bands: K_BAND x the envelope of the FP64 runs' spread + the form's floor
FLOOR = {"plain": 1e-5, "mixed": 3e-3}  # relative, the forms' one-step error levels


def ulp_perturb(a, seed):
    """Every coordinate moved by one float ulp up or down (seeded random signs)."""
    up = np.random.default_rng(seed).integers(0, 2, a.shape) == 1
    return np.where(up, np.nextafter(a, np.float32(np.inf)), np.nextafter(a, np.float32(-np.inf))).astype(np.float32)


def spread_envelope(ref, perturbed):
    """Running maximum over snapshots of the largest relative deviation of the perturbed FP64
    runs from the reference FP64 run (columns: mean density, max density, kinetic energy)."""
    dev = np.max([np.abs(b[:, :3] - ref[:, :3]) / np.abs(ref[:, :3]) for b in perturbed], axis=0)
    return np.maximum.accumulate(dev, axis=0)


def band_ratio(got, ref, env, floor):
    """Worst ratio of the form's relative deviation from the reference FP64 run to its band
    K_BAND * env + floor (<= 1 passes)."""
    dev = np.abs(got[:, :3] - ref[:, :3]) / np.abs(ref[:, :3])
    return float(np.max(dev / (K_BAND * env + floor)))


def f64_state(sphlib, ctx, n):
    x = np.zeros((n, 3)); v = np.zeros((n, 3)); r = np.zeros(n); a = np.zeros((n, 3))
    sphlib.load().sph_download_f64(ctx.h, sphlib._vp(x), sphlib._vp(v), sphlib._vp(r), None, sphlib._vp(a))
    return {"pos": x, "vel": v, "rho": r, "acc": a}


# ------------------------------------------------------------------------- 1M dam break
@pytest.mark.parametrize("cell_mult", [1, 2])
@pytest.mark.parametrize("start", ["lattice", "step250"])
def test_dam1m_one_step_vs_oracle(sphlib, oracle_mod, start, cell_mult):
    """The 1,000,000-particle dam break: one plain FP32 step per particle against the oracle
    (all host cores), within the 1e-5 band of helpers.py, from the initial lattice and from the
    compressed column 250 steps later, on cells of h and of h/2."""
    box = (5.0, 5.0, 2.5)
    pos = sphlib.dam_break_scene((100, 100, 100), box, seed=1)
    vel = np.zeros_like(pos)
    n = pos.shape[0]
    if start == "step250":
        ctx = sphlib.SphContext(box, n, gravity=G981)
        ctx.upload(pos)
        ctx.step(250)
        d = ctx.download()
        ctx.close()
        pos, vel = d["pos"], d["vel"]
    ctx = sphlib.SphContext(box, n, gravity=G981, flags=sphlib.SPH_FLAG_RECORD_ACC)
    ctx.set_cell_multiple(cell_mult)
    ctx.upload(pos, vel)
    ctx.step(1)
    got = ctx.download(acc=True)
    ctx.close()
    o = oracle_mod.Oracle(box, oracle_mod.REF, threads=os.cpu_count(), gravity=G981)
    o.add(pos, vel)
    o.step(1)
    ref = o.state()
    o.close()
    errs = rel_errors(got, ref)
    print(f"dam1m {start} cells h/{cell_mult}: normalised errors {errs}")
    if start == "lattice":
        assert_within(errs, f"dam1m/{start}/cells h/{cell_mult}")
        return
    # In the compressed column many particles sit near rest density, where p = k (rho - rho0)
    # cancels: the reference's own float arithmetic then deviates from the exact (FP64) step by up
    # to ~1.5e-5 of the acceleration scale A, so two float implementations cannot agree within
    # 1e-5 A everywhere. Required: density, pressure and positions within the band everywhere;
    # accelerations within the band for 99.99% of particles and within twice it for all; and the
    # GPU step's largest deviation from the FP64 step no larger than 1.25 times the oracle's.
    assert_within({k: v for k, v in errs.items() if k != "acc"}, f"dam1m/{start}/cells h/{cell_mult}")
    A = np.asarray(ref["ascale"], np.float64)
    c64 = sphlib.SphContext(box, n, precision=sphlib.SPH_F64, gravity=G981, flags=sphlib.SPH_FLAG_RECORD_ACC)
    c64.upload(pos, vel)
    c64.step(1)
    exact = f64_state(sphlib, c64, n)["acc"]
    c64.close()
    norm = lambda a, b: np.linalg.norm(np.asarray(a, np.float64) - np.asarray(b, np.float64), axis=1) / (1e-5 * A)
    e_go, e_gx, e_ox = norm(got["acc"], ref["acc"]), norm(got["acc"], exact), norm(ref["acc"], exact)
    print(f"  acceleration / (1e-5 A): GPU-oracle 99.99% {np.quantile(e_go, 0.9999):.3f} max {e_go.max():.3f}; "
          f"GPU-FP64 max {e_gx.max():.3f}; oracle-FP64 max {e_ox.max():.3f}")
    assert np.quantile(e_go, 0.9999) <= 1.0 and e_go.max() <= 2.0, (np.quantile(e_go, 0.9999), e_go.max())
    assert e_gx.max() <= 1.25 * e_ox.max(), (e_gx.max(), e_ox.max())


# ------------------------------------------------------------------------- 256 scenes
def batch256(sphlib):
    dims, boxes = sphlib.batch_plan(256, seed=3)
    parts = [sphlib.dam_break_scene(tuple(int(x) for x in d), tuple(float(x) for x in b), s)
             for s, (d, b) in enumerate(zip(dims, boxes))]
    return [tuple(float(x) for x in b) for b in boxes], parts


@pytest.mark.parametrize("form", ["plain", "mixed"])
def test_batch256_every_scene_vs_f64(sphlib, form):
    """The 256-scene batch, one step after 30 steps of flow: every scene of the batch against
    its own single-scene FP64 context started from the same state. Plain FP32: density within
    1e-5 relative, acceleration within 1e-5 of the scene's largest; mixed: density within 1e-3,
    acceleration within 1e-2 of the scene's largest (neighbour velocities and force factors are
    FP16; measured up to 5.6e-3)."""
    boxes, parts = batch256(sphlib)
    counts = [p.shape[0] for p in parts]
    prec = {"plain": sphlib.SPH_PLAIN_F32, "mixed": sphlib.SPH_MIXED}[form]
    warm = sphlib.SphContext(boxes, counts, gravity=G981)
    warm.upload(np.concatenate(parts), None, counts)
    warm.step(30)
    st = warm.download()
    warm.close()
    ctx = sphlib.SphContext(boxes, counts, precision=prec, gravity=G981, flags=sphlib.SPH_FLAG_RECORD_ACC)
    ctx.upload(st["pos"], st["vel"], counts)
    ctx.step(1)
    got = ctx.download(acc=True)
    ctx.close()
    off = np.concatenate([[0], np.cumsum(counts)])
    worst_rho = worst_acc = 0.0
    for s in range(256):
        sl = slice(off[s], off[s + 1])
        c = sphlib.SphContext(boxes[s], counts[s], precision=sphlib.SPH_F64, gravity=G981,
                              flags=sphlib.SPH_FLAG_RECORD_ACC)
        c.upload(st["pos"][sl], st["vel"][sl])
        c.step(1)
        ref = f64_state(sphlib, c, counts[s])
        c.close()
        worst_rho = max(worst_rho, float(np.max(np.abs(got["rho"][sl] - ref["rho"]) / ref["rho"])))
        amax = np.max(np.linalg.norm(ref["acc"], axis=1))
        worst_acc = max(worst_acc, float(np.max(np.linalg.norm(got["acc"][sl] - ref["acc"], axis=1)) / amax))
    print(f"batch256 {form}: worst density {worst_rho:.3e}, worst acceleration {worst_acc:.3e} of the scene's max")
    tol_rho, tol_acc = (1e-5, 1e-5) if form == "plain" else (1e-3, 1e-2)
    assert worst_rho < tol_rho and worst_acc < tol_acc, (worst_rho, worst_acc)


def test_batch256_scenes_vs_oracle(sphlib, oracle_mod):
    """Eight seeded scenes of the 256-scene batch, per particle against the oracle, one plain
    FP32 step of the whole batch from the initial lattices."""
    boxes, parts = batch256(sphlib)
    counts = [p.shape[0] for p in parts]
    ctx = sphlib.SphContext(boxes, counts, gravity=G981, flags=sphlib.SPH_FLAG_RECORD_ACC)
    ctx.upload(np.concatenate(parts), None, counts)
    ctx.step(1)
    got = ctx.download(acc=True)
    ctx.close()
    off = np.concatenate([[0], np.cumsum(counts)])
    for s in np.random.default_rng(8).choice(256, 8, replace=False):
        sl = slice(off[s], off[s + 1])
        o = oracle_mod.Oracle(boxes[s], oracle_mod.REF, threads=os.cpu_count(), gravity=G981)
        o.add(parts[s])
        o.step(1)
        ref = o.state()
        o.close()
        assert_within(rel_errors({k: v[sl] for k, v in got.items()}, ref), f"batch scene {s}")


# ------------------------------------------------------------------------- 16M, mixed
def test_dam16m_mixed_vs_f64_subsample(sphlib):
    """The 16M dam break with obstacles in the mixed form: one step against the FP64 run of
    the same state, on the seeded 1M subsample: density within 1e-3 relative, acceleration
    within 5e-3 of the subsample's largest (A), position within 4 float ulp + 5e-3 A dt^2."""
    s_ = 4.57
    box = (4 * s_, s_, s_)
    pos = sphlib.dam_break_scene((400, 200, 200), box, seed=4)
    rng = np.random.default_rng(48)
    obs = []
    for _ in range(8):
        size = rng.uniform(0.05, 0.2, 3) * s_
        cen = np.array([rng.uniform(0.05, 0.95) * box[0] / 2, rng.uniform(-0.5, 0.0) * box[1] / 2,
                        rng.uniform(-0.9, 0.9) * box[2] / 2])
        obs += list(cen - size / 2) + list(cen + size / 2)
    obs = [np.array(obs, np.float32)]
    n = pos.shape[0]
    sub = np.random.default_rng(5).choice(n, 1_000_000, replace=False)
    out = {}
    for name, prec in (("mixed", sphlib.SPH_MIXED), ("f64", sphlib.SPH_F64)):
        ctx = sphlib.SphContext(box, n, precision=prec, gravity=G981, obstacles=obs, flags=sphlib.SPH_FLAG_RECORD_ACC)
        ctx.upload(pos)
        ctx.step(1)
        st = f64_state(sphlib, ctx, n)
        out[name] = {k: v[sub] for k, v in st.items()}
        ctx.close()
    a, b = out["mixed"], out["f64"]
    rho_err = float(np.max(np.abs(a["rho"] - b["rho"]) / b["rho"]))
    amax = np.max(np.linalg.norm(b["acc"], axis=1))
    acc_err = float(np.max(np.linalg.norm(a["acc"] - b["acc"], axis=1)) / amax)
    bound = 4 * np.spacing(np.abs(b["pos"]).astype(np.float32)).astype(np.float64) + 5e-3 * amax * 1e-4
    pos_err = float(np.max(np.abs(a["pos"] - b["pos"]) / bound))
    print(f"dam16m mixed: density {rho_err:.3e}, acceleration {acc_err:.3e} of max, position {pos_err:.3f} of bound")
    assert rho_err < 1e-3 and acc_err < 5e-3 and pos_err <= 1.0, (rho_err, acc_err, pos_err)


# ------------------------------------------------------------------------- fountain bands
FOUNTAIN = {"box": (2.0, 2.0, 2.0), "per_step": 2000, "cap": 2_000_000, "center": (0.0, -1.0 + 0.0229, 0.0),
            "radius": 0.05, "speed": 5.0, "sigma": 0.2, "seed": 7}


def fountain_aggregates(sphlib, prec, steps, every, perturb=None):
    """Mean and max density, kinetic energy and particle count of the fountain every `every`
    steps. The emitter is the step's first phase: on the device, or (perturb = a seed) the same
    particles from the host generator with every coordinate moved by one float ulp."""
    f = FOUNTAIN
    ctx = sphlib.SphContext(f["box"], f["cap"], precision=prec, gravity=G981)
    ctx.upload(np.zeros((0, 3), np.float32), None, [0])
    out = []
    for step in range(steps):
        if ctx.n + f["per_step"] <= f["cap"]:
            if perturb is None:
                ctx.emit_fountain(0, f["seed"], step, f["per_step"], f["center"], f["radius"], f["speed"], f["sigma"])
            else:
                x, v = sphlib.fountain_emit(f["seed"], step, f["per_step"], f["center"], f["radius"], f["speed"],
                                            f["sigma"])
                ctx.append(0, ulp_perturb(x, perturb * 100003 + step), v)
        ctx.step(1)
        if step % every == every - 1:
            s = ctx.stats(0)
            out.append((s["rho_mean"], s["rho_max"], s["kinetic"], s["count"]))
    ctx.close()
    return np.array(out)


@pytest.fixture(scope="module")
def fountain_fp64(sphlib):
    """The fountain's FP64 run and its spread envelope (three one-ulp perturbed FP64 runs), 1,000
    steps, snapshots every 100."""
    ref = fountain_aggregates(sphlib, sphlib.SPH_F64, 1000, 100)
    pert = [fountain_aggregates(sphlib, sphlib.SPH_F64, 1000, 100, perturb=k) for k in (1, 2, 3)]
    for b in pert:
        assert np.array_equal(b[:, 3], ref[:, 3])
    return ref, spread_envelope(ref, pert)


@pytest.mark.parametrize("form", ["plain", "mixed"])
def test_fountain_bands_vs_f64(sphlib, fountain_fp64, form):
    """The fountain (2,000 particles a step into the 2 m box, extreme occupancy skew), 1,000
    steps: every 100 steps the form's mean and max density and kinetic energy stay within
    K_BAND times the FP64 spread envelope plus the form's floor; the particle counts are equal."""
    ref, env = fountain_fp64
    prec = {"plain": sphlib.SPH_PLAIN_F32, "mixed": sphlib.SPH_MIXED}[form]
    got = fountain_aggregates(sphlib, prec, 1000, 100)
    assert np.array_equal(got[:, 3], ref[:, 3])
    worst = band_ratio(got, ref, env, FLOOR[form])
    print(f"fountain {form}: envelope at step 1000 {env[-1]}, deviation "
          f"{np.abs(got[-1, :3] - ref[-1, :3]) / np.abs(ref[-1, :3])}, worst deviation / band {worst:.3f}")
    assert worst <= 1.0, worst


# ------------------------------------------------------------------------- all-pairs form
def test_all_pairs_vs_oracle_brute_and_reference_brute(sphlib, oracle_mod):
    """The all-pairs form (SPH_FLAG_ALL_PAIRS) against the oracle's all-pairs restatement
    (orc_brute_step, sph_brute.cl:9-57) per particle within the 1e-5 band, and against the
    reference's own brute-force kernels' golden outputs (density, pressure; acceleration away
    from the walls)."""
    from test_oracle import interior, ref_cl_cases

    for c in ref_cl_cases():
        if "brute_rho" not in c:
            continue
        box = tuple(float(x) for x in c["box"])
        ctx = sphlib.SphContext(box, c["pos"].shape[0], gravity=c["gravity"],
                                flags=sphlib.SPH_FLAG_ALL_PAIRS | sphlib.SPH_FLAG_RECORD_ACC)
        ctx.upload(c["pos"], c["vel"])
        ctx.step(1)
        got = ctx.download(acc=True)
        ctx.close()
        # the per-particle force scale A of the tolerance comes from the grid oracle's step
        og = oracle_mod.Oracle(box, oracle_mod.REF, threads=4, gravity=c["gravity"])
        og.add(c["pos"], c["vel"])
        og.step(1)
        ascale = og.state()["ascale"]
        og.close()
        o = oracle_mod.Oracle(box, oracle_mod.REF, threads=4, gravity=c["gravity"])
        o.add(c["pos"], c["vel"])
        o.brute_step()
        ref = o.state()
        ref["ascale"] = ascale
        o.close()
        assert_within(rel_errors(got, ref), c["name"] + "/oracle brute")
        inside = interior(c["pos"], box)
        errs = rel_errors({"rho": got["rho"], "p": got["p"]},
                          {"rho": c["brute_rho"], "p": c["brute_p"], "ascale": ref["ascale"]})
        errs.update(rel_errors({"acc": got["acc"][inside]}, {"rho": c["brute_rho"][inside],
                                                             "acc": c["brute_acc"][inside],
                                                             "ascale": ref["ascale"][inside]}))
        assert_within(errs, c["name"] + "/reference brute kernels")
