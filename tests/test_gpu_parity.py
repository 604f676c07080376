"""GPU parity of the CUDA step (through the C ABI) against the oracle.

Tolerances (see helpers.py): plain FP32 within 1e-5 relative to each quantity's scale;
the FP64 GPU run within 1e-10 of the FP64 oracle; the grid (cells, counts, sorted order)
bit-exact. Long runs are chaotic, so they are compared as bands on aggregates.
"""
import json
import os

import numpy as np
import pytest

from helpers import assert_within, rel_errors

pytestmark = pytest.mark.gpu

H32 = np.float32(0.0457)
C0_BOX = (1.0, 1.0, 0.5)
G981 = (0.0, -9.81, 0.0)


def c0_scene(sphlib, dims=(20, 20, 20), box=C0_BOX, seed=0):
    return sphlib.dam_break_scene(dims, box, seed)


def gpu_run(sphlib, box, pos, vel=None, steps=1, precision=0, gravity=None, flags=2, cell_mult=1):
    ctx = sphlib.SphContext(box, pos.shape[0], precision=precision, flags=flags, gravity=gravity)
    if cell_mult != 1:
        ctx.set_cell_multiple(cell_mult)
    ctx.upload(pos, vel)
    ctx.step(steps)
    out = ctx.download(acc=bool(flags & 2))
    ctx.close()
    return out


def oracle_run(O, box, pos, vel=None, steps=1, mode=None, gravity=None):
    o = O.Oracle(box, O.REF if mode is None else mode, threads=os.cpu_count(), gravity=gravity)
    o.add(pos, vel)
    o.step(steps)
    s = o.state64() if mode == O.F64 else o.state()
    s["ascale"] = o.state()["ascale"]
    return s


def cells_numpy(pos, box):
    """The reference's hash, vectorised in float64: floor((p + box/2.0) / h), clamped."""
    box = np.asarray(box, np.float32)
    res = np.ceil(box / H32).astype(np.int64)
    q = (pos.astype(np.float64) + box.astype(np.float64) / 2.0) / np.float64(H32)
    c = np.floor(q)
    c = np.where(q >= 0, c, 0)
    c = np.minimum(c, res - 1).astype(np.int64)
    return c[:, 0] + c[:, 1] * res[0] + c[:, 2] * res[0] * res[1], res


def scenes(sphlib, oracle_mod):
    rng = np.random.default_rng(11)
    out = {"ref_default_0.4": ((0.4, 0.4, 0.4), oracle_mod.reference_dam_break(0.4), None, None)}
    p = c0_scene(sphlib)
    out["c0_8000"] = (C0_BOX, p, None, G981)
    out["c0_8000_moving"] = (C0_BOX, p, rng.normal(0, 0.5, p.shape).astype(np.float32), G981)
    q = c0_scene(sphlib, dims=(12, 9, 14), box=(0.45, 0.5, 0.6), seed=5)
    q[:40] -= np.float32(0.02)  # some outside the min walls: clamped cells, wall forces
    out["outside_walls"] = ((0.45, 0.5, 0.6), q, rng.normal(0, 0.2, q.shape).astype(np.float32), None)
    # ~80 particles per cell: rows of ~250 candidates, beyond the four recorded mask words
    # (the force kernels' fallback that tests the remaining candidates itself)
    cl = (rng.random((1500, 3)) * 0.12 - 0.06).astype(np.float32)
    out["dense_clump"] = ((0.5, 0.5, 0.5), cl, rng.normal(0, 0.1, cl.shape).astype(np.float32), G981)
    return out


# ------------------------------------------------------------------------- grid
def test_grid_bit_exact(sphlib, oracle_mod):
    O = oracle_mod
    for name, (box, pos, vel, g) in scenes(sphlib, oracle_mod).items():
        ctx = sphlib.SphContext(box, pos.shape[0], gravity=g)
        ctx.upload(pos, vel)
        for rep in range(2):
            cur = ctx.download()["pos"] if rep else pos
            ctx.pass_grid()
            cell, counts, order = ctx.grid()
            o = O.Oracle(box, O.REF, threads=1)
            o.add(cur)
            o.update_grid()
            ocell, ocounts, oorder = o.grid()
            assert np.array_equal(cell, ocell.astype(np.uint32)), name
            assert np.array_equal(counts, ocounts.astype(np.uint32)), name
            assert np.array_equal(order, oorder.astype(np.uint32)), name
            ncell, _ = cells_numpy(cur, box)
            assert np.array_equal(cell.astype(np.int64), ncell), name
            # finish this step and re-check the grid of the moved particles
            ctx.pass_density()
            ctx.pass_forces()
            ctx.step(4)
        ctx.close()


@pytest.mark.parametrize("prec", ["plain", "mixed"])
def test_grid_reported_on_half_cells(sphlib, oracle_mod, prec):
    """On cells of h/2 the step's grid is finer, and sph_get_grid still reports the reference's
    grid (cells of size h: cell of every particle, counts, (cell, id) order) bit for bit, for a
    batch of scenes, before and after the particles move."""
    form = {"plain": sphlib.SPH_PLAIN_F32, "mixed": sphlib.SPH_MIXED}[prec]
    sc = scenes(sphlib, oracle_mod)
    names = ["c0_8000_moving", "outside_walls", "dense_clump"]
    boxes = [sc[k][0] for k in names]
    parts = [sc[k][1] for k in names]
    vels = np.concatenate([sc[k][2] for k in names])
    counts = [p.shape[0] for p in parts]
    ctx = sphlib.SphContext(boxes, counts, precision=form, gravity=G981)
    ctx.set_cell_multiple(2)
    assert ctx.cell_multiple() == 2
    ctx.upload(np.concatenate(parts), vels, counts)
    off = np.concatenate([[0], np.cumsum(counts)])
    for rep in range(2):
        cur = ctx.download()["pos"]
        ctx.pass_grid()
        cell, cnt, order = ctx.grid()
        cbase = 0
        for s_, (box, n) in enumerate(zip(boxes, counts)):
            o = oracle_mod.Oracle(box, oracle_mod.CANON, threads=1)
            o.add(cur[off[s_]:off[s_ + 1]])
            o.update_grid()
            ocell, ocounts, oorder = o.grid()
            assert np.array_equal(cell[off[s_]:off[s_ + 1]], ocell.astype(np.uint32)), (prec, rep, s_)
            assert np.array_equal(cnt[cbase:cbase + ocounts.size], ocounts.astype(np.uint32)), (prec, rep, s_)
            assert np.array_equal(order[off[s_]:off[s_ + 1]], oorder.astype(np.uint32)), (prec, rep, s_)
            cbase += ocounts.size
        ctx.pass_density()
        ctx.pass_forces()
        ctx.step(3)
    ctx.close()


def test_cell_multiple_errors(sphlib):
    """Cells of h/2 are for the plain and mixed grid forms and change between steps only."""
    f64 = sphlib.SphContext(C0_BOX, 100, precision=sphlib.SPH_F64)
    with pytest.raises(sphlib.SphError) as e:
        f64.set_cell_multiple(2)
    assert e.value.code == sphlib.SPH_ERR_UNSUPPORTED
    f64.close()
    ap = sphlib.SphContext(C0_BOX, 100, flags=sphlib.SPH_FLAG_ALL_PAIRS)
    with pytest.raises(sphlib.SphError) as e:
        ap.set_cell_multiple(2)
    assert e.value.code == sphlib.SPH_ERR_UNSUPPORTED
    ap.close()
    ctx = sphlib.SphContext(C0_BOX, 100)
    for bad in (0, 3, -1):
        with pytest.raises(sphlib.SphError) as e:
            ctx.set_cell_multiple(bad)
        assert e.value.code == sphlib.SPH_ERR_ARG
    ctx.set_cell_multiple(2)
    with pytest.raises(sphlib.SphError) as e:
        ctx.set_variant(0, 4)  # cells of h/2 run the record variants 7-11 only
    assert e.value.code == sphlib.SPH_ERR_ARG
    ctx.upload(c0_scene(sphlib, dims=(4, 5, 5)))
    ctx.pass_grid()
    with pytest.raises(sphlib.SphError) as e:
        ctx.set_cell_multiple(1)
    assert e.value.code == sphlib.SPH_ERR_STATE
    ctx.pass_density()
    ctx.pass_forces()
    ctx.set_cell_multiple(1)
    ctx.step(2)
    assert np.all(np.isfinite(ctx.download()["pos"]))
    ctx.close()


def test_cell_multiple_switch_between_steps(sphlib, oracle_mod):
    """Switching the cell multiple between steps re-hashes the held particles: a run that switches
    twice matches the oracle's run of the same steps within the one-step band per step."""
    box, pos, vel, g = scenes(sphlib, oracle_mod)["c0_8000_moving"]
    ctx = sphlib.SphContext(box, pos.shape[0], gravity=g, flags=sphlib.SPH_FLAG_RECORD_ACC)
    ctx.upload(pos, vel)
    for m in (2, 1, 2):
        cur = ctx.download()
        ctx.set_cell_multiple(m)
        ctx.step(1)
        got = ctx.download(acc=True)
        ref = oracle_run(oracle_mod, box, cur["pos"], cur["vel"], gravity=g)
        assert_within(rel_errors(got, ref), f"switch to cells h/{m}")
    ctx.close()


def test_grid_cell_faces(sphlib, oracle_mod):
    """Coordinates on and one ulp around every cell face hash exactly as the double formula."""
    box = (0.4, 0.4, 0.4)
    faces = [np.float32(np.float32(k) * H32 - np.float32(0.2)) for k in range(0, 10)]
    vals = []
    for f in faces:
        vals += [f, np.nextafter(f, np.float32(-1)), np.nextafter(f, np.float32(1))]
    vals = np.array(vals, np.float32)
    rng = np.random.default_rng(1)
    pos = np.stack([vals, rng.permutation(vals), rng.permutation(vals)], axis=1).astype(np.float32)
    ctx = sphlib.SphContext(box, pos.shape[0])
    ctx.upload(pos)
    ctx.pass_grid()
    cell, counts, order = ctx.grid()
    want, _ = cells_numpy(pos, box)
    assert np.array_equal(cell.astype(np.int64), want)
    o = oracle_mod.Oracle(box, oracle_mod.CANON, threads=1)
    o.add(pos)
    o.update_grid()
    assert np.array_equal(order, o.grid()[2].astype(np.uint32))
    ctx.close()


def crowded_scene(seed=4):
    """Cells far above rest occupancy: one cell of 2,500 particles (sorted in shared memory), one of
    20,000 (above the 4,096 that are sorted; those are counted), 40 cells of 100-160 (around the
    128 that are counted directly), and a sparse lattice around them."""
    rng = np.random.default_rng(seed)
    box = (0.6, 0.6, 0.6)
    h = float(H32)
    parts = []
    for cidx, n in (((2, 3, 4), 2500), ((8, 8, 8), 20000)):
        lo = np.array(cidx) * h - 0.3
        parts.append(lo + (0.05 + 0.9 * rng.random((n, 3))) * h)
    for k in range(40):
        cidx = rng.integers(0, 13, 3)
        lo = cidx * h - 0.3
        parts.append(lo + (0.05 + 0.9 * rng.random((int(rng.integers(100, 161)), 3))) * h)
    g = np.stack(np.meshgrid(*[np.arange(6) * 0.09 - 0.25] * 3, indexing="ij"), -1).reshape(-1, 3)
    parts.append(g)
    pos = np.concatenate(parts).astype(np.float32)
    return box, pos[rng.permutation(pos.shape[0])]


@pytest.mark.parametrize("prec", ["plain", "mixed", "f64"])
def test_grid_crowded_cells_bit_exact(sphlib, oracle_mod, prec):
    """The canonical (cell, id) order in cells of thousands of particles (sorted slot ids and a
    lower-bound rank) and of tens of thousands (counted) equals the oracle's grid bit for bit,
    in every precision form, before and after the particles move."""
    box, pos = crowded_scene()
    form = {"plain": sphlib.SPH_PLAIN_F32, "mixed": sphlib.SPH_MIXED, "f64": sphlib.SPH_F64}[prec]
    # a short time step keeps the crowded particles (pressures far above any physical state)
    # near their cells for the second grid pass, which starts from the force pass's hashes
    ctx = sphlib.SphContext(box, pos.shape[0], precision=form, params=sphlib.default_params(dt=1e-5, gravity=G981))
    ctx.upload(pos)
    # FP64 positions are compared from the upload only: their float copies could round across a face
    for rep in range(1 if prec == "f64" else 2):
        cur = ctx.download()["pos"] if rep else pos
        assert np.all(np.isfinite(cur))
        ctx.pass_grid()
        cell, counts, order = ctx.grid()
        assert counts.max() >= 20000 and np.sum(counts > 128) >= 15 and np.sum((counts > 32) & (counts <= 128)) >= 5
        o = oracle_mod.Oracle(box, oracle_mod.CANON, threads=1)
        o.add(cur)
        o.update_grid()
        ocell, ocounts, oorder = o.grid()
        assert np.array_equal(cell, ocell.astype(np.uint32)), (prec, rep)
        assert np.array_equal(counts, ocounts.astype(np.uint32)), (prec, rep)
        assert np.array_equal(order, oorder.astype(np.uint32)), (prec, rep)
        ctx.pass_density()
        ctx.pass_forces()
    ctx.close()


# ------------------------------------------------------------------------- one step
@pytest.mark.parametrize("cell_mult", [1, 2])
@pytest.mark.parametrize("name", ["ref_default_0.4", "c0_8000", "c0_8000_moving", "outside_walls", "dense_clump"])
def test_one_step_plain_vs_oracle(sphlib, oracle_mod, name, cell_mult):
    """One plain FP32 step per particle against the oracle, on the reference's cells of size h
    and on cells of h/2 (the same method, candidates summed in another order)."""
    box, pos, vel, g = scenes(sphlib, oracle_mod)[name]
    got = gpu_run(sphlib, box, pos, vel, gravity=g, cell_mult=cell_mult)
    ref = oracle_run(oracle_mod, box, pos, vel, gravity=g)
    assert_within(rel_errors(got, ref), f"{name}/cells h/{cell_mult}")


@pytest.mark.parametrize("name", ["ref_default_0.4", "c0_8000_moving", "outside_walls"])
def test_one_step_f64_vs_oracle_f64(sphlib, oracle_mod, name):
    O = oracle_mod
    box, pos, vel, g = scenes(sphlib, oracle_mod)[name]
    got = gpu_run(sphlib, box, pos, vel, gravity=g, precision=sphlib.SPH_F64)
    ref = oracle_run(O, box, pos, vel, gravity=g, mode=O.F64)
    assert np.max(np.abs(got["rho"] - ref["rho"]) / ref["rho"]) < 1e-12
    err = np.linalg.norm(got["acc"] - ref["acc"], axis=1) / ref["ascale"]
    assert err.max() < 1e-10
    assert np.abs(got["pos"] - ref["pos"]).max() < 1e-13


@pytest.mark.parametrize("name", ["ref_default_0.4", "c0_8000_moving"])
def test_one_step_plain_vs_f64_gpu(sphlib, oracle_mod, name):
    box, pos, vel, g = scenes(sphlib, oracle_mod)[name]
    a = gpu_run(sphlib, box, pos, vel, gravity=g)
    b = gpu_run(sphlib, box, pos, vel, gravity=g, precision=sphlib.SPH_F64)
    b["ascale"] = oracle_run(oracle_mod, box, pos, vel, gravity=g, mode=oracle_mod.F64)["ascale"]
    assert_within(rel_errors(a, b), name)


def _golden():
    with open(os.path.join(os.path.dirname(__file__), "golden", "analytic_cases.json")) as f:
        return json.load(f)["cases"]


@pytest.mark.parametrize("case", _golden(), ids=lambda c: c["name"])
def test_golden_cases_on_gpu(sphlib, case):
    pos = np.array(case["pos"], np.float32)
    vel = np.array(case["vel"], np.float32)
    got = gpu_run(sphlib, case["box"], pos, vel, gravity=case["gravity"])
    ref = {"rho": np.array(case["rho"]), "p": np.array(case["p"]), "acc": np.array(case["acc"]),
           "ascale": np.array(case["acc_scale"]), "pos": np.array(case["pos_new"]),
           "vel": np.array(case["vel_new"])}
    assert_within(rel_errors(got, ref), case["name"])
    g64 = gpu_run(sphlib, case["box"], pos, vel, gravity=case["gravity"], precision=sphlib.SPH_F64)
    np.testing.assert_allclose(g64["rho"], case["rho"], rtol=1e-12)
    err = np.linalg.norm(g64["acc"] - np.array(case["acc"]), axis=1) / np.array(case["acc_scale"])
    assert err.max() < 1e-11


# ------------------------------------------------------------------------- long runs
def dam8k_aggregates(sphlib, prec, pos, steps=200, every=10):
    c = sphlib.SphContext(C0_BOX, pos.shape[0], precision=prec, gravity=G981)
    c.upload(pos)
    out = []
    for s in range(steps):
        c.step(1)
        if s % every == every - 1:
            st = c.stats()
            out.append((st["rho_mean"], st["rho_max"], st["kinetic"], st["mass"]))
    d = c.download()
    assert np.all(np.isfinite(d["pos"])) and np.all(np.isfinite(d["rho"]))
    c.close()
    return np.array(out)


@pytest.fixture(scope="module")
def dam8k_fp64(sphlib):
    """The 8,000-particle dam break's FP64 run and the envelope of its chaotic spread: three FP64
    runs from the same lattice with every coordinate moved by one float ulp (random signs)."""
    from test_config_scale import spread_envelope, ulp_perturb

    pos = c0_scene(sphlib)
    ref = dam8k_aggregates(sphlib, sphlib.SPH_F64, pos)
    pert = [dam8k_aggregates(sphlib, sphlib.SPH_F64, ulp_perturb(pos, k)) for k in (1, 2, 3)]
    return pos, ref, spread_envelope(ref, pert)


@pytest.mark.parametrize("form", ["plain", "mixed"])
def test_bands_vs_f64_c0(sphlib, dam8k_fp64, form):
    """8,000-particle dam break, 200 steps: every 10 steps the form's mean and max density and
    kinetic energy stay within 3 times the FP64 runs' spread envelope plus the form's floor
    (1e-5 plain, 3e-3 mixed, relative); mass is exact."""
    from test_config_scale import FLOOR, band_ratio

    pos, ref, env = dam8k_fp64
    prec = {"plain": sphlib.SPH_PLAIN_F32, "mixed": sphlib.SPH_MIXED}[form]
    got = dam8k_aggregates(sphlib, prec, pos)
    assert np.array_equal(got[:, 3], ref[:, 3])
    worst = band_ratio(got, ref, env, FLOOR[form])
    print(f"dam8k {form}: worst deviation / band {worst:.3f}")
    assert worst <= 1.0, worst


# ------------------------------------------------------------------------- batches
def test_batch_equals_single_scenes(sphlib):
    """Scenes stepped together in one launch per pass give bit-identical results to each
    scene alone."""
    dims, boxes = sphlib.batch_plan(5, seed=9, nmin=500, nmax=6000)
    parts = [sphlib.dam_break_scene(tuple(int(x) for x in d), tuple(float(x) for x in b), seed=s)
             for s, (d, b) in enumerate(zip(dims, boxes))]
    counts = [p.shape[0] for p in parts]
    batch = sphlib.SphContext(boxes, counts, gravity=G981, flags=2)
    batch.upload(np.concatenate(parts), None, counts)
    batch.step(10)
    got = batch.download(acc=True)
    off = np.concatenate([[0], np.cumsum(counts)])
    for s, p in enumerate(parts):
        one = gpu_run(sphlib, boxes[s], p, steps=10, gravity=G981)
        for k in ("pos", "vel", "rho", "p", "acc"):
            assert np.array_equal(got[k][off[s]:off[s + 1]], one[k]), (s, k)
    batch.close()


def test_gravity_change_between_steps(sphlib, oracle_mod):
    """setGravityVector between steps (src/CBaseParticleSimulator.cpp:111-114; the G key,
    :154-179), for one scene of a batch or for all of them, takes effect at the next step. The
    batch with its gravity changed mid-run equals each scene run alone with the same changes,
    bit for bit, and the step after the last change matches the oracle under the new gravity."""
    O = oracle_mod
    boxes = [(0.4, 0.4, 0.4), (0.5, 0.3, 0.4)]
    parts = [O.reference_dam_break(0.4), sphlib.dam_break_scene((8, 6, 8), boxes[1], seed=3)]
    counts = [p.shape[0] for p in parts]
    off = np.concatenate([[0], np.cumsum(counts)])
    g1, g2 = (2.0, -5.0, 1.0), (0.0, -3.0, -2.0)
    batch = sphlib.SphContext(boxes, counts, gravity=G981, flags=sphlib.SPH_FLAG_RECORD_ACC)
    batch.upload(np.concatenate(parts), None, counts)
    batch.step(3)
    batch.set_gravity(g1, scene=1)
    batch.step(2)
    batch.set_gravity(g2)
    mid = batch.download()
    batch.step(1)
    got = batch.download(acc=True)
    batch.close()
    for s, p in enumerate(parts):
        one = sphlib.SphContext(boxes[s], p.shape[0], gravity=G981, flags=sphlib.SPH_FLAG_RECORD_ACC)
        one.upload(p)
        one.step(3)
        if s == 1:
            one.set_gravity(g1)
        one.step(2)
        one.set_gravity(g2)
        one.step(1)
        alone = one.download(acc=True)
        one.close()
        for k in ("pos", "vel", "rho", "p", "acc"):
            assert np.array_equal(got[k][off[s]:off[s + 1]], alone[k]), (s, k)
        o = O.Oracle(boxes[s], O.REF, threads=1, gravity=G981)
        o.add(mid["pos"][off[s]:off[s + 1]], mid["vel"][off[s]:off[s + 1]])
        o.set_gravity(g2)
        o.step(1)
        ref = o.state()
        o.close()
        assert_within(rel_errors({k: got[k][off[s]:off[s + 1]] for k in ("pos", "vel", "rho", "p", "acc")}, ref),
                      f"scene {s} after the gravity change")


def test_determinism(sphlib):
    pos = c0_scene(sphlib)
    a = gpu_run(sphlib, C0_BOX, pos, steps=25, gravity=G981)
    b = gpu_run(sphlib, C0_BOX, pos, steps=25, gravity=G981)
    for k in a:
        assert np.array_equal(a[k], b[k]), k


def test_graph_replay_matches_passes(sphlib):
    """sph_step (graph-captured steps) equals the pass-by-pass calls bit for bit."""
    pos = c0_scene(sphlib, dims=(10, 10, 10))
    a = gpu_run(sphlib, C0_BOX, pos, steps=19, gravity=G981)
    ctx = sphlib.SphContext(C0_BOX, pos.shape[0], gravity=G981, flags=2)
    ctx.upload(pos)
    for _ in range(19):
        ctx.pass_grid()
        ctx.pass_density()
        ctx.pass_forces()
    b = ctx.download(acc=True)
    for k in a:
        assert np.array_equal(a[k], b[k]), k


def test_caller_work_between_chained_passes(sphlib):
    """The step's kernels are chained launches (each may be scheduled while its predecessor
    drains, and waits for it before any other instruction). Work a caller enqueues on the
    context's stream between the passes (a kernel writing 256 MB, an event, a host wait) runs in
    stream order among them: the results equal those of the passes alone, bit for bit."""
    import torch

    pos = c0_scene(sphlib, dims=(20, 20, 20))
    a = gpu_run(sphlib, C0_BOX, pos, steps=12, gravity=G981)
    ctx = sphlib.SphContext(C0_BOX, pos.shape[0], gravity=G981, flags=2)
    ctx.upload(pos)
    ext = torch.cuda.ExternalStream(ctx.stream, device=torch.device("cuda:0"))
    filler = torch.empty(64 * 2**20, dtype=torch.float32, device="cuda:0")
    for k in range(12):
        for q, p in enumerate((ctx.pass_grid, ctx.pass_density, ctx.pass_forces)):
            with torch.cuda.stream(ext):
                filler.fill_(float(k + q))
                ev = torch.cuda.Event()
                ev.record(ext)
            if (k + q) % 5 == 0:
                ev.synchronize()
            p()
    b = ctx.download(acc=True)
    for key in a:
        assert np.array_equal(a[key], b[key]), key


# ------------------------------------------------------------------------- emitters, interface
def test_append_between_steps(sphlib, oracle_mod):
    box = (0.6, 0.6, 0.6)
    ctx = sphlib.SphContext(box, 5000)
    ctx.upload(np.zeros((0, 3), np.float32))
    added = []
    for k in range(6):
        xyz, vel = sphlib.fountain_emit(seed=4, step=k, n=100, center=(0.0, -0.29, 0.0), radius=0.05, speed=1.0,
                                        sigma=0.05)
        ctx.append(0, xyz, vel)
        added.append(xyz)
        ctx.step(1)
    assert ctx.n == 600 and list(ctx.counts()) == [600]
    d = ctx.download()
    assert np.all(np.isfinite(d["pos"]))
    # the first batch moved upward; ids stayed attached to their particles
    assert np.all(d["pos"][:100, 1] > added[0][:, 1])
    with pytest.raises(sphlib.SphError) as e:
        ctx.append(0, np.zeros((4401, 3), np.float32))
    assert e.value.code == sphlib.SPH_ERR_CAPACITY
    ctx.close()


def test_gpu_matches_reference_kernels(sphlib, oracle_mod):
    """One plain FP32 step on the golden states against the reference's own OpenCL kernels
    (density, pressure; acceleration away from the walls), within the 1e-5 parity band."""
    from test_oracle import interior, ref_cl_cases

    for c in ref_cl_cases():
        box = tuple(float(b) for b in c["box"])
        ctx = sphlib.SphContext(box, c["pos"].shape[0], flags=sphlib.SPH_FLAG_RECORD_ACC, gravity=c["gravity"])
        ctx.upload(c["pos"], c["vel"])
        ctx.step(1)
        got = ctx.download(acc=True)
        ctx.close()
        o = oracle_mod.Oracle(box, oracle_mod.REF, threads=4, gravity=c["gravity"])
        o.add(c["pos"], c["vel"])
        o.step(1)
        s = o.state()  # the per-particle force scale A
        inside = interior(c["pos"], box)
        errs = rel_errors({"rho": got["rho"], "p": got["p"]}, {"rho": c["rho"], "p": c["p"], "ascale": s["ascale"]})
        errs.update(rel_errors({"acc": got["acc"][inside]},
                               {"rho": c["rho"][inside], "acc": c["acc"][inside], "ascale": s["ascale"][inside]}))
        assert_within(errs, c["name"])


@pytest.mark.parametrize("prec", ["plain", "f64"])
def test_all_pairs_equals_grid(sphlib, prec):
    """The all-pairs form (the reference's brute-force simulator) and the grid form give the
    same bits over several steps: one scene with obstacles, then a batch of three scenes."""
    P = {"plain": sphlib.SPH_PLAIN_F32, "f64": sphlib.SPH_F64}[prec]
    box = (1.0, 1.0, 0.5)
    pos = sphlib.dam_break_scene((20, 20, 20), box, seed=0)
    obstacles = [np.array([0.1, -0.5, -0.1, 0.3, -0.3, 0.1], np.float32)]
    runs = []
    for flags in (0, sphlib.SPH_FLAG_ALL_PAIRS):
        ctx = sphlib.SphContext(box, pos.shape[0], precision=P, flags=flags | sphlib.SPH_FLAG_RECORD_ACC,
                                gravity=G981, obstacles=obstacles)
        ctx.upload(pos)
        ctx.step(12)
        runs.append(ctx.download(acc=True))
        if flags:
            with pytest.raises(sphlib.SphError) as e:
                ctx.set_variant(0, 3)
            assert e.value.code == sphlib.SPH_ERR_STATE
        ctx.close()
    for k in runs[0]:
        assert np.array_equal(runs[0][k], runs[1][k]), k
    dims, boxes = sphlib.batch_plan(3, seed=5, nmin=500, nmax=4000)
    parts = [sphlib.dam_break_scene(tuple(int(x) for x in d), tuple(float(x) for x in b), seed=s)
             for s, (d, b) in enumerate(zip(dims, boxes))]
    counts = [q.shape[0] for q in parts]
    runs = []
    for flags in (0, sphlib.SPH_FLAG_ALL_PAIRS):
        ctx = sphlib.SphContext(boxes, counts, precision=P, flags=flags, gravity=G981)
        ctx.upload(np.concatenate(parts), None, counts)
        ctx.step(7)
        runs.append(ctx.download())
        ctx.close()
    for k in runs[0]:
        assert np.array_equal(runs[0][k], runs[1][k]), k


@pytest.mark.parametrize("prec", ["plain", "f64", "mixed"])
def test_handoff_and_export(sphlib, prec):
    """The asynchronous handoff delivers the state of the moment it was queued while later
    steps run, leaves the run unchanged, and the device export gives the same float3 arrays."""
    import torch

    P = {"plain": sphlib.SPH_PLAIN_F32, "f64": sphlib.SPH_F64, "mixed": sphlib.SPH_MIXED}[prec]
    pos = c0_scene(sphlib, dims=(16, 16, 16))
    n = pos.shape[0]

    def now(ctx):
        if prec == "f64":
            import ctypes
            L = sphlib.load()
            x = np.zeros((n, 3)); v = np.zeros((n, 3))
            L.sph_download_f64(ctx.h, ctypes.c_void_p(x.ctypes.data), ctypes.c_void_p(v.ctypes.data), None, None, None)
            return x.astype(np.float32), v.astype(np.float32)
        d = ctx.download()
        return d["pos"], d["vel"]

    a = sphlib.SphContext(C0_BOX, n, precision=P, gravity=G981)
    a.upload(pos)
    a.step(5)
    ref_x, ref_v = now(a)
    a.step(9)
    fin_x, fin_v = now(a)
    b = sphlib.SphContext(C0_BOX, n, precision=P, gravity=G981)
    b.upload(pos)
    b.step(5)
    hx = torch.empty((n, 3), dtype=torch.float32).pin_memory()
    hv = torch.empty((n, 3), dtype=torch.float32).pin_memory()
    b.handoff_async(hx.data_ptr(), hv.data_ptr())
    b.step(9)  # queued behind the handoff's egress, overlapping its copy
    b.handoff_wait()
    assert b.handoff_ready()
    assert np.array_equal(hx.numpy(), ref_x) and np.array_equal(hv.numpy(), ref_v)
    got_x, got_v = now(b)
    assert np.array_equal(got_x, fin_x) and np.array_equal(got_v, fin_v)
    # a second handoff reuses the buffers after the first copy
    b.handoff_async(hx.data_ptr(), None)
    b.handoff_wait()
    assert np.array_equal(hx.numpy(), fin_x)
    dx = torch.full((n, 3), float("nan"), dtype=torch.float32, device="cuda")
    dv = torch.full((n, 3), float("nan"), dtype=torch.float32, device="cuda")
    side = torch.cuda.Stream()
    b.export_positions(dx.data_ptr(), dv.data_ptr(), side.cuda_stream)
    with torch.cuda.stream(side):
        sx, sv = dx.cpu(), dv.cpu()
    assert np.array_equal(sx.numpy(), fin_x) and np.array_equal(sv.numpy(), fin_v)
    a.close()
    b.close()


def test_splat_counts_and_depth(sphlib, tmp_path):
    """The point splat equals a numpy restatement of its pixel mapping (float32 add and
    multiply, floor, clamp) bit for bit, per axis, for one scene of a batch."""
    boxes = [(1.0, 1.0, 0.5), (0.6, 0.8, 0.7)]
    parts = [c0_scene(sphlib, dims=(16, 16, 16)), sphlib.dam_break_scene((9, 12, 10), boxes[1], 5)]
    counts = [q.shape[0] for q in parts]
    ctx = sphlib.SphContext(boxes, counts, gravity=G981)
    ctx.upload(np.concatenate(parts), None, counts)
    ctx.step(7)
    d = ctx.download()
    for scene in (0, 1):
        p = d["pos"][sum(counts[:scene]):sum(counts[:scene + 1])]
        box = np.asarray(boxes[scene], np.float32)
        for axis, (W, H) in zip((0, 1, 2), ((40, 30), (64, 48), (33, 77))):
            cnt, dep = ctx.splat(scene, axis, W, H)
            au, av = (1, 2) if axis == 0 else ((0, 2) if axis == 1 else (0, 1))
            fu = np.floor((p[:, au] + box[au] / np.float32(2)) * (np.float32(W) / box[au]))
            fv = np.floor((p[:, av] + box[av] / np.float32(2)) * (np.float32(H) / box[av]))
            u = np.clip(np.nan_to_num(fu, nan=0.0), 0, W - 1).astype(np.int64)
            v = np.clip(np.nan_to_num(fv, nan=0.0), 0, H - 1).astype(np.int64)
            want = np.zeros((H, W), np.uint32)
            np.add.at(want, (v, u), 1)
            wdep = np.full((H, W), np.inf, np.float32)
            np.minimum.at(wdep, (v, u), p[:, axis])
            assert np.array_equal(cnt, want), (scene, axis)
            assert np.array_equal(dep, wdep), (scene, axis)
            assert int(cnt.sum()) == counts[scene]
    path = sphlib.write_pgm(str(tmp_path / "splat.pgm"), cnt)
    raw = open(path, "rb").read()
    assert raw.startswith(b"P5\n33 77\n255\n") and len(raw) == len(b"P5\n33 77\n255\n") + 33 * 77
    ctx.close()


def test_online_tuning_keeps_the_bits(sphlib):
    """Online tuning switches force variants between real steps; with the cell multiple set by
    the caller (so that it stays) the run is bit-identical to one without online tuning, through
    sph_step (graphs between trials) and through the pass calls."""
    pos = c0_scene(sphlib, dims=(16, 16, 16))
    runs = []
    for mode in ("plain", "online_step", "online_passes"):
        ctx = sphlib.SphContext(C0_BOX, pos.shape[0], gravity=G981, flags=sphlib.SPH_FLAG_RECORD_ACC)
        ctx.set_cell_multiple(1)
        ctx.upload(pos)
        ctx.set_variant(0, 4)
        if mode != "plain":
            ctx.set_online_tuning(4)
        if mode == "online_passes":
            for _ in range(23):
                ctx.pass_grid()
                ctx.pass_density()
                ctx.pass_forces()
        else:
            ctx.step(11)
            ctx.step(12)
        if mode != "plain":
            assert ctx.variant()[1] in (7, 9, 10, 11)
        runs.append(ctx.download(acc=True))
        ctx.close()
    for r in runs[1:]:
        for k in runs[0]:
            assert np.array_equal(runs[0][k], r[k]), k
    with pytest.raises(sphlib.SphError) as e:
        sphlib.SphContext(C0_BOX, 10).set_online_tuning(3)
    assert e.value.code == sphlib.SPH_ERR_ARG
    # the mixed form: its four launch forms give the same bits, so online tuning keeps them too
    runs = []
    for mode in ("fixed", "online_step", "online_passes"):
        m = sphlib.SphContext(C0_BOX, pos.shape[0], precision=sphlib.SPH_MIXED, gravity=G981,
                              flags=sphlib.SPH_FLAG_RECORD_ACC)
        m.set_cell_multiple(1)
        m.upload(pos)
        m.set_variant(0, 0)
        if mode != "fixed":
            m.set_online_tuning(4)
        if mode == "online_passes":
            for _ in range(23):
                m.pass_grid()
                m.pass_density()
                m.pass_forces()
        else:
            m.step(11)
            m.step(12)
        if mode != "fixed":
            assert m.variant()[1] in (0, 1, 2, 3)
        runs.append(m.download(acc=True))
        m.close()
    for r in runs[1:]:
        for k in runs[0]:
            assert np.array_equal(runs[0][k], r[k]), ("mixed", k)
    m = sphlib.SphContext(C0_BOX, 10, precision=sphlib.SPH_MIXED)
    with pytest.raises(sphlib.SphError) as e:
        m.set_variant(0, 4)  # the mixed form has force variants 0-3 only
    assert e.value.code == sphlib.SPH_ERR_ARG
    m.close()


@pytest.mark.parametrize("prec", ["plain", "mixed"])
def test_online_tuning_across_cell_multiples(sphlib, oracle_mod, prec):
    """Unpinned, online tuning also tries the other cell multiple once per period and keeps the
    faster grid: every step still matches the oracle's step from the same state (plain: the 1e-5
    band; mixed: density within 1e-3 of the FP64 run), whichever grid ran it."""
    box, pos, vel, g = scenes(sphlib, oracle_mod)["c0_8000_moving"]
    form = {"plain": sphlib.SPH_PLAIN_F32, "mixed": sphlib.SPH_MIXED}[prec]
    ctx = sphlib.SphContext(box, pos.shape[0], precision=form, gravity=g, flags=sphlib.SPH_FLAG_RECORD_ACC)
    ctx.upload(pos, vel)
    ctx.set_online_tuning(4)
    seen = set()
    for k in range(12):
        cur = ctx.download()
        if k % 2:
            ctx.pass_grid()
            ctx.pass_density()
            ctx.pass_forces()
        else:
            ctx.step(1)
        got = ctx.download(acc=True)
        seen.add(ctx.cell_multiple())
        if prec == "plain":
            ref = oracle_run(oracle_mod, box, cur["pos"], cur["vel"], gravity=g)
            assert_within(rel_errors(got, ref), f"online step {k}")
        else:
            ref = gpu_run(sphlib, box, cur["pos"], cur["vel"], precision=sphlib.SPH_F64, gravity=g)
            assert np.max(np.abs(got["rho"] - ref["rho"]) / ref["rho"]) < 1e-3, k
    assert seen <= {1, 2}
    ctx.close()


def test_pinned_transfers_equal_staged_transfers(sphlib):
    """Uploads from and downloads into pinned host arrays go straight through kernels (no
    staging copy); they give the same bits as pageable arrays, for a batch, after a whole step
    and between passes (the two state layouts)."""
    import torch

    dims, boxes = sphlib.batch_plan(3, seed=9, nmin=500, nmax=3000)
    parts = [sphlib.dam_break_scene(tuple(int(x) for x in d), tuple(float(x) for x in b), seed=s)
             for s, (d, b) in enumerate(zip(dims, boxes))]
    counts = [q.shape[0] for q in parts]
    pos = np.concatenate(parts)
    vel = np.random.default_rng(3).normal(0, 0.1, pos.shape).astype(np.float32)
    n = pos.shape[0]
    px, pv = torch.from_numpy(pos.copy()).pin_memory(), torch.from_numpy(vel.copy()).pin_memory()
    runs = []
    for pinned in (False, True):
        ctx = sphlib.SphContext(boxes, counts, gravity=G981)
        if pinned:
            ctx.upload_raw(px.data_ptr(), pv.data_ptr(), counts)
        else:
            ctx.upload(pos, vel, counts)
        ctx.step(4)
        got = []
        for mid_step in (False, True):
            if mid_step:
                ctx.pass_grid()  # sorted layout
            if pinned:
                ox, ov = torch.empty((n, 3)).pin_memory(), torch.empty((n, 3)).pin_memory()
                ctx.download_raw(ox.data_ptr(), ov.data_ptr())
                got.append((ox.numpy().copy(), ov.numpy().copy()))
                # a pinned array that is not 16-byte aligned takes the staging path: same bits
                big = torch.empty(3 * n + 1).pin_memory()
                ctx.download_raw(big.data_ptr() + 4, ov.data_ptr())
                assert np.array_equal(big.numpy()[1:].reshape(n, 3), got[-1][0])
            else:
                d = ctx.download()
                got.append((d["pos"], d["vel"]))
        runs.append(got)
        ctx.close()
    for (a, b) in zip(runs[0], runs[1]):
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_fountain_emission_vs_oracle(sphlib, oracle_mod):
    """Emitter steps against the oracle: after each device emission, one GPU step and one
    oracle step from the same state, in the 1e-5 band. The jet is dense and fast, so whole
    trajectories diverge chaotically within a few steps; each step is compared from the
    common state instead. The first two steps also follow the oracle fed the host generator's
    particles (the device emitter's bits) without resynchronising."""
    box = (0.8, 0.8, 0.8)
    args = dict(center=(0.0, -0.38, 0.0), radius=0.03, speed=1.5, sigma=0.05)
    ctx = sphlib.SphContext(box, 4000, gravity=G981, flags=sphlib.SPH_FLAG_RECORD_ACC)
    ctx.upload(np.zeros((0, 3), np.float32))
    follow = oracle_mod.Oracle(box, oracle_mod.REF, threads=os.cpu_count(), gravity=G981)
    for k in range(6):
        ctx.emit_fountain(0, 21, k, 500, args["center"], args["radius"], args["speed"], args["sigma"])
        before = ctx.download()
        o = oracle_mod.Oracle(box, oracle_mod.REF, threads=os.cpu_count(), gravity=G981)
        o.add(before["pos"], before["vel"])
        o.step(1)
        ctx.step(1)
        got = ctx.download(acc=True)
        assert_within(rel_errors({q: got[q] for q in ("rho", "p", "acc", "pos", "vel")}, o.state()),
                      f"emission step {k}")
        if k < 2:
            xyz, vel = sphlib.fountain_emit(21, k, 500, **args)
            follow.add(xyz, vel)
            follow.step(1)
            assert_within(rel_errors({q: got[q] for q in ("rho", "p", "acc", "pos", "vel")}, follow.state()),
                          f"followed emission step {k}")
    ctx.close()


def test_device_emitter_equals_host_emitter(sphlib):
    """sph_emit_fountain generates on the device the same bits as the host generator, and a run
    fed by it equals a run fed by sph_append of the host-generated particles."""
    box = (0.6, 0.6, 0.6)
    args = dict(center=(0.0, -0.29, 0.0), radius=0.05, speed=1.0, sigma=0.05)
    a = sphlib.SphContext(box, 5000)
    b = sphlib.SphContext(box, 5000)
    for c in (a, b):
        c.upload(np.zeros((0, 3), np.float32))
    for k in range(6):
        xyz, vel = sphlib.fountain_emit(seed=4, step=k, n=333, **args)
        a.append(0, xyz, vel)
        b.emit_fountain(0, 4, k, 333, args["center"], args["radius"], args["speed"], args["sigma"])
        if k == 0:
            da, db = a.download(), b.download()
            assert np.array_equal(da["pos"], db["pos"]) and np.array_equal(da["vel"], db["vel"])
            assert np.array_equal(db["pos"], xyz) and np.array_equal(db["vel"], vel)
        a.step(1)
        b.step(1)
    da, db = a.download(), b.download()
    assert a.n == b.n == 6 * 333
    for k in ("pos", "vel", "rho"):
        assert np.array_equal(da[k], db[k]), k
    with pytest.raises(sphlib.SphError) as e:
        b.emit_fountain(0, 4, 7, 3003, args["center"], args["radius"], args["speed"], args["sigma"])
    assert e.value.code == sphlib.SPH_ERR_CAPACITY
    a.close()
    b.close()


def test_reference_shaped_simulator(sphlib, oracle_mod, tmp_path):
    """The CBaseParticleSimulator mirror: setupScene + step on the 0.4 m dam break matches the
    oracle, and the FOUNTAIN scenario emits 7 particles per step."""
    sim = sphlib.CCUDAParticleSimulator(0.4, sphlib.DAM_BREAK)
    sim.setupScene()
    assert sim.getParticlesCount() == 1620 and "sm_" in sim.getSelectedDevice()
    sim.step()
    t = sim.lastPassTimes()
    assert t[0] > 0 and t[1] > 0 and t[2] > 0 and t[3] == 0 and t[4] == 0
    got = sim.ctx.download()
    ref = oracle_run(oracle_mod, 0.4, oracle_mod.reference_dam_break(0.4))
    errs = rel_errors({k: got[k] for k in ("rho", "p", "pos", "vel")}, ref)
    assert_within(errs, "mirror")
    f = sphlib.CCUDAParticleSimulator(0.4, sphlib.FOUNTAIN)
    f.setupScene()
    for _ in range(5):
        f.step()
    assert f.getParticlesCount() == 35 and f.ctx.n == 35
    assert f.getMaxParticlesCount() == 1620
    # the profiling log: an event every 10 steps with the passes' event times, exported as the
    # reference's two CSV files
    for _ in range(20):
        sim.step()
    assert [e.iteration for e in sim.events] == [0, 10, 20]
    assert all(e.updateGrid > 0 and e.updateDensityPressure > 0 and e.updateForces > 0 for e in sim.events)
    assert sim.events[-1].fps > 0
    s, d = sim.exportLogs(str(tmp_path))
    assert os.path.basename(s) == "Dam break_0.4.csv" and open(s).read().count(";") == 4
    assert open(d).read().splitlines()[1].startswith("Grid;")


def test_empty_and_single_particle_scenes(sphlib):
    """A batch holding an empty scene, a lone particle and a small dam break: the lone particle
    has the self density m poly6(0) and falls with gravity exactly, the dam break equals a
    run of its own, and the empty scene stays empty."""
    boxes = [(0.3, 0.3, 0.3), (0.5, 0.5, 0.5), C0_BOX]
    dam = c0_scene(sphlib, dims=(8, 8, 8))
    lone = np.zeros((1, 3), np.float32)
    ctx = sphlib.SphContext(boxes, [10, 1, dam.shape[0]], gravity=G981, flags=sphlib.SPH_FLAG_RECORD_ACC)
    ctx.upload(np.concatenate([lone, dam]), None, [0, 1, dam.shape[0]])
    ctx.step(3)
    d = ctx.download(acc=True)
    assert list(ctx.counts()) == [0, 1, dam.shape[0]]
    h = np.float32(0.0457)
    self_rho = np.float32(0.02) * np.float32(315.0 / (64.0 * np.pi * float(h) ** 9)) * np.float32(h * h) ** 3
    assert abs(d["rho"][0] - self_rho) / self_rho < 1e-6
    assert np.allclose(d["acc"][0], np.float32(G981), rtol=1e-6, atol=0)
    st = ctx.stats(0)
    assert st["count"] == 0 and st["mass"] == 0.0
    ctx.close()
    one = sphlib.SphContext(C0_BOX, dam.shape[0], gravity=G981, flags=sphlib.SPH_FLAG_RECORD_ACC)
    one.upload(dam)
    one.step(3)
    e = one.download(acc=True)
    one.close()
    for k in e:
        assert np.array_equal(d[k][1:], e[k]), k


@pytest.mark.parametrize("prec", ["plain", "f64"])
def test_nan_particle_is_isolated(sphlib, prec):
    """A particle with a NaN coordinate in the host input fails every neighbour test (h^2 - r^2
    is NaN, not > 0): every other particle's state is bit-identical to a run without it, and
    the run does not fail. The NaN particle itself stays non-finite."""
    P = {"plain": sphlib.SPH_PLAIN_F32, "f64": sphlib.SPH_F64}[prec]
    pos = c0_scene(sphlib, dims=(12, 12, 12))
    vel = np.random.default_rng(6).normal(0, 0.2, pos.shape).astype(np.float32)
    n = pos.shape[0]
    bad = np.concatenate([pos, np.float32([[np.nan, -0.3, 0.05]])])
    badv = np.concatenate([vel, np.zeros((1, 3), np.float32)])
    out = []
    for p_, v_ in ((pos, vel), (bad, badv)):
        ctx = sphlib.SphContext(C0_BOX, p_.shape[0], precision=P, gravity=G981)
        ctx.upload(p_, v_)
        ctx.step(5)
        if prec == "f64":
            import ctypes
            x = np.zeros((p_.shape[0], 3)); v = np.zeros((p_.shape[0], 3)); r = np.zeros(p_.shape[0])
            sphlib.load().sph_download_f64(ctx.h, ctypes.c_void_p(x.ctypes.data), ctypes.c_void_p(v.ctypes.data),
                                           ctypes.c_void_p(r.ctypes.data), None, None)
            out.append({"pos": x, "vel": v, "rho": r})
        else:
            out.append(ctx.download())
        ctx.close()
    a, b = out
    for k in ("pos", "vel", "rho"):
        assert np.array_equal(a[k], b[k][:n]), k
    assert not np.all(np.isfinite(b["pos"][n]))


def test_errors_are_status_codes(sphlib):
    ctx = sphlib.SphContext((0.4, 0.4, 0.4), 10)
    with pytest.raises(sphlib.SphError) as e:
        ctx.step(1)
    assert e.value.code == sphlib.SPH_ERR_STATE
    with pytest.raises(sphlib.SphError) as e:
        ctx.upload(np.zeros((11, 3), np.float32))
    assert e.value.code == sphlib.SPH_ERR_CAPACITY
    ctx.upload(np.zeros((3, 3), np.float32) + np.float32([[0.0, 0, 0], [0.01, 0, 0], [0.0, 0.01, 0]]))
    with pytest.raises(sphlib.SphError) as e:
        ctx.pass_density()
    assert e.value.code == sphlib.SPH_ERR_STATE
    msgs = []
    sim = sphlib.CCUDAParticleSimulator(0.4, sphlib.DAM_BREAK)
    sim.errorOccured = msgs.append
    sim.setupScene()
    sim.ctx.pass_grid()  # leaves a pass in progress: the next step fails and stops the simulator
    sim.start()
    sim.step()
    assert msgs and not sim.running
    ctx.close()


def test_stats_fp64(sphlib):
    pos = c0_scene(sphlib, dims=(10, 10, 10))
    rng = np.random.default_rng(3)
    vel = rng.normal(0, 0.3, pos.shape).astype(np.float32)
    ctx = sphlib.SphContext(C0_BOX, pos.shape[0], gravity=G981)
    ctx.upload(pos, vel)
    ctx.step(3)
    s = ctx.stats()
    d = ctx.download()
    m = float(np.float32(0.02))
    v = d["vel"].astype(np.float64)
    assert s["count"] == 1000 and s["mass"] == m * 1000
    np.testing.assert_allclose(s["momentum"], m * v.sum(axis=0), rtol=1e-9, atol=1e-12)
    np.testing.assert_allclose(s["kinetic"], 0.5 * m * (v ** 2).sum(), rtol=1e-12)
    np.testing.assert_allclose(s["rho_mean"], d["rho"].astype(np.float64).mean(), rtol=1e-12)
    assert s["rho_max"] == float(d["rho"].max())
    ctx.close()


# ------------------------------------------------------------------------- full size
def test_full_size_1m_properties(sphlib):
    """The 1,000,000-particle dam break (100^3 lattice, 5 x 5 x 2.5 m): grid bit-exact against
    the vectorised double hash, canonical order, conservation and finiteness over 20 steps."""
    box = (5.0, 5.0, 2.5)
    pos = sphlib.dam_break_scene((100, 100, 100), box, seed=1)
    ctx = sphlib.SphContext(box, pos.shape[0], gravity=G981)
    ctx.upload(pos)
    for rep in range(2):
        cur = ctx.download()["pos"]
        ctx.pass_grid()
        cell, counts, order = ctx.grid()
        want, res = cells_numpy(cur, box)
        assert np.array_equal(cell.astype(np.int64), want)
        assert counts.sum() == 1_000_000 and counts.size == int(np.prod(res))
        assert np.array_equal(np.bincount(want, minlength=counts.size), counts)
        cs = cell[order].astype(np.int64)
        key = cs * (1 << 21) + order
        assert np.all(np.diff(key) > 0)  # ascending (cell, id): canonical and a permutation
        ctx.pass_density()
        ctx.pass_forces()
        ctx.step(19)
    s = ctx.stats()
    assert s["count"] == 1_000_000 and s["mass"] == float(np.float32(0.02)) * 1_000_000
    d = ctx.download()
    assert np.all(np.isfinite(d["pos"])) and np.all(np.isfinite(d["vel"]))
    # with the reference's soft equation of state (k = 3) the 2.3 m column compresses under
    # gravity: densities rise well above rest density; the FP64 run of the same 40 steps
    # must agree on the aggregates
    ctx64 = sphlib.SphContext(box, pos.shape[0], gravity=G981, precision=sphlib.SPH_F64)
    ctx64.upload(pos)
    ctx64.step(40)
    s64 = ctx64.stats()
    assert abs(s["rho_mean"] - s64["rho_mean"]) / s64["rho_mean"] < 1e-3
    assert abs(s["kinetic"] - s64["kinetic"]) / s64["kinetic"] < 1e-2
    np.testing.assert_allclose(s["rho_mean"], d["rho"].astype(np.float64).mean(), rtol=1e-9)
    ctx64.close()
    ctx.close()


def test_full_size_16m_with_obstacles(sphlib):
    """The largest configuration: 16,000,000 particles (400 x 200 x 200 lattice) in the
    4 x 1 x 1 m box scaled x4.57, with 8 box obstacles. One plain FP32 step against an FP64
    GPU step of the same state, compared on a 1M subsample (density 1e-5 relative,
    acceleration 1e-5 of the subsample's largest), then conservation over 5 more steps."""
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
    out = {}
    for name, prec in (("f32", sphlib.SPH_PLAIN_F32), ("f64", sphlib.SPH_F64)):
        ctx = sphlib.SphContext(box, n, precision=prec, gravity=G981, obstacles=obs,
                                flags=sphlib.SPH_FLAG_RECORD_ACC)
        ctx.upload(pos)
        ctx.step(1)
        if prec == sphlib.SPH_F64:
            import ctypes
            r = np.zeros(n); a = np.zeros((n, 3))
            sphlib.load().sph_download_f64(ctx.h, None, None, ctypes.c_void_p(r.ctypes.data), None,
                                           ctypes.c_void_p(a.ctypes.data))
            out[name] = {"rho": r, "acc": a}
        else:
            d = ctx.download(acc=True)
            out[name] = {"rho": d["rho"].astype(np.float64), "acc": d["acc"].astype(np.float64)}
            ctx.step(5)
            st = ctx.stats()
            assert st["count"] == n and st["mass"] == float(np.float32(0.02)) * n
            assert np.isfinite(st["kinetic"]) and np.isfinite(st["rho_max"])
        ctx.close()
    sub = np.random.default_rng(5).choice(n, 1_000_000, replace=False)
    a, b = out["f32"], out["f64"]
    assert np.max(np.abs(a["rho"][sub] - b["rho"][sub]) / b["rho"][sub]) < 1e-5
    amax = np.max(np.linalg.norm(b["acc"][sub], axis=1))
    assert np.max(np.linalg.norm(a["acc"][sub] - b["acc"][sub], axis=1)) / amax < 1e-5


# ------------------------------------------------------------------------- launch variants
def test_variants_bit_identical(sphlib, oracle_mod):
    """Every launch variant of the two neighbour passes computes the same bits."""
    for box, pos, vel, g in [scenes(sphlib, oracle_mod)["c0_8000_moving"],
                             scenes(sphlib, oracle_mod)["outside_walls"],
                             scenes(sphlib, oracle_mod)["dense_clump"]]:
        base = None
        for dv, fv in [(d, f) for d in (0, 1, 2, 4) for f in (0, 1, 2)] + [(0, f) for f in range(3, 12)]:
            if True:
                ctx = sphlib.SphContext(box, pos.shape[0], gravity=g, flags=2)
                ctx.set_variant(dv, fv)
                ctx.upload(pos, vel)
                ctx.step(6)
                out = ctx.download(acc=True)
                ctx.close()
                if base is None:
                    base = out
                for k in out:
                    assert np.array_equal(out[k], base[k]), (dv, fv, k)


@pytest.mark.parametrize("cell_mult", [1, 2])
def test_mixed_variants_bit_identical(sphlib, oracle_mod, cell_mult):
    """The mixed form's four force launch forms compute the same bits (also on the dense clump,
    whose rows run past the recorded mask words), on cells of h and of h/2."""
    for box, pos, vel, g in [scenes(sphlib, oracle_mod)["c0_8000_moving"],
                             scenes(sphlib, oracle_mod)["dense_clump"]]:
        base = None
        for fv in range(4):
            ctx = sphlib.SphContext(box, pos.shape[0], precision=sphlib.SPH_MIXED, gravity=g, flags=2)
            ctx.set_cell_multiple(cell_mult)
            ctx.set_variant(0, fv)
            ctx.upload(pos, vel)
            ctx.step(6)
            out = ctx.download(acc=True)
            ctx.close()
            if base is None:
                base = out
            for k in out:
                assert np.array_equal(out[k], base[k]), (fv, k)


def test_half_cell_variants_bit_identical(sphlib, oracle_mod):
    """On cells of h/2 the record variants 7 to 11 compute the same bits."""
    for box, pos, vel, g in [scenes(sphlib, oracle_mod)["c0_8000_moving"],
                             scenes(sphlib, oracle_mod)["dense_clump"]]:
        base = None
        for fv in (7, 8, 9, 10, 11):
            ctx = sphlib.SphContext(box, pos.shape[0], gravity=g, flags=2)
            ctx.set_cell_multiple(2)
            ctx.set_variant(0, fv)
            ctx.upload(pos, vel)
            ctx.step(6)
            out = ctx.download(acc=True)
            ctx.close()
            if base is None:
                base = out
            for k in out:
                assert np.array_equal(out[k], base[k]), (fv, k)


def test_mixed_half_cells_vs_f64(sphlib, oracle_mod):
    """The mixed form on cells of h/2, one step against the FP64 run: density within 1e-3."""
    for name in ("ref_default_0.4", "c0_8000_moving", "outside_walls"):
        box, pos, vel, g = scenes(sphlib, oracle_mod)[name]
        m = sphlib.SphContext(box, pos.shape[0], precision=sphlib.SPH_MIXED, flags=2, gravity=g)
        m.set_cell_multiple(2)
        m.upload(pos, vel)
        m.step(1)
        got = m.download(acc=True)
        m.close()
        ref = gpu_run(sphlib, box, pos, vel, steps=1, precision=sphlib.SPH_F64, gravity=g)
        assert np.max(np.abs(got["rho"] - ref["rho"]) / ref["rho"]) < 1e-3, name


def test_autotune_is_one_plain_step(sphlib, tmp_path, monkeypatch):
    monkeypatch.setenv("SPH_TUNE_CACHE", str(tmp_path / "tune.txt"))
    pos = c0_scene(sphlib)
    a = sphlib.SphContext(C0_BOX, pos.shape[0], gravity=G981, flags=2)
    a.upload(pos)
    dv, fv = a.autotune(reps=2)
    cm = a.cell_multiple()
    assert dv in (0, 1, 2, 4) and fv in (0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11) and cm in (1, 2)
    a.step(3)
    # the same four steps with the chosen cell multiple and variants, set by hand
    ref = sphlib.SphContext(C0_BOX, pos.shape[0], gravity=G981, flags=2)
    ref.set_cell_multiple(cm)
    ref.set_variant(dv, fv)
    ref.upload(pos)
    ref.step(4)
    b = ref.download(acc=True)
    ref.close()
    got = a.download(acc=True)
    for k in got:
        assert np.array_equal(got[k], b[k]), k
    line = (tmp_path / "tune.txt").read_text().strip().splitlines()[-1]
    assert line.endswith(f" {dv} {fv} {cm}") and "|b12" in line  # 8000 particles -> bucket 12
    # a new context of the same bucket picks the cached choice at upload
    c = sphlib.SphContext(C0_BOX, pos.shape[0], gravity=G981)
    c.upload(pos)
    assert c.variant() == (dv, fv) and c.cell_multiple() == cm
    a.close()
    c.close()
    # a cached line for cells of h/2 is applied before the upload's hash
    (tmp_path / "tune.txt").write_text(line.rsplit(" ", 3)[0] + " 0 9 2\n")
    d = sphlib.SphContext(C0_BOX, pos.shape[0], gravity=G981, flags=2)
    d.upload(pos)
    assert d.variant() == (0, 9) and d.cell_multiple() == 2
    d.step(2)
    e2 = gpu_run(sphlib, C0_BOX, pos, steps=2, gravity=G981, cell_mult=2)
    dd = d.download(acc=True)
    for k in dd:
        assert np.array_equal(dd[k], e2[k]), k
    d.close()


def test_upload_step_download_equals_resident(sphlib):
    """Stepping through host buffers (upload, step, download each step) reproduces the
    device-resident run bit for bit: the canonical sort makes the layout irrelevant."""
    pos = c0_scene(sphlib, dims=(12, 12, 12))
    ref = gpu_run(sphlib, C0_BOX, pos, steps=8, gravity=G981)
    ctx = sphlib.SphContext(C0_BOX, pos.shape[0], gravity=G981)
    x, v = pos, np.zeros_like(pos)
    for _ in range(8):
        ctx.upload(x, v)
        ctx.step(1)
        d = ctx.download()
        x, v = d["pos"], d["vel"]
    assert np.array_equal(x, ref["pos"]) and np.array_equal(v, ref["vel"])
    ctx.close()


# ------------------------------------------------------------------------- mixed precision
def mixed_vs_f64(sphlib, box, pos, vel=None, steps=1, gravity=G981):
    m = sphlib.SphContext(box, pos.shape[0], precision=sphlib.SPH_MIXED, flags=2, gravity=gravity)
    m.upload(pos, vel)
    m.step(steps)
    got = m.download(acc=True)
    got64 = {}
    L = sphlib.load()
    n = pos.shape[0]
    x64 = np.zeros((n, 3))
    L.sph_download_f64(m.h, sphlib._vp(x64), None, None, None, None)
    m.close()
    ref = gpu_run(sphlib, box, pos, vel, steps=steps, precision=sphlib.SPH_F64, gravity=gravity)
    return got, x64, ref


def test_mixed_one_step_vs_f64(sphlib, oracle_mod):
    """Mixed form, one step from an identical state, against the FP64 run: density within
    1e-3 relative, acceleration within 2e-3 of its scale A, position within 4 ulp + 2e-3 A dt^2
    (positions are gathered at h / 8192 = 5.6 um resolution, neighbour velocities in FP16)."""
    for name in ("ref_default_0.4", "c0_8000_moving", "outside_walls"):
        box, pos, vel, g = scenes(sphlib, oracle_mod)[name]
        got, x64, ref = mixed_vs_f64(sphlib, box, pos, vel, gravity=g)
        scale = oracle_run(oracle_mod, box, pos, vel, gravity=g, mode=oracle_mod.F64)["ascale"]
        rho_err = np.max(np.abs(got["rho"] - ref["rho"]) / ref["rho"])
        acc_err = np.max(np.linalg.norm(got["acc"] - ref["acc"], axis=1) / scale)
        bound = 4 * np.spacing(np.abs(ref["pos"]).astype(np.float32)).astype(np.float64) + \
            (2e-3 * scale * 1e-4)[:, None]
        pos_err = np.max(np.abs(x64 - ref["pos"]) / bound)
        assert rho_err < 1e-3 and acc_err < 2e-3 and pos_err <= 1.0, (name, rho_err, acc_err, pos_err)


def test_mixed_ten_steps_vs_f64(sphlib):
    """After 10 steps of the 8,000-particle dam break the mixed form's densities stay within
    1e-2 of the FP64 run per particle and its mean density within 1e-4 (the flow amplifies any
    first-step difference, the plain form's included)."""
    pos = c0_scene(sphlib)
    ref = gpu_run(sphlib, C0_BOX, pos, steps=10, precision=sphlib.SPH_F64, gravity=G981)
    mixed, _, _ = mixed_vs_f64(sphlib, C0_BOX, pos, steps=10)
    em = np.max(np.abs(mixed["rho"] - ref["rho"]) / ref["rho"])
    assert em < 1e-2, em
    assert abs(mixed["rho"].astype(np.float64).mean() - ref["rho"].mean()) / ref["rho"].mean() < 1e-4
    assert np.all(np.isfinite(mixed["pos"]))


def test_mixed_batch_and_append(sphlib):
    """The mixed form batches scenes and appends emitter particles like the plain form."""
    dims, boxes = sphlib.batch_plan(3, seed=4, nmin=500, nmax=3000)
    parts = [sphlib.dam_break_scene(tuple(int(x) for x in d), tuple(float(x) for x in b), seed=s)
             for s, (d, b) in enumerate(zip(dims, boxes))]
    counts = [p.shape[0] for p in parts]
    ctx = sphlib.SphContext(boxes, [c + 100 for c in counts], precision=sphlib.SPH_MIXED, gravity=G981)
    ctx.upload(np.concatenate(parts), None, counts)
    ctx.step(5)
    xyz, vel = sphlib.fountain_emit(seed=1, step=0, n=100, center=(0.0, 0.0, 0.0), radius=0.02, speed=0.5,
                                    sigma=0.01)
    ctx.append(1, xyz, vel)
    ctx.step(5)
    d = ctx.download()
    assert ctx.n == sum(counts) + 100 and np.all(np.isfinite(d["pos"])) and np.all(np.isfinite(d["rho"]))
    ctx.close()


def test_one_step_with_obstacles_vs_oracle(sphlib, oracle_mod):
    """Box obstacles (no reference counterpart: nearest-face push-out with the wall constants,
    restated in the oracle): one plain FP32 step against the oracle, particles inside, beside
    and straddling two obstacles."""
    box = (0.6, 0.5, 0.5)
    obstacles = np.array([[-0.05, -0.25, -0.05, 0.05, -0.1, 0.05],
                          [0.12, -0.2, -0.2, 0.2, 0.0, -0.1]], np.float32)
    rng = np.random.default_rng(21)
    pos = sphlib.dam_break_scene((14, 10, 10), box, seed=8)
    pos[:, 0] += np.float32(0.22)  # lattice across both obstacles
    vel = rng.normal(0, 0.3, pos.shape).astype(np.float32)
    ctx = sphlib.SphContext(box, pos.shape[0], flags=2, gravity=G981, obstacles=[obstacles])
    ctx.upload(pos, vel)
    ctx.step(1)
    got = ctx.download(acc=True)
    ctx.close()
    o = oracle_mod.Oracle(box, oracle_mod.REF, threads=os.cpu_count(), gravity=G981, obstacles=obstacles)
    o.add(pos, vel)
    o.step(1)
    ref = o.state()
    inside = np.zeros(pos.shape[0], bool)
    for ob in obstacles:
        inside |= np.all((pos > ob[:3] - 0.01) & (pos < ob[3:] + 0.01), axis=1)
    assert inside.sum() > 20  # the case exercises the obstacle response
    assert_within(rel_errors(got, ref), "obstacles")
