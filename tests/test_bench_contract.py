"""The benchmark's reference arm runs on the host alone: its JSON line keeps the keys the
benchmark line promises (value, unit, impl, cpu_baseline, e2e with zero transfer bytes)."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_line():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "0", "--threads", "2"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e"):
        assert k in line, k
    assert line["impl"] == "reference" and line["steps"] == 1 and line["value"] > 0
    assert line["cpu_baseline"]["value"] == line["value"] and line["cpu_baseline"]["cores"] == 2
    assert line["cpu_baseline"]["kind"] in ("port", "reference")
    assert line["e2e"] == {"value": line["value"], "unit": line["unit"], "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
    assert "workload" in line["config"]


def test_byte_model_matches_the_documented_totals():
    """bench.py's algorithmic bytes per step: 360 N + 40 C with the force records (variants 7 and
    up), the density pass 116 N + 4 C and the force pass 156 N + 12 C; the 1M dam break's cell
    count is 110 x 110 x 55."""
    sys.path.insert(0, ROOT)
    import bench

    N, C = 1_000_000, bench.grid_cells(bench.BOX)
    assert C == 110 * 110 * 55
    for v in (7, 9, 10, 11):
        ab = bench.alg_bytes(N, C, 4, v)
        assert ab["density"] == 116 * N + 4 * C and ab["forces"] == 156 * N + 12 * C
        assert sum(ab.values()) == 360 * N + 40 * C
    keys = {(k, m) for k in ("k_forces", "k_density") for m in (1, 2)}
    assert set(bench.TRAFFIC) == keys and set(bench.ISSUE) == keys


def test_reference_arm_loads_no_product_library():
    """The reference arm builds its scene from the oracle's restatement and times only the
    oracle: the product library is never mapped into its process."""
    code = ("import sys, runpy; sys.argv = ['bench.py', '--impl', 'reference', '--steps', '1', '--warmup', '2', "
            "'--threads', '2']\n"
            "try:\n    runpy.run_path('bench.py', run_name='__main__')\nexcept SystemExit:\n    pass\n"
            "maps = open('/proc/self/maps').read()\n"
            "print('PRODUCT_MAPPED' if 'libsph_gb300' in maps else 'PRODUCT_NOT_MAPPED')\n")
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    out = r.stdout.strip().splitlines()
    assert out[-1] == "PRODUCT_NOT_MAPPED"
    line = json.loads(out[-2])
    assert line["warmup"] == 2  # the requested warm-up, not a capped one


def test_compulsory_bytes():
    """The roofline's algorithmic bytes: density 24 B, forces 72 B per particle, the step 196 B per
    particle plus 12 B per cell (plain FP32)."""
    sys.path.insert(0, ROOT)
    import bench

    N, C = 1_000_000, bench.grid_cells(bench.BOX)
    cb = bench.compulsory_bytes(N, C)
    assert cb == {"density": 24 * N, "forces": 72 * N, "step": 196 * N + 12 * C}
    assert bench.timed_steps(20, 500) == list(range(0, 500, 25))
    assert bench.timed_steps(500, 500) == list(range(500))


def test_rehash_launch_count():
    """bench.py's count of rehash launches per step from the cell multiple of every step: a
    trial on the other multiple switches in at its start and back at its end (two launches in
    that step); a switch that stays is the next step's one launch."""
    sys.path.insert(0, ROOT)
    import bench

    assert bench.rehash_steps([1, 1, 1, 2, 1, 1, 2, 2, 2, 1]) == [0, 0, 0, 2, 0, 0, 1, 0, 0, 1]
    assert bench.rehash_steps([2, 2, 2]) == [0, 0, 0]
    assert bench.rehash_steps([]) == []
