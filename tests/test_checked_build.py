"""The checked library (SPH_CHECKED: device bounds checks on every counting-sort scatter,
neighbour row, neighbour index and id-ordered target, and guard regions after every array of
the pool) runs the workloads clean and gives the same bits as the production library. It
stands in for a sanitizer run: the checks skip a bad access and report it instead of
faulting. The checked library runs in a child process (one library per process)."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import json, sys, numpy as np
sys.path.insert(0, sys.argv[1]); sys.path.insert(0, sys.argv[1] + "/gmu-water-simulation_gb300")
import sphcuda
out = {}
flags = 0
rng = np.random.default_rng(11)
clump = (rng.random((1500, 3)) * 0.12 - 0.06).astype(np.float32)
lattice = sphcuda.dam_break_scene((12, 12, 12), (1.0, 1.0, 0.5), 2)
g = (0.0, -9.81, 0.0)
variants = [(d, f) for d in (0, 1, 2, 4) for f in (0, 1, 2)] + [(0, f) for f in range(3, 12)]
for name, box, pos in (("clump", (0.5, 0.5, 0.5), clump), ("lattice", (1.0, 1.0, 0.5), lattice)):
    for dv, fv in variants:
        ctx = sphcuda.SphContext(box, pos.shape[0], gravity=g)
        ctx.set_variant(dv, fv)
        ctx.upload(pos)
        ctx.step(4)
        d = ctx.download()
        flags |= ctx.debug_check()
        out[f"{name}/{dv},{fv}"] = d["pos"].tobytes().hex()
        ctx.close()
for form in (sphcuda.SPH_MIXED, sphcuda.SPH_F64):
    ctx = sphcuda.SphContext((1.0, 1.0, 0.5), lattice.shape[0] + 200, precision=form, gravity=g)
    ctx.upload(lattice)
    ctx.step(3)
    ctx.emit_fountain(0, 5, 0, 200, (0.0, -0.2, 0.0), 0.03, 0.5, 0.05)
    ctx.step(3)
    flags |= ctx.debug_check()
    ctx.close()
ctx = sphcuda.SphContext((1.0, 1.0, 0.5), lattice.shape[0], gravity=g, flags=sphcuda.SPH_FLAG_ALL_PAIRS)
ctx.upload(lattice)
ctx.step(3)
flags |= ctx.debug_check()
ctx.close()
# the allocation-free grid build (its checks are collected by the next context's check)
import ctypes, torch
L = sphcuda.load()
for box, pos in (((0.5, 0.5, 0.5), clump), ((1.0, 1.0, 0.5), lattice)):
    n = pos.shape[0]
    res = [int(np.ceil(np.float32(b) / np.float32(0.0457))) for b in box]
    xyz = torch.from_numpy(np.ascontiguousarray(pos)).cuda()
    oc = torch.empty(n, dtype=torch.int32, device="cuda")
    os_ = torch.empty(res[0] * res[1] * res[2] + 1, dtype=torch.int32, device="cuda")
    oo = torch.empty(n, dtype=torch.int32, device="cuda")
    rc = L.sph_grid_build_noalloc(ctypes.c_void_p(xyz.data_ptr()), n, (ctypes.c_float * 3)(*box), 0.0457,
                                  ctypes.c_void_p(oc.data_ptr()), ctypes.c_void_p(os_.data_ptr()),
                                  ctypes.c_void_p(oo.data_ptr()), None)
    torch.cuda.synchronize()
    assert rc == 0
    out[f"noalloc/{box}"] = oo.cpu().numpy().tobytes().hex()
ctx = sphcuda.SphContext((0.4, 0.4, 0.4), 10)
flags |= ctx.debug_check()
ctx.close()
print(json.dumps({"flags": flags, "out": out}))
"""


def run_child(lib):
    env = dict(os.environ, SPH_LIBRARY=lib)
    r = subprocess.run([sys.executable, "-c", CHILD, ROOT], capture_output=True, text=True, env=env, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    return json.loads(r.stdout.strip().splitlines()[-1])


def test_checked_library_exports_the_check(sphlib):
    """Both libraries export sph_debug_check; the production one answers unsupported."""
    assert os.path.exists(sphlib.LIB_CHECKED_PATH)
    import ctypes
    L = ctypes.CDLL(sphlib.LIB_CHECKED_PATH)
    assert hasattr(L, "sph_debug_check") and hasattr(sphlib.load(), "sph_debug_check")


@pytest.mark.gpu
def test_checked_build_is_clean_and_identical(sphlib):
    checked = run_child(sphlib.LIB_CHECKED_PATH)
    assert checked["flags"] == 0
    plain_lib = os.path.join(os.path.dirname(sphlib.LIB_CHECKED_PATH), "libsph_gb300.so")
    env = dict(os.environ, SPH_LIBRARY=plain_lib)
    r = subprocess.run([sys.executable, "-c", CHILD.replace("flags |= ctx.debug_check()", "pass"), ROOT],
                       capture_output=True, text=True, env=env, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    plain = json.loads(r.stdout.strip().splitlines()[-1])
    assert checked["out"].keys() == plain["out"].keys()
    for k in plain["out"]:
        assert checked["out"][k] == plain["out"][k], k


@pytest.mark.gpu
def test_production_library_reports_no_checks(sphlib):
    ctx = sphlib.SphContext((0.4, 0.4, 0.4), 10)
    with pytest.raises(sphlib.SphError) as e:
        ctx.debug_check()
    assert e.value.code == sphlib.SPH_ERR_UNSUPPORTED
    ctx.close()
