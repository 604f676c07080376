"""The C-ABI library loads, exports every function include/sph_cuda.h declares, and its
host-side argument checks report errors without a GPU (no compute call is made here)."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "sph_cuda.h")


def header_functions():
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(sph_[a-z0-9_]+)\s*\(", txt)))


def test_header_lists_match(sphlib):
    assert sorted(sphlib.EXPORTS) == header_functions()


def test_every_declared_symbol_is_exported(sphlib):
    L = sphlib.load()
    for name in header_functions():
        assert hasattr(L, name), name
    out = subprocess.run(["nm", "-D", "--defined-only", sphlib.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT (sph_\w+)", out))
    assert set(header_functions()) <= exported


def test_params_default(sphlib):
    p = sphlib.default_params()
    assert p.struct_size == ctypes.sizeof(sphlib.sph_params)
    assert p.h == np.float32(0.0457) and p.mass == np.float32(0.02) and p.viscosity == np.float32(3.5)
    assert p.gas_stiffness == 3.0 and p.rest_density == np.float32(998.29)
    assert p.dt == np.float32(0.01) and p.gravity[1] == np.float32(-9.80665)
    assert p.wall_k == 10000.0 and p.wall_damping == np.float32(-0.9) and p.wall_radius == np.float32(0.01)
    assert p.precision == sphlib.SPH_PLAIN_F32


def _create(sphlib, box=(1.0, 1.0, 1.0), cap=10, n_scenes=1, **kw):
    L = sphlib.load()
    p = sphlib.default_params(**kw)
    descs = (sphlib.sph_scene_desc * max(n_scenes, 1))()
    for s in range(max(n_scenes, 1)):
        for a in range(3):
            descs[s].box[a] = box[a]
        descs[s].max_particles = cap
    h = ctypes.c_void_p()
    rc = L.sph_batch_create(ctypes.byref(p), n_scenes, descs, ctypes.byref(h))
    return rc, h, L.sph_last_error(None).decode()


def test_argument_errors_without_gpu(sphlib):
    rc, h, msg = _create(sphlib, box=(1.0, -1.0, 1.0))
    assert rc == sphlib.SPH_ERR_ARG and "box" in msg and not h.value
    rc, h, msg = _create(sphlib, n_scenes=0)
    assert rc == sphlib.SPH_ERR_ARG
    rc, h, msg = _create(sphlib, h=0.0)
    assert rc == sphlib.SPH_ERR_ARG and "h" in msg
    rc, h, msg = _create(sphlib, precision=7)
    assert rc == sphlib.SPH_ERR_UNSUPPORTED
    p = sphlib.default_params()
    p.struct_size = 4
    hh = ctypes.c_void_p()
    box = (ctypes.c_float * 3)(1, 1, 1)
    rc = sphlib.load().sph_create(ctypes.byref(p), box, 10, ctypes.byref(hh))
    assert rc == sphlib.SPH_ERR_ARG and b"struct_size" in sphlib.load().sph_last_error(None)
    # the all-pairs form: no mixed-precision variant, small scenes only
    rc, h, msg = _create(sphlib, precision=sphlib.SPH_MIXED, flags=sphlib.SPH_FLAG_ALL_PAIRS)
    assert rc == sphlib.SPH_ERR_UNSUPPORTED and "all-pairs" in msg
    rc, h, msg = _create(sphlib, cap=131073, flags=sphlib.SPH_FLAG_ALL_PAIRS)
    assert rc == sphlib.SPH_ERR_CAPACITY and "131072" in msg
    # NULL context pointers are rejected, never dereferenced
    L = sphlib.load()
    assert L.sph_step(None, 1) == sphlib.SPH_ERR_ARG
    assert L.sph_pass_grid(None) == sphlib.SPH_ERR_ARG
    assert L.sph_download(None, None, None, None, None, None) == sphlib.SPH_ERR_ARG
    assert L.sph_num_particles(None) == 0


def test_create_without_gpu_reports_cuda_error(sphlib):
    """With no GPU the context cannot be created; the call fails with a message, no crash."""
    try:
        import torch

        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        pytest.skip("a GPU is present")
    rc, h, msg = _create(sphlib)
    assert rc == sphlib.SPH_ERR_CUDA and msg
    with pytest.raises(sphlib.SphError):
        sphlib.SphContext([1.0, 1.0, 1.0], 10)


def test_memory_required_and_limit(sphlib, monkeypatch):
    """The device memory of a configuration is known on the host, and a context above
    SPH_DEVICE_MEMORY_LIMIT is refused with SPH_ERR_NOMEM before any device work."""
    L = sphlib.load()

    def required(cap, box=(5.0, 5.0, 2.5), **kw):
        p = sphlib.default_params(**kw)
        d = (sphlib.sph_scene_desc * 1)()
        for a in range(3):
            d[0].box[a] = box[a]
        d[0].max_particles = cap
        out = ctypes.c_uint64()
        rc = L.sph_memory_required(ctypes.byref(p), 1, d, ctypes.byref(out))
        return rc, out.value

    rc, b1 = required(1_000_000)
    assert rc == sphlib.SPH_OK and 250e6 < b1 < 450e6  # ~330 B per particle + ~50 B per cell
    rc, b2 = required(2_000_000)
    assert rc == sphlib.SPH_OK and 1.8 < b2 / b1 < 2.0
    rc, b3 = required(1_000_000, precision=sphlib.SPH_F64)
    assert rc == sphlib.SPH_OK and b3 > b1
    rc, _ = required(0)
    assert rc == sphlib.SPH_ERR_ARG
    monkeypatch.setenv("SPH_DEVICE_MEMORY_LIMIT", str(b1 - 1))
    rc, h, msg = _create(sphlib, box=(5.0, 5.0, 2.5), cap=1_000_000)
    assert rc == sphlib.SPH_ERR_NOMEM and "SPH_DEVICE_MEMORY_LIMIT" in msg and not h.value
