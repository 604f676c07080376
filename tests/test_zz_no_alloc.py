"""The grid build that allocates no device memory (sph_grid_build_noalloc), for callers that
cannot allocate while running (a host whose GPU memory belongs to its own pool allocator, or a
real-time per-frame callback that must not stall on an allocation). Its cells, cell starts and
sorted order must equal the grid of the context entry points (sph_pass_grid + sph_get_grid) on
the same positions; the grid is compared bit for bit, the tolerance of every grid test here.
Two calls in a row check that the shared scratch array is cleared between calls.
This file runs last so that a failure here leaves every other test already run."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

H = np.float32(0.0457)


def context_grid(sphlib, box, pos):
    ctx = sphlib.SphContext(box, pos.shape[0])
    ctx.upload(pos)
    ctx.pass_grid()
    cell, counts, order = ctx.grid()
    ctx.close()
    return cell, counts, order


def crowded(seed=9):
    """One cell of 3,000 particles (its slot ids sorted before the rank) in a sparse lattice."""
    rng = np.random.default_rng(seed)
    h = float(H)
    clump = np.array([3, 4, 2]) * h - 0.3 + (0.05 + 0.9 * rng.random((3000, 3))) * h
    g = np.stack(np.meshgrid(*[np.arange(5) * 0.1 - 0.2] * 3, indexing="ij"), -1).reshape(-1, 3)
    pos = np.concatenate([clump, g]).astype(np.float32)
    return (0.6, 0.6, 0.6), pos[rng.permutation(pos.shape[0])]


def test_noalloc_grid_matches_context_grid(sphlib):
    torch = pytest.importorskip("torch")
    L = sphlib.load()
    cases = [((1.0, 1.0, 0.5), sphlib.dam_break_scene((20, 20, 20), (1.0, 1.0, 0.5), seed=0)),
             ((0.45, 0.5, 0.6), sphlib.dam_break_scene((12, 9, 14), (0.45, 0.5, 0.6), seed=5) - np.float32(0.01)),
             crowded()]
    # calls in a row, different scenes and grids; the last writes its cell starts to an array
    # that is 4- but not 16-byte aligned (the scan then takes its scalar path)
    for (box, pos), offset in zip(cases + cases[:1], (0, 0, 0, 1)):
        n = pos.shape[0]
        res = [int(np.ceil(np.float32(b) / H)) for b in box]
        ncells = res[0] * res[1] * res[2]
        xyz = torch.from_numpy(np.ascontiguousarray(pos)).cuda()
        out_cell = torch.empty(n, dtype=torch.int32, device="cuda")
        start_buf = torch.empty(ncells + 1 + offset, dtype=torch.int32, device="cuda")
        out_start = start_buf[offset:]
        out_order = torch.empty(n, dtype=torch.int32, device="cuda")
        boxa = (ctypes.c_float * 3)(*box)
        stream = torch.cuda.current_stream().cuda_stream
        rc = L.sph_grid_build_noalloc(ctypes.c_void_p(xyz.data_ptr()), n, boxa, float(H),
                                      ctypes.c_void_p(out_cell.data_ptr()), ctypes.c_void_p(out_start.data_ptr()),
                                      ctypes.c_void_p(out_order.data_ptr()), ctypes.c_void_p(stream))
        torch.cuda.synchronize()
        assert rc == sphlib.SPH_OK
        assert (out_start.data_ptr() % 16 != 0) == (offset == 1)
        cell, counts, order = context_grid(sphlib, box, pos)
        start = out_start.cpu().numpy().astype(np.int64)
        assert np.array_equal(out_cell.cpu().numpy().astype(np.uint32), cell)
        assert start[-1] == n and np.array_equal(np.diff(start).astype(np.uint32), counts)
        assert np.array_equal(out_order.cpu().numpy().astype(np.uint32), order)


def test_noalloc_allocates_nothing(sphlib):
    """After the first call on the device (the setup call), further calls leave the device's free
    memory unchanged: no allocation by the library or by the CUDA runtime on its behalf."""
    torch = pytest.importorskip("torch")
    L = sphlib.load()
    box = (1.0, 1.0, 0.5)
    pos = sphlib.dam_break_scene((20, 20, 20), box, seed=3)
    n = pos.shape[0]
    res = [int(np.ceil(np.float32(b) / H)) for b in box]
    xyz = torch.from_numpy(np.ascontiguousarray(pos)).cuda()
    out_cell = torch.empty(n, dtype=torch.int32, device="cuda")
    out_start = torch.empty(res[0] * res[1] * res[2] + 1, dtype=torch.int32, device="cuda")
    out_order = torch.empty(n, dtype=torch.int32, device="cuda")
    boxa = (ctypes.c_float * 3)(*box)
    stream = torch.cuda.current_stream().cuda_stream

    def call():
        rc = L.sph_grid_build_noalloc(ctypes.c_void_p(xyz.data_ptr()), n, boxa, float(H),
                                      ctypes.c_void_p(out_cell.data_ptr()), ctypes.c_void_p(out_start.data_ptr()),
                                      ctypes.c_void_p(out_order.data_ptr()), ctypes.c_void_p(stream))
        torch.cuda.synchronize()
        assert rc == sphlib.SPH_OK

    call()  # the setup call
    first = out_order.clone()
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(3):
        call()
    assert torch.cuda.mem_get_info()[0] == free0
    assert torch.equal(out_order, first)


def test_noalloc_rejects_sizes_beyond_its_limit(sphlib):
    L = sphlib.load()
    box = (ctypes.c_float * 3)(100.0, 100.0, 100.0)  # 2189^3 cells: beyond 1,048,576
    one = ctypes.c_void_p(1)  # never dereferenced: the size check comes first
    rc = L.sph_grid_build_noalloc(one, 10, box, float(H), one, one, one, None)
    assert rc == sphlib.SPH_ERR_CAPACITY
    box = (ctypes.c_float * 3)(1.0, 1.0, 1.0)
    rc = L.sph_grid_build_noalloc(one, (1 << 20) + 1, box, float(H), one, one, one, None)
    assert rc == sphlib.SPH_ERR_CAPACITY
    # a quotient beyond int range on every axis (its product would wrap) and an infinite box
    box = (ctypes.c_float * 3)(1e30, 1e30, 1e30)
    assert L.sph_grid_build_noalloc(one, 10, box, float(H), one, one, one, None) == sphlib.SPH_ERR_CAPACITY
    box = (ctypes.c_float * 3)(float("inf"), 1.0, 1.0)
    assert L.sph_grid_build_noalloc(one, 10, box, float(H), one, one, one, None) == sphlib.SPH_ERR_ARG
    box = (ctypes.c_float * 3)(1.0, float("nan"), 1.0)
    assert L.sph_grid_build_noalloc(one, 10, box, float(H), one, one, one, None) == sphlib.SPH_ERR_ARG
    box = (ctypes.c_float * 3)(1.0, 1.0, 1.0)
    assert L.sph_grid_build_noalloc(one, 10, box, float("inf"), one, one, one, None) == sphlib.SPH_ERR_ARG
