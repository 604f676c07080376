"""ctypes binding of the oracle (test infrastructure only; never the product path).

The oracle is a CPU restatement of the reference's serial SPH step
(src/CCPUParticleSimulator.cpp:9-229); see sph_oracle.c for the line-by-line
citations. The reference's CPU simulator cannot be built here (Qt5/Qt3D absent) and ships
no golden vectors. Its own OpenCL grid kernels (resources/kernels/sph_grid.cl,
sph_common.cl) compile for the CPU through oracle/ref_cl where the reference tree is present
(build_ref): they pin this restatement's density, pressure and forces and generate the golden
vectors under tests/golden/. The walls, integration and cell hash are pinned to analytic
known answers and to the reference's scene-count assert.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this module.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")

REF, CANON, F64 = 0, 1, 2

_lib = None


CFLAGS = ["-std=gnu11", "-O2", "-fPIC", "-shared", "-fopenmp", "-Wall", "-Wextra", "-Wno-unused-parameter",
          # no fused multiply-add: the reference's x86-64 build has none
          "-ffp-contract=off"]


def build(force=False):
    """Compile liboracle.so from sph_oracle.c with gcc (one translation unit)."""
    src = os.path.join(HERE, "sph_oracle.c")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        tmp = LIB_PATH + ".tmp"
        subprocess.check_call([os.environ.get("CC", "gcc"), *CFLAGS, "-o", tmp, src, "-lm"])
        os.replace(tmp, LIB_PATH)
    return LIB_PATH


# The reference's own OpenCL kernels compiled for the CPU (oracle/ref_cl): built only where the
# reference tree is present, into oracle/_ref/ (not committed, not usable on another machine).
# The kernels' directory (resources/kernels of the reference tree) comes from the caller or from
# SPH_REF_KERNELS; without either, an already built library is used if there is one.
REF_DIR = os.path.join(HERE, "_ref")
REF_LIB = os.path.join(REF_DIR, "librefcl.so")
_ref = None


def build_ref(kernels_dir=None, force=False):
    """Compile oracle/ref_cl/ref_cl.cpp, which includes sph_common.cl, sph_grid.cl and
    sph_brute.cl from kernels_dir (default: $SPH_REF_KERNELS) where they lie, into
    oracle/_ref/librefcl.so. Returns the path, or None when neither the kernels nor a built
    library are present."""
    kernels_dir = kernels_dir or os.environ.get("SPH_REF_KERNELS")
    if not kernels_dir:
        return REF_LIB if os.path.exists(REF_LIB) else None
    srcs = [os.path.join(kernels_dir, f) for f in ("sph_common.cl", "sph_grid.cl", "sph_brute.cl")]
    if not all(os.path.exists(f) for f in srcs):
        return REF_LIB if os.path.exists(REF_LIB) else None
    here = os.path.join(HERE, "ref_cl")
    deps = srcs + [os.path.join(here, f) for f in ("ref_cl.cpp", "cl_shim.h")]
    if force or not os.path.exists(REF_LIB) or os.path.getmtime(REF_LIB) < max(os.path.getmtime(f) for f in deps):
        os.makedirs(REF_DIR, exist_ok=True)
        tmp = REF_LIB + ".tmp"
        subprocess.check_call([os.environ.get("CXX", "g++"), "-std=c++17", "-O2", "-fPIC", "-shared",
                               "-ffp-contract=off", "-Wno-unknown-pragmas", "-Wno-unused-value",
                               "-Wno-unused-variable", "-I", here, "-I", kernels_dir,
                               os.path.join(here, "ref_cl.cpp"), "-o", tmp])
        os.replace(tmp, REF_LIB)
    return REF_LIB


def ref_lib():
    """The compiled reference kernels, or None where they were not built."""
    global _ref
    if _ref is None:
        if not os.path.exists(REF_LIB):
            return None
        try:
            L = ctypes.CDLL(REF_LIB)
        except OSError:  # built for another machine
            return None
        fp = ctypes.POINTER(ctypes.c_float)
        L.refcl_density_forces.argtypes = [ctypes.c_int, fp, fp, fp, fp, fp, fp, fp]
        L.refcl_density_forces.restype = ctypes.c_int
        L.refcl_brute_density_forces.argtypes = [ctypes.c_int, fp, fp, fp, fp, fp, fp]
        L.refcl_brute_density_forces.restype = ctypes.c_int
        _ref = L
    return _ref


def ref_density_forces(pos, vel, box, gravity):
    """The reference's density_pressure_step and forces_step (sph_grid.cl) for one state:
    (rho, p, acc before the walls), in input order."""
    L = ref_lib()
    if L is None:
        raise RuntimeError("reference kernels not built (oracle.build_ref)")
    pos = np.ascontiguousarray(pos, np.float32).reshape(-1, 3)
    vel = np.ascontiguousarray(vel, np.float32).reshape(-1, 3)
    n = pos.shape[0]
    b = np.ascontiguousarray(np.broadcast_to(np.asarray(box, np.float32), (3,)))
    g = np.ascontiguousarray(gravity, np.float32)
    rho, p, acc = np.zeros(n, np.float32), np.zeros(n, np.float32), np.zeros((n, 3), np.float32)
    rc = L.refcl_density_forces(n, _f(pos), _f(vel), _f(b), _f(g), _f(rho), _f(p), _f(acc))
    if rc:
        raise ValueError("refcl_density_forces failed")
    return rho, p, acc


def ref_brute_density_forces(pos, vel, gravity):
    """The reference's all-pairs density_pressure_step and forces_step (sph_brute.cl) for one
    state: (rho, p, acc before the walls), in input order."""
    L = ref_lib()
    if L is None:
        raise RuntimeError("reference kernels not built (oracle.build_ref)")
    pos = np.ascontiguousarray(pos, np.float32).reshape(-1, 3)
    vel = np.ascontiguousarray(vel, np.float32).reshape(-1, 3)
    n = pos.shape[0]
    g = np.ascontiguousarray(gravity, np.float32)
    rho, p, acc = np.zeros(n, np.float32), np.zeros(n, np.float32), np.zeros((n, 3), np.float32)
    if L.refcl_brute_density_forces(n, _f(pos), _f(vel), _f(g), _f(rho), _f(p), _f(acc)):
        raise ValueError("refcl_brute_density_forces failed")
    return rho, p, acc


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        vp, fp, ip, dp = ctypes.c_void_p, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_double)
        L.orc_create.restype = vp
        L.orc_create.argtypes = [ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_int, ctypes.c_int]
        L.orc_destroy.argtypes = [vp]
        L.orc_set_gravity.argtypes = [vp, ctypes.c_float, ctypes.c_float, ctypes.c_float]
        L.orc_set_dt.argtypes = [vp, ctypes.c_float]
        L.orc_set_obstacles.argtypes = [vp, ctypes.c_int, fp]
        L.orc_count.argtypes = [vp]
        L.orc_count.restype = ctypes.c_int
        L.orc_get_res.argtypes = [vp, ip]
        L.orc_add_particles.argtypes = [vp, ctypes.c_int, fp, fp]
        L.orc_add_particles.restype = ctypes.c_int
        for name in ("orc_update_grid", "orc_density", "orc_forces", "orc_integrate", "orc_brute_step"):
            getattr(L, name).argtypes = [vp]
        L.orc_step.argtypes = [vp, ctypes.c_int]
        L.orc_get_state.argtypes = [vp, fp, fp, fp, fp, fp, fp]
        L.orc_get_state_f64.argtypes = [vp, dp, dp, dp, dp, dp]
        L.orc_set_state.argtypes = [vp, fp, fp]
        L.orc_get_grid.argtypes = [vp, ip, ip, ip]
        L.orc_grid_res.argtypes = [ctypes.c_float]
        L.orc_grid_res.restype = ctypes.c_int
        L.orc_cell_axis.argtypes = [ctypes.c_float, ctypes.c_float, ctypes.c_int]
        L.orc_cell_axis.restype = ctypes.c_int
        L.orc_reference_dam_break.argtypes = [ctypes.c_float, fp, ctypes.c_int]
        L.orc_reference_dam_break.restype = ctypes.c_int
        L.orc_reference_dam_break_count.argtypes = [ctypes.c_float]
        L.orc_reference_dam_break_count.restype = ctypes.c_uint
        _lib = L
    return _lib


def _f(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float)) if a is not None else None


def _d(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)) if a is not None else None


def _i(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)) if a is not None else None


def reference_dam_break(box):
    """Positions of the reference's DAM_BREAK scene for a cubic box (float32, id order)."""
    L = lib()
    n = L.orc_reference_dam_break(ctypes.c_float(box), None, 0)
    out = np.zeros((n, 3), np.float32)
    L.orc_reference_dam_break(ctypes.c_float(box), _f(out), n)
    return out


def reference_dam_break_count(box):
    return int(lib().orc_reference_dam_break_count(ctypes.c_float(box)))


def grid_res(box):
    return int(lib().orc_grid_res(ctypes.c_float(box)))


def cell_axis(p, box, res):
    return int(lib().orc_cell_axis(ctypes.c_float(p), ctypes.c_float(box), res))


class Oracle:
    """One scene of the restated CPU simulator. Particles are kept in id order."""

    def __init__(self, box, mode=REF, threads=None, gravity=None, dt=None, obstacles=None):
        L = lib()
        if np.isscalar(box):
            box = (box, box, box)
        self.box = tuple(float(b) for b in box)
        self.mode = mode
        threads = threads or (os.cpu_count() or 1)
        self.h = L.orc_create(ctypes.c_float(self.box[0]), ctypes.c_float(self.box[1]),
                              ctypes.c_float(self.box[2]), mode, threads)
        if gravity is not None:
            L.orc_set_gravity(self.h, *[ctypes.c_float(g) for g in gravity])
        if dt is not None:
            L.orc_set_dt(self.h, ctypes.c_float(dt))
        if obstacles is not None and len(obstacles):
            ob = np.ascontiguousarray(obstacles, np.float32).reshape(-1, 6)
            L.orc_set_obstacles(self.h, ob.shape[0], _f(ob))

    def set_gravity(self, g):
        """setGravityVector (src/CBaseParticleSimulator.cpp:111-114): used from the next step."""
        lib().orc_set_gravity(self.h, *[ctypes.c_float(v) for v in g])

    def close(self):
        if self.h:
            lib().orc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def n(self):
        return lib().orc_count(self.h)

    @property
    def res(self):
        r = np.zeros(3, np.int32)
        lib().orc_get_res(self.h, _i(r))
        return tuple(int(v) for v in r)

    def add(self, pos, vel=None):
        pos = np.ascontiguousarray(pos, np.float32).reshape(-1, 3)
        vel = None if vel is None else np.ascontiguousarray(vel, np.float32).reshape(-1, 3)
        return lib().orc_add_particles(self.h, pos.shape[0], _f(pos), _f(vel))

    def set_state(self, pos, vel):
        pos = np.ascontiguousarray(pos, np.float32).reshape(-1, 3)
        vel = np.ascontiguousarray(vel, np.float32).reshape(-1, 3)
        assert pos.shape[0] == self.n
        lib().orc_set_state(self.h, _f(pos), _f(vel))

    def step(self, n=1):
        lib().orc_step(self.h, n)

    def update_grid(self):
        lib().orc_update_grid(self.h)

    def density(self):
        lib().orc_density(self.h)

    def forces(self):
        lib().orc_forces(self.h)

    def integrate(self):
        lib().orc_integrate(self.h)

    def brute_step(self):
        lib().orc_brute_step(self.h)

    def state(self):
        n = self.n
        out = {k: np.zeros((n, 3), np.float32) for k in ("pos", "vel", "acc")}
        out.update({k: np.zeros(n, np.float32) for k in ("rho", "p", "ascale")})
        lib().orc_get_state(self.h, _f(out["pos"]), _f(out["vel"]), _f(out["acc"]),
                            _f(out["rho"]), _f(out["p"]), _f(out["ascale"]))
        return out

    def state64(self):
        n = self.n
        out = {k: np.zeros((n, 3), np.float64) for k in ("pos", "vel", "acc")}
        out.update({k: np.zeros(n, np.float64) for k in ("rho", "p")})
        lib().orc_get_state_f64(self.h, _d(out["pos"]), _d(out["vel"]), _d(out["acc"]),
                                _d(out["rho"]), _d(out["p"]))
        return out

    def grid(self):
        """(cell of each particle, count of each cell, canonical (cell, id) order)."""
        X, Y, Z = self.res
        cell = np.zeros(self.n, np.int32)
        counts = np.zeros(X * Y * Z, np.int32)
        order = np.zeros(self.n, np.int32)
        lib().orc_get_grid(self.h, _i(cell), _i(counts), _i(order))
        return cell, counts, order
