"""ctypes binding of libsph_gb300.so (include/sph_cuda.h) and a Python mirror of the
reference's simulator interface.

`SphContext` wraps one C-ABI context (one or many scenes). `CCUDAParticleSimulator`
mirrors CBaseParticleSimulator (include/CBaseParticleSimulator.h:29-110) for the CUDA
backend: setupScene, step, setGravityVector, getSelectedDevice, the five pass methods
returning milliseconds, and the DAM_BREAK / FOUNTAIN scenarios.

The library is the only compute path: there is no CPU fallback, and importing this module
on a machine without the built library raises.
"""
import ctypes
import math
import os
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
# SPH_LIBRARY selects another build of the library, e.g. lib/libsph_gb300_checked.so (bounds
# checks and guarded allocations, reported by sph_debug_check)
LIB_PATH = os.environ.get("SPH_LIBRARY") or os.path.join(HERE, "lib", "libsph_gb300.so")
LIB_CHECKED_PATH = os.path.join(HERE, "lib", "libsph_gb300_checked.so")

SPH_OK = 0
SPH_ERR_ARG, SPH_ERR_CUDA, SPH_ERR_CAPACITY, SPH_ERR_STATE, SPH_ERR_NOMEM, SPH_ERR_UNSUPPORTED, SPH_ERR_DEVICE = (
    -1, -2, -3, -4, -5, -6, -7)
SPH_PLAIN_F32, SPH_F64, SPH_MIXED = 0, 1, 2
SPH_FLAG_PROFILE, SPH_FLAG_RECORD_ACC, SPH_FLAG_ALL_PAIRS = 1, 2, 4

# every symbol the header declares
EXPORTS = (
    "sph_params_default", "sph_create", "sph_batch_create", "sph_memory_required", "sph_debug_check", "sph_destroy", "sph_last_error", "sph_device_name",
    "sph_stream", "sph_set_variant", "sph_get_variant", "sph_set_cell_multiple", "sph_get_cell_multiple", "sph_autotune",
    "sph_set_online_tuning", "sph_grid_build_noalloc",
    "sph_upload", "sph_append", "sph_emit_fountain", "sph_set_gravity", "sph_step", "sph_pass_grid", "sph_pass_density",
    "sph_pass_forces", "sph_pass_times", "sph_get_counts", "sph_num_scenes", "sph_num_particles",
    "sph_get_resolution", "sph_download", "sph_download_f64", "sph_handoff_async", "sph_handoff_ready",
    "sph_handoff_wait", "sph_export_positions", "sph_splat", "sph_get_grid", "sph_stats",
    "sph_scene_reference_dam_break", "sph_scene_lattice", "sph_scene_batch_plan", "sph_scene_fountain_emit",
)


class sph_params(ctypes.Structure):
    _fields_ = [
        ("struct_size", ctypes.c_uint32), ("h", ctypes.c_float), ("mass", ctypes.c_float),
        ("gas_stiffness", ctypes.c_float), ("rest_density", ctypes.c_float), ("viscosity", ctypes.c_float),
        ("dt", ctypes.c_float), ("gravity", ctypes.c_float * 3), ("wall_k", ctypes.c_float),
        ("wall_damping", ctypes.c_float), ("wall_radius", ctypes.c_float), ("precision", ctypes.c_int32),
        ("flags", ctypes.c_uint32), ("device", ctypes.c_int32),
    ]


class sph_scene_desc(ctypes.Structure):
    _fields_ = [
        ("box", ctypes.c_float * 3), ("max_particles", ctypes.c_uint32), ("n_obstacles", ctypes.c_uint32),
        ("obstacles", ctypes.POINTER(ctypes.c_float)),
    ]


class SphError(RuntimeError):
    """Raised on a non-zero status (the reference's CLException counterpart)."""

    def __init__(self, code, msg):
        super().__init__(f"sph error {code}: {msg}")
        self.code = code


_lib = None


def load(path=None):
    """Load the built library (never builds; build with sph_build.py or __graft_entry__.build)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise ImportError(f"{path} is missing: build it with gmu-water-simulation_gb300/sph_build.py")
    L = ctypes.CDLL(path)
    vp, u32, i32, f = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_int32, ctypes.c_float
    fp, dp, up, ip = (ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_double),
                      ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(ctypes.c_int32))
    sig = {
        "sph_params_default": (None, [ctypes.POINTER(sph_params)]),
        "sph_create": (i32, [ctypes.POINTER(sph_params), fp, u32, ctypes.POINTER(vp)]),
        "sph_batch_create": (i32, [ctypes.POINTER(sph_params), u32, ctypes.POINTER(sph_scene_desc),
                                   ctypes.POINTER(vp)]),
        "sph_memory_required": (i32, [ctypes.POINTER(sph_params), u32, ctypes.POINTER(sph_scene_desc),
                                      ctypes.POINTER(ctypes.c_uint64)]),
        "sph_debug_check": (i32, [vp, up]),
        "sph_destroy": (None, [vp]),
        "sph_last_error": (ctypes.c_char_p, [vp]),
        "sph_device_name": (ctypes.c_char_p, [vp]),
        "sph_stream": (vp, [vp]),
        "sph_set_variant": (i32, [vp, i32, i32]),
        "sph_get_variant": (i32, [vp, ip]),
        "sph_set_cell_multiple": (i32, [vp, i32]),
        "sph_get_cell_multiple": (i32, [vp]),
        "sph_autotune": (i32, [vp, i32]),
        "sph_set_online_tuning": (i32, [vp, i32]),
        "sph_grid_build_noalloc": (i32, [vp, u32, fp, f, vp, vp, vp, vp]),
        "sph_upload": (i32, [vp, vp, vp, up]),
        "sph_append": (i32, [vp, u32, vp, vp, u32]),
        "sph_emit_fountain": (i32, [vp, u32, ctypes.c_uint64, u32, u32, fp, f, f, f]),
        "sph_set_gravity": (i32, [vp, i32, fp]),
        "sph_step": (i32, [vp, i32]),
        "sph_pass_grid": (i32, [vp]), "sph_pass_density": (i32, [vp]), "sph_pass_forces": (i32, [vp]),
        "sph_pass_times": (i32, [vp, dp]),
        "sph_get_counts": (i32, [vp, up]),
        "sph_num_scenes": (u32, [vp]),
        "sph_num_particles": (ctypes.c_uint64, [vp]),
        "sph_get_resolution": (i32, [vp, u32, ip]),
        "sph_download": (i32, [vp, vp, vp, vp, vp, vp]),
        "sph_download_f64": (i32, [vp, vp, vp, vp, vp, vp]),
        "sph_handoff_async": (i32, [vp, vp, vp]),
        "sph_handoff_ready": (i32, [vp]),
        "sph_handoff_wait": (i32, [vp]),
        "sph_export_positions": (i32, [vp, vp, vp, vp]),
        "sph_splat": (i32, [vp, u32, i32, u32, u32, vp, vp, vp]),
        "sph_get_grid": (i32, [vp, up, up, up]),
        "sph_stats": (i32, [vp, u32, dp]),
        "sph_scene_reference_dam_break": (ctypes.c_int64, [f, fp, ctypes.c_uint64]),
        "sph_scene_lattice": (i32, [up, fp, f, f, ctypes.c_uint64, fp]),
        "sph_scene_batch_plan": (i32, [u32, ctypes.c_uint64, u32, u32, f, f, up, fp]),
        "sph_scene_fountain_emit": (i32, [ctypes.c_uint64, u32, u32, fp, f, f, f, fp, fp]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def _p(a, t=ctypes.c_float):
    return None if a is None else a.ctypes.data_as(ctypes.POINTER(t))


def _vp(a):
    return None if a is None else ctypes.c_void_p(a.ctypes.data)


def default_params(**kw):
    p = sph_params()
    load().sph_params_default(ctypes.byref(p))
    for k, v in kw.items():
        if k == "gravity":
            for a in range(3):
                p.gravity[a] = v[a]
        else:
            setattr(p, k, v)
    return p


# ----------------------------------------------------------------- scene generators
def reference_dam_break(box):
    L = load()
    n = L.sph_scene_reference_dam_break(ctypes.c_float(box), None, 0)
    out = np.zeros((n, 3), np.float32)
    L.sph_scene_reference_dam_break(ctypes.c_float(box), _p(out), n)
    return out


def lattice(dims, box, spacing, jitter, seed):
    dims_a = np.ascontiguousarray(dims, np.uint32)
    box_a = np.ascontiguousarray(box, np.float32)
    out = np.zeros((int(np.prod(dims_a, dtype=np.int64)), 3), np.float32)
    rc = load().sph_scene_lattice(_p(dims_a, ctypes.c_uint32), _p(box_a), spacing, jitter, seed, _p(out))
    if rc:
        raise SphError(rc, "sph_scene_lattice")
    return out


def batch_plan(n_scenes, seed, nmin=2000, nmax=64000, amin=0.5, amax=2.0):
    dims = np.zeros((n_scenes, 3), np.uint32)
    boxes = np.zeros((n_scenes, 3), np.float32)
    rc = load().sph_scene_batch_plan(n_scenes, seed, nmin, nmax, amin, amax, _p(dims, ctypes.c_uint32), _p(boxes))
    if rc:
        raise SphError(rc, "sph_scene_batch_plan")
    return dims, boxes


def fountain_emit(seed, step, n, center, radius, speed, sigma):
    c = np.ascontiguousarray(center, np.float32)
    xyz = np.zeros((n, 3), np.float32)
    vel = np.zeros((n, 3), np.float32)
    rc = load().sph_scene_fountain_emit(seed, step, n, _p(c), radius, speed, sigma, _p(xyz), _p(vel))
    if rc:
        raise SphError(rc, "sph_scene_fountain_emit")
    return xyz, vel


H = 0.0457
SPACING = np.float32(np.float32(H) / np.float32(2.0))  # 0.5 h, the reference lattice spacing


def dam_break_scene(dims, box, seed, jitter=0.01):
    """A jittered lattice anchored at the box's min corner (the synthetic dam breaks)."""
    return lattice(dims, box, float(SPACING), jitter, seed)


# ----------------------------------------------------------------- context
class SphContext:
    """One context of the C ABI: one or more scenes stepped together on one GPU."""

    def __init__(self, boxes, max_particles, precision=SPH_PLAIN_F32, flags=0, gravity=None, device=0,
                 obstacles=None, params=None):
        L = load()
        boxes = np.atleast_2d(np.asarray(boxes, np.float32))
        caps = np.atleast_1d(np.asarray(max_particles, np.uint64))
        if caps.size == 1 and boxes.shape[0] > 1:
            caps = np.repeat(caps, boxes.shape[0])
        p = params or default_params()
        p.precision = precision
        p.flags = flags
        p.device = device
        if gravity is not None:
            for a in range(3):
                p.gravity[a] = gravity[a]
        self.params = p
        self.precision = precision
        self.flags = flags
        S = boxes.shape[0]
        descs = (sph_scene_desc * S)()
        self._obs_keep = []
        for s in range(S):
            for a in range(3):
                descs[s].box[a] = float(boxes[s, a])
            descs[s].max_particles = int(caps[s])
            ob = None if obstacles is None else obstacles[s]
            if ob is not None and len(ob):
                arr = np.ascontiguousarray(ob, np.float32).reshape(-1, 6)
                self._obs_keep.append(arr)
                descs[s].n_obstacles = arr.shape[0]
                descs[s].obstacles = _p(arr)
        h = ctypes.c_void_p()
        rc = L.sph_batch_create(ctypes.byref(p), S, descs, ctypes.byref(h))
        if rc:
            raise SphError(rc, L.sph_last_error(None).decode())
        self.h = h
        self.n_scenes = S
        self.boxes = boxes

    # error helper
    def _ck(self, rc):
        if rc:
            raise SphError(rc, load().sph_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None):
            load().sph_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def device_name(self):
        return load().sph_device_name(self.h).decode()

    @property
    def stream(self):
        """The cudaStream_t handle (int) this context launches on."""
        return load().sph_stream(self.h) or 0

    @property
    def n(self):
        return int(load().sph_num_particles(self.h))

    def counts(self):
        c = np.zeros(self.n_scenes, np.uint32)
        self._ck(load().sph_get_counts(self.h, _p(c, ctypes.c_uint32)))
        return c

    def resolution(self, scene=0):
        r = np.zeros(3, np.int32)
        self._ck(load().sph_get_resolution(self.h, scene, _p(r, ctypes.c_int32)))
        return tuple(int(v) for v in r)

    def upload(self, xyz, vel=None, counts=None):
        xyz = np.ascontiguousarray(xyz, np.float32).reshape(-1, 3)
        vel = None if vel is None else np.ascontiguousarray(vel, np.float32).reshape(-1, 3)
        if counts is None:
            counts = [xyz.shape[0]]
        counts = np.ascontiguousarray(counts, np.uint32)
        self._ck(load().sph_upload(self.h, _vp(xyz), _vp(vel), _p(counts, ctypes.c_uint32)))

    def upload_raw(self, xyz_ptr, vel_ptr, counts):
        """Upload from raw host pointers (e.g. pinned buffers)."""
        counts = np.ascontiguousarray(counts, np.uint32)
        self._ck(load().sph_upload(self.h, ctypes.c_void_p(xyz_ptr), ctypes.c_void_p(vel_ptr) if vel_ptr else None,
                                   _p(counts, ctypes.c_uint32)))

    def append(self, scene, xyz, vel=None):
        xyz = np.ascontiguousarray(xyz, np.float32).reshape(-1, 3)
        vel = None if vel is None else np.ascontiguousarray(vel, np.float32).reshape(-1, 3)
        self._ck(load().sph_append(self.h, scene, _vp(xyz), _vp(vel), xyz.shape[0]))

    def emit_fountain(self, scene, seed, step, n, center, radius, speed, sigma):
        """Disc emitter on the device (the same particles as fountain_emit)."""
        c = np.ascontiguousarray(center, np.float32)
        self._ck(load().sph_emit_fountain(self.h, scene, seed, step, n, _p(c), radius, speed, sigma))

    def set_gravity(self, g, scene=-1):
        g = np.ascontiguousarray(g, np.float32)
        self._ck(load().sph_set_gravity(self.h, scene, _p(g)))

    def step(self, n=1):
        self._ck(load().sph_step(self.h, n))

    def pass_grid(self):
        self._ck(load().sph_pass_grid(self.h))

    def pass_density(self):
        self._ck(load().sph_pass_density(self.h))

    def pass_forces(self):
        self._ck(load().sph_pass_forces(self.h))

    def set_variant(self, density, forces):
        self._ck(load().sph_set_variant(self.h, density, forces))

    def variant(self):
        v = np.zeros(2, np.int32)
        self._ck(load().sph_get_variant(self.h, _p(v, ctypes.c_int32)))
        return int(v[0]), int(v[1])

    def set_cell_multiple(self, m):
        """Step grid of cells h / m (1: the reference's cells; 2: cells of h/2, 125-cell stencil)."""
        self._ck(load().sph_set_cell_multiple(self.h, m))

    def cell_multiple(self):
        m = load().sph_get_cell_multiple(self.h)
        if m < 0:
            self._ck(m)
        return m

    def autotune(self, reps=3):
        self._ck(load().sph_autotune(self.h, reps))
        return self.variant()

    def set_online_tuning(self, period):
        """Re-time the force variants every `period` steps (0 = off)."""
        self._ck(load().sph_set_online_tuning(self.h, period))

    def debug_check(self):
        """Device check flags since the last call (checked library only; 0 = clean)."""
        f = np.zeros(1, np.uint32)
        self._ck(load().sph_debug_check(self.h, _p(f, ctypes.c_uint32)))
        return int(f[0])

    def pass_times(self):
        ms = np.zeros(5, np.float64)
        self._ck(load().sph_pass_times(self.h, _p(ms, ctypes.c_double)))
        return ms

    def download(self, acc=False):
        n = self.n
        f64 = self.precision == SPH_F64
        dt = np.float64 if f64 else np.float32
        out = {"pos": np.zeros((n, 3), dt), "vel": np.zeros((n, 3), dt), "rho": np.zeros(n, dt),
               "p": np.zeros(n, dt)}
        if acc:
            out["acc"] = np.zeros((n, 3), dt)
        fn = load().sph_download_f64 if f64 else load().sph_download
        self._ck(fn(self.h, _vp(out["pos"]), _vp(out["vel"]), _vp(out["rho"]), _vp(out["p"]),
                    _vp(out.get("acc"))))
        return out

    def download_raw(self, xyz_ptr, vel_ptr, rho_ptr=None, p_ptr=None):
        self._ck(load().sph_download(self.h, ctypes.c_void_p(xyz_ptr), ctypes.c_void_p(vel_ptr),
                                     ctypes.c_void_p(rho_ptr) if rho_ptr else None,
                                     ctypes.c_void_p(p_ptr) if p_ptr else None, None))

    def handoff_async(self, xyz_ptr, vel_ptr=None):
        """Queue the id-ordered positions (and velocities) into host memory at raw pointers
        (pinned for an asynchronous copy); see handoff_ready / handoff_wait."""
        self._ck(load().sph_handoff_async(self.h, ctypes.c_void_p(xyz_ptr),
                                          ctypes.c_void_p(vel_ptr) if vel_ptr else None))

    def handoff_ready(self):
        rc = load().sph_handoff_ready(self.h)
        if rc < 0:
            self._ck(rc)
        return rc == 1

    def handoff_wait(self):
        self._ck(load().sph_handoff_wait(self.h))

    def export_positions(self, dev_xyz_ptr, dev_vel_ptr=None, consumer_stream=None):
        """Id-ordered float3 positions (and velocities) into device arrays at raw pointers."""
        self._ck(load().sph_export_positions(self.h, ctypes.c_void_p(dev_xyz_ptr),
                                             ctypes.c_void_p(dev_vel_ptr) if dev_vel_ptr else None,
                                             ctypes.c_void_p(consumer_stream) if consumer_stream else None))

    def splat_raw(self, scene, axis, width, height, dev_count_ptr, dev_depth_ptr, consumer_stream=None):
        """Point splat into device images at raw pointers (see sph_splat)."""
        self._ck(load().sph_splat(self.h, scene, axis, width, height,
                                  ctypes.c_void_p(dev_count_ptr) if dev_count_ptr else None,
                                  ctypes.c_void_p(dev_depth_ptr) if dev_depth_ptr else None,
                                  ctypes.c_void_p(consumer_stream) if consumer_stream else None))

    def splat(self, scene, axis, width, height):
        """(counts, depth) images of one scene as (height, width) numpy arrays; the device
        buffers are torch tensors (device memory plumbing only)."""
        import torch

        cnt = torch.empty((height, width), dtype=torch.int32, device="cuda")
        dep = torch.empty((height, width), dtype=torch.float32, device="cuda")
        s = torch.cuda.current_stream()
        self.splat_raw(scene, axis, width, height, cnt.data_ptr(), dep.data_ptr(), s.cuda_stream)
        return cnt.cpu().numpy().view(np.uint32), dep.cpu().numpy()

    def grid(self):
        """(cell of each particle, count of each cell, sorted ids) of the last grid pass."""
        n = self.n
        ncells = sum(int(np.prod(self.resolution(s))) for s in range(self.n_scenes))
        cell = np.zeros(n, np.uint32)
        counts = np.zeros(ncells, np.uint32)
        order = np.zeros(n, np.uint32)
        self._ck(load().sph_get_grid(self.h, _p(cell, ctypes.c_uint32), _p(counts, ctypes.c_uint32),
                                     _p(order, ctypes.c_uint32)))
        return cell, counts, order

    def stats(self, scene=0):
        out = np.zeros(8, np.float64)
        self._ck(load().sph_stats(self.h, scene, _p(out, ctypes.c_double)))
        return {"mass": out[0], "momentum": out[1:4].copy(), "kinetic": out[4], "rho_mean": out[5],
                "rho_max": out[6], "count": int(out[7])}


def write_pgm(path, image, vmax=None):
    """An image (row 0 at the smallest coordinate) as an 8-bit binary PGM, row 0 at the bottom."""
    a = np.asarray(image, np.float64)
    a = np.where(np.isfinite(a), a, 0.0)
    top = float(vmax if vmax is not None else (a.max() if a.size and a.max() > 0 else 1.0))
    g = np.clip(np.round(a / top * 255.0), 0, 255).astype(np.uint8)[::-1]
    with open(path, "wb") as f:
        f.write(f"P5\n{g.shape[1]} {g.shape[0]}\n255\n".encode())
        f.write(g.tobytes())
    return path


# ----------------------------------------------------------------- reference-shaped simulator
DAM_BREAK, FOUNTAIN = 0, 1  # include/CBaseParticleSimulator.h:21-25


class ProfilingEvent:
    """One step's pass times in ms and the frame rate (sProfilingEvent, include/SProfilingEvent.h:7-31)."""

    __slots__ = ("iteration", "fps", "updateGrid", "updateDensityPressure", "updateForces", "updateCollisions",
                 "integrate")

    def __init__(self, iteration, fps=0.0, updateGrid=0.0, updateDensityPressure=0.0, updateForces=0.0,
                 updateCollisions=0.0, integrate=0.0):
        self.iteration = iteration
        self.fps = fps
        self.updateGrid = updateGrid
        self.updateDensityPressure = updateDensityPressure
        self.updateForces = updateForces
        self.updateCollisions = updateCollisions
        self.integrate = integrate

    def together(self):
        return self.updateGrid + self.updateDensityPressure + self.updateForces + self.updateCollisions + self.integrate


def _qnum(v):
    """A double as QString::number formats it (format 'g', 6 significant digits)."""
    return f"{float(v):g}"


DETAIL_LABELS = ("Grid", "Density + pressure", "Forces", "Collisions", "Integrate")


def export_logs(events, directory, scenario, box_size, simulation_type):
    """Appends the two profiling logs of MainWindow::exportLogs (src/mainwindow.cpp:310-368):
    `<scenario>_<box>.csv`, one line `type;together;together;...;` per export, and
    `<scenario>_<box>_detail.csv`, the type, one `label;v;v;...;` line per pass and two blank
    lines. Returns the two paths."""
    os.makedirs(directory, exist_ok=True)
    stem = os.path.join(directory, f"{scenario}_{_qnum(box_size)}")
    summary, detail = stem + ".csv", stem + "_detail.csv"
    with open(summary, "a") as f:
        f.write(f"{simulation_type};" + "".join(_qnum(e.together()) + ";" for e in events) + "\n")
    cols = ("updateGrid", "updateDensityPressure", "updateForces", "updateCollisions", "integrate")
    with open(detail, "a") as f:
        f.write(f"{simulation_type}\n")
        for label, col in zip(DETAIL_LABELS, cols):
            f.write(f"{label};" + "".join(_qnum(getattr(e, col)) + ";" for e in events) + "\n")
        f.write("\n\n")
    return summary, detail


class CCUDAParticleSimulator:
    """Mirror of CBaseParticleSimulator for the CUDA backend (Qt-free).

    ctor(boxSize, scenario) builds the grid and walls of a cubic box
    (src/CBaseParticleSimulator.cpp:3-36); setupScene() adds the scenario's particles
    (:38-65); step() runs the passes in the reference's order (:116-144); a failing step
    stops the simulator and reports through `errorOccured` like
    CGPUBaseParticleSimulator::step (src/CGPUBaseParticleSimulator.cpp:28-37).
    """

    def __init__(self, boxSize, scenario=DAM_BREAK, precision=SPH_PLAIN_F32, profile=True, device=0):
        self.m_boxSize = np.float32(boxSize)
        self.m_scenario = scenario
        self.precision = precision
        self.flags = SPH_FLAG_PROFILE if profile else 0
        self.device = device
        self.ctx = None
        self.m_particlesCount = 0
        self.m_maxParticlesCount = 0
        self.totalIteration = 0
        self.running = False
        self.errorOccured = None  # callable(str), the errorOccured signal
        self._gravity = np.array([0.0, -9.80665, 0.0], np.float32)
        self._times = np.zeros(5)
        self._pending = None
        # profiling log (include/CBaseParticleSimulator.h:54-55): one event every 10 steps
        self.events = []
        self.eventLoggerStride = 10
        self.iterationSincePaused = 0
        self._t0 = time.perf_counter()

    def getSelectedDevice(self):
        return self.ctx.device_name if self.ctx else ""

    def getParticlesCount(self):
        return self.m_particlesCount

    def getMaxParticlesCount(self):
        return self.m_maxParticlesCount

    def setupScene(self):
        b = float(self.m_boxSize)
        half = np.float64(np.float32(H) / np.float32(2.0))
        calculated = int(math.ceil(b / half) * math.ceil(b / half) * math.ceil(b / 4 / half))
        if self.m_scenario == DAM_BREAK:
            xyz = reference_dam_break(b)
            assert xyz.shape[0] == calculated  # src/CBaseParticleSimulator.cpp:56
            self.m_maxParticlesCount = xyz.shape[0]
        else:
            xyz = np.zeros((0, 3), np.float32)
            self.m_maxParticlesCount = calculated
        self.ctx = SphContext([b, b, b], max(self.m_maxParticlesCount, 1), precision=self.precision,
                              flags=self.flags, gravity=self._gravity, device=self.device)
        self.ctx.upload(xyz)
        self.m_particlesCount = xyz.shape[0]

    def setGravityVector(self, g):
        self._gravity = np.asarray(g, np.float32)
        if self.ctx:
            self.ctx.set_gravity(self._gravity)

    def _generateParticles(self):
        """FOUNTAIN emitter (src/CBaseParticleSimulator.cpp:187-210): 7 particles per step."""
        if self.m_scenario != FOUNTAIN:
            return
        per = 7
        if self.m_particlesCount >= self.m_maxParticlesCount - per:
            return
        hp = np.float32(np.float32(H) / np.float32(2.0))
        q = np.float32(np.float32(H) / np.float32(4))
        oy = np.float32(-self.m_boxSize / np.float32(2.0))
        pts = np.array([[0, oy, 0], [-hp, oy, 0], [hp, oy, 0], [-q, oy, -hp], [q, oy, -hp], [-q, oy, hp],
                        [q, oy, hp]], np.float32)
        vel = np.tile(np.array([0.0, self.m_boxSize * np.float32(3.2), 0.0], np.float32), (per, 1))
        self.ctx.append(0, pts, vel)
        self.m_particlesCount += per

    def _pass_time(self, k):
        # each pass returns its own milliseconds (0 when profiling is off): a profiled pass call
        # waits for its work, so its time is known when it returns
        return float(self.ctx.pass_times()[k]) if self.flags & SPH_FLAG_PROFILE else 0.0

    def updateGrid(self):
        self.ctx.pass_grid()
        return self._pass_time(0)

    def updateDensityPressure(self):
        self.ctx.pass_density()
        return self._pass_time(1)

    def updateForces(self):
        self.ctx.pass_forces()
        return self._pass_time(2)

    def updateCollisions(self):
        return 0.0  # fused into the force pass

    def integrate(self):
        return 0.0  # fused into the force pass

    def step(self):
        try:
            self._generateParticles()
            t = [self.updateGrid(), self.updateDensityPressure(), self.updateForces(), self.updateCollisions(),
                 self.integrate()]
            if self.flags & SPH_FLAG_PROFILE:
                self._times = np.array(t)
                if self.totalIteration % self.eventLoggerStride == 0:
                    self.events.append(ProfilingEvent(self.totalIteration, self.getFps(), *self._times))
            self.totalIteration += 1
            self.iterationSincePaused += 1
        except SphError as exc:
            self.running = False
            if self.errorOccured:
                self.errorOccured(str(exc))
            else:
                raise

    def lastPassTimes(self):
        """(grid, density, forces, collisions, integrate) ms of the last step."""
        return self._times

    def getFps(self):
        """Steps per second since the simulation was last started (CBaseParticleSimulator::getFps)."""
        el = time.perf_counter() - self._t0
        return self.iterationSincePaused / el if el > 0 else 0.0

    def exportLogs(self, directory, simulationType="GPU CUDA", scenarioName=None):
        """The profiling logs of MainWindow::exportLogs for this simulator's events."""
        name = scenarioName or ("Dam break" if self.m_scenario == DAM_BREAK else "Fountain")
        return export_logs(self.events, directory, name, float(self.m_boxSize), simulationType)

    def start(self):
        self.running = True
        self.iterationSincePaused = 0
        self._t0 = time.perf_counter()

    def stop(self):
        self.running = False
