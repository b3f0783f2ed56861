"""GB300 (sm_103a) explicit APIC / MLS-MPM snow step behind the C ABI of
``include/rd_mpm.h`` - Python host side.

Two layers, both thin ctypes front ends over ``librd_mpm.so`` (built in-tree
from ``csrc/`` by :func:`build`):

* :class:`Simulation` - one ``rd_handle``: particle upload/download, the fused
  step, the reference's individual stages, the grid.
* :class:`LagrangeEulerView` - the reference's simulation class
  (realtime-deformations/material_point_method.hpp:174-233) with its method
  names, so a ``main.cpp``-style driver reads the same.

There is no CPU fallback: every call goes to the CUDA library and fails loudly
(``RuntimeError``) when it is missing or returns an error.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
REPO_DIR = os.path.dirname(PKG_DIR)
CSRC = os.path.join(PKG_DIR, "csrc")
# RD_BOUNDS_CHECK=1 in the environment selects the bounds-checked build
# (librd_mpm_checked.so, compiled with -DRD_BOUNDS_CHECK) for this process.
CHECKED = os.environ.get("RD_BOUNDS_CHECK") == "1"
LIB_PATH = os.path.join(PKG_DIR, "librd_mpm_checked.so" if CHECKED else "librd_mpm.so")
HEADER = os.path.join(REPO_DIR, "include", "rd_mpm.h")

NVCC_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-lineinfo", "-std=c++17",
              "-Xcompiler", "-fPIC,-ffp-contract=off", "-shared"]

RD_OK, RD_INVALID_ARG, RD_OOM, RD_CUDA_ERROR, RD_DEVICE_FAULT_FLAG, RD_TIMEOUT, RD_NOT_SUPPORTED, RD_TOO_LARGE = range(8)
STATUS_NAMES = {0: "RD_OK", 1: "RD_INVALID_ARG", 2: "RD_OOM", 3: "RD_CUDA_ERROR",
                4: "RD_DEVICE_FAULT_FLAG", 5: "RD_TIMEOUT", 6: "RD_NOT_SUPPORTED", 7: "RD_TOO_LARGE"}
RD_FP32, RD_FP64 = 0, 1
RD_HOST, RD_DEVICE = 0, 1
RD_BC_NONE, RD_BC_STICKY = 0, 1
FLAG_OUT_OF_DOMAIN, FLAG_NONFINITE, FLAG_BAD_WORK, FLAG_WAIT_TIMEOUT = 1, 2, 4, 8
STAGES = {"rasterize": 0, "forces": 1, "grid_velocities": 2, "collisions": 3,
          "deformation": 4, "particle_velocities": 5, "positions": 6, "volumes": 7}

# Every symbol include/rd_mpm.h declares.
EXPORTS = ("rd_default_params", "rd_create", "rd_destroy", "rd_set_particles", "rd_get_particles",
           "rd_init_volumes", "rd_step", "rd_stage", "rd_get_grid", "rd_device_xyzs", "rd_get_flags",
           "rd_clear_flags", "rd_synchronize", "rd_get_stream", "rd_last_error", "rd_debug_sort", "rd_debug_wait_timeout",
           "rd_debug_bounds_violations",
           "rd_set_kernel_timing", "rd_kernel_timing", "rd_launch_count", "rd_graph_replays", "rd_io_bytes", "rd_host_alloc", "rd_host_free", "rd_batch_create",
           "rd_batch_num_scenes", "rd_batch_set_particles", "rd_batch_get_particles", "rd_batch_get_grid",
           "rd_batch_step", "rd_set_graphs", "rd_autotune", "rd_tune_trials", "rd_tune_key", "rd_tune_cache_get",
           "rd_tune_cache_put", "rd_set_tuning", "rd_get_tuning",
           "rd_adjoint_record", "rd_adjoint_backward", "rd_set_colliders", "rd_move_colliders",
           "rd_set_colors", "rd_device_colors", "rd_splat", "rd_initialize_particles", "rd_get_diagnostics",
           "rd_rasterize_noalloc", "rd_rasterize_noalloc_flags", "rd_default_implicit_opts", "rd_time_integration",
           "rd_implicit_energy")
KERNELS = ("keys", "scan", "scatter", "grid_clear", "p2g", "g2p2g", "adj_g2p", "adj_p2g")


def _sources():
    return [os.path.join(CSRC, f) for f in sorted(os.listdir(CSRC)) if f.endswith((".cu", ".cuh", ".h"))] + [HEADER]


def bounds_violations():
    """(count, checked): accesses out of range skipped so far in this process
    by the bounds-checked build (rd_debug_bounds_violations); checked is False
    for the normal build, whose count is 0."""
    c, k = ctypes.c_uint64(), ctypes.c_int32()
    st = lib().rd_debug_bounds_violations(ctypes.byref(c), ctypes.byref(k))
    if st != RD_OK:
        raise RuntimeError(f"rd_debug_bounds_violations: {STATUS_NAMES.get(st, st)}")
    return c.value, bool(k.value)


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile ``csrc/rd_mpm.cu`` for sm_103a into ``librd_mpm.so`` (in-tree;
    ``librd_mpm_checked.so`` with RD_BOUNDS_CHECK=1 in the environment)."""
    newest = max(os.path.getmtime(f) for f in _sources())
    if not force and os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= newest:
        return LIB_PATH
    tmp = LIB_PATH + f".tmp{os.getpid()}"
    cmd = ["nvcc", *NVCC_FLAGS, *(["-DRD_BOUNDS_CHECK"] if CHECKED else []), os.path.join(CSRC, "rd_mpm.cu"), "-o", tmp]
    if verbose:
        print(" ".join(cmd))
    subprocess.check_call(cmd, cwd=CSRC)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


class Params(ctypes.Structure):
    """Mirror of ``rd_params``."""
    _fields_ = [("max_i", ctypes.c_int32), ("max_j", ctypes.c_int32), ("max_k", ctypes.c_int32),
                ("num_particles", ctypes.c_int32), ("h", ctypes.c_double), ("E", ctypes.c_double),
                ("nu", ctypes.c_double), ("xi", ctypes.c_double), ("theta_c", ctypes.c_double),
                ("theta_s", ctypes.c_double), ("gravity", ctypes.c_double * 3), ("bc", ctypes.c_int32),
                ("bc_width", ctypes.c_int32), ("lagged_b", ctypes.c_int32), ("track_fp", ctypes.c_int32),
                ("precision", ctypes.c_int32), ("device", ctypes.c_int32)]


class _Particles(ctypes.Structure):
    _fields_ = [(k, ctypes.c_void_p) for k in ("x", "v", "B", "FE", "FP", "Jp", "mass", "volume")]


_LIB = None
_LIB_LOCK = threading.Lock()


RD_COLLIDE_REFERENCE, RD_COLLIDE_COULOMB = 0, 1


class Collider(ctypes.Structure):
    """rd_collider: a box mesh spanning [-1, 1]^3 placed by T R S, with a velocity."""
    _fields_ = [("translation", ctypes.c_double * 3), ("rotation", ctypes.c_double * 4),
                ("scale", ctypes.c_double * 3), ("velocity", ctypes.c_double * 3)]


RD_INIT_REFERENCE, RD_INIT_PARALLEL = 0, 1


class InitSpec(ctypes.Structure):
    _fields_ = [("origin", ctypes.c_double * 3), ("velocity", ctypes.c_double * 3), ("radius", ctypes.c_double),
                ("mass", ctypes.c_double), ("seed", ctypes.c_uint32), ("mode", ctypes.c_int32)]


class Diagnostics(ctypes.Structure):
    _fields_ = [("particle_mass", ctypes.c_double), ("particle_momentum", ctypes.c_double * 3),
                ("grid_mass", ctypes.c_double), ("grid_momentum", ctypes.c_double * 3),
                ("used_cells", ctypes.c_int64), ("average_particle_density", ctypes.c_double),
                ("average_deformation_gradient", ctypes.c_double * 9)]


class View(ctypes.Structure):
    """rd_view: camera of the point-splat image."""
    _fields_ = [("view_projection", ctypes.c_float * 16), ("camera_right", ctypes.c_float * 3),
                ("camera_up", ctypes.c_float * 3), ("width", ctypes.c_int32), ("height", ctypes.c_int32),
                ("background", ctypes.c_uint32), ("max_radius", ctypes.c_int32)]


def look_at_view(eye, target, up=(0.0, 1.0, 0.0), fovy_deg=45.0, width=512, height=512, near=0.01, far=10.0,
                 background=0xFF201A18, max_radius=0) -> View:
    """A perspective camera like glm::lookAt / glm::perspective, as an rd_view."""
    eye, target, up = (np.asarray(a, np.float64) for a in (eye, target, up))
    f = target - eye
    f /= np.linalg.norm(f)
    r = np.cross(f, up)
    r /= np.linalg.norm(r)
    u = np.cross(r, f)
    view = np.eye(4)
    view[0, :3], view[1, :3], view[2, :3] = r, u, -f
    view[:3, 3] = [-r @ eye, -u @ eye, f @ eye]
    t = 1.0 / np.tan(np.radians(fovy_deg) / 2)
    proj = np.zeros((4, 4))
    proj[0, 0], proj[1, 1] = t / (width / height), t
    proj[2, 2], proj[2, 3] = -(far + near) / (far - near), -2 * far * near / (far - near)
    proj[3, 2] = -1.0
    vp = proj @ view
    v = View()
    v.view_projection[:] = list(vp.T.reshape(-1).astype(np.float32))  # column-major
    v.camera_right[:] = list(r.astype(np.float32))
    v.camera_up[:] = list(u.astype(np.float32))
    v.width, v.height, v.background, v.max_radius = width, height, background, max_radius
    return v


def save_ppm(path: str, image: np.ndarray):
    """Writes an (h, w, 4) rgba8 image as a binary PPM (alpha dropped)."""
    h, w = image.shape[:2]
    with open(path, "wb") as f:
        f.write(b"P6\n%d %d\n255\n" % (w, h))
        f.write(np.ascontiguousarray(image[:, :, :3]).tobytes())


class Grads(ctypes.Structure):
    _fields_ = [("v0", ctypes.c_void_p), ("E", ctypes.POINTER(ctypes.c_double)),
                ("nu", ctypes.POINTER(ctypes.c_double)), ("theta_c", ctypes.POINTER(ctypes.c_double)),
                ("theta_s", ctypes.POINTER(ctypes.c_double))]


class TuneResult(ctypes.Structure):
    _fields_ = [("particles_per_item", ctypes.c_int32), ("ctas_per_sm", ctypes.c_int32),
                ("ms_per_step", ctypes.c_double), ("trials", ctypes.c_int32), ("scatter", ctypes.c_int32),
                ("from_cache", ctypes.c_int32)]


class ImplicitOpts(ctypes.Structure):
    _fields_ = [("max_iters", ctypes.c_int32), ("history", ctypes.c_int32), ("grad_tol", ctypes.c_double),
                ("step_tol", ctypes.c_double), ("mu0", ctypes.c_double), ("lambda0", ctypes.c_double),
                ("xi", ctypes.c_double), ("hardening", ctypes.c_int32), ("ls_max_iters", ctypes.c_int32)]


class ImplicitResult(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int32), ("evaluations", ctypes.c_int32), ("converged", ctypes.c_int32),
                ("unknowns", ctypes.c_int32), ("energy_start", ctypes.c_double), ("energy", ctypes.c_double),
                ("grad_norm", ctypes.c_double)]


HARDENING_REFERENCE, HARDENING_INTENDED = 0, 1


def implicit_opts(**kw) -> ImplicitOpts:
    """rd_default_implicit_opts (the reference's L-BFGS settings and constants)
    with the given fields replaced."""
    o = ImplicitOpts()
    lib().rd_default_implicit_opts(ctypes.byref(o))
    for k, v in kw.items():
        if not hasattr(o, k):
            raise TypeError(f"unknown implicit option {k}")
        setattr(o, k, v)
    return o


class TuneTrial(ctypes.Structure):
    _fields_ = [("particles_per_item", ctypes.c_int32), ("ctas_per_sm", ctypes.c_int32),
                ("scatter", ctypes.c_int32), ("ms_per_step", ctypes.c_double)]


SCATTER_LANE_PAIRS, SCATTER_RECORD_PAIRS = 0, 1
SCATTER_NAMES = {SCATTER_LANE_PAIRS: "lane_pairs", SCATTER_RECORD_PAIRS: "record_pairs"}


def _tune_dict(r):
    return {"particles_per_item": r.particles_per_item, "ctas_per_sm": r.ctas_per_sm, "ms_per_step": r.ms_per_step,
            "trials": r.trials, "scatter": SCATTER_NAMES.get(r.scatter, r.scatter), "from_cache": bool(r.from_cache)}


def tune_cache_get(path: str, key: str):
    """rd_tune_cache_get: the cached point for `key` in the file, or None."""
    r, found = TuneResult(), ctypes.c_int32(0)
    st = lib().rd_tune_cache_get(os.fsencode(path), key.encode(), ctypes.byref(r), ctypes.byref(found))
    if st != RD_OK:
        raise RDError(st, "rd_tune_cache_get")
    return _tune_dict(r) if found.value else None


def tune_cache_put(path: str, key: str, particles_per_item: int, ctas_per_sm: int, scatter: int = 0,
                   ms_per_step: float = 0.0):
    """rd_tune_cache_put: appends one point for `key` to the file."""
    r = TuneResult(int(particles_per_item), int(ctas_per_sm), float(ms_per_step), 0, int(scatter), 0)
    st = lib().rd_tune_cache_put(os.fsencode(path), key.encode(), ctypes.byref(r))
    if st != RD_OK:
        raise RDError(st, "rd_tune_cache_put")


def lib():
    """The loaded CUDA library; raises if it has not been built."""
    global _LIB
    with _LIB_LOCK:
        if _LIB is None:
            if not os.path.exists(LIB_PATH):
                raise RuntimeError(f"CUDA library not built: {LIB_PATH} (run build())")
            L = ctypes.CDLL(LIB_PATH)
            vp, st = ctypes.c_void_p, ctypes.c_int
            L.rd_default_params.argtypes = [ctypes.POINTER(Params)]
            L.rd_default_params.restype = None
            L.rd_create.argtypes = [ctypes.POINTER(Params), ctypes.POINTER(vp)]
            L.rd_destroy.argtypes = [vp]
            L.rd_set_particles.argtypes = [vp, ctypes.POINTER(_Particles), ctypes.c_int]
            L.rd_get_particles.argtypes = [vp, ctypes.POINTER(_Particles), ctypes.c_int]
            L.rd_init_volumes.argtypes = [vp]
            L.rd_step.argtypes = [vp, ctypes.c_double, ctypes.c_int32]
            L.rd_stage.argtypes = [vp, ctypes.c_int32, ctypes.c_double]
            L.rd_get_grid.argtypes = [vp, vp, vp, vp, ctypes.c_int]
            L.rd_device_xyzs.argtypes = [vp, ctypes.POINTER(vp)]
            L.rd_get_flags.argtypes = [vp, ctypes.POINTER(ctypes.c_uint32)]
            L.rd_clear_flags.argtypes = [vp]
            L.rd_synchronize.argtypes = [vp]
            L.rd_get_stream.argtypes = [vp, ctypes.POINTER(vp)]
            L.rd_last_error.argtypes = [vp, ctypes.c_char_p, ctypes.c_size_t]
            L.rd_debug_sort.argtypes = [vp, vp, vp, ctypes.c_int]
            L.rd_debug_wait_timeout.argtypes = [vp, ctypes.c_int32, ctypes.POINTER(ctypes.c_int32)]
            L.rd_debug_bounds_violations.argtypes = [ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_int32)]
            L.rd_launch_count.argtypes = [vp, ctypes.POINTER(ctypes.c_uint64)]
            L.rd_graph_replays.argtypes = [vp, ctypes.POINTER(ctypes.c_uint64)]
            L.rd_io_bytes.argtypes = [vp, ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64)]
            L.rd_host_alloc.argtypes = [ctypes.c_size_t, ctypes.POINTER(vp)]
            L.rd_host_free.argtypes = [vp]
            L.rd_rasterize_noalloc.argtypes = [ctypes.POINTER(Params), ctypes.POINTER(_Particles), vp, vp]
            L.rd_rasterize_noalloc_flags.argtypes = [ctypes.POINTER(ctypes.c_uint32)]
            L.rd_batch_create.argtypes = [ctypes.POINTER(Params), ctypes.c_int32, ctypes.POINTER(vp)]
            L.rd_batch_num_scenes.argtypes = [vp, ctypes.POINTER(ctypes.c_int32)]
            L.rd_batch_set_particles.argtypes = [vp, ctypes.c_int32, ctypes.POINTER(_Particles), ctypes.c_int]
            L.rd_batch_get_particles.argtypes = [vp, ctypes.c_int32, ctypes.POINTER(_Particles), ctypes.c_int]
            L.rd_batch_get_grid.argtypes = [vp, ctypes.c_int32, vp, vp, ctypes.c_int]
            L.rd_batch_step.argtypes = [vp, ctypes.c_double, ctypes.c_int32]
            L.rd_set_graphs.argtypes = [vp, ctypes.c_int]
            L.rd_autotune.argtypes = [vp, ctypes.c_double, ctypes.c_int32, ctypes.c_char_p, ctypes.POINTER(TuneResult)]
            L.rd_tune_trials.argtypes = [vp, ctypes.POINTER(TuneTrial), ctypes.c_int32, ctypes.POINTER(ctypes.c_int32)]
            L.rd_tune_key.argtypes = [vp, ctypes.c_char_p, ctypes.c_size_t]
            L.rd_tune_cache_get.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.POINTER(TuneResult),
                                            ctypes.POINTER(ctypes.c_int32)]
            L.rd_tune_cache_put.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.POINTER(TuneResult)]
            L.rd_set_tuning.argtypes = [vp, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32]
            L.rd_default_implicit_opts.argtypes = [ctypes.POINTER(ImplicitOpts)]
            L.rd_default_implicit_opts.restype = None
            L.rd_time_integration.argtypes = [vp, ctypes.c_double, ctypes.POINTER(ImplicitOpts),
                                              ctypes.POINTER(ImplicitResult)]
            L.rd_implicit_energy.argtypes = [vp, ctypes.c_double, ctypes.POINTER(ImplicitOpts), vp, vp, ctypes.c_int,
                                             ctypes.POINTER(ctypes.c_double)]
            L.rd_get_tuning.argtypes = [vp, ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int32),
                                        ctypes.POINTER(ctypes.c_int32)]
            L.rd_get_diagnostics.argtypes = [vp, ctypes.c_int32, ctypes.POINTER(Diagnostics)]
            L.rd_initialize_particles.argtypes = [vp, ctypes.POINTER(InitSpec), ctypes.POINTER(ctypes.c_int32)]
            L.rd_set_colors.argtypes = [vp, vp, ctypes.c_int]
            L.rd_device_colors.argtypes = [vp, ctypes.POINTER(vp)]
            L.rd_splat.argtypes = [vp, ctypes.POINTER(View), vp, ctypes.c_int]
            L.rd_set_colliders.argtypes = [vp, ctypes.POINTER(Collider), ctypes.c_int32, ctypes.c_int32, ctypes.c_double]
            L.rd_move_colliders.argtypes = [vp, ctypes.c_double]
            L.rd_adjoint_record.argtypes = [vp, ctypes.c_double, ctypes.c_int32, ctypes.c_int32]
            L.rd_adjoint_backward.argtypes = [vp, vp, vp, ctypes.c_int, ctypes.POINTER(Grads)]
            L.rd_set_kernel_timing.argtypes = [vp, ctypes.c_int]
            L.rd_kernel_timing.argtypes = [vp, ctypes.c_int, ctypes.POINTER(ctypes.c_uint64),
                                           ctypes.POINTER(ctypes.c_double)]
            for name in EXPORTS:
                if name != "rd_default_params":
                    getattr(L, name).restype = st
            _LIB = L
    return _LIB


def default_params() -> Params:
    p = Params()
    lib().rd_default_params(ctypes.byref(p))
    return p


def make_params(max_i, max_j, max_k, num_particles, h, *, E=1.4e5, nu=0.2, xi=10.0, theta_c=2.5e-2,
                theta_s=5.0e-3, gravity=(0.0, -9.8, 0.0), bc=RD_BC_NONE, bc_width=3, lagged_b=1,
                track_fp=0, precision=RD_FP32, device=0) -> Params:
    p = Params()
    p.max_i, p.max_j, p.max_k, p.num_particles = max_i, max_j, max_k, num_particles
    p.h, p.E, p.nu, p.xi, p.theta_c, p.theta_s = h, E, nu, xi, theta_c, theta_s
    p.gravity = (ctypes.c_double * 3)(*gravity)
    p.bc, p.bc_width, p.lagged_b, p.track_fp, p.precision, p.device = bc, bc_width, lagged_b, track_fp, precision, device
    return p


class RDError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


class Simulation:
    """One ``rd_handle``.  Arrays are numpy on the host (float32 for RD_FP32,
    float64 for RD_FP64) or, for ``where=RD_DEVICE``, raw device pointers."""

    def __init__(self, params: Params):
        self.params = params
        self.n = params.num_particles
        self.dtype = np.float64 if params.precision == RD_FP64 else np.float32
        self._h = ctypes.c_void_p()
        L = lib()
        s = L.rd_create(ctypes.byref(params), ctypes.byref(self._h))
        if s != RD_OK:
            raise RDError(s, "rd_create failed")

    def close(self):
        if self._h:
            lib().rd_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def handle(self):
        return self._h

    def _check(self, status, what):
        if status != RD_OK:
            buf = ctypes.create_string_buffer(512)
            lib().rd_last_error(self._h, buf, 512)
            raise RDError(status, f"{what}: {buf.value.decode(errors='replace')}")

    def _arr(self, a, shape):
        if a is None:
            return None
        return np.ascontiguousarray(np.asarray(a, self.dtype).reshape(shape))

    def _particles_in(self, n, x, v, mass, B, FE, FP, Jp, volume):
        arrs = {"x": self._arr(x, (n, 3)), "v": self._arr(v, (n, 3)), "B": self._arr(B, (n, 9)),
                "FE": self._arr(FE, (n, 9)), "FP": self._arr(FP, (n, 9)), "Jp": self._arr(Jp, (n,)),
                "mass": self._arr(mass, (n,)), "volume": self._arr(volume, (n,))}
        ps = _Particles(**{k: (a.ctypes.data if a is not None else None) for k, a in arrs.items()})
        return ps, arrs

    def _particles_out(self, n, fields, out):
        shapes = {"x": (n, 3), "v": (n, 3), "B": (n, 9), "FE": (n, 9), "FP": (n, 9), "Jp": (n,),
                  "mass": (n,), "volume": (n,)}
        if out is None:
            out = {k: np.zeros(shapes[k], self.dtype) for k in fields}
        for k in fields:
            a = out[k]
            if a.shape != shapes[k] or a.dtype != self.dtype or not a.flags.c_contiguous:
                raise ValueError(f"out[{k!r}] must be a contiguous {self.dtype.__name__} array of shape {shapes[k]}")
        ps = _Particles(**{k: (out[k].ctypes.data if k in fields else None) for k in shapes})
        return ps, out

    def set_particles(self, x, v, mass, B=None, FE=None, FP=None, Jp=None, volume=None, sync=True,
                      mapped=False):
        """Copies host arrays in (rd_set_particles).  Arrays in page-locked
        memory (torch ``pin_memory``) are read in place by the packing kernel,
        the others go through a device staging buffer.  With sync=False the
        call returns once the work is queued; the arrays must stay alive and
        unchanged until the handle's stream reaches them.  mapped=True passes
        the arrays as device-accessible pointers (RD_DEVICE) without the
        page-locked check."""
        ps, self._pending = self._particles_in(self.n, x, v, mass, B, FE, FP, Jp, volume)
        self._check(lib().rd_set_particles(self._h, ctypes.byref(ps), RD_DEVICE if mapped else RD_HOST),
                    "rd_set_particles")
        if sync:
            self._check(lib().rd_synchronize(self._h), "rd_synchronize")

    def get_particles(self, fields=("x", "v", "B", "FE", "FP", "Jp", "mass", "volume"), out=None, mapped=False):
        """Copies the particle state out in the original particle order
        (rd_get_particles).  ``out`` may supply the destination arrays;
        page-locked ones are written in place by the unpacking kernel.  With
        mapped=True (``out`` device-accessible, e.g. pinned host memory) the
        call returns without waiting: synchronize() before reading."""
        ps, out = self._particles_out(self.n, fields, out)
        self._check(lib().rd_get_particles(self._h, ctypes.byref(ps), RD_DEVICE if mapped else RD_HOST),
                    "rd_get_particles")
        return out

    def init_volumes(self):
        self._check(lib().rd_init_volumes(self._h), "rd_init_volumes")

    def step(self, dt: float, nsteps: int = 1):
        self._check(lib().rd_step(self._h, float(dt), int(nsteps)), "rd_step")

    def stage(self, name: str, dt: float = 0.0):
        self._check(lib().rd_stage(self._h, STAGES[name], float(dt)), f"rd_stage({name})")

    def time_integration(self, dt: float, **opts) -> dict:
        """rd_time_integration: the grid velocities replaced by the minimiser of
        the reference's implicit energy (options as rd_implicit_opts fields)."""
        o, r = implicit_opts(**opts), ImplicitResult()
        self._check(lib().rd_time_integration(self._h, float(dt), ctypes.byref(o), ctypes.byref(r)),
                    "rd_time_integration")
        return {k: getattr(r, k) for k, _ in ImplicitResult._fields_}

    def implicit_energy(self, vel, dt: float, grad: bool = False, **opts):
        """rd_implicit_energy at the dense velocity field vel (cells x 3):
        the energy, and (energy, gradient) with grad."""
        p = self.params
        nc = p.max_i * p.max_j * p.max_k
        v = np.ascontiguousarray(np.asarray(vel, self.dtype).reshape(nc, 3))
        g = np.zeros((nc, 3), self.dtype) if grad else None
        e = ctypes.c_double()
        o = implicit_opts(**opts)
        self._check(lib().rd_implicit_energy(self._h, float(dt), ctypes.byref(o), v.ctypes.data,
                                             g.ctypes.data if grad else None, RD_HOST, ctypes.byref(e)),
                    "rd_implicit_energy")
        return (e.value, g) if grad else e.value

    def get_grid(self, force: bool = False):
        p = self.params
        nc = p.max_i * p.max_j * p.max_k
        m = np.zeros(nc, self.dtype)
        v = np.zeros((nc, 3), self.dtype)
        f = np.zeros((nc, 3), self.dtype) if force else None
        self._check(lib().rd_get_grid(self._h, m.ctypes.data, v.ctypes.data,
                                      f.ctypes.data if f is not None else None, RD_HOST), "rd_get_grid")
        out = {"mass": m, "vel": v}
        if f is not None:
            out["force"] = f
        return out

    def device_xyzs(self) -> int:
        ptr = ctypes.c_void_p()
        self._check(lib().rd_device_xyzs(self._h, ctypes.byref(ptr)), "rd_device_xyzs")
        return ptr.value

    def flags(self) -> int:
        f = ctypes.c_uint32()
        self._check(lib().rd_get_flags(self._h, ctypes.byref(f)), "rd_get_flags")
        return f.value

    def clear_flags(self):
        self._check(lib().rd_clear_flags(self._h), "rd_clear_flags")

    def synchronize(self):
        self._check(lib().rd_synchronize(self._h), "rd_synchronize")

    def stream(self) -> int:
        s = ctypes.c_void_p()
        self._check(lib().rd_get_stream(self._h, ctypes.byref(s)), "rd_get_stream")
        return s.value or 0

    def debug_sort(self):
        """(block key per particle in original order, original index per sorted slot)."""
        keys = np.zeros(self.n, np.uint32)
        order = np.zeros(self.n, np.uint32)
        self._check(lib().rd_debug_sort(self._h, keys.ctypes.data, order.ctypes.data, RD_HOST), "rd_debug_sort")
        return keys, order

    def set_kernel_timing(self, enable: bool):
        self._check(lib().rd_set_kernel_timing(self._h, int(enable)), "rd_set_kernel_timing")

    def kernel_timing(self):
        """{kernel name: (launches, total ms)} since timing was enabled."""
        out = {}
        for k, name in enumerate(KERNELS):
            n, ms = ctypes.c_uint64(), ctypes.c_double()
            self._check(lib().rd_kernel_timing(self._h, k, ctypes.byref(n), ctypes.byref(ms)), "rd_kernel_timing")
            out[name] = (n.value, ms.value)
        return out

    def launch_count(self) -> int:
        c = ctypes.c_uint64()
        self._check(lib().rd_launch_count(self._h, ctypes.byref(c)), "rd_launch_count")
        return c.value

    def debug_wait_timeout(self, tries: int = 64) -> bool:
        """Runs the tile-copy wait against an mbarrier nothing arrives at;
        True when it gave up (and raised RD_FLAG_WAIT_TIMEOUT)."""
        g = ctypes.c_int32()
        self._check(lib().rd_debug_wait_timeout(self._h, int(tries), ctypes.byref(g)), "rd_debug_wait_timeout")
        return bool(g.value)

    def graph_replays(self) -> int:
        """Two-step CUDA graphs replayed so far."""
        c = ctypes.c_uint64()
        self._check(lib().rd_graph_replays(self._h, ctypes.byref(c)), "rd_graph_replays")
        return c.value

    def io_bytes(self):
        """(in place, staged): particle bytes that set_particles / get_particles
        moved straight from and to page-locked host arrays, and through the
        device staging buffer (rd_io_bytes)."""
        a, b = ctypes.c_uint64(), ctypes.c_uint64()
        self._check(lib().rd_io_bytes(self._h, ctypes.byref(a), ctypes.byref(b)), "rd_io_bytes")
        return a.value, b.value

    @property
    def num_scenes(self) -> int:
        return 1

    def set_colliders(self, colliders, mode: int = RD_COLLIDE_REFERENCE, friction: float = 0.5):
        """Box colliders for the grid update (rd_set_colliders): dicts with
        translation, rotation (unit quaternion w, x, y, z), scale (half extents)
        and velocity."""
        arr = (Collider * max(1, len(colliders)))()
        for k, c in enumerate(colliders):
            arr[k].translation[:] = list(c["translation"])
            arr[k].rotation[:] = list(c.get("rotation", (1.0, 0.0, 0.0, 0.0)))
            arr[k].scale[:] = list(c["scale"])
            arr[k].velocity[:] = list(c.get("velocity", (0.0, 0.0, 0.0)))
        self._check(lib().rd_set_colliders(self._h, arr, len(colliders), int(mode), float(friction)),
                    "rd_set_colliders")

    def move_colliders(self, dt: float):
        self._check(lib().rd_move_colliders(self._h, float(dt)), "rd_move_colliders")

    def diagnostics(self, scene: int = 0) -> dict:
        """rd_get_diagnostics: the reference's momentum / mass / density / F
        diagnostics of one scene, reduced on the device."""
        d = Diagnostics()
        self._check(lib().rd_get_diagnostics(self._h, int(scene), ctypes.byref(d)), "rd_get_diagnostics")
        return {"particle_mass": d.particle_mass, "particle_momentum": np.array(d.particle_momentum[:]),
                "grid_mass": d.grid_mass, "grid_momentum": np.array(d.grid_momentum[:]), "used_cells": d.used_cells,
                "average_particle_density": d.average_particle_density,
                "average_deformation_gradient": np.array(d.average_deformation_gradient[:]).reshape(3, 3)}

    def initialize_particles(self, origin, velocity, radius: float = 0.2, mass: float = 6e-5, seed: int = 1,
                             mode: int = RD_INIT_REFERENCE) -> int:
        """rd_initialize_particles: the reference's jittered sphere generated on the
        device; returns how many kept points found no particle."""
        sp = InitSpec()
        sp.origin[:] = list(origin)
        sp.velocity[:] = list(velocity)
        sp.radius, sp.mass, sp.seed, sp.mode = radius, mass, seed, mode
        more = ctypes.c_int32()
        self._check(lib().rd_initialize_particles(self._h, ctypes.byref(sp), ctypes.byref(more)),
                    "rd_initialize_particles")
        return more.value

    def set_colors(self, rgba):
        """n x 4 uint8 colours in original particle order (the viewer's colour stream)."""
        a = np.ascontiguousarray(np.asarray(rgba, np.uint8).reshape(self.n, 4))
        self._check(lib().rd_set_colors(self._h, a.ctypes.data, RD_HOST), "rd_set_colors")
        self.synchronize()

    def splat(self, view: View) -> np.ndarray:
        """rd_splat: the point-splat image of the current particles, (h, w, 4) uint8."""
        img = np.zeros((view.height, view.width, 4), np.uint8)
        self._check(lib().rd_splat(self._h, ctypes.byref(view), img.ctypes.data, RD_HOST), "rd_splat")
        return img

    def adjoint_record(self, dt: float, steps: int, checkpoint_every: int = 10):
        """rd_adjoint_record: `steps` steps from the current state, keeping
        checkpoints for the reverse pass; the handle then holds the final state."""
        self._check(lib().rd_adjoint_record(self._h, float(dt), int(steps), int(checkpoint_every)),
                    "rd_adjoint_record")

    def adjoint_backward(self, grad_x, grad_v=None) -> dict:
        """rd_adjoint_backward: dL/dx (and dL/dv) of the final state, n x 3 in
        original order -> {"v0": dL/dv of the start state, "E", "nu",
        "theta_c", "theta_s": one value per scene}."""
        gx = self._arr(grad_x, (self.n, 3))
        gv = self._arr(grad_v, (self.n, 3))
        ns = self.num_scenes
        out = {"v0": np.zeros((self.n, 3), self.dtype)}
        for k in ("E", "nu", "theta_c", "theta_s"):
            out[k] = np.zeros(ns, np.float64)
        dp = ctypes.POINTER(ctypes.c_double)
        g = Grads(out["v0"].ctypes.data, *(out[k].ctypes.data_as(dp) for k in ("E", "nu", "theta_c", "theta_s")))
        self._check(lib().rd_adjoint_backward(self._h, gx.ctypes.data, gv.ctypes.data if gv is not None else None,
                                              RD_HOST, ctypes.byref(g)), "rd_adjoint_backward")
        return out

    def set_graphs(self, enable: bool):
        self._check(lib().rd_set_graphs(self._h, int(enable)), "rd_set_graphs")

    def autotune(self, dt: float, steps: int = 10, cache: str | None = None) -> dict:
        """rd_autotune: picks the work-item size, CTAs per SM and scatter layout
        by timing, or from the cache file `cache` when it holds this handle's key."""
        r = TuneResult()
        path = os.fsencode(cache) if cache else None
        self._check(lib().rd_autotune(self._h, float(dt), int(steps), path, ctypes.byref(r)), "rd_autotune")
        return _tune_dict(r)

    def tune_trials(self) -> list:
        """rd_tune_trials: every point the last autotune timed."""
        n = ctypes.c_int32(0)
        self._check(lib().rd_tune_trials(self._h, None, 0, ctypes.byref(n)), "rd_tune_trials")
        arr = (TuneTrial * max(n.value, 1))()
        self._check(lib().rd_tune_trials(self._h, arr, n.value, ctypes.byref(n)), "rd_tune_trials")
        return [{"particles_per_item": t.particles_per_item, "ctas_per_sm": t.ctas_per_sm,
                 "scatter": SCATTER_NAMES.get(t.scatter, t.scatter), "ms_per_step": t.ms_per_step}
                for t in arr[:n.value]]

    def tune_key(self) -> str:
        buf = ctypes.create_string_buffer(512)
        self._check(lib().rd_tune_key(self._h, buf, 512), "rd_tune_key")
        return buf.value.decode()

    def set_tuning(self, particles_per_item: int = 0, ctas_per_sm: int = 0, scatter: int = SCATTER_LANE_PAIRS):
        self._check(lib().rd_set_tuning(self._h, int(particles_per_item), int(ctas_per_sm), int(scatter)),
                    "rd_set_tuning")

    def tuning(self):
        """(particles per item, CTAs per SM, scatter layout)."""
        a, b, c = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
        self._check(lib().rd_get_tuning(self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)), "rd_get_tuning")
        return a.value, b.value, c.value


class Batch(Simulation):
    """Several independent scenes in one handle (rd_batch_create): one sort and
    one fused kernel per step for all of them.  Scene s is described by its own
    ``Params``; its particles are set and read per scene."""

    def __init__(self, scenes):
        scenes = list(scenes)
        if not scenes:
            raise ValueError("a batch needs at least one scene")
        self.scene_params = scenes
        self.params = scenes[0]
        self.counts = [p.num_particles for p in scenes]
        self.offsets = [int(o) for o in np.cumsum([0] + self.counts)[:-1]]
        self.n = int(sum(self.counts))
        self.dtype = np.float64 if scenes[0].precision == RD_FP64 else np.float32
        self._h = ctypes.c_void_p()
        arr = (Params * len(scenes))(*scenes)
        s = lib().rd_batch_create(arr, len(scenes), ctypes.byref(self._h))
        if s != RD_OK:
            raise RDError(s, "rd_batch_create failed")

    @property
    def nscenes(self) -> int:
        return len(self.scene_params)

    @property
    def num_scenes(self) -> int:
        return len(self.scene_params)

    def set_particles(self, scene, x, v, mass, B=None, FE=None, FP=None, Jp=None, volume=None, sync=True):
        ps, self._pending = self._particles_in(self.counts[scene], x, v, mass, B, FE, FP, Jp, volume)
        self._check(lib().rd_batch_set_particles(self._h, int(scene), ctypes.byref(ps), RD_HOST),
                    "rd_batch_set_particles")
        if sync:
            self._check(lib().rd_synchronize(self._h), "rd_synchronize")

    def get_particles(self, scene, fields=("x", "v", "B", "FE", "FP", "Jp", "mass", "volume"), out=None):
        ps, out = self._particles_out(self.counts[scene], fields, out)
        self._check(lib().rd_batch_get_particles(self._h, int(scene), ctypes.byref(ps), RD_HOST),
                    "rd_batch_get_particles")
        return out

    def get_grid(self, scene):
        p = self.scene_params[scene]
        nc = p.max_i * p.max_j * p.max_k
        m = np.zeros(nc, self.dtype)
        v = np.zeros((nc, 3), self.dtype)
        self._check(lib().rd_batch_get_grid(self._h, int(scene), m.ctypes.data, v.ctypes.data, RD_HOST),
                    "rd_batch_get_grid")
        return {"mass": m, "vel": v}


class LagrangeEulerView:
    """The reference's ``MaterialPointMethod::LagrangeEulerView`` interface
    (material_point_method.hpp:174-233) over :class:`Simulation`.

    ``h`` replaces the global ``WeightCalculator::h`` that the reference reads at
    construction (material_point_method.hpp:177).  Stage methods run the
    corresponding GPU stage; :meth:`step` is the fused fast path that the seven
    stage calls of main.cpp:192-218 amount to.  :meth:`getParticles` returns a
    host copy (dict of arrays) synchronised from the device.
    """

    def __init__(self, max_i: int, max_j: int, max_k: int, particlesNum: int, h: float = 0.05, **kw):
        self.MAX_I, self.MAX_J, self.MAX_K = max_i, max_j, max_k
        kw.setdefault("track_fp", 1)
        self.sim = Simulation(make_params(max_i, max_j, max_k, particlesNum, h, **kw))
        self.h = h

    def getNumParticles(self) -> int:
        return self.sim.n

    def setParticles(self, x, v, mass, **kw):
        self.sim.set_particles(x, v, mass, **kw)

    def getParticles(self):
        return self.sim.get_particles()

    def rasterizeParticlesToGrid(self):
        self.sim.stage("rasterize")

    def computeParticleVolumesAndDensities(self):
        self.sim.stage("volumes")

    def computeExplicitGridForces(self):
        self.sim.stage("forces")

    def gridVelocitiesUpdate(self, timeDelta: float):
        self.sim.stage("grid_velocities", timeDelta)

    def gridBasedCollisions(self, timeDelta: float, objects=()):
        """objects: box colliders as dicts (translation, rotation (w, x, y, z),
        scale, velocity), the reference's MeshCollider fields; uploaded when
        they change."""
        objs = [dict(c) for c in objects]
        if objs != getattr(self, "_colliders", []):
            self.sim.set_colliders(objs)
            self._colliders = objs
        self.sim.stage("collisions", timeDelta)

    def timeIntegration(self, timeDelta: float, **opts):
        """material_point_method.cpp:212-233 (rd_time_integration)."""
        return self.sim.time_integration(timeDelta, **opts)

    def updateDeformationGradient(self, timeDelta: float):
        self.sim.stage("deformation", timeDelta)

    def updateParticleVelocities(self):
        self.sim.stage("particle_velocities")

    def updateParticlePositions(self, timeDelta: float):
        self.sim.stage("positions", timeDelta)

    def step(self, timeDelta: float, nsteps: int = 1):
        self.sim.step(timeDelta, nsteps)
