"""ctypes front end for the CPU oracles.  TEST INFRASTRUCTURE ONLY.

Two oracles live here; the product path never imports this module.

* ``OracleSim`` wraps ``mpm_oracle.c`` (the C restatement of the reference's
  step, FP32 or FP64), built by ``build_oracle()`` into ``oracle/_build``.
* ``RefSim`` wraps ``oracle/_ref/librd_ref.so``: the reference's own
  ``LagrangeEulerView`` compiled headless from its sources by
  ``oracle/ref/build_ref.sh``.  It exists only where the reference sources were
  available at build time on this machine's architecture.

Both use the reference's state: positions, velocities, APIC ``B`` (the kernels
carry ``C = B * DpInverse``), full ``F_E`` and ``F_P`` (row-major 3x3), mass and
volume; grids are dense ``MAX_I*MAX_J*MAX_K`` in the reference's index order.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF_SO = os.path.join(HERE, "_ref", "librd_ref.so")


def build_oracle(force: bool = False) -> None:
    """Compile the FP32 and FP64 restatements (gcc, no FMA contraction so the
    FP32 oracle rounds like the reference's x86-64 build on any host)."""
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(HERE, "mpm_oracle.c")
    for real in ("float", "double"):
        out = os.path.join(BUILD, f"liborc_{real}.so")
        if not force and os.path.exists(out) and os.path.getmtime(out) >= os.path.getmtime(src):
            continue
        subprocess.check_call(["gcc", "-O2", "-fPIC", "-shared", "-std=c11", "-ffp-contract=off",
                               f"-DORC_REAL={real}", src, "-o", out + ".tmp", "-lm"])
        os.replace(out + ".tmp", out)


# Copy of the reference sources the headless build needs (oracle/ref/stage_tree.sh),
# for machines without a checkout of the reference; git-ignored.
TREE = os.path.join(HERE, "_ref", "tree")


def _holds_sources(root) -> bool:
    return bool(root) and os.path.isfile(os.path.join(root, "realtime-deformations", "material_point_method.cpp"))


def reference_root():
    """The directory holding the reference's ``realtime-deformations/`` sources:
    ``$RD_REFERENCE_ROOT`` when set, else ``$RD_REFERENCE_DEFAULT`` as this
    repository's build recipe exports it for its own checkout, else the staged
    copy ``oracle/_ref/tree``; None when none holds them."""
    for root in (os.environ.get("RD_REFERENCE_ROOT"), os.environ.get("RD_REFERENCE_DEFAULT"), TREE):
        if _holds_sources(root):
            return root
    return None


def start_ref_build(root=None):
    """Starts building the headless reference from the sources under ``root``
    (default ``reference_root()``) in the background and returns the process,
    or None when no sources are found.  Building from a checkout first stages
    the copy ``oracle/_ref/tree`` that another machine builds from."""
    root = root or reference_root()
    if not _holds_sources(root):
        return None
    if os.path.realpath(root) != os.path.realpath(TREE):
        subprocess.check_call(["bash", os.path.join(HERE, "ref", "stage_tree.sh"), root],
                              stdout=subprocess.DEVNULL)
    return subprocess.Popen(["bash", os.path.join(HERE, "ref", "build_ref.sh"), root])


def build_ref(root=None) -> bool:
    """Build the headless reference from the sources under ``root`` (default
    ``reference_root()``) if they are present.  Returns whether
    ``librd_ref.so`` is usable afterwards."""
    proc = start_ref_build(root)
    if proc is not None and proc.wait() != 0:
        raise subprocess.CalledProcessError(proc.returncode, "build_ref.sh")
    return ref_available()


def ref_available() -> bool:
    if not os.path.exists(REF_SO):
        return False
    try:
        ctypes.CDLL(REF_SO)
    except OSError:  # e.g. built for another architecture
        return False
    return True


def reference_dinv(h: float) -> np.float32:
    """DpInverse[0][0] as the reference computes it: glm::inverse of
    mat3(1) * (1/3f) * h * h in FP32 (material_point_method.hpp:177,
    glm type_mat3x3.inl compute_inverse)."""
    f = np.float32
    d = f(f(f(1.0) * f(1.0 / 3.0)) * f(h)) * f(h)
    dd = f(d * d)
    one_over_det = f(f(1.0) / f(d * dd))
    return f(dd * one_over_det)


@dataclass
class Params:
    mi: int
    mj: int
    mk: int
    h: float
    E: float = 1.4e5
    nu: float = 0.2
    xi: float = 10.0
    theta_c: float = 2.5e-2
    theta_s: float = 5.0e-3
    gravity: tuple = (0.0, -9.8, 0.0)
    bc: int = 0
    bc_width: int = 3
    lagged_c: int = 1


class _CParams(ctypes.Structure):
    _fields_ = [("mi", ctypes.c_int), ("mj", ctypes.c_int), ("mk", ctypes.c_int),
                ("h", ctypes.c_double), ("dinv", ctypes.c_double),
                ("E", ctypes.c_double), ("nu", ctypes.c_double), ("xi", ctypes.c_double),
                ("theta_c", ctypes.c_double), ("theta_s", ctypes.c_double),
                ("gravity", ctypes.c_double * 3),
                ("bc", ctypes.c_int), ("bc_width", ctypes.c_int), ("lagged_c", ctypes.c_int)]


class _CState(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int)] + [(k, ctypes.c_void_p) for k in ("x", "v", "B", "FE", "FP", "mass", "vol")]


class _CGrid(ctypes.Structure):
    _fields_ = [(k, ctypes.c_void_p) for k in ("mass", "vel", "force")]


_LIBS: dict = {}


def _lib(dtype):
    key = np.dtype(dtype).name
    if key not in _LIBS:
        build_oracle()
        real = "float" if key == "float32" else "double"
        lib = ctypes.CDLL(os.path.join(BUILD, f"liborc_{real}.so"))
        P, S, G = ctypes.POINTER(_CParams), ctypes.POINTER(_CState), ctypes.POINTER(_CGrid)
        rt = ctypes.c_float if real == "float" else ctypes.c_double
        lib.orc_rasterize.argtypes = [P, S, G]
        lib.orc_volumes.argtypes = [P, S, G]
        lib.orc_forces.argtypes = [P, S, G]
        lib.orc_grid_velocities.argtypes = [P, rt, G]
        lib.orc_update_F.argtypes = [P, rt, S]
        lib.orc_g2p.argtypes = [P, S, G]
        lib.orc_advect.argtypes = [P, rt, S]
        lib.orc_init.argtypes = [P, S, G]
        lib.orc_step.argtypes = [P, rt, ctypes.c_int, S, G]
        lib.orc_svd3.argtypes = [ctypes.c_void_p] * 4
        lib.orc_set_colliders.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_double]
        lib.orc_move_colliders.argtypes = [ctypes.c_double]
        lib.orc_collisions.argtypes = [P, G]
        lib.orc_weight.argtypes = [rt]
        lib.orc_weight.restype = rt
        lib.orc_implicit_energy.argtypes = [P, S, G, rt, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                            ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
        lib.orc_implicit_energy.restype = ctypes.c_double
        _LIBS[key] = lib
    return _LIBS[key]


class OracleSim:
    """The C restatement, FP32 (``dtype=np.float32``) or FP64."""

    def __init__(self, params: Params, x, v, mass, B=None, FE=None, FP=None, vol=None,
                 dtype=np.float32):
        self.p = params
        self.dtype = np.dtype(dtype)
        self.lib = _lib(self.dtype)
        n = len(mass)
        dt_ = self.dtype

        def arr(a, shape, fill=None):
            if a is None:
                out = np.zeros(shape, dt_)
                if fill is not None:
                    out[:] = fill
                return out
            return np.array(a, dtype=dt_, copy=True).reshape(shape)  # never alias the caller's arrays

        eye = np.eye(3, dtype=dt_).reshape(9)
        self.x = arr(x, (n, 3))
        self.v = arr(v, (n, 3))
        self.B = arr(B, (n, 9))
        self.FE = arr(FE, (n, 9), eye)
        self.FP = arr(FP, (n, 9), eye)
        self.mass = arr(mass, (n,))
        self.vol = arr(vol, (n,))
        nc = params.mi * params.mj * params.mk
        self.gmass = np.zeros(nc, dt_)
        self.gvel = np.zeros((nc, 3), dt_)
        self.gforce = np.zeros((nc, 3), dt_)
        self._cp = _CParams(params.mi, params.mj, params.mk, float(params.h),
                            float(reference_dinv(params.h)) if self.dtype == np.float32 else 3.0 / params.h ** 2,
                            params.E, params.nu, params.xi, params.theta_c, params.theta_s,
                            (ctypes.c_double * 3)(*params.gravity), params.bc, params.bc_width, params.lagged_c)
        self._cs = _CState(n, *(a.ctypes.data for a in (self.x, self.v, self.B, self.FE, self.FP, self.mass, self.vol)))
        self._cg = _CGrid(self.gmass.ctypes.data, self.gvel.ctypes.data, self.gforce.ctypes.data)

    @property
    def dinv(self) -> float:
        return self._cp.dinv

    def init(self):
        self.lib.orc_init(ctypes.byref(self._cp), ctypes.byref(self._cs), ctypes.byref(self._cg))

    def stage(self, name: str, dt: float = 0.0):
        cp, cs, cg = ctypes.byref(self._cp), ctypes.byref(self._cs), ctypes.byref(self._cg)
        L = self.lib
        {"rasterize": lambda: L.orc_rasterize(cp, cs, cg),
         "volumes": lambda: L.orc_volumes(cp, cs, cg),
         "forces": lambda: L.orc_forces(cp, cs, cg),
         "grid_velocities": lambda: L.orc_grid_velocities(cp, dt, cg),
         "collisions": lambda: L.orc_collisions(cp, cg),
         "update_F": lambda: L.orc_update_F(cp, dt, cs),
         "g2p": lambda: L.orc_g2p(cp, cs, cg),
         "advect": lambda: L.orc_advect(cp, dt, cs)}[name]()

    def step(self, dt: float, nsteps: int = 1):
        self.lib.orc_step(ctypes.byref(self._cp), dt, nsteps, ctypes.byref(self._cs), ctypes.byref(self._cg))

    def set_colliders(self, colliders, mode: int = 0, mu: float = 0.5):
        """Box colliders (orc_set_colliders; one set per oracle library, shared
        by every OracleSim of this precision)."""
        spec = collider_spec(colliders)
        self.lib.orc_set_colliders(len(colliders), spec.ctypes.data if len(colliders) else None, mode, mu)
        self._spec = spec

    def move_colliders(self, dt: float):
        self.lib.orc_move_colliders(dt)

    def implicit_energy(self, vel, dt: float, mu0: float = 1.0, lambda0: float = 1.0, xi: float = 10.0,
                        hardening: int = 0, grad: bool = False):
        """The implicit integration's energy (orc_implicit_energy) at the dense
        grid velocities vel (cells x 3) against the current grid (masses and
        v*), and its gradient (cells x 3) when grad is set."""
        v = np.ascontiguousarray(np.asarray(vel, self.dtype).reshape(-1, 3))
        g = np.zeros_like(v) if grad else None
        e = self.lib.orc_implicit_energy(ctypes.byref(self._cp), ctypes.byref(self._cs), ctypes.byref(self._cg), dt,
                                         mu0, lambda0, xi, hardening, v.ctypes.data,
                                         g.ctypes.data if grad else None)
        return (e, g) if grad else e

    @property
    def C(self):
        return self.B * self.dtype.type(self.dinv)

    @property
    def Jp(self):
        return np.linalg.det(self.FP.reshape(-1, 3, 3).astype(np.float64))


def implicit_lbfgs(fg, x0, max_iters=50, history=8, grad_tol=1e-2, step_tol=1e-2, ls_max_iters=200):
    """The L-BFGS of rd_time_integration restated in numpy (FP64), for the
    parity test of the device solver: Nocedal & Wright 7.2 with the two-loop
    recursion scaled by s.y / y.y, a backtracking Armijo line search (factor
    0.7, constant 1e-4) from a unit step, and steepest descent with a step of
    min(1, 1 / |g|_inf) whenever the direction does not descend - as the
    reference's vendored minimiser (external/mcloptlib LBFGS.hpp,
    Backtracking.hpp) is configured by mathy.hpp:10-36.  fg(x) -> (E, grad).
    Returns (x, E, iterations, converged) with converged 1 (a tolerance),
    0 (max_iters) or -1 (line search failed)."""
    x = np.array(x0, np.float64)
    fx, g = fg(x)
    pairs = []
    gamma, alpha_init = 1.0, 1.0
    converged, k = 0, 0
    while k < max_iters:
        x_old, g_old = x.copy(), g.copy()
        q = g.copy()
        alphas = []
        for s, y in reversed(pairs):
            rho = 1.0 / np.dot(y, s)
            a = rho * np.dot(q, s)
            alphas.append((rho, a))
            q -= a * y
        q *= gamma
        for (s, y), (rho, a) in zip(pairs, reversed(alphas)):
            beta = rho * np.dot(q, y)
            q += (a - beta) * s
        direction = np.dot(g, q)
        if not direction > 0.0:
            q = g.copy()
            pairs = []
            gmax = np.max(np.abs(g))
            alpha_init = min(1.0, 1.0 / gmax) if gmax > 0 else 1.0
            direction = np.dot(g, q)
        a, ls = alpha_init, 0
        while ls < ls_max_iters:
            fa, _ = fg(x - a * q)
            if fa <= fx - 1e-4 * a * direction:
                break
            a *= 0.7
            ls += 1
        if ls >= ls_max_iters:
            converged = -1
            break
        x = x - a * q
        step = a * np.linalg.norm(q)
        if np.linalg.norm(g) < grad_tol or step < step_tol:
            converged = 1
            fx = fa
            k += 1
            break
        fx, g = fg(x)
        s, y = x - x_old, g - g_old
        pairs.append((s, y))
        if len(pairs) > history:
            pairs.pop(0)
        yy = np.dot(y, y)
        if not abs(yy) > 0.0:
            k += 1
            break
        gamma = np.dot(s, y) / yy
        alpha_init = 1.0
        k += 1
    fx, g = fg(x)
    return x, fx, k, converged


def collider_spec(colliders) -> np.ndarray:
    """Flat float64 array, 13 per collider: translation (3), rotation as a
    unit quaternion (w, x, y, z), scale (half extents, 3), velocity (3)."""
    rows = [list(c["translation"]) + list(c["rotation"]) + list(c["scale"]) + list(c.get("velocity", (0, 0, 0)))
            for c in colliders]
    return np.ascontiguousarray(np.asarray(rows, np.float64).reshape(-1))


def svd3(F: np.ndarray):
    """The oracle's FP64 SVD of one 3x3 matrix: returns W, s, Z."""
    lib = _lib(np.float32)
    F = np.ascontiguousarray(F, np.float64).reshape(9)
    W, s, Z = np.zeros(9), np.zeros(3), np.zeros(9)
    lib.orc_svd3(F.ctypes.data, W.ctypes.data, s.ctypes.data, Z.ctypes.data)
    return W.reshape(3, 3), s, Z.reshape(3, 3)


class RefSim:
    """The reference's own LagrangeEulerView, built headless (FP32 only)."""

    _lib = None

    @classmethod
    def lib(cls):
        if cls._lib is None:
            L = ctypes.CDLL(REF_SO)
            vp, fp = ctypes.c_void_p, ctypes.POINTER(ctypes.c_float)
            L.rdref_create.restype = vp
            L.rdref_create.argtypes = [ctypes.c_int] * 4 + [ctypes.c_float]
            L.rdref_destroy.argtypes = [vp]
            L.rdref_dp_inverse.restype = ctypes.c_float
            L.rdref_dp_inverse.argtypes = [vp]
            L.rdref_set_params.argtypes = [ctypes.c_float] * 4 + [ctypes.c_double] * 2 + [ctypes.c_int]
            L.rdref_set_particles.argtypes = [vp] + [ctypes.c_void_p] * 7
            L.rdref_get_particles.argtypes = [vp] + [ctypes.c_void_p] * 6
            L.rdref_get_grid.argtypes = [vp] + [ctypes.c_void_p] * 3
            L.rdref_stage.argtypes = [vp, ctypes.c_int, ctypes.c_float]
            L.rdref_init.argtypes = [vp]
            L.rdref_step.argtypes = [vp, ctypes.c_float, ctypes.c_int]
            L.rdref_get_mass.argtypes = [vp, ctypes.c_void_p]
            L.rdref_initialize_particles.argtypes = [vp, ctypes.c_uint] + [ctypes.c_float] * 6
            L.rdref_set_colliders.argtypes = [ctypes.c_int, ctypes.c_void_p]
            L.rdref_move_colliders.argtypes = [ctypes.c_float]
            L.rdref_energy.argtypes = [vp, ctypes.c_void_p, ctypes.c_float]
            L.rdref_energy.restype = ctypes.c_float
            L.rdref_time_integration.argtypes = [vp, ctypes.c_float]
            cls._lib = L
        return cls._lib

    STAGES = {"rasterize": 0, "forces": 1, "grid_velocities": 2, "collisions": 3,
              "update_F": 4, "g2p": 5, "advect": 6, "volumes": 7}

    def __init__(self, params: Params, x=None, v=None, mass=None, B=None, FE=None, FP=None, vol=None, p4: int = 1,
                 n: int | None = None):
        if params.bc != 0 or params.lagged_c != 1 or tuple(params.gravity[::2]) != (0.0, 0.0):
            raise ValueError("the reference has no walls, lagged-B order only and gravity along y")
        L = self.lib()
        self.p = params
        self.n = len(mass) if mass is not None else int(n)
        L.rdref_set_params(params.E, params.nu, params.xi, params.gravity[1], params.theta_c, params.theta_s, p4)
        self.h = L.rdref_create(params.mi, params.mj, params.mk, self.n, params.h)
        if mass is not None:
            f32 = lambda a, s: None if a is None else np.ascontiguousarray(np.asarray(a, np.float32).reshape(s))
            ins = [f32(x, (self.n, 3)), f32(v, (self.n, 3)), f32(mass, (self.n,)), f32(B, (self.n, 9)),
                   f32(FE, (self.n, 9)), f32(FP, (self.n, 9)), f32(vol, (self.n,))]
            L.rdref_set_particles(self.h, *[None if a is None else a.ctypes.data for a in ins])
        self.p4 = p4

    def set_colliders(self, colliders):
        """The reference's own MeshColliders for the collision stage (one list
        per process, shared by every RefSim)."""
        spec = collider_spec(colliders)
        self.lib().rdref_set_colliders(len(colliders), spec.ctypes.data if len(colliders) else None)

    def move_colliders(self, dt: float):
        self.lib().rdref_move_colliders(dt)

    def initialize_particles(self, origin, velocity, seed: int = 1):
        """The reference's initializeParticles (material_point_method.cpp:18-63)."""
        self.lib().rdref_initialize_particles(self.h, seed, *origin, *velocity)

    def __del__(self):
        if getattr(self, "h", None):
            self.lib().rdref_destroy(self.h)
            self.h = None

    @property
    def dinv(self) -> float:
        return self.lib().rdref_dp_inverse(self.h)

    def _params(self):
        p = self.p
        self.lib().rdref_set_params(p.E, p.nu, p.xi, p.gravity[1], p.theta_c, p.theta_s, self.p4)

    def init(self):
        self._params()
        self.lib().rdref_init(self.h)

    def stage(self, name: str, dt: float = 0.0):
        self._params()
        self.lib().rdref_stage(self.h, self.STAGES[name], dt)

    def step(self, dt: float, nsteps: int = 1):
        self._params()
        self.lib().rdref_step(self.h, dt, nsteps)

    def particles(self):
        n = self.n
        out = {k: np.zeros(s, np.float32) for k, s in
               (("x", (n, 3)), ("v", (n, 3)), ("B", (n, 9)), ("FE", (n, 9)), ("FP", (n, 9)), ("vol", (n,)))}
        self.lib().rdref_get_particles(self.h, *(out[k].ctypes.data for k in ("x", "v", "B", "FE", "FP", "vol")))
        return out

    def masses(self):
        """Particle masses (the harness reads them through rdref_get_mass)."""
        m = np.zeros(self.n, np.float32)
        self.lib().rdref_get_mass(self.h, m.ctypes.data)
        return m

    def energy(self, vel, dt: float) -> float:
        """The reference's implicit Energy at the dense grid velocities vel."""
        v = np.ascontiguousarray(np.asarray(vel, np.float32).reshape(-1, 3))
        return float(self.lib().rdref_energy(self.h, v.ctypes.data, dt))

    def time_integration(self, dt: float):
        """The reference's timeIntegration: its LBFGS minimiser of Energy
        written to the grid velocities."""
        self.lib().rdref_time_integration(self.h, dt)

    def grid(self):
        nc = self.p.mi * self.p.mj * self.p.mk
        m, v, f = np.zeros(nc, np.float32), np.zeros((nc, 3), np.float32), np.zeros((nc, 3), np.float32)
        self.lib().rdref_get_grid(self.h, m.ctypes.data, v.ctypes.data, f.ctypes.data)
        return {"mass": m, "vel": v, "force": f}


def splat_image(xyzs, rgba, vp, right, up, width, height, background, max_radius=32):
    """Restatement of rd_splat (test infrastructure): float32 numpy version of
    project / splat_radius / the (depth, id) minimum / sphere shading.  xyzs:
    n x 4 (x, y, z, size), rgba: n uint32, vp: 16 column-major.  Returns the
    (h, w) uint32 image and the (h, w) id map (-1 where empty)."""
    f = np.float32
    xyzs = np.asarray(xyzs, f)
    M = np.asarray(vp, f).reshape(4, 4).T  # row-major clip = M @ (x, y, z, 1)
    right, up = np.asarray(right, f), np.asarray(up, f)

    def project(p):
        c = p @ M[:, :3].T + M[:, 3]
        iw = f(1) / c[:, 3]
        px = (c[:, 0] * iw * f(0.5) + f(0.5)) * f(width)
        py = (f(0.5) - c[:, 1] * iw * f(0.5)) * f(height)
        depth = c[:, 2] * iw * f(0.5) + f(0.5)
        return px, py, depth, c[:, 3]

    pos, size = xyzs[:, :3], xyzs[:, 3:4]
    px, py, depth, w = project(pos)
    ax, ay, _, _ = project(pos + right * size * f(0.5))
    bx, by, _, _ = project(pos + up * size * f(0.5))
    r = np.maximum(np.sqrt((ax - px) ** 2 + (ay - py) ** 2), np.sqrt((bx - px) ** 2 + (by - py) ** 2))
    r = np.minimum(r, f(max_radius))
    key = np.full(width * height, np.iinfo(np.uint64).max, np.uint64)
    ok = (w > 0) & (depth >= 0) & (depth <= 1) & (r > 0)
    dbits = depth.view(np.uint32).astype(np.uint64)
    for i in np.nonzero(ok)[0]:
        x0, x1 = max(0, int(np.floor(px[i] - r[i]))), min(width - 1, int(np.floor(px[i] + r[i])))
        y0, y1 = max(0, int(np.floor(py[i] - r[i]))), min(height - 1, int(np.floor(py[i] + r[i])))
        if x1 < x0 or y1 < y0:
            continue
        ys, xs = np.mgrid[y0:y1 + 1, x0:x1 + 1]
        dx, dy = xs.astype(f) + f(0.5) - px[i], ys.astype(f) + f(0.5) - py[i]
        m = dx * dx + dy * dy <= r[i] * r[i]
        lin = (ys * width + xs)[m]
        np.minimum.at(key, lin, (dbits[i] << np.uint64(32)) | np.uint64(i))
    empty = key == np.iinfo(np.uint64).max
    ids = np.where(empty, -1, (key & np.uint64(0xffffffff)).astype(np.int64))
    img = np.full(width * height, background, np.uint32)
    pix = np.nonzero(~empty)[0]
    pid = ids[pix]
    xs, ys = (pix % width).astype(f), (pix // width).astype(f)
    dx, dy = xs + f(0.5) - px[pid], ys + f(0.5) - py[pid]
    rr = r[pid]
    q = np.where(rr > 0, np.minimum(f(1), (dx * dx + dy * dy) / (rr * rr)), f(1))
    shade = f(0.35) + f(0.65) * np.sqrt(f(1) - q)
    c = np.asarray(rgba, np.uint32)[pid]
    chan = [np.minimum(f(255), ((c >> s) & 0xff).astype(f) * shade + f(0.5)).astype(np.uint32) for s in (0, 8, 16)]
    img[pix] = chan[0] | (chan[1] << 8) | (chan[2] << 16) | np.uint32(0xff000000)
    return img.reshape(height, width), ids.reshape(height, width)
