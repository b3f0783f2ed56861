"""Seeded synthetic scenes for the benchmark and the parity tests.

The reference ships no dataset; its own scene (initializeParticles,
realtime-deformations/material_point_method.cpp:18-63) is a jittered
8-particles-per-cell sphere.  The scenes here are the workloads the step is
measured on, generated from a seed with numpy's PCG64 so every run sees the
same particles:

* ``snowball``      8,192 particles uniform in a sphere r = 0.1 at
                    (0.5, 0.6, 0.5), 64^3 grid, dx = 1/64, v0 = (0, -2, 0),
                    rho = 400, E = 1.4e5, nu = 0.2, theta = (2.5e-2, 7.5e-3),
                    xi = 10, dt = 1e-4, sticky walls of 3 cells, 200 steps.
* ``two_balls``     two spheres r = 0.15 at (0.3, 0.5, 0.5) and
                    (0.7, 0.55, 0.5), v0 = +-(3, 0, 0), 8 particles per cell
                    jittered on a 128^3 grid (about 4.7e5 particles), same
                    material, dt and walls, 500 steps.
* ``two_balls_1m``  the same two spheres holding 1.1M particles (uniform,
                    about 18.6 per cell), the particle count the two-ball
                    workload is quoted at.
* ``cube``          65,536 particles uniform in a 0.2-side cube at
                    (0.5, 0.6, 0.5), 64^3 grid, 50 steps.

Batches (lists of scenes stepped together):

* ``uneven_snowballs``  64 snowballs, each with a log-uniform 4,096-262,144
                    particles on a 32^3-128^3 grid (drawn from the seed), per
                    scene E ~ U[5e4, 3e5], nu ~ U[0.15, 0.3], v0 ~ N(0, 1)^3,
                    300 steps.  The radius is set by the particle count at 8
                    particles per cell, r = (3 N / (32 pi))^(1/3) cells, and a
                    grid drawn too small for the ball is raised to
                    2 r + 24 cells.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np


@dataclass
class Scene:
    name: str
    grid: tuple
    h: float
    x: np.ndarray
    v: np.ndarray
    mass: np.ndarray
    dt: float
    steps: int
    material: dict = field(default_factory=dict)
    bc: int = 1
    bc_width: int = 3

    @property
    def n(self) -> int:
        return len(self.mass)

    def params(self, **over):
        """Keyword arguments for ``make_params``."""
        kw = dict(self.material)
        kw.update(bc=self.bc, bc_width=self.bc_width)
        kw.update(over)
        return kw


SNOW = dict(E=1.4e5, nu=0.2, xi=10.0, theta_c=2.5e-2, theta_s=7.5e-3, gravity=(0.0, -9.8, 0.0))


def uniform_ball(rng, n, center, r):
    out = np.empty((0, 3))
    while len(out) < n:
        p = rng.uniform(-r, r, size=(2 * n, 3))
        p = p[np.einsum("ij,ij->i", p, p) <= r * r]
        out = np.concatenate([out, p])
    return out[:n] + np.asarray(center)


def jittered_ball(rng, center, r, h, ppc_side=2):
    """Particles at the ppc_side^3 sub-cell centres of every cell, each jittered
    uniformly within its sub-cell, kept where inside the sphere."""
    c = np.asarray(center, np.float64)
    lo = np.floor((c - r) / h).astype(int)
    hi = np.ceil((c + r) / h).astype(int)
    ii, jj, kk = np.meshgrid(*[np.arange(lo[a], hi[a]) for a in range(3)], indexing="ij")
    cells = np.stack([ii.ravel(), jj.ravel(), kk.ravel()], 1).astype(np.float64)
    s = (np.arange(ppc_side) + 0.5) / ppc_side
    sub = np.stack(np.meshgrid(s, s, s, indexing="ij"), -1).reshape(-1, 3)
    pts = (cells[:, None, :] + sub[None, :, :]).reshape(-1, 3)
    pts += rng.uniform(-0.5 / ppc_side, 0.5 / ppc_side, size=pts.shape)
    pts *= h
    d = pts - c
    return pts[np.einsum("ij,ij->i", d, d) <= r * r]


def snowball(seed: int = 0, n: int = 8192, grid: int = 64, steps: int = 200) -> Scene:
    rng = np.random.default_rng(seed)
    r, rho = 0.1, 400.0
    x = uniform_ball(rng, n, (0.5, 0.6, 0.5), r)
    v = np.tile([0.0, -2.0, 0.0], (n, 1))
    m = np.full(n, rho * 4.0 / 3.0 * np.pi * r ** 3 / n)
    return Scene("snowball", (grid,) * 3, 1.0 / grid, x.astype(np.float32), v.astype(np.float32),
                 m.astype(np.float32), 1e-4, steps, dict(SNOW))


def _two_ball_state(xa, xb, rho, r):
    x = np.concatenate([xa, xb])
    v = np.concatenate([np.tile([3.0, 0.0, 0.0], (len(xa), 1)), np.tile([-3.0, 0.0, 0.0], (len(xb), 1))])
    vol = 4.0 / 3.0 * np.pi * r ** 3
    m = np.concatenate([np.full(len(xa), rho * vol / len(xa)), np.full(len(xb), rho * vol / len(xb))])
    return x, v, m


def two_balls(seed: int = 0, grid: int = 128, steps: int = 500) -> Scene:
    rng = np.random.default_rng(seed)
    h, r = 1.0 / grid, 0.15
    xa = jittered_ball(rng, (0.3, 0.5, 0.5), r, h)
    xb = jittered_ball(rng, (0.7, 0.55, 0.5), r, h)
    x, v, m = _two_ball_state(xa, xb, 400.0, r)
    return Scene("two_balls", (grid,) * 3, h, x.astype(np.float32), v.astype(np.float32),
                 m.astype(np.float32), 1e-4, steps, dict(SNOW))


def two_balls_1m(seed: int = 0, n: int = 1_100_000, grid: int = 128, steps: int = 500) -> Scene:
    rng = np.random.default_rng(seed)
    r = 0.15
    xa = uniform_ball(rng, n // 2, (0.3, 0.5, 0.5), r)
    xb = uniform_ball(rng, n - n // 2, (0.7, 0.55, 0.5), r)
    x, v, m = _two_ball_state(xa, xb, 400.0, r)
    return Scene("two_balls_1m", (grid,) * 3, 1.0 / grid, x.astype(np.float32), v.astype(np.float32),
                 m.astype(np.float32), 1e-4, steps, dict(SNOW))


def cube(seed: int = 0, n: int = 65536, grid: int = 64, steps: int = 50) -> Scene:
    rng = np.random.default_rng(seed)
    side, rho = 0.2, 400.0
    x = rng.uniform(-side / 2, side / 2, size=(n, 3)) + np.array([0.5, 0.6, 0.5])
    v = np.zeros((n, 3))
    m = np.full(n, rho * side ** 3 / n)
    return Scene("cube", (grid,) * 3, 1.0 / grid, x.astype(np.float32), v.astype(np.float32),
                 m.astype(np.float32), 1e-4, steps, dict(SNOW))


def perturbed_state(rng, n, scale_B=1.0, scale_F=1e-3, dinv=1.0):
    """Non-trivial APIC B and near-identity F_E / F_P for parity cases that
    exercise the affine transfer, the stress and the plastic SVD."""
    B = rng.normal(0.0, scale_B, size=(n, 9)) / dinv
    FE = np.eye(3).reshape(1, 9) + rng.normal(0.0, scale_F, size=(n, 9))
    FP = np.eye(3).reshape(1, 9) + rng.normal(0.0, scale_F, size=(n, 9))
    return B.astype(np.float32), FE.astype(np.float32), FP.astype(np.float32)


def uneven_snowballs(seed: int = 0, nscenes: int = 64, n_lo: int = 4096, n_hi: int = 262144, g_lo: int = 32,
                     g_hi: int = 128, steps: int = 300, ppc: float = 8.0) -> list:
    rng = np.random.default_rng(seed)
    out = []
    for s in range(nscenes):
        n = int(round(np.exp(rng.uniform(np.log(n_lo), np.log(n_hi)))))
        g = int(rng.integers(g_lo, g_hi + 1))
        r_cells = (3.0 * n / (4.0 * np.pi * ppc)) ** (1.0 / 3.0)
        g = max(g, int(np.ceil(2.0 * r_cells + 24.0)))
        h = 1.0 / g
        r = r_cells * h
        mat = dict(SNOW, E=float(rng.uniform(5e4, 3e5)), nu=float(rng.uniform(0.15, 0.3)))
        v0 = rng.normal(0.0, 1.0, size=3)
        x = uniform_ball(rng, n, (0.5, 0.55, 0.5), r)
        v = np.tile(v0, (n, 1))
        m = np.full(n, 400.0 * 4.0 / 3.0 * np.pi * r ** 3 / n)
        out.append(Scene(f"uneven_snowballs[{s}]", (g,) * 3, h, x.astype(np.float32), v.astype(np.float32),
                         m.astype(np.float32), 1e-4, steps, mat))
    return out


BATCHES = {"uneven_snowballs": uneven_snowballs}

SCENES = {"snowball": snowball, "two_balls": two_balls, "two_balls_1m": two_balls_1m, "cube": cube}
