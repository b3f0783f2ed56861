"""torch.autograd front end of the reverse-mode rollout (rd_adjoint_record /
rd_adjoint_backward).  It only moves tensors across the C ABI: the forward
rollout and every gradient come from the CUDA kernels.

    spec = RolloutSpec(grid=(64,)*3, h=1/64, x0=x, mass=m, dt=1e-4, steps=50, every=10)
    xT = rollout(v0, E, nu, spec)            # v0 [N,3], E and nu 0-d tensors
    loss = ((xT.mean(0) - target) ** 2).sum()
    loss.backward()                           # v0.grad, E.grad, nu.grad

``batch_rollout`` does the same for a list of scenes stepped in one batch
handle, with per-scene E, theta_c and theta_s tensors.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np
import torch

from . import RD_FP32, RD_FP64, Batch, Simulation, make_params


@dataclass
class RolloutSpec:
    grid: tuple
    h: float
    x0: np.ndarray
    mass: np.ndarray
    dt: float
    steps: int
    every: int = 10
    material: dict = field(default_factory=dict)  # xi, theta_c, theta_s, gravity (E, nu come as tensors)
    bc: int = 1
    bc_width: int = 3
    precision: int = RD_FP32
    FE0: np.ndarray | None = None
    device: int = 0

    @property
    def dtype(self):
        return np.float64 if self.precision == RD_FP64 else np.float32


def _params(spec: RolloutSpec, **over):
    kw = dict(spec.material)
    kw.update(over)
    return make_params(*spec.grid, len(spec.mass), spec.h, bc=spec.bc, bc_width=spec.bc_width,
                       precision=spec.precision, device=spec.device, **kw)


class MPMRollout(torch.autograd.Function):
    @staticmethod
    def forward(ctx, v0, E, nu, spec: RolloutSpec):
        sim = Simulation(_params(spec, E=float(E), nu=float(nu)))
        sim.set_particles(spec.x0, v0.detach().cpu().numpy().astype(spec.dtype), spec.mass, FE=spec.FE0)
        sim.init_volumes()
        sim.adjoint_record(spec.dt, spec.steps, spec.every)
        xT = sim.get_particles(("x",))["x"]
        ctx.sim = sim
        ctx.meta = (v0.dtype, v0.device, E.dtype, nu.dtype)
        return torch.from_numpy(xT).to(device=v0.device, dtype=v0.dtype)

    @staticmethod
    def backward(ctx, gx):
        vdt, dev, edt, ndt = ctx.meta
        g = ctx.sim.adjoint_backward(gx.detach().cpu().numpy().astype(ctx.sim.dtype))
        ctx.sim.close()
        return (torch.from_numpy(g["v0"]).to(device=dev, dtype=vdt), torch.tensor(g["E"][0], dtype=edt),
                torch.tensor(g["nu"][0], dtype=ndt), None)


def rollout(v0: torch.Tensor, E: torch.Tensor, nu: torch.Tensor, spec: RolloutSpec) -> torch.Tensor:
    """Final positions [N, 3] of `spec.steps` steps from (x0, v0) with Young's
    modulus E and Poisson ratio nu; differentiable in v0, E and nu."""
    return MPMRollout.apply(v0, E, nu, spec)


class MPMBatchRollout(torch.autograd.Function):
    @staticmethod
    def forward(ctx, E, theta_c, theta_s, specs):
        ps = [_params(s, E=float(E[i]), theta_c=float(theta_c[i]), theta_s=float(theta_s[i]))
              for i, s in enumerate(specs)]
        b = Batch(ps)
        for i, s in enumerate(specs):
            b.set_particles(i, s.x0, np.zeros((len(s.mass), 3), s.dtype) if s.v0 is None else s.v0, s.mass, FE=s.FE0)
        b.init_volumes()
        b.adjoint_record(specs[0].dt, specs[0].steps, specs[0].every)
        xs = [torch.from_numpy(b.get_particles(i, ("x",))["x"]) for i in range(len(specs))]
        ctx.b = b
        ctx.counts = [len(s.mass) for s in specs]
        return torch.cat(xs).to(dtype=E.dtype)

    @staticmethod
    def backward(ctx, gx):
        g = ctx.b.adjoint_backward(gx.detach().cpu().numpy().astype(ctx.b.dtype))
        ctx.b.close()
        t = lambda k: torch.from_numpy(g[k]).to(dtype=gx.dtype)  # noqa: E731
        return t("E"), t("theta_c"), t("theta_s"), None


@dataclass
class BatchSceneSpec(RolloutSpec):
    v0: np.ndarray | None = None


def batch_rollout(E: torch.Tensor, theta_c: torch.Tensor, theta_s: torch.Tensor, specs) -> torch.Tensor:
    """Final positions of every scene (concatenated in scene order) of a batch
    rollout; differentiable in the per-scene E, theta_c and theta_s."""
    return MPMBatchRollout.apply(E, theta_c, theta_s, list(specs))
