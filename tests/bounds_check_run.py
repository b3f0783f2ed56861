"""Workloads for the bounds-checked build of the library (test infrastructure).

Run with RD_BOUNDS_CHECK=1 in the environment, so that the package loads
librd_mpm_checked.so (compiled with -DRD_BOUNDS_CHECK): the fused step, the
P2G, batches, stage mode, the sorted upload and the adjoint run over the edge
cases the other tests use (particles outside the domain, on the clamp planes,
moving several cells a step, grids of partial 4x4x4 blocks, FP64 with the full
F_P), and one step is compared with the oracle.  Prints one JSON line: the
accesses out of range the checked sites skipped (rd_debug_bounds_violations),
each workload's device flags and the oracle comparison."""
import json
import os
import sys

import numpy as np

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, REPO)
import __graft_entry__ as graft  # noqa: E402

pkg = graft.load_package()
assert pkg.CHECKED, "run with RD_BOUNDS_CHECK=1"
pkg.build()
orc = graft.load_oracle()
orc.build_oracle()
from rd_gb300 import scenes  # noqa: E402

out = {"flags": {}}


def sim_of(sc, **over):
    return pkg.Simulation(pkg.make_params(*sc.grid, sc.n, sc.h, **sc.params(**over)))


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


# the snowball with its walls: one step against the oracle, then a rollout
sc = scenes.snowball(seed=1, n=4000, grid=32)
s = sim_of(sc)
s.set_particles(sc.x, sc.v, sc.mass)
s.init_volumes()
kw = sc.params()
o = orc.OracleSim(orc.Params(*sc.grid, float(sc.h), **{k: v for k, v in kw.items() if k not in ("track_fp", "precision")}),
                  sc.x, sc.v, sc.mass)
o.init()
s.step(sc.dt, 1)
o.step(sc.dt, 1)
got = s.get_particles(("x", "v"))
out["oracle_one_step"] = max(rel(got["x"], o.x), rel(got["v"], o.v))
s.step(sc.dt, 20)
s.synchronize()
out["flags"]["snowball"] = s.flags()

# edge cases on grids of partial 4x4x4 blocks (30 = 7 x 4 + 2, 37 = 9 x 4 + 1):
# one particle outside the domain, several on the clamp planes, several moving
# three cells a step; the fused steps, then the seven stages
for G in (30, 37):
    h = 1.0 / G
    rng = np.random.default_rng(G)
    x = scenes.uniform_ball(rng, 3000, (0.5, 0.5, 0.5), 0.2).astype(np.float32)
    v = rng.normal(0, 1.0, (3000, 3)).astype(np.float32)
    x[0] = (0.3 * h, 0.5, 0.5)
    lo, hi = 3 * h, (G - 3) * h
    x[1:9] = np.array([[lo, 0.5, 0.5], [hi, 0.5, 0.5], [0.5, lo, 0.5], [0.5, hi, 0.5], [0.5, 0.5, lo],
                       [0.5, 0.5, hi], [lo, lo, lo], [hi, hi, hi]], np.float32)
    v[10:40] = (rng.normal(0, 1.0, (30, 3)) * (3 * h / 1e-4)).astype(np.float32)
    e = pkg.Simulation(pkg.make_params(G, G, G, 3000, h))
    e.set_particles(x, v, np.full(3000, 1e-4, np.float32))
    e.init_volumes()
    e.step(1e-4, 6)
    for name in ("rasterize", "forces", "grid_velocities", "collisions", "deformation", "particle_velocities",
                 "positions"):
        e.stage(name, 1e-4)
    e.synchronize()
    out["flags"][f"edges_{G}"] = e.flags()

# a batch of uneven scenes
batch = scenes.uneven_snowballs(seed=3, nscenes=3, n_lo=1500, n_hi=6000, g_lo=24, g_hi=40)
b = pkg.Batch([pkg.make_params(*q.grid, q.n, q.h, **q.params()) for q in batch])
for i, q in enumerate(batch):
    b.set_particles(i, q.x, q.v, q.mass)
b.init_volumes()
b.step(batch[0].dt, 10)
b.synchronize()
out["flags"]["batch"] = b.flags()

# FP64 with the full plastic F_P
f = scenes.snowball(seed=2, n=2000, grid=24)
d = sim_of(f, precision=pkg.RD_FP64, track_fp=1)
d.set_particles(f.x.astype(np.float64), f.v.astype(np.float64), f.mass.astype(np.float64))
d.init_volumes()
d.step(f.dt, 5)
d.synchronize()
out["flags"]["fp64_track_fp"] = d.flags()

# the sorted upload from page-locked arrays, after a step
import torch  # noqa: E402

st = s.get_particles(("x", "v", "B", "FE", "Jp", "mass", "volume"))
pin = {k: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy() for k, a in st.items()}
s.set_particles(pin["x"], pin["v"], pin["mass"], B=pin["B"], FE=pin["FE"], Jp=pin["Jp"], volume=pin["volume"])
s.step(sc.dt, 3)
s.get_particles(("x",))
s.synchronize()
out["flags"]["sorted_upload"] = s.flags()

# reverse mode
a = sim_of(scenes.snowball(seed=4, n=1500, grid=24), precision=pkg.RD_FP64)
q = scenes.snowball(seed=4, n=1500, grid=24)
a.set_particles(q.x.astype(np.float64), q.v.astype(np.float64), q.mass.astype(np.float64))
a.init_volumes()
a.adjoint_record(1e-4, 8, 3)
a.adjoint_backward(np.ones((q.n, 3)))
a.synchronize()
out["flags"]["adjoint"] = a.flags()

count, checked = pkg.bounds_violations()
out["violations"], out["checked"] = int(count), bool(checked)
print(json.dumps(out), flush=True)
