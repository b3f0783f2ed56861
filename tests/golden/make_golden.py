"""Generates the golden fixtures in this directory from the reference itself:
the headless build of brocbyte/realtime-deformations' own LagrangeEulerView
(oracle/ref/build_ref.sh), driven through oracle/oracle.py's RefSim.

    python tests/golden/make_golden.py [REFERENCE_ROOT]

Fixtures (all FP32, matrices row-major n x 9, grids as sparse cell lists):

* ref_scene_20.npz - the reference's own scene (main.cpp:48-54,170): 20^3 grid,
  h = 0.05, 2147 particles from initializeParticles((0.5, 0.6, 0.5),
  (0, -200, 0)) with rand() seed 1, dt = 1e-5.  Inputs, volumes after the
  init rasterize, the state after 1 step (unmodified reference) with that
  step's grid, and after 3 steps with the plastic split of F_E itself (P4).
* perturbed_16.npz - 512 particles in a sphere on a 16^3 grid, h = 1/16,
  random velocities, random APIC B and near-identity F_E, F_P, dt = 1e-4:
  the state after 1 and 2 steps (P4) and the step-1 grid.
* colliders_32.npz - 1200 particles of a ball falling (v ~ (0.4, -3, 0.3))
  onto the reference's own MeshCollider boxes, a floor box and a box turned
  45 degrees about z moving at (0.1, 0, 0), on a 32^3 grid, dt = 1e-4: the
  grid after the collision stage of step 1 and the state after 3 steps, the
  boxes moved before each step as main.cpp:188 does (P4).
* implicit_12.npz - the reference's implicit time integration (timeIntegration,
  material_point_method.cpp:212-233, which its driver never calls): 40 particles
  in a ball on a 12^3 grid, h = 1/12, random velocities and near-identity F_E,
  after init and a rasterize; its Energy at v* and at three perturbed velocity
  fields (dt = 1e-3), and the grid velocities its L-BFGS leaves, dense.

    python tests/golden/make_golden.py [REFERENCE_ROOT] [fixture ...]
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
from oracle import oracle as orc  # noqa: E402


def sparse_grid(g):
    idx = np.nonzero((g["mass"] != 0) | np.any(g["force"] != 0, axis=1) | np.any(g["vel"] != 0, axis=1))[0]
    return {"grid_idx": idx.astype(np.int32), "grid_mass": g["mass"][idx], "grid_vel": g["vel"][idx],
            "grid_force": g["force"][idx]}


def state(prefix, p):
    return {f"{prefix}_{k}": v for k, v in p.items()}


def ref_scene():
    P = orc.Params(20, 20, 20, 0.05)
    r = orc.RefSim(P, n=2147, p4=0)
    r.initialize_particles((0.5, 0.6, 0.5), (0.0, -200.0, 0.0), seed=1)
    p0 = r.particles()
    m0 = r.masses()
    assert np.all(m0 > 0), "initializer left particles unplaced"
    out = {"grid": np.array([20, 20, 20]), "h": np.float32(0.05), "dt": np.float32(1e-5), "n": 2147,
           "x0": p0["x"], "v0": p0["v"], "m0": m0}
    r.init()
    out["vol0"] = r.particles()["vol"]
    r.step(1e-5, 1)
    out.update(state("s1", r.particles()))
    out.update(sparse_grid(r.grid()))
    r.p4 = 1
    r.step(1e-5, 2)
    out.update(state("s3", r.particles()))
    return out


def perturbed():
    rng = np.random.default_rng(1234)
    n, G = 512, 16
    h = np.float32(1.0 / G)
    P = orc.Params(G, G, G, float(h))
    dinv = float(orc.reference_dinv(h))
    d = rng.normal(size=(4 * n, 3))
    d = d / np.linalg.norm(d, axis=1, keepdims=True) * (rng.uniform(size=(4 * n, 1)) ** (1 / 3)) * 0.22
    x = (d[:n] + np.array([0.5, 0.5, 0.5])).astype(np.float32)
    v = rng.normal(0, 1.0, (n, 3)).astype(np.float32)
    m = rng.uniform(0.5e-4, 1.5e-4, n).astype(np.float32)
    B = (rng.normal(0, 0.5, (n, 9)) / dinv).astype(np.float32)
    FE = (np.eye(3).reshape(1, 9) + rng.normal(0, 4e-3, (n, 9))).astype(np.float32)
    FP = (np.eye(3).reshape(1, 9) + rng.normal(0, 4e-3, (n, 9))).astype(np.float32)
    r = orc.RefSim(P, x, v, m, B, FE, FP, p4=1)
    out = {"grid": np.array([G, G, G]), "h": h, "dt": np.float32(1e-4), "n": n,
           "x0": x, "v0": v, "m0": m, "B0": B, "FE0": FE, "FP0": FP}
    r.init()
    out["vol0"] = r.particles()["vol"]
    r.step(1e-4, 1)
    out.update(state("s1", r.particles()))
    out.update(sparse_grid(r.grid()))
    r.step(1e-4, 1)
    out.update(state("s2", r.particles()))
    return out


def colliders():
    rng = np.random.default_rng(77)
    G, n = 32, 1200
    h = np.float32(1.0 / G)
    d = rng.normal(size=(n, 3))
    d = d / np.linalg.norm(d, axis=1, keepdims=True) * (rng.uniform(size=(n, 1)) ** (1 / 3)) * 0.12
    x = (d + np.array([0.5, 0.31, 0.5])).astype(np.float32)
    v = (np.array([0.4, -3.0, 0.3]) + rng.normal(0, 0.3, (n, 3))).astype(np.float32)
    m = np.full(n, 1e-4, np.float32)
    s, c = np.sin(np.radians(22.5)), np.cos(np.radians(22.5))
    cols = [dict(translation=(0.5, -0.2, 0.5), rotation=(1, 0, 0, 0), scale=(0.4, 0.4, 0.4), velocity=(0, 0, 0)),
            dict(translation=(0.33, 0.33, 0.5), rotation=(c, 0, 0, s), scale=(0.06, 0.06, 0.3), velocity=(0.1, 0, 0))]
    P = orc.Params(G, G, G, float(h))
    r = orc.RefSim(P, x, v, m, p4=1)
    r.set_colliders(cols)
    out = {"grid": np.array([G, G, G]), "h": h, "dt": np.float32(1e-4), "n": n, "x0": x, "v0": v, "m0": m,
           "colliders": orc.collider_spec(cols)}
    r.init()
    out["vol0"] = r.particles()["vol"]
    for st in ("rasterize", "forces", "grid_velocities", "collisions"):
        r.stage(st, 1e-4)
    g = r.grid()
    idx = np.nonzero(g["mass"] != 0)[0]
    out["s1_grid_idx"] = idx.astype(np.int32)
    out["s1_grid_mass"] = g["mass"][idx]
    out["s1_grid_vel"] = g["vel"][idx]
    # the state after 3 full steps from the initial state
    r2 = orc.RefSim(P, x, v, m, p4=1)
    r2.init()
    for _ in range(3):
        r2.move_colliders(1e-4)
        r2.step(1e-4, 1)
    out.update(state("s3", r2.particles()))
    r.set_colliders([])
    return out


def implicit():
    rng = np.random.default_rng(3)
    G, n, dt = 12, 40, 1e-3
    h = 1.0 / G
    d = rng.normal(size=(n, 3))
    d = d / np.linalg.norm(d, axis=1, keepdims=True) * rng.uniform(size=(n, 1)) ** (1 / 3) * 0.12
    x = (d + 0.5).astype(np.float32)
    v = rng.normal(0, 0.5, (n, 3)).astype(np.float32)
    m = np.full(n, 1e-3, np.float32)
    FE = (np.eye(3).reshape(1, 9) + 0.02 * rng.normal(size=(n, 9))).astype(np.float32)
    r = orc.RefSim(orc.Params(G, G, G, h), x, v, m, FE=FE, p4=1)
    r.init()
    r.stage("rasterize")
    g = r.grid()
    used = g["mass"] != 0
    fields = [g["vel"]] + [(g["vel"] + s * rng.normal(size=g["vel"].shape) * used[:, None]).astype(np.float32)
                           for s in (0.1, 1.0, 10.0)]
    energies = np.array([r.energy(f, dt) for f in fields], np.float32)
    r.time_integration(dt)
    vel_ref = r.grid()["vel"]
    return {"grid": np.array([G, G, G]), "h": np.float32(h), "dt": np.float32(dt), "n": n, "x0": x, "v0": v,
            "m0": m, "FE0": FE, "vol0": r.particles()["vol"], "gmass": g["mass"], "vstar": g["vel"],
            "fields": np.stack(fields), "energies": energies, "vel_ref": vel_ref}


FIXTURES = {"ref_scene_20": ref_scene, "perturbed_16": perturbed, "colliders_32": colliders, "implicit_12": implicit}


def main():
    # usage: make_golden.py REFERENCE_ROOT [fixture ...]; REFERENCE_ROOT "-" takes
    # $RD_REFERENCE_ROOT (oracle.reference_root())
    root = sys.argv[1] if len(sys.argv) > 1 and sys.argv[1] != "-" else orc.reference_root()
    names = sys.argv[2:] or list(FIXTURES)
    if not root or not orc.build_ref(root):
        raise SystemExit("headless reference not available")
    for name in names:
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **FIXTURES[name]())


if __name__ == "__main__":
    main()
