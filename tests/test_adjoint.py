"""Reverse mode (rd_adjoint_record / rd_adjoint_backward): gradients of a
rollout against central finite differences of the FP64 build, invariance to
the checkpoint interval, FP32 against FP64, the torch.autograd front end and
batches.  The FD bar is 1e-4 relative."""
import numpy as np
import pytest

from conftest import rel

pytestmark = pytest.mark.gpu

FD_TOL = 1e-4


def plastic_scene(seed=0, n=1500, grid=24):
    """A ball with random velocities and elastic strains beyond the clamp
    bounds, so the plastic split, the stress and the grid all carry gradient."""
    from rd_gb300 import scenes
    rng = np.random.default_rng(seed)
    h = 1.0 / grid
    x = scenes.uniform_ball(rng, n, (0.5, 0.5, 0.5), 0.15)
    v = rng.normal(0.0, 0.5, (n, 3))
    m = np.full(n, 400.0 * 4.0 / 3.0 * np.pi * 0.15 ** 3 / n)
    FE = np.eye(3).reshape(1, 9) + 0.02 * rng.normal(size=(n, 9))
    c = rng.normal(size=(n, 3))  # loss L = sum c . x_T
    return dict(grid=(grid,) * 3, h=h, x=x, v=v, m=m, FE=FE, c=c, rng=rng)


MAT = dict(E=1.4e5, nu=0.2, xi=10.0, theta_c=2.5e-2, theta_s=7.5e-3, gravity=(0.0, -9.8, 0.0), bc=1, bc_width=3)


def run(pkg, sc, v0, steps=12, every=4, precision=1, grads=True, **mat):
    kw = dict(MAT)
    kw.update(mat)
    dt_ = np.float64 if precision == 1 else np.float32
    sim = pkg.Simulation(pkg.make_params(*sc["grid"], len(sc["m"]), sc["h"], precision=precision, **kw))
    sim.set_particles(sc["x"].astype(dt_), v0.astype(dt_), sc["m"].astype(dt_), FE=sc["FE"].astype(dt_))
    sim.init_volumes()
    sim.adjoint_record(1e-4, steps, every)
    xT = sim.get_particles(("x",))["x"].astype(np.float64)
    loss = float(np.sum(sc["c"] * xT))
    g = sim.adjoint_backward(sc["c"].astype(dt_)) if grads else None
    assert sim.flags() == 0
    sim.close()
    return loss, g


def rel_err(a, b):
    return abs(a - b) / max(abs(a), abs(b), 1e-300)


def test_gradients_match_central_differences_fp64(built_pkg):
    sc = plastic_scene()
    L0, g = run(built_pkg, sc, sc["v"])
    # v0 along two random directions
    for k in range(2):
        e = sc["rng"].normal(size=sc["v"].shape)
        eps = 1e-5
        fd = (run(built_pkg, sc, sc["v"] + eps * e, grads=False)[0] - run(built_pkg, sc, sc["v"] - eps * e, grads=False)[0]) / (2 * eps)
        ad = float(np.sum(g["v0"] * e))
        assert rel_err(fd, ad) < FD_TOL, (k, fd, ad)
    # material parameters
    for name, base, eps in (("E", 1.4e5, 1.0), ("nu", 0.2, 1e-6), ("theta_c", 2.5e-2, 1e-7), ("theta_s", 7.5e-3, 1e-7)):
        lp = run(built_pkg, sc, sc["v"], grads=False, **{name: base + eps})[0]
        lm = run(built_pkg, sc, sc["v"], grads=False, **{name: base - eps})[0]
        fd = (lp - lm) / (2 * eps)
        ad = float(g[name][0])
        assert abs(ad) > 0, name
        assert rel_err(fd, ad) < FD_TOL, (name, fd, ad)


def test_gradients_from_identity_elastic_F_match_central_differences_fp64(built_pkg):
    """Every scene starts with F_E = I: all three singular values tie at 1
    in the first steps, where the split's backward takes its tie branch."""
    sc = plastic_scene(seed=7)
    sc["FE"] = np.tile(np.eye(3).reshape(1, 9), (len(sc["m"]), 1))
    L0, g = run(built_pkg, sc, sc["v"])
    for k in range(2):
        e = sc["rng"].normal(size=sc["v"].shape)
        eps = 1e-5
        fd = (run(built_pkg, sc, sc["v"] + eps * e, grads=False)[0] - run(built_pkg, sc, sc["v"] - eps * e, grads=False)[0]) / (2 * eps)
        ad = float(np.sum(g["v0"] * e))
        assert rel_err(fd, ad) < FD_TOL, (k, fd, ad)
    for name, base, eps in (("E", 1.4e5, 1.0), ("theta_s", 7.5e-3, 1e-7)):
        lp = run(built_pkg, sc, sc["v"], grads=False, **{name: base + eps})[0]
        lm = run(built_pkg, sc, sc["v"], grads=False, **{name: base - eps})[0]
        fd = (lp - lm) / (2 * eps)
        assert rel_err(fd, float(g[name][0])) < FD_TOL, (name, fd, float(g[name][0]))


def test_checkpoint_interval_does_not_change_gradients(built_pkg):
    sc = plastic_scene(seed=1, n=800, grid=20)
    ref = run(built_pkg, sc, sc["v"], steps=9, every=9)[1]
    for every in (1, 4):
        g = run(built_pkg, sc, sc["v"], steps=9, every=every)[1]
        assert rel(g["v0"], ref["v0"]) < 1e-10
        for k in ("E", "nu", "theta_c", "theta_s"):
            assert rel_err(g[k][0], ref[k][0]) < 1e-10


def test_fp32_gradients_track_fp64(built_pkg):
    sc = plastic_scene(seed=2, n=1500)
    g64 = run(built_pkg, sc, sc["v"], precision=1)[1]
    g32 = run(built_pkg, sc, sc["v"], precision=0)[1]
    assert rel(g32["v0"], g64["v0"]) < 1e-3
    for k in ("E", "nu"):
        assert rel_err(g32[k][0], g64[k][0]) < 1e-2


def test_record_is_invalidated_by_a_step(built_pkg):
    sc = plastic_scene(seed=3, n=500, grid=16)
    sim = built_pkg.Simulation(built_pkg.make_params(*sc["grid"], len(sc["m"]), sc["h"], **MAT))
    sim.set_particles(sc["x"], sc["v"], sc["m"])
    sim.init_volumes()
    with pytest.raises(built_pkg.RDError):
        sim.adjoint_backward(sc["c"])
    sim.adjoint_record(1e-4, 3, 2)
    sim.step(1e-4, 1)
    with pytest.raises(built_pkg.RDError):
        sim.adjoint_backward(sc["c"])


def test_torch_autograd_centroid_loss(built_pkg):
    import torch
    import importlib
    ag = importlib.import_module(built_pkg.__name__ + ".autograd")
    from rd_gb300 import scenes
    sc = scenes.cube(seed=0, n=4096, grid=32, steps=20)
    spec = ag.RolloutSpec(grid=sc.grid, h=sc.h, x0=sc.x, mass=sc.mass, dt=sc.dt, steps=20, every=5,
                          material={k: v for k, v in sc.material.items() if k not in ("E", "nu")})
    v0 = torch.tensor(np.random.default_rng(0).normal(0, 1, (sc.n, 3)).astype(np.float32), requires_grad=True)
    E = torch.tensor(1.4e5, dtype=torch.float64, requires_grad=True)
    nu = torch.tensor(0.2, dtype=torch.float64, requires_grad=True)
    target = torch.tensor([0.55, 0.3, 0.5])
    xT = ag.rollout(v0, E, nu, spec)
    loss = ((xT.mean(0) - target) ** 2).sum()
    loss.backward()
    # the same through the handle directly: dL/dx_T = 2 (centroid - target) / N for every particle
    cen = xT.detach().numpy().astype(np.float64).mean(0)
    gx = np.tile(2.0 * (cen - target.numpy()) / sc.n, (sc.n, 1)).astype(np.float32)
    sim = built_pkg.Simulation(built_pkg.make_params(*sc.grid, sc.n, sc.h, **sc.params()))
    sim.set_particles(sc.x, v0.detach().numpy(), sc.mass)
    sim.init_volumes()
    sim.adjoint_record(sc.dt, 20, 5)
    g = sim.adjoint_backward(gx)
    assert rel(v0.grad.numpy(), g["v0"]) < 1e-5
    assert rel_err(float(E.grad), g["E"][0]) < 1e-4 or abs(float(E.grad)) < 1e-12
    # with no walls reached, the centroid moves with the mean velocity: dL/dv0 = dt steps dL/dx_T
    assert rel(g["v0"], gx * sc.dt * 20) < 1e-3


def test_batch_gradients_match_single_scenes(built_pkg):
    from rd_gb300 import scenes
    batch = scenes.uneven_snowballs(seed=3, nscenes=3, n_lo=600, n_hi=2000, g_lo=16, g_hi=28)
    rng = np.random.default_rng(4)
    cs = [rng.normal(size=(s.n, 3)) for s in batch]
    params = [built_pkg.make_params(*s.grid, s.n, s.h, precision=1, **s.params()) for s in batch]
    b = built_pkg.Batch(params)
    for i, s in enumerate(batch):
        b.set_particles(i, s.x.astype(np.float64), s.v.astype(np.float64), s.mass.astype(np.float64))
    b.init_volumes()
    b.adjoint_record(1e-4, 8, 3)
    gb = b.adjoint_backward(np.concatenate(cs))
    off = 0
    for i, s in enumerate(batch):
        one = built_pkg.Simulation(params[i])
        one.set_particles(s.x.astype(np.float64), s.v.astype(np.float64), s.mass.astype(np.float64))
        one.init_volumes()
        one.adjoint_record(1e-4, 8, 3)
        g1 = one.adjoint_backward(cs[i])
        assert rel(gb["v0"][off:off + s.n], g1["v0"]) < 1e-9
        for k in ("E", "nu", "theta_c", "theta_s"):
            # theta gradients vanish when almost no particle is clamped: floor at 1e-15
            assert abs(gb[k][i] - g1[k][0]) <= 1e-9 * max(abs(gb[k][i]), abs(g1[k][0])) + 1e-15, (k, gb[k][i], g1[k][0])
        off += s.n
