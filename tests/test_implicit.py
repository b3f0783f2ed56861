"""Implicit time integration (rd_time_integration): the energy the reference
minimises in timeIntegration (material_point_method.cpp:160-233), its
gradient, and the L-BFGS minimiser on the device.

* CPU: the oracle's restatement of Energy against the reference's own, built
  headless (the pin), and its analytic gradient against central differences.
* GPU: energy and gradient against the oracle (FP32 and FP64 builds), against
  the reference's values in the golden fixture, the device's L-BFGS iterate by
  iterate against the same algorithm on the oracle's FP64 energy, and against
  the minimiser the reference's own L-BFGS found (it stops early on its loose
  tolerances: the device reaches a lower energy)."""
import numpy as np
import pytest

from conftest import golden, rel

DT = 1e-3


def scene(orc, dtype=np.float32, seed=3, n=40, G=12, mass=1e-3, fe_noise=0.02):
    from rd_gb300 import scenes
    rng = np.random.default_rng(seed)
    h = 1.0 / G
    x = scenes.uniform_ball(rng, n, (0.5, 0.5, 0.5), 0.12).astype(np.float32)
    v = rng.normal(0, 0.5, (n, 3)).astype(np.float32)
    m = np.full(n, mass, np.float32)
    FE = (np.eye(3).reshape(1, 9) + fe_noise * rng.normal(size=(n, 9))).astype(np.float32)
    o = orc.OracleSim(orc.Params(G, G, G, h), x, v, m, FE=FE, dtype=dtype)
    o.init()
    o.stage("rasterize")
    return dict(G=G, h=h, x=x, v=v, m=m, FE=FE, rng=rng), o


def test_oracle_energy_matches_reference(orc):
    if not orc.ref_available():
        pytest.skip("headless reference not built on this machine")
    sc, o = scene(orc)
    r = orc.RefSim(orc.Params(sc["G"], sc["G"], sc["G"], sc["h"]), sc["x"], sc["v"], sc["m"], FE=sc["FE"], p4=1)
    r.init()
    r.stage("rasterize")
    g = r.grid()
    assert rel(g["mass"], o.gmass) < 1e-6
    used = (g["mass"] != 0)[:, None]
    for s in (0.0, 0.1, 1.0, 10.0):
        vel = (g["vel"] + s * sc["rng"].normal(size=g["vel"].shape) * used).astype(np.float32)
        e_ref = r.energy(vel, DT)
        assert abs(o.implicit_energy(vel, DT) - e_ref) <= 1e-6 * abs(e_ref), s


def test_oracle_gradient_matches_central_differences(orc):
    sc, o = scene(orc, np.float64)
    used = (o.gmass != 0)[:, None]
    rng = sc["rng"]
    for hardening in (0, 1):
        vel = o.gvel + 0.3 * rng.normal(size=o.gvel.shape) * used
        e, g = o.implicit_energy(vel, DT, hardening=hardening, grad=True)
        assert np.all(g[~used[:, 0]] == 0)
        d = rng.normal(size=vel.shape) * used
        eps = 1e-5
        fd = (o.implicit_energy(vel + eps * d, DT, hardening=hardening) -
              o.implicit_energy(vel - eps * d, DT, hardening=hardening)) / (2 * eps)
        assert abs(fd - np.sum(g * d)) <= 1e-6 * abs(fd), (hardening, fd, np.sum(g * d))


def gpu_sim(pkg, sc, precision=0):
    dt_ = np.float64 if precision else np.float32
    sim = pkg.Simulation(pkg.make_params(sc["G"], sc["G"], sc["G"], len(sc["m"]), sc["h"], precision=precision))
    sim.set_particles(sc["x"].astype(dt_), sc["v"].astype(dt_), sc["m"].astype(dt_), FE=sc["FE"].astype(dt_))
    sim.init_volumes()
    sim.stage("rasterize")
    return sim


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1])
def test_gpu_energy_and_gradient_match_oracle(built_pkg, orc, precision):
    dtype = np.float64 if precision else np.float32
    sc, o = scene(orc, dtype)
    sim = gpu_sim(built_pkg, sc, precision)
    grd = sim.get_grid()
    assert rel(grd["mass"], o.gmass) < 1e-6 and rel(grd["vel"], o.gvel) < 1e-5
    # both evaluate against the same grid: the device's rasterize rounds
    # differently, and at v = v* only the elastic part of the gradient is left
    o.gmass[:] = grd["mass"]
    o.gvel[:] = grd["vel"]
    used = (o.gmass != 0)[:, None]
    tol = 1e-10 if precision else 2e-5
    for hardening in (0, 1):
        for s in (0.0, 0.3, 3.0):
            vel = (o.gvel + s * sc["rng"].normal(size=o.gvel.shape) * used).astype(dtype)
            e_o, g_o = o.implicit_energy(vel, DT, hardening=hardening, grad=True)
            e_g, g_g = sim.implicit_energy(vel, DT, grad=True, hardening=hardening)
            assert abs(e_g - e_o) <= tol * abs(e_o), (hardening, s, e_g, e_o)
            assert rel(g_g, g_o) < tol, (hardening, s, rel(g_g, g_o))
    # the query leaves the grid as it was
    assert np.array_equal(sim.get_grid()["vel"], grd["vel"])


@pytest.mark.gpu
def test_gpu_energy_matches_reference_fixture(built_pkg):
    g = golden("implicit_12.npz")
    G = int(g["grid"][0])
    sim = built_pkg.Simulation(built_pkg.make_params(G, G, G, int(g["n"]), float(g["h"])))
    sim.set_particles(g["x0"], g["v0"], g["m0"], FE=g["FE0"])
    sim.init_volumes()
    sim.stage("rasterize")
    assert rel(sim.get_particles(("volume",))["volume"], g["vol0"]) < 1e-6
    grd = sim.get_grid()
    assert rel(grd["mass"], g["gmass"]) < 1e-6 and rel(grd["vel"], g["vstar"]) < 1e-5
    for f, e_ref in zip(g["fields"], g["energies"]):
        assert abs(sim.implicit_energy(f, float(g["dt"])) - e_ref) <= 1e-5 * abs(e_ref)


@pytest.mark.gpu
def test_gpu_lbfgs_follows_the_oracle_lbfgs_fp64(built_pkg, orc):
    """The device's L-BFGS against the same algorithm in numpy (oracle
    implicit_lbfgs) on the oracle's FP64 energy: 25 iterations from v* on the
    reference's own implicit scene (golden fixture; the reference's hardening,
    dt = 1e-3), the same iterate at the end.  The energy is badly conditioned
    (nodes at the cloud's edge carry almost no mass), so iterates are compared
    rather than a converged minimiser."""
    g = golden("implicit_12.npz")
    G, dt = int(g["grid"][0]), float(g["dt"])
    sim = built_pkg.Simulation(built_pkg.make_params(G, G, G, int(g["n"]), float(g["h"]), precision=1))
    sim.set_particles(*(g[k].astype(np.float64) for k in ("x0", "v0", "m0")), FE=g["FE0"].astype(np.float64))
    sim.init_volumes()
    sim.stage("rasterize")
    grd = sim.get_grid()
    o = orc.OracleSim(orc.Params(G, G, G, float(g["h"])), g["x0"], g["v0"], g["m0"], FE=g["FE0"], dtype=np.float64)
    o.init()
    o.stage("rasterize")
    o.gmass[:] = grd["mass"]
    o.gvel[:] = grd["vel"]
    used = o.gmass != 0

    def fg(z):
        vel = np.zeros(o.gvel.shape)
        vel[used] = z.reshape(-1, 3)
        e, gr = o.implicit_energy(vel, dt, grad=True)
        return e, gr[used].ravel()

    opts = dict(max_iters=25, grad_tol=0.0, step_tol=0.0)
    x, e, iters, conv = orc.implicit_lbfgs(fg, o.gvel[used].ravel(), **opts)
    res = sim.time_integration(dt, **opts)
    assert (res["iterations"], res["converged"]) == (iters, conv) == (25, 0)
    assert res["unknowns"] == 3 * int(np.count_nonzero(used))
    assert abs(res["energy"] - e) <= 1e-9 * abs(e), (res["energy"], e)
    assert res["energy"] < res["energy_start"]
    assert rel(sim.get_grid()["vel"][used].ravel(), x) < 1e-7


@pytest.mark.gpu
def test_gpu_minimiser_goes_below_the_references(built_pkg, orc):
    """The reference's own scene for its implicit path (golden fixture): with
    its default settings the device's L-BFGS lowers the energy and stops on
    the same tolerances; run further, it reaches a lower energy than the
    minimiser the reference's L-BFGS (finite-difference gradients) left."""
    g = golden("implicit_12.npz")
    G, dt = int(g["grid"][0]), float(g["dt"])
    o = orc.OracleSim(orc.Params(G, G, G, float(g["h"])), g["x0"], g["v0"], g["m0"], FE=g["FE0"], dtype=np.float64)
    o.init()
    o.stage("rasterize")
    e_ref = o.implicit_energy(g["vel_ref"].astype(np.float64), dt)
    for opts in ({}, {"max_iters": 400, "grad_tol": 0.0, "step_tol": 0.0}):
        sim = built_pkg.Simulation(built_pkg.make_params(G, G, G, int(g["n"]), float(g["h"])))
        sim.set_particles(g["x0"], g["v0"], g["m0"], FE=g["FE0"])
        sim.init_volumes()
        sim.stage("rasterize")
        res = sim.time_integration(dt, **opts)
        e_dev = o.implicit_energy(sim.get_grid()["vel"].astype(np.float64), dt)
        assert res["energy"] < res["energy_start"], res
        assert abs(res["energy"] - e_dev) <= 1e-5 * abs(e_dev)
        if opts:
            assert e_dev < e_ref, (e_dev, e_ref)
        else:
            assert res["converged"] == 1 and res["iterations"] <= 50, res
    assert sim.flags() == 0


@pytest.mark.gpu
def test_facade_time_integration_in_the_stage_order(built_pkg):
    """LagrangeEulerView.timeIntegration between the grid-velocity and the
    collision stages, then the rest of the step."""
    from rd_gb300 import scenes
    sc = scenes.snowball(seed=2, n=2000, grid=24)
    view = built_pkg.LagrangeEulerView(24, 24, 24, sc.n, h=sc.h)
    view.setParticles(sc.x, sc.v, sc.mass)
    view.rasterizeParticlesToGrid()
    view.computeParticleVolumesAndDensities()
    view.rasterizeParticlesToGrid()
    view.computeExplicitGridForces()
    view.gridVelocitiesUpdate(sc.dt)
    res = view.timeIntegration(sc.dt)
    assert res["energy"] <= res["energy_start"] and res["unknowns"] > 0
    view.gridBasedCollisions(sc.dt, [])
    view.updateDeformationGradient(sc.dt)
    view.updateParticleVelocities()
    view.updateParticlePositions(sc.dt)
    p = view.getParticles()
    assert np.all(np.isfinite(p["x"])) and np.all(np.isfinite(p["v"]))
