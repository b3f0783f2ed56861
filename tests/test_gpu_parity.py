"""GPU parity: the sm_103a step through the C ABI against the oracle (the C
restatement, pinned to the reference) and against the reference's own golden
outputs.  Tolerances are norm-wise relative errors ||gpu - ref|| / ||ref||
per field; 1e-5 is the one-step bar for FP32 with reordered atomics."""
import numpy as np
import pytest

from conftest import b_scale, golden, rel, rel_floor

pytestmark = pytest.mark.gpu

TOL1 = 1e-5  # one step, FP32


def make_sim(pkg, grid, n, h, **kw):
    return pkg.Simulation(pkg.make_params(*grid, n, h, **kw))


def oracle_params(orc, grid, h, **kw):
    kw = dict(kw)
    kw.pop("track_fp", None)
    kw.pop("precision", None)
    if "lagged_b" in kw:
        kw["lagged_c"] = kw.pop("lagged_b")
    return orc.Params(*grid, float(h), **kw)


def small_snowball(pkg, seed=0, n=3000, grid=32):
    from rd_gb300 import scenes
    return scenes.snowball(seed=seed, n=n, grid=grid)


def perturbed_inputs(orc, seed, n, grid, r=0.2, scale_B=0.3, scale_F=3e-3):
    from rd_gb300 import scenes
    rng = np.random.default_rng(seed)
    h = np.float32(1.0 / grid)
    x = scenes.uniform_ball(rng, n, (0.5, 0.5, 0.5), r).astype(np.float32)
    v = rng.normal(0, 1.0, (n, 3)).astype(np.float32)
    m = rng.uniform(0.5e-4, 1.5e-4, n).astype(np.float32)
    B, FE, FP = scenes.perturbed_state(rng, n, scale_B, scale_F, float(orc.reference_dinv(h)))
    return h, x, v, m, B, FE, FP


def compare_particles(got, o, h, tol, fields=("x", "v", "B", "FE", "Jp")):
    errs = {}
    for k in fields:
        if k == "B":
            errs[k] = rel_floor(got["B"], o.B, b_scale(o.v, h))
        elif k == "Jp":
            errs[k] = rel(got["Jp"], o.Jp)
        else:
            errs[k] = rel(got[k], getattr(o, k))
    bad = {k: v for k, v in errs.items() if not v < tol}
    assert not bad, f"errors {errs}"
    return errs


# ----------------------------------------------------------------- sorting
def test_block_keys_bit_exact_against_cpu_sort(built_pkg):
    from rd_gb300 import scenes
    sc = scenes.snowball(seed=7)
    sim = make_sim(built_pkg, sc.grid, sc.n, sc.h)
    sim.set_particles(sc.x, sc.v, sc.mass)
    keys, order = sim.debug_sort()
    h = np.float32(sc.h)
    nb = (np.array(sc.grid) + 3) // 4

    def cpu_keys(x):
        base = (x / h).astype(np.int32)  # IEEE FP32 divide, truncation (ivec3(pos / h))
        blk = ((base[:, 0] // 4) * nb[1] + base[:, 1] // 4) * nb[2] + base[:, 2] // 4
        cell = ((base[:, 0] % 4) * 4 + base[:, 1] % 4) * 4 + base[:, 2] % 4
        return (blk * 64 + cell).astype(np.int64)

    cpu = cpu_keys(sc.x)
    assert np.array_equal(keys, cpu.astype(np.uint32))
    assert np.array_equal(np.sort(order), np.arange(sc.n))
    assert np.array_equal(keys[order], np.sort(cpu, kind="stable").astype(np.uint32))
    # after steps the sort still matches the CPU keys of the new positions
    sim.init_volumes()
    sim.step(sc.dt, 3)
    x = sim.get_particles(("x",))["x"]
    keys, order = sim.debug_sort()
    cpu = cpu_keys(x)
    assert np.array_equal(keys, cpu.astype(np.uint32))
    assert np.array_equal(keys[order], np.sort(cpu).astype(np.uint32))


# ----------------------------------------------------------------- golden vectors
def test_reference_scene_golden_one_step(built_pkg):
    """The reference's own main.cpp scene (2147 particles, 20^3, dt = 1e-5)
    against the reference's outputs."""
    g = golden("ref_scene_20.npz")
    grid = tuple(int(v) for v in g["grid"])
    sim = make_sim(built_pkg, grid, int(g["n"]), float(g["h"]), track_fp=1)
    sim.set_particles(g["x0"], g["v0"], g["m0"])
    sim.init_volumes()
    got = sim.get_particles()
    assert rel(got["volume"], g["vol0"]) < 1e-6
    sim.step(float(g["dt"]), 1)
    got = sim.get_particles()
    assert rel(got["x"], g["s1_x"]) < TOL1
    assert rel(got["v"], g["s1_v"]) < TOL1
    assert rel_floor(got["B"], g["s1_B"], b_scale(g["s1_v"], float(g["h"]))) < TOL1
    assert rel(got["FE"], g["s1_FE"]) < TOL1
    assert rel(got["FP"], g["s1_FP"]) < TOL1
    grd = sim.get_grid()
    idx = g["grid_idx"]
    assert rel(grd["mass"][idx], g["grid_mass"]) < 1e-6
    assert np.count_nonzero(grd["mass"]) == np.count_nonzero(g["grid_mass"])
    assert rel(grd["vel"][idx], g["grid_vel"]) < TOL1
    sim.step(float(g["dt"]), 2)
    got = sim.get_particles()
    for k in ("x", "v", "FE", "FP"):
        assert rel(got[k], g[f"s3_{k}"]) < 1e-5, k


def test_perturbed_golden_one_step(built_pkg):
    """Random APIC B, near-identity F_E and F_P: exercises the affine transfer,
    the stress and the plastic split against the reference's outputs."""
    g = golden("perturbed_16.npz")
    grid = tuple(int(v) for v in g["grid"])
    sim = make_sim(built_pkg, grid, int(g["n"]), float(g["h"]), track_fp=1)
    sim.set_particles(g["x0"], g["v0"], g["m0"], B=g["B0"], FE=g["FE0"], FP=g["FP0"])
    sim.init_volumes()
    assert rel(sim.get_particles(("volume",))["volume"], g["vol0"]) < 1e-6
    sim.step(float(g["dt"]), 1)
    got = sim.get_particles()
    for k in ("x", "v", "B", "FE", "FP"):
        assert rel(got[k], g[f"s1_{k}"]) < TOL1, k
    grd = sim.get_grid()
    idx = g["grid_idx"]
    assert rel(grd["mass"][idx], g["grid_mass"]) < 1e-6
    mom_gpu = grd["mass"][idx, None].astype(np.float64) * grd["vel"][idx]
    mom_ref = g["grid_mass"][:, None].astype(np.float64) * g["grid_vel"]
    assert rel(mom_gpu, mom_ref) < TOL1


# ----------------------------------------------------------------- oracle parity
@pytest.mark.parametrize("bc", [0, 1])
def test_one_step_snowball_matches_oracle(built_pkg, orc, bc):
    sc = small_snowball(built_pkg, seed=1)
    kw = sc.params(bc=bc)
    sim = make_sim(built_pkg, sc.grid, sc.n, sc.h, **kw)
    sim.set_particles(sc.x, sc.v, sc.mass)
    sim.init_volumes()
    o = orc.OracleSim(oracle_params(orc, sc.grid, sc.h, **kw), sc.x, sc.v, sc.mass)
    o.init()
    assert rel(sim.get_particles(("volume",))["volume"], o.vol) < 1e-6
    sim.step(sc.dt, 1)
    o.step(sc.dt, 1)
    compare_particles(sim.get_particles(), o, sc.h, TOL1)
    grd = sim.get_grid()
    assert rel(grd["mass"], o.gmass) < 1e-6
    assert rel(grd["mass"][:, None] * grd["vel"], o.gmass[:, None] * o.gvel) < TOL1


@pytest.mark.parametrize("seed", [11, 12])
def test_one_step_perturbed_matches_oracle(built_pkg, orc, seed):
    h, x, v, m, B, FE, FP = perturbed_inputs(orc, seed, 4000, 32)
    sim = make_sim(built_pkg, (32, 32, 32), len(m), float(h), theta_s=7.5e-3)
    sim.set_particles(x, v, m, B=B, FE=FE, FP=FP)
    sim.init_volumes()
    o = orc.OracleSim(orc.Params(32, 32, 32, float(h), theta_s=7.5e-3), x, v, m, B, FE, FP)
    o.init()
    sim.step(1e-4, 1)
    o.step(1e-4, 1)
    compare_particles(sim.get_particles(), o, float(h), TOL1)


@pytest.mark.parametrize("track_fp", [0, 1])
def test_unclamped_and_clamped_warps_match_oracle(built_pkg, orc, track_fp):
    """The fused step's two ways to the stress: warps whose particles are all
    inside the clamp take F_E = F_E* and the stress without an SVD, other
    warps the SVD.  The half x < 0.5 of the ball holds F_E within 1e-3 of a
    rotation (no particle clamped, so its warps go the direct way), the other
    half F_E spread past both clamp bounds (most warps there have a clamped
    particle).  Three steps against the FP64 oracle: with strong stresses and
    random velocities the FP32 oracle's own grid velocities are ~1e-5 from
    the FP64 ones, so the FP32 step is held to the FP64 oracle and to no
    larger an error than the FP32 oracle makes."""
    h, x, v, m, B, FE, FP = perturbed_inputs(orc, 17, 5000, 32, scale_B=0.1, scale_F=1e-3)
    rng = np.random.default_rng(18)
    ang = rng.normal(0, 1.0, (len(m), 3))
    for i in range(len(m)):  # a rotation times a stretch
        a = ang[i]
        K = np.array([[0, -a[2], a[1]], [a[2], 0, -a[0]], [-a[1], a[0], 0]])
        t = np.linalg.norm(a)
        R = np.eye(3) + np.sin(t) / t * K + (1 - np.cos(t)) / t ** 2 * K @ K
        spread = 1e-3 if x[i, 0] < 0.5 else 2e-2
        FE[i] = (R @ (np.eye(3) + rng.normal(0, spread, (3, 3)))).reshape(9).astype(np.float32)
    right = x[:, 0] >= 0.5
    sv = np.linalg.svd(FE.reshape(-1, 3, 3).astype(np.float64), compute_uv=False)
    assert np.all((sv[~right] > 0.98) & (sv[~right] < 1.005))
    assert np.mean(np.any((sv[right] < 0.975) | (sv[right] > 1.0075), axis=1)) > 0.3
    sim = make_sim(built_pkg, (32, 32, 32), len(m), float(h), track_fp=track_fp)
    sim.set_particles(x, v, m, B=B, FE=FE, FP=FP)
    sim.init_volumes()
    P = orc.Params(32, 32, 32, float(h))
    o64 = orc.OracleSim(P, x, v, m, B, FE, FP, dtype=np.float64)
    o32 = orc.OracleSim(P, x, v, m, B, FE, FP)
    for o in (o64, o32):
        o.init()
        o.step(1e-4, 3)
    sim.step(1e-4, 3)
    got = sim.get_particles()
    compare_particles(got, o64, float(h), TOL1)
    if track_fp:
        assert rel(got["FP"], o64.FP) < 5e-5
    grd = sim.get_grid()
    assert rel(grd["mass"], o64.gmass) < 1e-6
    for k, own in (("v", rel(o32.v, o64.v)), ("gvel", rel(o32.gvel, o64.gvel))):
        err = rel(got["v"], o64.v) if k == "v" else rel(grd["vel"], o64.gvel)
        assert err < TOL1 and err <= 1.5 * own, (k, err, own)
    assert sim.flags() == 0


def test_stagewise_matches_oracle(built_pkg, orc):
    """rd_stage runs the reference's seven stages one at a time; each one's grid
    and particle state agree with the oracle's same stage."""
    h, x, v, m, B, FE, FP = perturbed_inputs(orc, 21, 3000, 24)
    sim = make_sim(built_pkg, (24, 24, 24), len(m), float(h), track_fp=1)
    sim.set_particles(x, v, m, B=B, FE=FE, FP=FP)
    sim.init_volumes()
    o = orc.OracleSim(orc.Params(24, 24, 24, float(h)), x, v, m, B, FE, FP)
    o.init()
    stages = [("rasterize", "rasterize", 0.0), ("forces", "forces", 0.0),
              ("grid_velocities", "grid_velocities", 1e-4), ("collisions", None, 1e-4),
              ("deformation", "update_F", 1e-4), ("particle_velocities", "g2p", 0.0),
              ("positions", "advect", 1e-4)]
    for gname, oname, dt in stages:
        sim.stage(gname, dt)
        if oname:
            o.stage(oname, dt)
        grd = sim.get_grid(force=True)
        assert rel(grd["mass"], o.gmass) < 1e-6, gname
        assert rel(grd["vel"], o.gvel) < TOL1, gname
        assert rel(grd["force"], o.gforce) < TOL1, gname
        got = sim.get_particles()
        for k in ("x", "v", "FE", "FP"):
            assert rel(got[k], getattr(o, k)) < TOL1, (gname, k)
        assert rel_floor(got["B"], o.B, b_scale(o.v, float(h))) < TOL1, gname


def test_rollout_matches_oracle_and_conserves_mass(built_pkg, orc):
    sc = small_snowball(built_pkg, seed=3, n=4000)
    kw = sc.params()
    sim = make_sim(built_pkg, sc.grid, sc.n, sc.h, **kw)
    sim.set_particles(sc.x, sc.v, sc.mass)
    sim.init_volumes()
    o = orc.OracleSim(oracle_params(orc, sc.grid, sc.h, **kw), sc.x, sc.v, sc.mass)
    o.init()
    total = float(np.sum(sc.mass, dtype=np.float64))
    for _ in range(20):
        sim.step(sc.dt, 1)
        o.step(sc.dt, 1)
        gm = sim.get_grid()["mass"]
        assert abs(float(np.sum(gm, dtype=np.float64)) - total) / total < 1e-6
    compare_particles(sim.get_particles(), o, sc.h, 1e-4)
    assert sim.flags() == 0


def test_textbook_order_matches_oracle(built_pkg, orc):
    h, x, v, m, B, FE, FP = perturbed_inputs(orc, 31, 3000, 32)
    sim = make_sim(built_pkg, (32, 32, 32), len(m), float(h), lagged_b=0)
    sim.set_particles(x, v, m, B=B, FE=FE, FP=FP)
    sim.init_volumes()
    o = orc.OracleSim(orc.Params(32, 32, 32, float(h), lagged_c=0), x, v, m, B, FE, FP)
    o.init()
    sim.step(1e-4, 1)
    o.step(1e-4, 1)
    compare_particles(sim.get_particles(), o, float(h), TOL1)


def test_track_fp_full_plastic_matrix(built_pkg, orc):
    h, x, v, m, B, FE, FP = perturbed_inputs(orc, 41, 2000, 24)
    sim = make_sim(built_pkg, (24, 24, 24), len(m), float(h), track_fp=1)
    sim.set_particles(x, v, m, B=B, FE=FE, FP=FP)
    sim.init_volumes()
    o = orc.OracleSim(orc.Params(24, 24, 24, float(h)), x, v, m, B, FE, FP)
    o.init()
    sim.step(1e-4, 2)
    o.step(1e-4, 2)
    got = sim.get_particles()
    assert rel(got["FP"], o.FP) < 5e-5
    assert rel(got["Jp"], o.Jp) < 1e-5


def test_fp64_build_matches_fp64_oracle(built_pkg, orc):
    h, x, v, m, B, FE, FP = perturbed_inputs(orc, 51, 1500, 24)
    sim = make_sim(built_pkg, (24, 24, 24), len(m), float(h), precision=built_pkg.RD_FP64, track_fp=1)
    sim.set_particles(x, v, m, B=B, FE=FE, FP=FP)
    sim.init_volumes()
    o = orc.OracleSim(orc.Params(24, 24, 24, float(h)), x, v, m, B, FE, FP, dtype=np.float64)
    o.init()
    sim.step(1e-4, 3)
    o.step(1e-4, 3)
    got = sim.get_particles()
    for k in ("x", "v", "B", "FE", "FP"):
        assert rel(got[k], getattr(o, k)) < 1e-10, k
    # the FP32 kernels' error against the FP64 oracle on the same inputs
    s32 = make_sim(built_pkg, (24, 24, 24), len(m), float(h))
    s32.set_particles(x, v, m, B=B, FE=FE, FP=FP)
    s32.init_volumes()
    s32.step(1e-4, 1)
    o1 = orc.OracleSim(orc.Params(24, 24, 24, float(h)), x, v, m, B, FE, FP, dtype=np.float64)
    o1.init()
    o1.step(1e-4, 1)
    g32 = s32.get_particles()
    for k in ("x", "v", "FE"):
        assert rel(g32[k], getattr(o1, k)) < 2e-5, k


# ----------------------------------------------------------------- edge cases
def test_empty_particle_set(built_pkg):
    sim = make_sim(built_pkg, (16, 16, 16), 0, 1 / 16)
    sim.set_particles(np.zeros((0, 3)), np.zeros((0, 3)), np.zeros(0))
    sim.init_volumes()
    sim.step(1e-4, 3)
    assert sim.get_particles()["x"].shape == (0, 3)
    assert float(sim.get_grid()["mass"].sum()) == 0.0
    assert sim.flags() == 0


def test_single_particle(built_pkg, orc):
    x = np.array([[0.5123, 0.4987, 0.5031]], np.float32)
    v = np.array([[0.3, -0.2, 0.1]], np.float32)
    m = np.array([1e-3], np.float32)
    sim = make_sim(built_pkg, (16, 16, 16), 1, 1 / 16)
    sim.set_particles(x, v, m)
    sim.init_volumes()
    o = orc.OracleSim(orc.Params(16, 16, 16, 1 / 16), x, v, m)
    o.init()
    sim.step(1e-4, 2)
    o.step(1e-4, 2)
    compare_particles(sim.get_particles(), o, 1 / 16, TOL1)


def test_dense_block_overflows_work_items(built_pkg, orc):
    """3000 particles inside one 4x4x4-cell block: one block spans many work
    items of at most 256 particles."""
    rng = np.random.default_rng(61)
    G = 32
    h = 1.0 / G
    x = (rng.uniform(16 * h, 20 * h - 1e-4, (3000, 3))).astype(np.float32)
    v = rng.normal(0, 0.5, (3000, 3)).astype(np.float32)
    m = np.full(3000, 1e-5, np.float32)
    sim = make_sim(built_pkg, (G, G, G), 3000, h)
    sim.set_particles(x, v, m)
    keys, _ = sim.debug_sort()
    assert len(np.unique(keys // 64)) == 1  # a single block
    sim.init_volumes()
    o = orc.OracleSim(orc.Params(G, G, G, h), x, v, m)
    o.init()
    sim.step(1e-4, 1)
    o.step(1e-4, 1)
    compare_particles(sim.get_particles(), o, h, TOL1)


def test_particles_on_nodes_and_clamp_boundaries(built_pkg, orc):
    """Positions exactly on grid nodes (fractional offset 0, so the +2 weight is
    0) and exactly on the clamp planes 3h and (MAX-3)h."""
    G = 24
    h = np.float32(1.0 / G)
    pts = []
    for i in (3, 5, 10, 21):
        for j in (3, 8, 21):
            for k in (3, 12, 21):
                pts.append([i * h, j * h, k * h])
    x = np.array(pts, np.float32)
    n = len(x)
    rng = np.random.default_rng(71)
    v = rng.normal(0, 1, (n, 3)).astype(np.float32)
    m = np.full(n, 1e-4, np.float32)
    sim = make_sim(built_pkg, (G, G, G), n, float(h))
    sim.set_particles(x, v, m)
    sim.init_volumes()
    o = orc.OracleSim(orc.Params(G, G, G, float(h)), x, v, m)
    o.init()
    sim.step(1e-4, 2)
    o.step(1e-4, 2)
    compare_particles(sim.get_particles(), o, float(h), TOL1)
    assert sim.flags() == 0


def test_out_of_domain_particle_is_flagged_not_fatal(built_pkg):
    """A particle whose stencil leaves the grid (the reference would index out of
    bounds) drops those nodes, raises RD_FLAG_OUT_OF_DOMAIN, and is clamped back
    into the domain by the position update."""
    G = 16
    h = 1.0 / G
    x = np.array([[0.5, 0.5, 0.5], [0.3 * h, 0.5, 0.5]], np.float32)
    sim = make_sim(built_pkg, (G, G, G), 2, h)
    sim.set_particles(x, np.zeros((2, 3), np.float32), np.full(2, 1e-4, np.float32))
    sim.init_volumes()
    sim.step(1e-4, 1)
    assert sim.flags() & built_pkg.FLAG_OUT_OF_DOMAIN
    got = sim.get_particles()
    assert np.all(np.isfinite(got["x"])) and got["x"][1, 0] >= 3 * h - 1e-7
    sim.clear_flags()
    assert sim.flags() == 0


def test_facade_stage_calls_match_fused_step(built_pkg, orc):
    """The reference's call sequence (main.cpp:53-54,192-218) through the
    LagrangeEulerView facade agrees with the oracle and with rd_step."""
    sc = small_snowball(built_pkg, seed=5, n=2500, grid=24)
    view = built_pkg.LagrangeEulerView(24, 24, 24, sc.n, h=sc.h, theta_s=7.5e-3)
    view.setParticles(sc.x, sc.v, sc.mass)
    view.rasterizeParticlesToGrid()
    view.computeParticleVolumesAndDensities()
    for _ in range(2):
        view.rasterizeParticlesToGrid()
        view.computeExplicitGridForces()
        view.gridVelocitiesUpdate(sc.dt)
        view.gridBasedCollisions(sc.dt, [])
        view.updateDeformationGradient(sc.dt)
        view.updateParticleVelocities()
        view.updateParticlePositions(sc.dt)
    o = orc.OracleSim(orc.Params(24, 24, 24, sc.h, theta_s=7.5e-3), sc.x, sc.v, sc.mass)
    o.init()
    o.step(sc.dt, 2)
    compare_particles(view.getParticles(), o, sc.h, TOL1)
    fused = built_pkg.LagrangeEulerView(24, 24, 24, sc.n, h=sc.h, theta_s=7.5e-3)
    fused.setParticles(sc.x, sc.v, sc.mass)
    fused.rasterizeParticlesToGrid()
    fused.computeParticleVolumesAndDensities()
    fused.step(sc.dt, 2)
    a, b = view.getParticles(), fused.getParticles()
    for k in ("x", "v", "FE", "FP"):
        assert rel(a[k], b[k]) < TOL1, k


def test_kernels_launch_natively(built_pkg):
    sc = small_snowball(built_pkg, seed=6, n=1000, grid=16)
    sim = make_sim(built_pkg, sc.grid, sc.n, sc.h)
    sim.set_particles(sc.x, sc.v, sc.mass)
    c0 = sim.launch_count()
    sim.init_volumes()
    sim.step(sc.dt, 4)
    assert sim.launch_count() - c0 >= 4 * 4


def test_step_size_change_rebuilds_next_grid(built_pkg, orc):
    """The fused kernel builds the next step's grid with this step's dt; a call
    with another dt must not reuse it."""
    sc = small_snowball(built_pkg, seed=8, n=3000)
    kw = sc.params()
    sim = make_sim(built_pkg, sc.grid, sc.n, sc.h, **kw)
    sim.set_particles(sc.x, sc.v, sc.mass)
    sim.init_volumes()
    o = orc.OracleSim(oracle_params(orc, sc.grid, sc.h, **kw), sc.x, sc.v, sc.mass)
    o.init()
    for dt, k in ((1e-4, 2), (5e-5, 2), (1e-4, 1)):
        sim.step(dt, k)
        o.step(dt, k)
    compare_particles(sim.get_particles(), o, sc.h, 2e-5)


def test_fast_particles_leave_their_block(built_pkg, orc):
    """Particles moving more than a cell per step leave the fused kernel's
    9^3 next-step tile and are scattered straight to the grid."""
    rng = np.random.default_rng(81)
    G, n = 32, 1500
    h = 1.0 / G
    x = rng.uniform(0.35, 0.65, (n, 3)).astype(np.float32)
    v = rng.normal(0, 1, (n, 3)).astype(np.float32)
    v[::7] *= 600.0  # |v| dt ~ 3-6 cells for every 7th particle
    m = np.full(n, 1e-4, np.float32)
    kw = dict(gravity=(0.0, 0.0, 0.0))
    sim = make_sim(built_pkg, (G, G, G), n, h, **kw)
    sim.set_particles(x, v, m)
    sim.init_volumes()
    o = orc.OracleSim(orc.Params(G, G, G, h, **kw), x, v, m)
    o.init()
    for _ in range(3):
        sim.step(1e-4, 1)
        o.step(1e-4, 1)
        gm = sim.get_grid()["mass"]
        assert abs(float(gm.sum(dtype=np.float64)) - float(m.sum(dtype=np.float64))) < 1e-6 * float(m.sum())
    compare_particles(sim.get_particles(), o, h, 2e-5)


def test_large_host_transfers_round_trip(built_pkg):
    """A 300,000-particle state goes to the device and back exactly, and after
    steps have permuted the slots the staged download (copied out of a device
    buffer) equals the mapped one (the unpacking kernel writing pinned memory
    directly), both in particle id order."""
    import torch
    from rd_gb300 import scenes
    sc = scenes.two_balls_1m(n=300_000)
    rng = np.random.default_rng(9)
    B = (0.01 * rng.normal(size=(sc.n, 9))).astype(np.float32)
    FE = (np.eye(3).reshape(1, 9) + 1e-3 * rng.normal(size=(sc.n, 9))).astype(np.float32)
    sim = built_pkg.Simulation(built_pkg.make_params(*sc.grid, sc.n, sc.h, **sc.params()))
    sim.set_particles(sc.x, sc.v, sc.mass, B=B, FE=FE)
    got = sim.get_particles(("x", "v", "B", "FE", "mass"))
    for k, ref in (("x", sc.x), ("v", sc.v), ("B", B), ("FE", FE), ("mass", sc.mass)):
        assert np.array_equal(got[k].reshape(ref.shape), ref), k
    sim.init_volumes()
    sim.step(sc.dt, 3)
    fields = ("x", "v", "B", "FE", "Jp", "mass", "volume")
    chunked = sim.get_particles(fields)
    shapes = {k: chunked[k].shape for k in fields}
    pinned = {k: torch.empty(shapes[k], dtype=torch.float32, pin_memory=True).numpy() for k in fields}
    sim.get_particles(fields, out=pinned, mapped=True)
    sim.synchronize()
    for k in fields:
        assert np.array_equal(chunked[k], pinned[k]), k
    assert sim.flags() == 0


# ----------------------------------------------------------------- full size
def test_full_size_two_ball_workload_properties(built_pkg):
    """The benchmark's 1.1M-particle two-ball workload (128^3) at full size,
    10 fused steps, checked through properties that hold at any size: every
    particle comes back with its own mass; total grid mass equals particle
    mass; linear momentum changes by the gravity impulse only (the MLS force
    and the APIC affine term sum to zero over each particle's stencil, and no
    particle is near a wall yet), within FP32 rounding; the block keys of the
    final positions equal a CPU computation bit for bit and the sort is a
    permutation in key order; no status flag."""
    from rd_gb300 import scenes
    sc = scenes.two_balls_1m()
    steps = 10
    sim = make_sim(built_pkg, sc.grid, sc.n, sc.h, **sc.params())
    sim.set_particles(sc.x, sc.v, sc.mass)
    sim.init_volumes()
    sim.step(sc.dt, steps)
    out = sim.get_particles(("x", "v", "FE", "Jp", "mass"))
    assert sim.flags() == 0
    assert np.array_equal(out["mass"], sc.mass)
    for k in ("x", "v", "FE", "Jp"):
        assert np.all(np.isfinite(out[k])), k
    m = sc.mass.astype(np.float64)
    total = float(m.sum())
    gm = sim.get_grid()["mass"]
    assert abs(float(np.sum(gm, dtype=np.float64)) - total) / total < 1e-6
    v = out["v"].astype(np.float64)
    p0 = (m[:, None] * sc.v.astype(np.float64)).sum(0)
    p = (m[:, None] * v).sum(0)
    want = p0 + total * steps * sc.dt * np.array([0.0, -9.8, 0.0])
    scale = float((m * np.linalg.norm(v, axis=1)).sum())
    assert np.abs(p - want).max() < 1e-5 * scale, (p, want)
    keys, order = sim.debug_sort()
    h = np.float32(sc.h)
    nb = (np.array(sc.grid) + 3) // 4
    base = (out["x"] / h).astype(np.int32)
    blk = ((base[:, 0] // 4) * nb[1] + base[:, 1] // 4) * nb[2] + base[:, 2] // 4
    cell = ((base[:, 0] % 4) * 4 + base[:, 1] % 4) * 4 + base[:, 2] % 4
    cpu = (blk * 64 + cell).astype(np.int64)
    assert np.array_equal(keys, cpu.astype(np.uint32))
    assert np.array_equal(np.sort(order), np.arange(sc.n))
    assert np.all(np.diff(keys[order].astype(np.int64)) >= 0)
