"""Box colliders (gridBasedCollisions, material_point_method.cpp:264-304) on the
GPU: against the compiled reference's own MeshCollider boxes (golden fixture
colliders_32.npz, made by tests/golden/make_golden.py) and against the oracle
in both rules."""
import numpy as np
import pytest

from conftest import golden, rel

pytestmark = pytest.mark.gpu


def fixture_colliders(g):
    spec = g["colliders"].reshape(-1, 13)
    return [dict(translation=c[0:3], rotation=c[3:7], scale=c[7:10], velocity=c[10:13]) for c in spec]


def make(pkg, g, **kw):
    G = tuple(int(a) for a in g["grid"])
    sim = pkg.Simulation(pkg.make_params(*G, int(g["n"]), float(g["h"]), theta_s=5e-3, **kw))
    sim.set_particles(g["x0"], g["v0"], g["m0"])
    return sim


def test_collision_stage_matches_reference_golden(built_pkg):
    g = golden("colliders_32.npz")
    sim = make(built_pkg, g)
    sim.set_colliders(fixture_colliders(g), built_pkg.RD_COLLIDE_REFERENCE, 0.5)
    sim.init_volumes()
    assert rel(sim.get_particles(("volume",))["volume"], g["vol0"]) < 1e-6
    dt = float(g["dt"])
    for st in ("rasterize", "forces", "grid_velocities", "collisions"):
        sim.stage(st, dt)
    grd = sim.get_grid()
    idx = g["s1_grid_idx"]
    assert rel(grd["mass"][idx], g["s1_grid_mass"]) < 1e-6
    assert rel(grd["vel"][idx], g["s1_grid_vel"]) < 1e-5


def test_fused_steps_with_moving_boxes_match_reference_golden(built_pkg):
    g = golden("colliders_32.npz")
    sim = make(built_pkg, g)
    sim.set_colliders(fixture_colliders(g), built_pkg.RD_COLLIDE_REFERENCE, 0.5)
    sim.init_volumes()
    dt = float(g["dt"])
    for _ in range(3):
        sim.move_colliders(dt)  # main.cpp:188, before the stages
        sim.step(dt, 1)
    got = sim.get_particles()
    assert rel(got["x"], g["s3_x"]) < 1e-6
    assert rel(got["v"], g["s3_v"]) < 2e-5
    assert rel(got["FE"], g["s3_FE"]) < 1e-5
    assert sim.flags() == 0


@pytest.mark.parametrize("mode", [0, 1])
def test_fused_step_matches_oracle_both_rules(built_pkg, orc, mode):
    g = golden("colliders_32.npz")
    cols = fixture_colliders(g)
    G = tuple(int(a) for a in g["grid"])
    sim = make(built_pkg, g)
    sim.set_colliders(cols, mode, 0.5)
    sim.init_volumes()
    o = orc.OracleSim(orc.Params(*G, float(g["h"]), theta_s=5e-3), g["x0"], g["v0"], g["m0"])
    o.set_colliders(cols, mode, 0.5)
    try:
        o.init()
        dt = float(g["dt"])
        for _ in range(2):
            sim.step(dt, 1)
            o.step(dt, 1)
        got = sim.get_particles()
        assert rel(got["x"], o.x) < 1e-6
        assert rel(got["v"], o.v) < 1e-5
        grd = sim.get_grid()  # the last step's grid velocities, colliders applied
        assert rel(grd["vel"], o.gvel) < 1e-5
    finally:
        o.set_colliders([])


def test_no_colliders_after_reset_and_unsupported_uses(built_pkg):
    g = golden("colliders_32.npz")
    a, b = make(built_pkg, g), make(built_pkg, g)
    a.set_colliders(fixture_colliders(g))
    a.set_colliders([])
    for s in (a, b):
        s.init_volumes()
        s.step(1e-4, 4)
    assert rel(a.get_particles(("x",))["x"], b.get_particles(("x",))["x"]) < 1e-6
    a.set_colliders(fixture_colliders(g))
    with pytest.raises(built_pkg.RDError):
        a.adjoint_record(1e-4, 2, 1)  # no collider backward
    from rd_gb300 import scenes
    sc = scenes.snowball(n=500, grid=16)
    batch = built_pkg.Batch([built_pkg.make_params(*sc.grid, sc.n, sc.h)] * 2)
    with pytest.raises(built_pkg.RDError):
        batch.set_colliders(fixture_colliders(g))
