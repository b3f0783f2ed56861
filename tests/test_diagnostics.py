"""The reference's diagnostics as device reductions (rd_get_diagnostics,
material_point_method.cpp:352-443), conservation through them, and failure
handling: argument checks without a GPU, NaN injection on one."""
import ctypes

import numpy as np
import pytest

from conftest import rel


def test_oversize_and_invalid_requests_fail_before_any_device_work(built_pkg):
    pkg = built_pkg
    L = pkg.lib()
    h = ctypes.c_void_p()
    p = pkg.make_params(64, 64, 64, (1 << 30), 1.0 / 64)  # 2^30 particles
    assert L.rd_create(ctypes.byref(p), ctypes.byref(h)) == pkg.RD_TOO_LARGE
    p = pkg.make_params(4, 64, 64, 10, 1.0 / 64)  # a grid too small for the stencil
    assert L.rd_create(ctypes.byref(p), ctypes.byref(h)) == pkg.RD_INVALID_ARG
    p = pkg.make_params(64, 64, 64, 10, -1.0)
    assert L.rd_create(ctypes.byref(p), ctypes.byref(h)) == pkg.RD_INVALID_ARG
    assert L.rd_step(None, 1e-4, 1) == pkg.RD_INVALID_ARG
    assert L.rd_batch_create(ctypes.byref(p), 0, ctypes.byref(h)) == pkg.RD_INVALID_ARG


@pytest.mark.gpu
def test_diagnostics_match_the_exported_state_and_conserve(built_pkg):
    from rd_gb300 import scenes
    sc = scenes.snowball(seed=5, n=6000, grid=32)
    kw = sc.params(bc=0, gravity=(0.0, 0.0, 0.0))
    sim = built_pkg.Simulation(built_pkg.make_params(*sc.grid, sc.n, sc.h, track_fp=1, **kw))
    rng = np.random.default_rng(1)
    v = sc.v + rng.normal(0, 0.5, sc.v.shape).astype(np.float32)
    sim.set_particles(sc.x, v, sc.mass)
    sim.init_volumes()
    d0 = sim.diagnostics()
    sim.step(sc.dt, 10)
    d = sim.diagnostics()
    p = sim.get_particles(("v", "mass", "volume", "FE", "FP"))
    m = p["mass"].astype(np.float64)
    assert rel(d["particle_mass"], np.sum(m)) < 1e-9
    assert rel(d["particle_momentum"], (m[:, None] * p["v"]).sum(0)) < 1e-6
    assert rel(d["average_particle_density"], np.mean(m / p["volume"])) < 1e-6
    F = np.einsum("nij,njk->nik", p["FE"].reshape(-1, 3, 3).astype(np.float64), p["FP"].reshape(-1, 3, 3))
    assert rel(d["average_deformation_gradient"], F.mean(0)) < 1e-6
    g = sim.get_grid()
    gm = g["mass"].astype(np.float64)
    assert rel(d["grid_mass"], gm.sum()) < 1e-6
    assert rel(d["grid_momentum"], (gm[:, None] * g["vel"]).sum(0)) < 1e-5
    assert d["used_cells"] == int(np.count_nonzero(gm))
    # conservation without gravity or walls: mass exactly moved, momentum kept
    assert rel(d["grid_mass"], d["particle_mass"]) < 1e-6
    assert rel(d["particle_momentum"], d0["particle_momentum"]) < 1e-4
    assert rel(d["grid_momentum"], d["particle_momentum"]) < 1e-5


@pytest.mark.gpu
def test_nan_injection_is_flagged_and_the_handle_recovers(built_pkg):
    from rd_gb300 import scenes
    sc = scenes.snowball(seed=6, n=3000, grid=32)
    sim = built_pkg.Simulation(built_pkg.make_params(*sc.grid, sc.n, sc.h, **sc.params()))
    v = sc.v.copy()
    v[17, 1] = np.nan
    sim.set_particles(sc.x, v, sc.mass)
    sim.init_volumes()
    sim.step(sc.dt, 2)
    assert sim.flags() & built_pkg.FLAG_NONFINITE
    sim.clear_flags()
    sim.set_particles(sc.x, sc.v, sc.mass)
    sim.init_volumes()
    sim.step(sc.dt, 5)
    assert sim.flags() == 0
    assert np.all(np.isfinite(sim.get_particles(("x",))["x"]))


@pytest.mark.gpu
def test_tile_copy_wait_gives_up_and_the_handle_keeps_working(built_pkg):
    """The fused kernel's wait for a TMA tile copy is bounded: against an
    mbarrier that nothing arrives at it gives up, raises the flag and the
    context stays usable (the next steps run and are flag-free)."""
    from rd_gb300 import scenes
    sc = scenes.snowball(seed=7, n=2000, grid=32)
    sim = built_pkg.Simulation(built_pkg.make_params(*sc.grid, sc.n, sc.h, **sc.params()))
    sim.set_particles(sc.x, sc.v, sc.mass)
    sim.init_volumes()
    assert sim.debug_wait_timeout(tries=32)
    assert sim.flags() & built_pkg.FLAG_WAIT_TIMEOUT
    sim.clear_flags()
    sim.step(sc.dt, 4)
    assert sim.flags() == 0
    assert np.all(np.isfinite(sim.get_particles(("x",))["x"]))
