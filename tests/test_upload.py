"""rd_set_particles from page-locked host memory on a single-scene handle
that has stepped: the upload sorts on the way in (k_pack_keys, the scan, k_pack_place puts every particle
straight into its sorted slot), so the first step's P2G reads the particles
in order and nothing is reordered.  Checked against the same state uploaded to
a fresh handle (one-pass k_pack; the first step sorts with k_scatter and
reorders in k_p2g) and against the oracle (material_point_method.cpp:94-350)
one step on."""
import numpy as np
import pytest

from conftest import b_scale, rel, rel_floor

pytestmark = pytest.mark.gpu

FIELDS = ("x", "v", "B", "FE", "Jp", "mass", "volume")


def make(pkg, sc, precision=0):
    return pkg.Simulation(pkg.make_params(*sc.grid, sc.n, sc.h, precision=precision, **sc.params()))


def stepped_state(pkg, sc, precision=0, steps=2):
    """A handle after `steps` steps of the scene, and a changed copy of its
    state (velocities rotated and scaled), so the uploaded grid is new."""
    sim = make(pkg, sc, precision)
    dtype = np.float64 if precision else np.float32
    sim.set_particles(*(a.astype(dtype) for a in (sc.x, sc.v, sc.mass)))
    sim.init_volumes()
    sim.step(sc.dt, steps)
    st = sim.get_particles(FIELDS)
    st["v"] = np.ascontiguousarray(1.5 * st["v"][:, [2, 0, 1]])
    return sim, st


def upload(sim, st, pinned=False, mapped=False):
    if pinned:
        import torch
        st = {k: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy() for k, a in st.items()}
    sim.set_particles(st["x"], st["v"], st["mass"], B=st["B"], FE=st["FE"], Jp=st["Jp"], volume=st["volume"],
                      mapped=mapped)
    return st


def same_state(a, b, h, tol):
    for k in ("x", "v", "FE", "Jp"):
        assert rel(a[k], b[k]) < tol, (k, rel(a[k], b[k]))
    assert rel_floor(a["B"], b["B"], b_scale(b["v"], h)) < tol


@pytest.mark.parametrize("route", ["pageable", "pinned", "mapped"])
@pytest.mark.parametrize("precision", [0, 1])
def test_upload_after_a_step_matches_a_fresh_handle(built_pkg, route, precision):
    """Page-locked arrays (read in place, RD_HOST or as device pointers) take
    the sorted upload; pageable ones go through the staging buffer and the
    one-pass route."""
    from rd_gb300 import scenes
    sc = scenes.snowball(seed=5, n=6000, grid=32)
    a, st = stepped_state(built_pkg, sc, precision)
    kept = upload(a, st, route != "pageable", mapped=route == "mapped")
    with pytest.raises(built_pkg.RDError):
        a.get_grid()  # nothing to export before a step, as after any upload
    b = make(built_pkg, sc, precision)
    upload(b, st)
    l0 = a.launch_count()
    a.step(sc.dt, 1)
    if route == "pageable":
        assert a.launch_count() - l0 > 2
    else:
        # sorted, and both grids cleared, during the upload: the step is k_p2g and the fused kernel
        assert a.launch_count() - l0 == 2
    a.step(sc.dt, 2)
    b.step(sc.dt, 3)
    same_state(a.get_particles(FIELDS), b.get_particles(FIELDS), sc.h, 1e-10 if precision else 1e-5)
    ga, gb = a.get_grid(), b.get_grid()
    assert rel(ga["mass"], gb["mass"]) < 1e-6
    assert a.flags() == 0 and b.flags() == 0
    del kept


def test_upload_then_another_dt(built_pkg):
    """After a sorted upload the steps may change dt (each change rasterizes
    the grid again)."""
    from rd_gb300 import scenes
    sc = scenes.snowball(seed=6, n=5000, grid=32)
    a, st = stepped_state(built_pkg, sc)
    kept = upload(a, st, pinned=True)
    b = make(built_pkg, sc)
    upload(b, st)
    for dt, k in ((0.5 * sc.dt, 2), (sc.dt, 2)):
        a.step(dt, k)
        b.step(dt, k)
    same_state(a.get_particles(FIELDS), b.get_particles(FIELDS), sc.h, 2e-5)
    del kept


def test_upload_after_a_step_matches_oracle(built_pkg, orc):
    from rd_gb300 import scenes
    sc = scenes.snowball(seed=7, n=6000, grid=32)
    a, st = stepped_state(built_pkg, sc)
    upload(a, st, pinned=True)
    a.step(sc.dt, 1)
    kw = dict(sc.params())
    kw.pop("track_fp", None)
    kw.pop("precision", None)
    if "lagged_b" in kw:
        kw["lagged_c"] = kw.pop("lagged_b")
    FP = (np.cbrt(st["Jp"].astype(np.float64))[:, None] * np.eye(3).reshape(1, 9)).astype(np.float32)
    o = orc.OracleSim(orc.Params(*sc.grid, float(sc.h), **kw), st["x"], st["v"], st["mass"], st["B"], st["FE"], FP,
                      vol=st["volume"])
    o.step(sc.dt, 1)
    got = a.get_particles(FIELDS)
    for k in ("x", "v", "FE"):
        assert rel(got[k], getattr(o, k)) < 1e-5, k
    assert rel_floor(got["B"], o.B, b_scale(o.v, sc.h)) < 1e-5
    grd = a.get_grid()
    assert rel(grd["mass"], o.gmass) < 1e-6


def test_upload_with_a_particle_outside_the_domain(built_pkg):
    """A particle whose stencil leaves the grid, uploaded after a step: the same
    flags and the same state as through a fresh handle."""
    from rd_gb300 import scenes
    sc = scenes.snowball(seed=8, n=3000, grid=32)
    a, st = stepped_state(built_pkg, sc)
    st["x"][17] = (0.3 * sc.h, 0.5, 0.5)
    kept = upload(a, st, pinned=True)
    b = make(built_pkg, sc)
    upload(b, st)
    a.step(sc.dt, 2)
    b.step(sc.dt, 2)
    assert a.flags() == b.flags() and a.flags() & built_pkg.FLAG_OUT_OF_DOMAIN
    same_state(a.get_particles(FIELDS), b.get_particles(FIELDS), sc.h, 1e-5)
    del kept
