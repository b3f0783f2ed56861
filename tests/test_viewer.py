"""Headless viewer feed (main.cpp:255-271): the xyzs and colour streams, and the
CUDA point-splat image against its numpy restatement."""
import numpy as np
import pytest


def test_look_at_view_centres_the_target(pkg):
    v = pkg.look_at_view((0.5, 0.5, 2.0), (0.5, 0.5, 0.5), width=64, height=48)
    M = np.asarray(list(v.view_projection), np.float64).reshape(4, 4).T
    c = M @ np.array([0.5, 0.5, 0.5, 1.0])
    assert abs(c[0] / c[3]) < 1e-6 and abs(c[1] / c[3]) < 1e-6 and -1 < c[2] / c[3] < 1


@pytest.mark.gpu
def test_splat_matches_restatement(built_pkg, orc):
    from rd_gb300 import scenes
    sc = scenes.snowball(seed=2, n=3000, grid=32)
    sim = built_pkg.Simulation(built_pkg.make_params(*sc.grid, sc.n, sc.h))
    sim.set_particles(sc.x, sc.v, sc.mass)
    rng = np.random.default_rng(0)
    rgba = rng.integers(0, 256, (sc.n, 4), dtype=np.uint8)
    sim.set_colors(rgba)
    view = built_pkg.look_at_view((0.62, 0.72, 0.95), (0.5, 0.6, 0.5), width=160, height=120)
    img = sim.splat(view)
    xyzs = np.concatenate([sc.x, np.full((sc.n, 1), 0.02, np.float32)], axis=1)
    ref, ids = orc.splat_image(xyzs, rgba.view(np.uint32).reshape(-1), list(view.view_projection),
                               list(view.camera_right), list(view.camera_up), 160, 120, view.background)
    got = img.view(np.uint32).reshape(120, 160)
    assert (ids >= 0).mean() > 0.1  # the ball covers part of the image
    same = got == ref
    assert same.mean() > 0.99, same.mean()
    # where they differ it is a disc edge: both pixels are covered or both background
    assert np.all((got[~same] == view.background) == (ref[~same] == view.background)) or (~same).mean() < 0.002
    # the streams drawParticles would upload
    assert sim.device_xyzs() != 0
