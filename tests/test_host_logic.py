"""Host-side logic behind the benchmark numbers, on the CPU: the seeded scenes
are reproducible and start inside the domain the step keeps particles in, and
the roofline helpers read and scale the committed ncu record."""
import json

import numpy as np
import pytest

import bench


def _inside_clamp(sc):
    """All particles within [3h, (M - 3)h] on every axis (the advection clamp,
    material_point_method.cpp:381-388), so the first step moves no particle by
    clamping alone."""
    h = sc.h
    lo = 3.0 * h
    hi = (np.asarray(sc.grid, np.float64) - 3.0) * h
    x = sc.x.astype(np.float64)
    return bool(np.all(x >= lo) and np.all(x <= hi))


def test_headline_scene_is_seeded_and_inside_the_domain():
    from rd_gb300 import scenes
    a, b = scenes.two_balls_1m(seed=0), scenes.two_balls_1m(seed=0)
    assert a.n == 1_100_000 and a.grid == (128, 128, 128)
    assert np.array_equal(a.x, b.x) and np.array_equal(a.mass, b.mass)
    assert not np.array_equal(a.x, scenes.two_balls_1m(seed=1).x)
    assert _inside_clamp(a)
    # each half fills its sphere and carries half of the total mass
    c = np.array([[0.3, 0.5, 0.5], [0.7, 0.55, 0.5]])
    half = a.n // 2
    for k, part in enumerate((slice(0, half), slice(half, a.n))):
        d = np.linalg.norm(a.x[part].astype(np.float64) - c[k], axis=1)
        assert d.max() <= 0.15 + 1e-6
    m = a.mass.astype(np.float64)
    assert abs(m[:half].sum() - m[half:].sum()) / m.sum() < 1e-6
    assert np.all(a.v[:half, 0] == 3.0) and np.all(a.v[half:, 0] == -3.0)


def test_uneven_batch_scenes_fit_their_grids():
    from rd_gb300 import scenes
    batch = scenes.uneven_snowballs(seed=0)
    again = scenes.uneven_snowballs(seed=0)
    assert len(batch) == 64
    ns = np.array([s.n for s in batch])
    assert ns.min() >= 4096 and ns.max() <= 262144
    assert ns.sum() == sum(s.n for s in again)
    for s, t in zip(batch, again):
        assert s.grid == t.grid and np.array_equal(s.x, t.x)
        assert 32 <= s.grid[0] and s.grid[0] == s.grid[1] == s.grid[2]
        assert _inside_clamp(s), s.name
        # radius set by the particle count at 8 per cell
        r = np.linalg.norm(s.x.astype(np.float64) - [0.5, 0.55, 0.5], axis=1).max() / s.h
        assert r <= (3.0 * s.n / (32.0 * np.pi)) ** (1.0 / 3.0) + 1e-3
        assert 5e4 <= s.material["E"] <= 3e5 and 0.15 <= s.material["nu"] <= 0.3


def test_captured_traffic_scales_by_particles():
    rec = None
    for line in open(bench.os.path.join(bench.REPO, "profiles", "traffic.txt")):
        f = line.split()
        if line.startswith("#") or len(f) < 5:
            continue
        if f[0] == "k_g2p2g" and f[1] == "two_balls_1m":
            rec = (int(f[2]), int(f[3]) + int(f[4]))
    assert rec is not None
    assert bench.captured_traffic("k_g2p2g", "two_balls_1m", rec[0]) == pytest.approx(rec[1])
    assert bench.captured_traffic("k_g2p2g", "two_balls_1m", rec[0] // 2) == pytest.approx(rec[1] / 2, rel=1e-6)
    assert bench.captured_traffic("k_g2p2g", "no_such_workload", 10) is None
    # the record agrees with the kernel's algorithmic bytes per particle within
    # 10% (DRAM traffic can fall below them: part of the written state is still
    # in the 129 MB L2 when the kernel ends, and the active nodes' bytes are not
    # counted here)
    bpp, bpc = bench.KERNEL_BYTES["g2p2g"]
    assert abs(rec[1] / (bpp * rec[0]) - 1.0) < 0.10


def test_captured_issue_scales_by_particles_and_fits_the_kernel():
    """profiles/issue.txt: the warp instructions of the fused kernel's launch
    (mean over the bench's timed launches), scaled by particle count, with the
    record it came from; between 60 and 200 warp instructions a particle (a
    gather, a split and a scatter per particle cannot take fewer, and more would
    mean a capture of another kernel)."""
    rec = None
    for line in open(bench.os.path.join(bench.REPO, "profiles", "issue.txt")):
        f = line.split()
        if line.startswith("#") or len(f) < 5:
            continue
        if f[0] == "k_g2p2g" and f[1] == "two_balls_1m":
            rec = (int(f[2]), int(f[3]), f[4])
    assert rec is not None
    inst, src = bench.captured_issue("k_g2p2g", "two_balls_1m", rec[0])
    assert inst == pytest.approx(rec[1]) and src == rec[2]
    assert bench.os.path.exists(bench.os.path.join(bench.REPO, src))
    half, _ = bench.captured_issue("k_g2p2g", "two_balls_1m", rec[0] // 2)
    assert half == pytest.approx(rec[1] / 2, rel=1e-6)
    assert bench.captured_issue("k_g2p2g", "no_such_workload", 10) == (None, None)
    assert 60.0 <= rec[1] / rec[0] <= 200.0


def test_peak_reads_the_measured_file_or_falls_back(tmp_path, monkeypatch):
    monkeypatch.setattr(bench, "REPO", str(tmp_path))
    assert bench.measured_peak_hbm() == (6800.0, "fallback")
    (tmp_path / "MEASURED_PEAKS.json").write_text(json.dumps({"hbm_gbs": 6686.0}))
    assert bench.measured_peak_hbm() == (6686.0, "measured")


def _worker_that_dies(conn, what, core):
    """A reference run that ends without a result (exit code 3)."""
    import os
    os._exit(3)


def _worker_that_answers(conn, what, core):
    conn.send({"what": what, "kind": "test"})
    conn.close()


def test_next_rows_reference_runs_apart_and_survives_a_dying_child(monkeypatch):
    """bench.measure_next_rows times the reference's code in a spawned process:
    a child that answers is passed through, one that dies is reported
    unavailable with its exit code and the caller goes on."""
    orc = bench.graft.load_oracle()
    monkeypatch.setattr(orc, "ref_available", lambda: True)
    assert bench._next_rows_reference("colliders", 60.0, _worker_that_answers) == {"what": "colliders",
                                                                                   "kind": "test"}
    out = bench._next_rows_reference("colliders", 60.0, _worker_that_dies)
    assert "unavailable" in out and "exit code 3" in out["unavailable"]

