"""Batches of uneven scenes in one handle (rd_batch_*), CUDA-graph replay and
the autotuner.  Every scene of a batch must step exactly as it does alone:
against the oracle for the physics, against a single-scene handle for the
batching itself."""
import numpy as np
import pytest

from conftest import b_scale, rel, rel_floor

pytestmark = pytest.mark.gpu


def small_batch(seed=5, nscenes=5):
    """Uneven scenes: particle counts, grid sizes, materials and velocities all differ."""
    from rd_gb300 import scenes
    return scenes.uneven_snowballs(seed=seed, nscenes=nscenes, n_lo=1500, n_hi=12000, g_lo=24, g_hi=48)


def scene_params(pkg, sc, **over):
    return pkg.make_params(*sc.grid, sc.n, sc.h, **sc.params(**over))


def oracle_of(orc, sc):
    kw = sc.params()
    o = orc.OracleSim(orc.Params(*sc.grid, float(sc.h), **kw), sc.x, sc.v, sc.mass)
    o.init()
    return o


def make_batch(pkg, batch, **over):
    b = pkg.Batch([scene_params(pkg, sc, **over) for sc in batch])
    for s, sc in enumerate(batch):
        b.set_particles(s, sc.x, sc.v, sc.mass)
    b.init_volumes()
    return b


def compare(got, o, h, tol):
    errs = {"x": rel(got["x"], o.x), "v": rel(got["v"], o.v),
            "B": rel_floor(got["B"], o.B, b_scale(o.v, h)), "FE": rel(got["FE"], o.FE), "Jp": rel(got["Jp"], o.Jp)}
    assert all(e < tol for e in errs.values()), errs
    return errs


def test_batch_one_step_matches_oracle_per_scene(built_pkg, orc):
    batch = small_batch()
    b = make_batch(built_pkg, batch)
    assert b.nscenes == len(batch)
    orcs = [oracle_of(orc, sc) for sc in batch]
    for s, o in enumerate(orcs):
        assert rel(b.get_particles(s, ("volume",))["volume"], o.vol) < 1e-6
    b.step(batch[0].dt, 1)
    for s, (sc, o) in enumerate(zip(batch, orcs)):
        o.step(sc.dt, 1)
        compare(b.get_particles(s), o, sc.h, 1e-5)
        g = b.get_grid(s)
        assert rel(g["mass"], o.gmass) < 1e-6
        assert rel(g["mass"][:, None] * g["vel"], o.gmass[:, None] * o.gvel) < 1e-5
    assert b.flags() == 0


def test_batch_rollout_matches_single_scene_handles(built_pkg):
    """20 steps (graph replay included): each scene of the batch against the
    same scene in its own handle; only the order of FP32 atomics differs."""
    batch = small_batch(seed=6)
    b = make_batch(built_pkg, batch)
    singles = []
    for sc in batch:
        s = built_pkg.Simulation(scene_params(built_pkg, sc))
        s.set_particles(sc.x, sc.v, sc.mass)
        s.init_volumes()
        s.step(sc.dt, 20)
        singles.append(s)
    b.step(batch[0].dt, 20)
    for s, (sc, single) in enumerate(zip(batch, singles)):
        got, ref = b.get_particles(s), single.get_particles()
        for k in ("x", "v", "FE", "Jp"):
            assert rel(got[k], ref[k]) < 2e-5, (s, k, rel(got[k], ref[k]))
        assert rel_floor(got["B"], ref["B"], b_scale(ref["v"], sc.h)) < 2e-5
        total = float(np.sum(sc.mass, dtype=np.float64))
        gm = b.get_grid(s)["mass"]
        assert abs(float(np.sum(gm, dtype=np.float64)) - total) / total < 1e-6
    assert b.flags() == 0


def test_graph_replay_matches_eager_launches(built_pkg):
    from rd_gb300 import scenes
    sc = scenes.snowball(seed=4, n=6000, grid=32)
    out = []
    for graphs in (True, False):
        s = built_pkg.Simulation(scene_params(built_pkg, sc))
        s.set_graphs(graphs)
        s.set_particles(sc.x, sc.v, sc.mass)
        s.init_volumes()
        s.step(sc.dt, 3)
        l0 = s.launch_count()
        s.step(sc.dt, 10)
        # steady steps: tile prefix (summing the tiles itself on a grid this
        # small), scan, scatter, grid clear and the fused kernel
        assert s.launch_count() - l0 == 50
        out.append(s.get_particles())
    for k in ("x", "v", "FE", "Jp"):
        assert rel(out[0][k], out[1][k]) < 1e-5


@pytest.mark.parametrize("precision", [0, 1])
def test_steady_steps_replay_graphs_in_batches_and_single_scenes(built_pkg, precision):
    """dt = 1e-4 has no exact FP32 value: the batch's scene table, built with
    dt in the arithmetic type, still counts as current for the graph."""
    batch = small_batch(seed=8, nscenes=3)
    dt_ = np.float64 if precision else np.float32
    handles = [built_pkg.Batch([scene_params(built_pkg, sc, precision=precision) for sc in batch]),
               built_pkg.Simulation(scene_params(built_pkg, batch[0], precision=precision))]
    for i, sc in enumerate(batch):
        handles[0].set_particles(i, sc.x.astype(dt_), sc.v.astype(dt_), sc.mass.astype(dt_))
    sc = batch[0]
    handles[1].set_particles(sc.x.astype(dt_), sc.v.astype(dt_), sc.mass.astype(dt_))
    for h in handles:
        h.init_volumes()
        h.step(1e-4, 3)
        r0 = h.graph_replays()
        h.step(1e-4, 10)
        assert h.graph_replays() - r0 == 5
        assert h.flags() == 0


def test_autotune_picks_a_valid_pair_and_restores_state(built_pkg):
    batch = small_batch(seed=7, nscenes=4)
    dt = batch[0].dt
    tuned = make_batch(built_pkg, batch)
    ref = make_batch(built_pkg, batch)
    r = tuned.autotune(dt, steps=4)
    assert r["particles_per_item"] in (64, 128, 192, 256)
    assert r["trials"] >= 8 and r["ms_per_step"] > 0 and not r["from_cache"]
    trials = tuned.tune_trials()
    assert len(trials) == r["trials"]
    assert {t["scatter"] for t in trials} == {"lane_pairs", "record_pairs"}
    assert min(t["ms_per_step"] for t in trials) == pytest.approx(r["ms_per_step"])
    layout = {"lane_pairs": built_pkg.SCATTER_LANE_PAIRS, "record_pairs": built_pkg.SCATTER_RECORD_PAIRS}
    assert tuned.tuning() == (r["particles_per_item"], r["ctas_per_sm"], layout[r["scatter"]])
    tuned.step(dt, 5)
    ref.step(dt, 5)
    for s in range(len(batch)):
        a, c = tuned.get_particles(s), ref.get_particles(s)
        for k in ("x", "v", "Jp"):
            assert rel(a[k], c[k]) < 1e-5, (s, k)


def test_autotune_cache_round_trip(built_pkg, tmp_path):
    """A tuned point goes to the cache file under the handle's key; a second
    handle of the same scenes takes it from there without timing."""
    batch = small_batch(seed=10, nscenes=3)
    dt = batch[0].dt
    cache = str(tmp_path / "tune.txt")
    first = make_batch(built_pkg, batch)
    r1 = first.autotune(dt, steps=3, cache=cache)
    assert not r1["from_cache"] and r1["trials"] > 0
    second = make_batch(built_pkg, batch)
    assert second.tune_key() == first.tune_key()
    r2 = second.autotune(dt, steps=3, cache=cache)
    assert r2["from_cache"] and r2["trials"] == 0 and second.tune_trials() == []
    for k in ("particles_per_item", "ctas_per_sm", "scatter"):
        assert r2[k] == r1[k], k
    assert second.tuning() == first.tuning()


@pytest.mark.parametrize("wp,scatter", [(64, 0), (128, 0), (192, 0), (128, 1), (256, 1)])
def test_item_size_and_scatter_layout_do_not_change_results(built_pkg, orc, wp, scatter):
    from rd_gb300 import scenes
    sc = scenes.snowball(seed=8, n=5000, grid=32)
    s = built_pkg.Simulation(scene_params(built_pkg, sc))
    s.set_tuning(wp, 1, scatter)
    assert s.tuning()[2] == scatter
    s.set_particles(sc.x, sc.v, sc.mass)
    s.init_volumes()
    o = oracle_of(orc, sc)
    s.step(sc.dt, 1)
    o.step(sc.dt, 1)
    compare(s.get_particles(), o, sc.h, 1e-5)


def test_batch_rejects_single_scene_calls_and_unset_scenes(built_pkg):
    pkg = built_pkg
    batch = small_batch(seed=9, nscenes=3)
    b = pkg.Batch([scene_params(pkg, sc) for sc in batch])
    with pytest.raises(pkg.RDError):
        b.step(1e-4, 1)  # scene particles not set
    for s, sc in enumerate(batch):
        b.set_particles(s, sc.x, sc.v, sc.mass)
    with pytest.raises(pkg.RDError):
        b.stage("rasterize")
    with pytest.raises(pkg.RDError):
        pkg.Simulation.set_particles(b, np.zeros((b.n, 3)), np.zeros((b.n, 3)), np.ones(b.n))
    with pytest.raises(pkg.RDError):
        pkg.Batch([scene_params(pkg, sc, track_fp=1) for sc in batch])
    with pytest.raises(pkg.RDError):
        b.set_particles(-1, batch[-1].x, batch[-1].v, batch[-1].mass)  # no scene -1
    b.init_volumes()
    b.step(1e-4, 2)
    assert b.flags() == 0


def test_pinned_host_buffers_are_used_in_place_and_match_staged_copies(built_pkg):
    """rd_set_particles / rd_get_particles with pageable host arrays (copied
    through the device staging buffer), with page-locked ones under RD_HOST
    (read and written in place by the pack and unpack kernels) and with
    page-locked ones passed as device-accessible pointers (RD_DEVICE) give
    the same state; rd_io_bytes tells the first two routes apart."""
    import torch
    from rd_gb300 import scenes
    sc = scenes.snowball(seed=12, n=4000, grid=32)
    src = {"x": sc.x, "v": sc.v, "mass": sc.mass}
    shapes = {"x": (sc.n, 3), "v": (sc.n, 3), "FE": (sc.n, 9)}
    state_bytes = sum(a.size * 4 for a in src.values())
    out_bytes = sum(int(np.prod(s)) * 4 for s in shapes.values())
    out = []
    for route in ("pageable", "pinned", "mapped"):
        pin = route != "pageable"
        arr = {k: (torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy() if pin else np.array(a))
               for k, a in src.items()}
        res = {k: (torch.empty(s, dtype=torch.float32).pin_memory().numpy() if pin else np.empty(s, np.float32))
               for k, s in shapes.items()}
        s = built_pkg.Simulation(scene_params(built_pkg, sc))
        s.set_particles(arr["x"], arr["v"], arr["mass"], mapped=route == "mapped")
        s.init_volumes()
        s.step(sc.dt, 3)
        s.get_particles(("x", "v", "FE"), out=res, mapped=route == "mapped")
        s.synchronize()
        in_place, staged = s.io_bytes()
        if route == "pageable":
            assert (in_place, staged) == (0, state_bytes + out_bytes)
        elif route == "pinned":
            assert (in_place, staged) == (state_bytes + out_bytes, 0)
        else:  # RD_DEVICE: not host I/O
            assert (in_place, staged) == (0, 0)
        out.append({k: a.copy() for k, a in res.items()})
        assert s.flags() == 0
    for o in out[1:]:
        for k in shapes:
            assert rel(o[k], out[0][k]) < 1e-6, k
