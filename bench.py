#!/usr/bin/env python3
"""Benchmark of the explicit APIC / MLS-MPM snow step on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload two_balls_1m|two_balls|snowball|cube]

One "step" is one full MPM step (sort, P2G with the MLS force, grid update,
G2P with the plastic SVD and advection) over every particle of the workload.
The metric is particle-steps per second.  Prints one JSON line (rank 0).

* ours (default): the CUDA path through the C ABI.  ``value`` is timed with
  CUDA events on the handle's stream with the particle state resident in HBM;
  ``e2e`` times the same steps through the C ABI with the whole particle state
  moved in from page-locked host memory and back out every step (the pack and
  unpack kernels read and write it in place; pageable arrays, copied through
  a staging buffer, are reported beside it); ``roofline``
  comes from a second pass of the same steps with per-kernel CUDA events.
  Multi-GPU (torchrun): one independent replica per GPU (the step has no
  exchange between scenes), barrier-bracketed, max over ranks.
* reference: the reference's CPU step on this host's cores - the headless
  build of the reference where it is loadable here, else the C restatement of
  it - one independent replica per core, each step a bounded sample of the
  workload's particles on the workload's grid.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

import __graft_entry__ as graft  # noqa: E402

# Bytes the step must move per particle-step and per active grid cell-step
# (FP32): the particle state read once (x 12, v 12, B 36, F_E 36, J_P 4, m 4,
# V 4) and written once (x, v, B, F_E, J_P); per active cell P2G writes (m, mv)
# 16 B, the grid update reads 16 and writes v 12, G2P reads v 12.
STEP_BYTES_PER_PARTICLE = 208
STEP_BYTES_PER_CELL = 44
# Per kernel (FP32, what each kernel must move per particle / per active cell):
#   k_p2g (first step only) reads x, m, v, V, B, F_E, J_P (108 B), writes the
#     particle to its sorted slot for the fused kernel (108 B and its id, 4 B)
#     and adds (m, p) into its cells (16 B);
#   k_g2p2g reads x, m, V, B, F_E, J_P (96 B), writes the particle at its sorted
#     slot (x, m, v, V, B, F_E, J_P: 108 B) and its next block key (4 B); it
#     reads this step's cell (m, p) (16 B) and adds the next step's (16 B).
KERNEL_BYTES = {"p2g": (108 + 112, 16), "g2p2g": (96 + 108 + 4, 32)}


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=500)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=("ours", "reference"), default="ours")
    ap.add_argument("--workload", default="two_balls_1m")
    ap.add_argument("--e2e-steps", type=int, default=50)
    ap.add_argument("--cpu-baseline", type=int, default=1, help="time the single-core CPU baseline (rank 0, N=1)")
    ap.add_argument("--adjoint", type=int, default=1, help="measure forward + adjoint on the 65,536-particle cube")
    ap.add_argument("--only", choices=("batched", "adjoint", "batched_adjoint", "snowball", "implicit", "profile",
                                       "profile_batched", "next_rows"),
                    default=None,
                    help="run one secondary measurement alone and print its JSON; 'profile' only initialises "
                         "the workload and runs --warmup + --steps steps (for ncu captures), 'profile_batched' "
                         "the same for the 64-scene batch at its default tuning")
    ap.add_argument("--snowball", type=int, default=1, help="measure the 8,192-particle snowball on 64^3")
    ap.add_argument("--link", type=int, default=1, help="measure the host link (pinned copies each way)")
    ap.add_argument("--implicit", type=int, default=1, help="time timeIntegration (implicit L-BFGS)")
    ap.add_argument("--next-rows", type=int, default=1,
                    help="time the colliders, the initialiser and the viewer feed against the reference")
    ap.add_argument("--batch-steps", type=int, default=-1,
                    help="timed steps of the batched-forward workload (64 uneven scenes); -1: as many as "
                         "--steps, so the batch and the plain forward it is compared with run equally long; "
                         "0 skips it")
    return ap.parse_args()


def dist_init(backend):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group(backend=backend)
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(ws, value, device=None):
    if ws == 1:
        return value
    import torch
    import torch.distributed as dist
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons while running."""
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                                          "-lms", "100", "-i", str(self.gpu)], stdout=open(self.path, "w"),
                                         stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        time.sleep(0.25)
        if self.proc:
            self.proc.terminate()
            self.proc.wait()

    def summary(self):
        rows = []
        if self.path and os.path.exists(self.path):
            for line in open(self.path):
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
            os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None

        sm = [num(r[1]) for r in rows if num(r[1]) is not None]
        smax = [num(r[2]) for r in rows if num(r[2]) is not None]
        loaded = [s for s in sm if smax and s > 0.5 * max(smax)] or sm
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(loaded) if loaded else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": reasons, "samples": len(rows),
                "power_w_max": max((num(r[3]) or 0.0) for r in rows)}


def measured_peak_hbm():
    path = os.path.join(REPO, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def make_scene(name, seed):
    graft.load_package()  # also in spawned worker processes
    from rd_gb300 import scenes
    return scenes.SCENES[name](seed=seed)


def captured_traffic(kernel, workload, particles):
    """DRAM bytes per launch of `kernel` from the ncu record in profiles/traffic.txt,
    scaled by particle count to this workload, or None."""
    path = os.path.join(REPO, "profiles", "traffic.txt")
    try:
        for line in open(path):
            f = line.split()
            if len(f) >= 5 and not line.startswith("#") and f[0] == kernel and f[1] == workload:
                return (int(f[3]) + int(f[4])) * particles / int(f[2])
    except OSError:
        pass
    return None


def captured_issue(kernel, workload, particles):
    """Warp instructions per launch of `kernel` (ncu smsp__inst_executed.sum)
    from profiles/issue.txt, scaled by particle count to this workload, and the
    record's source, or (None, None)."""
    path = os.path.join(REPO, "profiles", "issue.txt")
    try:
        for line in open(path):
            f = line.split()
            if len(f) >= 5 and not line.startswith("#") and f[0] == kernel and f[1] == workload:
                return int(f[3]) * particles / int(f[2]), f[4]
    except OSError:
        pass
    return None, None


def cpu_model():
    """The host CPU's model string (lscpu, else /proc/cpuinfo)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    import platform
    return platform.machine()


def pin_to_core(core):
    """Restricts this process to one core (as taskset does); returns the
    previous affinity to restore, or None where affinity cannot be set."""
    try:
        old = os.sched_getaffinity(0)
        os.sched_setaffinity(0, {core})
        return old
    except (AttributeError, OSError):
        return None


def oracle_for(orc, sc):
    """The reference's CPU step for the workload: its headless build where it is
    loadable here (it has no grid walls, so it steps without them), else the C
    restatement (with the workload's walls).  Returns (sim, kind)."""
    mat = {k: v for k, v in sc.material.items()}
    if orc.ref_available():
        return orc.RefSim(orc.Params(*sc.grid, sc.h, **mat), sc.x, sc.v, sc.mass, p4=1), "reference"
    P = orc.Params(*sc.grid, sc.h, bc=sc.bc, bc_width=sc.bc_width, **mat)
    return orc.OracleSim(P, sc.x, sc.v, sc.mass), "port"


def cpu_baseline_single_core(sc, seconds_hint=20.0):
    """The oracle (the headless reference where loadable, else the C
    restatement) timed on one pinned core for one full step of the workload
    after its init; returns (particle-steps/s, kind, sample description)."""
    orc = graft.load_oracle()
    orc.build_oracle()
    sim, kind = oracle_for(orc, sc)
    sim.init()
    core = sorted(os.sched_getaffinity(0))[-1] if hasattr(os, "sched_getaffinity") else 0
    old = pin_to_core(core)
    try:
        t0 = time.perf_counter()
        sim.step(sc.dt, 1)
        dt = time.perf_counter() - t0
    finally:
        if old is not None:
            os.sched_setaffinity(0, old)
    pinned = f"pinned to core {core}" if old is not None else "unpinned"
    return sc.n / dt, kind, (f"1 step of all {sc.n} particles after init, single thread {pinned} "
                             f"({dt:.1f} s) on {cpu_model()}")


def measure_link(local, nbytes=1 << 30, reps=3):
    """The host link alone: one cudaMemcpyAsync of `nbytes` from page-locked
    host memory to the device and one back, CUDA events on one stream, best of
    `reps`; GB/s each way."""
    import torch
    host = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
    dev = torch.empty(nbytes, dtype=torch.uint8, device=torch.device("cuda", local))
    st = torch.cuda.Stream(device=local)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    best = {"h2d": float("inf"), "d2h": float("inf")}
    with torch.cuda.stream(st):
        for _ in range(reps + 1):
            for way in ("h2d", "d2h"):
                e0.record(st)
                if way == "h2d":
                    dev.copy_(host, non_blocking=True)
                else:
                    host.copy_(dev, non_blocking=True)
                e1.record(st)
                e1.synchronize()
                best[way] = min(best[way], e0.elapsed_time(e1))
    del host, dev
    return {k: nbytes / (v / 1e3) / 1e9 for k, v in best.items()}


def measure_snowball(pkg, local, warmup):
    """The 8,192-particle snowball on 64^3 for its 200 steps (graph-pair replay):
    a launch- and latency-bound step, autotuned first (small work items give
    more CTAs); CUDA events on the handle's stream."""
    import torch
    graft.load_package()
    from rd_gb300 import scenes
    sc = scenes.snowball()
    sim = pkg.Simulation(pkg.make_params(*sc.grid, sc.n, sc.h, device=local, **sc.params()))
    stream = torch.cuda.ExternalStream(sim.stream(), device=local)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    sim.set_particles(sc.x, sc.v, sc.mass)
    sim.init_volumes()
    tune = sim.autotune(sc.dt, steps=20)
    tune["candidates"] = sim.tune_trials()
    best = None
    for _ in range(3):
        sim.set_particles(sc.x, sc.v, sc.mass)
        sim.init_volumes()
        sim.step(sc.dt, warmup)
        sim.synchronize()
        l0, r0 = sim.launch_count(), sim.graph_replays()
        e0.record(stream)
        sim.step(sc.dt, sc.steps)
        e1.record(stream)
        e1.synchronize()
        ms = e0.elapsed_time(e1)
        if best is None or ms < best[0]:
            best = (ms, sim.launch_count() - l0, sim.graph_replays() - r0)
    flags = sim.flags()
    sim.close()
    ms, launches, replays = best
    return {"value": sc.n * sc.steps / (ms / 1e3), "unit": "particle-steps/s", "steps": sc.steps,
            "warmup": warmup, "ms_per_step": ms / sc.steps, "gpu_launches": launches, "graph_replays": replays,
            "flags": flags, "timing": "best of 3 passes from the initial state", "tuning": tune,
            "workload": "snowball: 8,192 particles uniform in a sphere r = 0.1 at (0.5, 0.6, 0.5), 64^3, "
                        "v0 = (0, -2, 0), sticky walls, 200 steps, FP32"}


def implicit_ball(n, G, seed=3):
    """A ball of n particles (r = 0.12 at the centre) on a G^3 grid with random
    velocities and near-identity F_E: the shape of the reference's own test of
    timeIntegration (40 particles on 12^3)."""
    from rd_gb300 import scenes
    rng = np.random.default_rng(seed)
    x = scenes.uniform_ball(rng, n, (0.5, 0.5, 0.5), 0.12).astype(np.float32)
    v = rng.normal(0, 0.5, (n, 3)).astype(np.float32)
    m = np.full(n, 1e-3, np.float32)
    FE = (np.eye(3).reshape(1, 9) + 0.02 * rng.normal(size=(n, 9))).astype(np.float32)
    return x, v, m, FE


def measure_implicit(pkg, local, reps=5):
    """timeIntegration (the implicit L-BFGS over the grid velocities) at the
    reference's settings: on its own test's shape (40 particles, 12^3, dt 1e-3)
    against the reference's timeIntegration timed on one host core, and on the
    8,192-particle snowball on 64^3 after one explicit grid update.  Host wall
    time per call (the solver's host loop reads every dot product back)."""
    graft.load_package()
    from rd_gb300 import scenes
    out = {}
    G, n, dt = 12, 40, 1e-3
    x, v, m, FE = implicit_ball(n, G)
    sim = pkg.Simulation(pkg.make_params(G, G, G, n, 1.0 / G, device=local))
    best, res = None, None
    for _ in range(reps):
        sim.set_particles(x, v, m, FE=FE)
        sim.init_volumes()
        sim.stage("rasterize")
        sim.synchronize()
        t0 = time.perf_counter()
        res = sim.time_integration(dt)
        el = time.perf_counter() - t0
        best = el if best is None or el < best else best
    vel_ours = sim.get_grid()["vel"].astype(np.float64)
    sim.close()
    # both minimisers' results scored by one energy: the oracle's, FP64, at
    # the v* of this state (the reference's Energy reads v* from the grid it
    # overwrites, so its own value afterwards leaves out the kinetic term)
    orc = graft.load_oracle()
    o = orc.OracleSim(orc.Params(G, G, G, 1.0 / G), x, v, m, FE=FE, dtype=np.float64)
    o.init()
    o.stage("rasterize")
    small = {"workload": f"ball of {n} particles on {G}^3 (the reference's implicit test shape), dt {dt}, FP32, "
                         "the reference's L-BFGS settings",
             "ms_per_call": best * 1e3, "iterations": res["iterations"], "evaluations": res["evaluations"],
             "unknowns": res["unknowns"], "energy_start": res["energy_start"], "energy": res["energy"],
             "energy_fp64": o.implicit_energy(vel_ours, dt), "converged": res["converged"]}
    if orc.ref_available():
        r = orc.RefSim(orc.Params(G, G, G, 1.0 / G), x, v, m, FE=FE, p4=1)
        r.init()
        r.stage("rasterize")
        core = sorted(os.sched_getaffinity(0))[-1] if hasattr(os, "sched_getaffinity") else 0
        old = pin_to_core(core)
        try:
            t0 = time.perf_counter()
            r.time_integration(dt)
            el = time.perf_counter() - t0
        finally:
            if old is not None:
                os.sched_setaffinity(0, old)
        small["reference"] = {"ms_per_call": el * 1e3,
                              "energy_fp64": o.implicit_energy(r.grid()["vel"].astype(np.float64), dt), "cores": 1,
                              "cpu_model": cpu_model(),
                              "kind": "reference: its timeIntegration (L-BFGS on finite-difference gradients of "
                                      "Energy), compiled headless on this host"}
    else:
        small["reference"] = {"unavailable": "the headless reference build is not present on this host"}
    out["reference_shape"] = small
    sc = scenes.snowball()
    sim = pkg.Simulation(pkg.make_params(*sc.grid, sc.n, sc.h, device=local, **sc.params()))
    best = None
    for _ in range(3):
        sim.set_particles(sc.x, sc.v, sc.mass)
        sim.init_volumes()
        for st in ("rasterize", "forces"):
            sim.stage(st)
        sim.stage("grid_velocities", sc.dt)
        sim.synchronize()
        t0 = time.perf_counter()
        res = sim.time_integration(sc.dt)
        el = time.perf_counter() - t0
        best = el if best is None or el < best else best
    flags = sim.flags()
    sim.close()
    out["snowball"] = {"workload": "snowball: 8,192 particles, 64^3, after rasterize, forces and the grid update, "
                                   "FP32, the reference's L-BFGS settings",
                       "ms_per_call": best * 1e3, "iterations": res["iterations"],
                       "evaluations": res["evaluations"], "unknowns": res["unknowns"],
                       "energy_start": res["energy_start"], "energy": res["energy"],
                       "converged": res["converged"],
                       "particle_evaluations_per_s": sc.n * res["evaluations"] / best, "flags": flags}
    return out


def _next_rows_reference_worker(conn, what, core):
    """Child process (spawned): times the reference's own code for one of
    measure_next_rows' rows on one pinned core and sends the result back."""
    try:
        graft.load_package()
        from rd_gb300 import scenes
        orc = graft.load_oracle()
        pin_to_core(core)
        if what in ("colliders", "colliders_port"):
            sc = scenes.snowball()
            kw = sc.params()
            P = orc.Params(*sc.grid, float(sc.h), **{k: v for k, v in kw.items()
                                                     if k in ("E", "nu", "xi", "theta_c", "theta_s", "gravity")})
            if what == "colliders":
                r = orc.RefSim(P, sc.x, sc.v, sc.mass, p4=1)
                r.set_colliders(_NEXT_ROWS_COLLIDERS)
            else:
                orc.build_oracle()
                r = orc.OracleSim(P, sc.x, sc.v, sc.mass)
                r.set_colliders(_NEXT_ROWS_COLLIDERS, 0, 0.5)
            r.init()
            nref = 10
            t0 = time.perf_counter()
            for _ in range(nref):
                r.move_colliders(sc.dt)
                r.step(sc.dt, 1)
            el = time.perf_counter() - t0
            conn.send({"value": sc.n * nref / el, "ms_per_step": el / nref * 1e3, "cores": 1,
                       "kind": "reference" if what == "colliders" else "port",
                       "sample": f"{nref} steps from the initial state"})
        else:
            G, n = 20, 2147
            r = orc.RefSim(orc.Params(G, G, G, 1.0 / G), n=n, p4=1)
            t0 = time.perf_counter()
            r.initialize_particles((0.5, 0.6, 0.5), (0.0, -200.0, 0.0), seed=1)
            el = time.perf_counter() - t0
            conn.send({"ms_per_call": el * 1e3, "cores": 1, "kind": "reference"})
    except Exception as e:
        conn.send({"unavailable": f"{type(e).__name__}: {e}"})
    conn.close()


def _next_rows_reference(what, timeout_s=120.0, worker=None):
    """_next_rows_reference_worker (or `worker`, with the same arguments) in its
    own spawned process, so that a failure of the reference's code cannot end
    the benchmark: a process that ends without sending a result, or runs past
    timeout_s, is reported `unavailable` with its exit code."""
    import multiprocessing as mp
    orc = graft.load_oracle()
    if what != "colliders_port" and not orc.ref_available():
        return {"unavailable": "the headless reference build is not present on this host"}
    core = sorted(os.sched_getaffinity(0))[-1] if hasattr(os, "sched_getaffinity") else 0
    ctx = mp.get_context("spawn")
    parent, child = ctx.Pipe(duplex=False)
    proc = ctx.Process(target=worker or _next_rows_reference_worker, args=(child, what, core))
    proc.start()
    child.close()
    res = None
    try:
        if parent.poll(timeout_s):
            res = parent.recv()
    except EOFError:  # the child ended without a result
        res = None
    proc.join(10.0)
    if proc.is_alive():
        proc.kill()
        proc.join()
    if res is None:
        return {"unavailable": f"the reference's process ended with exit code {proc.exitcode} and no result"}
    return res


_S22, _C22 = float(np.sin(np.radians(22.5))), float(np.cos(np.radians(22.5)))
# the colliders of measure_next_rows: a floor box under the falling snowball and a
# turned box moving through its path (MeshCollider boxes, material_point_method.hpp:74-93)
_NEXT_ROWS_COLLIDERS = [
    dict(translation=(0.5, 0.28, 0.5), rotation=(1, 0, 0, 0), scale=(0.3, 0.2, 0.3), velocity=(0, 0, 0)),
    dict(translation=(0.36, 0.52, 0.5), rotation=(_C22, 0, 0, _S22), scale=(0.05, 0.05, 0.2), velocity=(0.5, 0, 0))]


def measure_next_rows(pkg, local, reps=3):
    """The rows that widen the path beyond the step, each on the GPU and, where
    the reference has the code, against the reference compiled on this host
    and timed on one core:
    * box colliders (gridBasedCollisions with the reference's MeshCollider
      boxes, moved every step as main.cpp:188 does): the 8,192-particle
      snowball falling on a floor box beside a turned, moving box, 200 fused
      steps (CUDA events), against the same scene without colliders and
      against the reference's step with the same boxes;
    * the particle initialiser (initializeParticles): the reference's rand()
      stream replayed on the device for its own scene (2,147 particles, 20^3,
      seed 1), and the parallel generator filling a 0.2-radius ball on 128^3,
      against the reference's initializeParticles on the same scenes;
    * the viewer feed: the xyzs stream and the point-splat image (1280 x 720,
      to host memory) of the 1.1M-particle two-ball state, host wall time per
      frame, beside a numpy fill of the same xyzs and rgba arrays."""
    import torch
    graft.load_package()
    from rd_gb300 import scenes
    out = {}
    # box colliders
    sc = scenes.snowball()
    kw = sc.params(bc=pkg.RD_BC_NONE)
    cols = _NEXT_ROWS_COLLIDERS
    steps = 200
    res = {}
    for name, cl in (("with_colliders", cols), ("without", [])):
        best = None
        for _ in range(reps):
            sim = pkg.Simulation(pkg.make_params(*sc.grid, sc.n, sc.h, device=local, **kw))
            sim.set_particles(sc.x, sc.v, sc.mass)
            sim.set_colliders(cl, pkg.RD_COLLIDE_REFERENCE, 0.5)
            sim.init_volumes()
            st = torch.cuda.ExternalStream(sim.stream(), device=local)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            sim.synchronize()
            e0.record(st)
            for _ in range(steps):
                if cl:
                    sim.move_colliders(sc.dt)
                sim.step(sc.dt, 1)
            e1.record(st)
            e1.synchronize()
            ms = e0.elapsed_time(e1) / steps
            best = ms if best is None or ms < best else best
            flags = sim.flags()
            sim.close()
        res[name] = {"ms_per_step": best, "value": sc.n / (best / 1e3), "flags": flags}
    colliders = {"workload": "snowball (8,192 particles, 64^3, no walls) falling on a floor box and past a turned box "
                             "moving at 0.5 m/s, the reference's collision rule, friction 0.5, 200 steps",
                 "unit": "particle-steps/s", "value": res["with_colliders"]["value"],
                 "ms_per_step": res["with_colliders"]["ms_per_step"],
                 "ms_per_step_without_colliders": res["without"]["ms_per_step"],
                 "flags": res["with_colliders"]["flags"]}
    colliders["reference"] = _next_rows_reference("colliders")
    if "unavailable" in colliders["reference"]:
        # the C restatement with the same boxes and rule, where the reference's
        # own collision step did not run
        colliders["port"] = _next_rows_reference("colliders_port")
    out["colliders"] = colliders
    # the particle initialiser
    init = {}
    for name, (G, n, origin, vel, radius, mode) in {
            "reference_scene": (20, 2147, (0.5, 0.6, 0.5), (0.0, -200.0, 0.0), 0.2, pkg.RD_INIT_REFERENCE),
            "ball_128": (128, 500000, (0.5, 0.5, 0.5), (0.0, -1.0, 0.0), 0.2, pkg.RD_INIT_PARALLEL)}.items():
        sim = pkg.Simulation(pkg.make_params(G, G, G, n, 1.0 / G, device=local))
        best = None
        for _ in range(reps + 1):
            sim.synchronize()
            t0 = time.perf_counter()
            more = sim.initialize_particles(origin, vel, radius=radius, mass=6e-5 if G == 20 else 1e-6, seed=1,
                                            mode=mode)
            sim.synchronize()
            el = time.perf_counter() - t0
            best = el if best is None or el < best else best
        sim.close()
        entry = {"particles": n, "grid": G, "ms_per_call": best * 1e3, "mode": "reference rand() stream" if
                 mode == pkg.RD_INIT_REFERENCE else "parallel hash generator", "kept_without_particle": more}
        if G == 20:
            entry["reference"] = _next_rows_reference("initializer")
        init[name] = entry
    out["initializer"] = init
    # the viewer feed
    sc = scenes.two_balls_1m()
    sim = pkg.Simulation(pkg.make_params(*sc.grid, sc.n, sc.h, device=local, **sc.params()))
    sim.set_particles(sc.x, sc.v, sc.mass)
    rgba = np.random.default_rng(0).integers(0, 256, (sc.n, 4), dtype=np.uint8)
    sim.set_colors(rgba)
    view = pkg.look_at_view((0.5, 0.6, 1.6), (0.5, 0.5, 0.5), width=1280, height=720)
    best_x, best_s = None, None
    for _ in range(reps + 1):
        sim.synchronize()
        t0 = time.perf_counter()
        sim.device_xyzs()
        sim.synchronize()
        ex = time.perf_counter() - t0
        t0 = time.perf_counter()
        img = sim.splat(view)
        es = time.perf_counter() - t0
        best_x = ex if best_x is None or ex < best_x else best_x
        best_s = es if best_s is None or es < best_s else best_s
    covered = float(np.mean(img.view(np.uint32).reshape(720, 1280) != view.background))
    sim.close()
    x = sc.x
    t0 = time.perf_counter()
    xyzs = np.empty((sc.n, 4), np.float32)
    xyzs[:, :3] = x
    xyzs[:, 3] = 0.01
    rgb = np.ascontiguousarray(rgba)
    el = time.perf_counter() - t0
    out["viewer_feed"] = {"workload": "1.1M-particle two-ball state, 1280 x 720 image to host memory",
                          "ms_xyzs": best_x * 1e3, "ms_splat_to_host": best_s * 1e3, "image_covered": covered,
                          "numpy_fill_ms": el * 1e3, "numpy_fill_kind": "port: the per-frame xyzs / rgba arrays "
                          "main.cpp:257-271 fills, filled by numpy on one core", "rgba_bytes": int(rgb.nbytes)}
    return out


def measure_batched(pkg, local, steps, warmup, plain_value):
    """Batched forward: the 64 uneven snowballs in one handle (one sort and one
    fused kernel per step for all scenes), autotuned, CUDA-graph replay; CUDA
    events on the handle's stream around `steps` steps after `warmup`."""
    import torch
    graft.load_package()
    from rd_gb300 import scenes
    batch = scenes.uneven_snowballs(seed=0)
    b = pkg.Batch([pkg.make_params(*s.grid, s.n, s.h, device=local, **s.params()) for s in batch])
    dt = batch[0].dt

    def reset():
        for i, s in enumerate(batch):
            b.set_particles(i, s.x, s.v, s.mass)
        b.init_volumes()

    reset()
    tune = b.autotune(dt, steps=5)
    tune["candidates"] = b.tune_trials()
    reset()
    b.step(dt, warmup)
    stream = torch.cuda.ExternalStream(b.stream(), device=local)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    b.synchronize()
    l0 = b.launch_count()
    e0.record(stream)
    b.step(dt, steps)
    e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1)
    launches = b.launch_count() - l0
    flags = b.flags()
    # per-kernel split of the same steps (events around each launch, no graphs)
    reset()
    b.step(dt, warmup)
    b.set_kernel_timing(True)
    b.step(dt, steps)
    kt = b.kernel_timing()
    b.set_kernel_timing(False)
    b.close()
    value = b.n * steps / (ms / 1e3)
    # the same scenes as plain forwards, one handle after the other
    seq_steps = min(steps, 50)
    seq_ms = 0.0
    for s in batch:
        one = pkg.Simulation(pkg.make_params(*s.grid, s.n, s.h, device=local, **s.params()))
        one.set_particles(s.x, s.v, s.mass)
        one.init_volumes()
        one.step(dt, warmup)
        st = torch.cuda.ExternalStream(one.stream(), device=local)
        one.synchronize()
        e0.record(st)
        one.step(dt, seq_steps)
        e1.record(st)
        e1.synchronize()
        seq_ms += e0.elapsed_time(e1)
        one.close()
    seq_value = b.n * seq_steps / (seq_ms / 1e3)
    # the plain forward at the batch's particle density: the two-ball scene at 8
    # particles per cell (474,282 particles; the 1.1M headline scene holds ~18.6)
    tb = scenes.two_balls()
    one = pkg.Simulation(pkg.make_params(*tb.grid, tb.n, tb.h, device=local, **tb.params()))
    one.set_particles(tb.x, tb.v, tb.mass)
    one.init_volumes()
    one.step(tb.dt, warmup)
    st = torch.cuda.ExternalStream(one.stream(), device=local)
    one.synchronize()
    e0.record(st)
    one.step(tb.dt, steps)
    e1.record(st)
    e1.synchronize()
    dens_value = tb.n * steps / (e0.elapsed_time(e1) / 1e3)
    one.close()
    return {"value": value, "unit": "particle-steps/s", "vs_plain_forward": value / plain_value,
            "plain_forward_8_per_cell": dens_value, "vs_plain_forward_8_per_cell": value / dens_value,
            "plain_forward_one_scene_at_a_time": seq_value, "vs_one_scene_at_a_time": value / seq_value,
            "steps": steps, "warmup": warmup, "ms_per_step": ms / steps, "gpu_launches": launches,
            "scenes": len(batch), "particles": b.n, "grid_nodes": int(sum(np.prod(s.grid) for s in batch)),
            "particles_range": [min(s.n for s in batch), max(s.n for s in batch)],
            "grid_range": [min(s.grid[0] for s in batch), max(s.grid[0] for s in batch)],
            "tuning": tune, "graphs": True, "flags": flags,
            "kernels_ms_per_step": {k: v[1] / steps for k, v in kt.items() if v[0]},
            "workload": "uneven_snowballs (seed 0): log-uniform 4k-262k particles, 32^3-128^3 grids, "
                        "E ~ U[5e4,3e5], nu ~ U[0.15,0.3], v0 ~ N(0,1)^3"}


def measure_adjoint(pkg, local, reps=3):
    """Forward + adjoint: the 65,536-particle cube on 64^3 for 50 steps,
    checkpoint every 10, loss ||centroid(x_T) - (0.55, 0.3, 0.5)||^2, gradients
    with respect to v0 (per particle), E and nu; against the plain forward of
    the same 50 steps, both timed on the host clock around synchronised calls
    (best of `reps`): the record and the backward are the timed library calls,
    the loss and dL/dx_T are computed on the host between them, untimed."""
    graft.load_package()
    from rd_gb300 import scenes
    sc = scenes.cube(seed=0)
    steps, every = 50, 10
    target = np.array([0.55, 0.3, 0.5])
    sim = pkg.Simulation(pkg.make_params(*sc.grid, sc.n, sc.h, device=local, **sc.params()))

    def start():
        sim.set_particles(sc.x, sc.v, sc.mass)
        sim.init_volumes()
        sim.synchronize()

    t_fwd, t_fa, t_rec = [], [], []
    for _ in range(reps + 1):  # the first round warms up
        start()
        t0 = time.perf_counter()
        sim.step(sc.dt, steps)
        sim.synchronize()
        t_fwd.append(time.perf_counter() - t0)
        start()
        t0 = time.perf_counter()
        sim.adjoint_record(sc.dt, steps, every)
        sim.synchronize()
        t1 = time.perf_counter()
        xT = sim.get_particles(("x",))["x"].astype(np.float64)  # the loss, on the host, untimed
        gx = np.tile(2.0 * (xT.mean(0) - target) / sc.n, (sc.n, 1)).astype(np.float32)
        t2 = time.perf_counter()
        g = sim.adjoint_backward(gx)
        t_fa.append((t1 - t0) + (time.perf_counter() - t2))
        t_rec.append(t1 - t0)
    # per-kernel split of one forward + adjoint (events around each launch)
    start()
    sim.set_kernel_timing(True)
    sim.adjoint_record(sc.dt, steps, every)
    xT = sim.get_particles(("x",))["x"].astype(np.float64)
    sim.adjoint_backward(np.tile(2.0 * (xT.mean(0) - target) / sc.n, (sc.n, 1)).astype(np.float32))
    kt = sim.kernel_timing()
    sim.set_kernel_timing(False)
    sim.close()
    fwd, fa, rec = min(t_fwd[1:]), min(t_fa[1:]), min(t_rec[1:])
    return {"value": sc.n * steps / fa, "unit": "particle-steps/s (forward + adjoint)",
            "ms_forward": fwd * 1e3, "ms_forward_adjoint": fa * 1e3, "ms_record": rec * 1e3,
            "ratio_vs_forward": fa / fwd, "steps": steps, "checkpoint_every": every,
            "kernels_ms": {k: v[1] for k, v in kt.items() if v[0]},
            "grad_v0_norm": float(np.linalg.norm(g["v0"])), "grad_E": float(g["E"][0]), "grad_nu": float(g["nu"][0]),
            "workload": "cube: 65,536 particles in a 0.2 cube at (0.5, 0.6, 0.5), 64^3, 50 steps, "
                        "loss ||centroid(x_T) - (0.55, 0.3, 0.5)||^2, FP32"}


def measure_batched_adjoint(pkg, local):
    """Batched forward + adjoint: 32 snowballs of log-uniform 16k-131k particles
    on 64^3-96^3 grids, compressed past the clamp by an inward radial velocity,
    100 steps, checkpoint every 10; per-scene loss = mean
    squared position error against a target rollout run at E = 2e5,
    theta = (2e-2, 5e-3); gradients w.r.t. each scene's E, theta_c, theta_s.
    Host-clock time of the two library calls, the record and the backward
    (the loss and its gradient dL/dx_T are computed on the host between them,
    untimed), against the batched forward of the same steps."""
    graft.load_package()
    from rd_gb300 import scenes
    batch = scenes.uneven_snowballs(seed=1, nscenes=32, n_lo=16384, n_hi=131072, g_lo=64, g_hi=96, steps=100)
    steps, every, dt = 100, 10, batch[0].dt

    # per-particle velocity noise (the same in the target and the fitted
    # rollout) so that the balls deform and the material parameters matter,
    # and an inward radial velocity 5 (x - c) / s, which compresses each ball
    # by ~5% over the rollout, past both compression clamps (2e-2, 2.5e-2),
    # so the clamp's subgradient carries the theta_c gradient
    rng = np.random.default_rng(2)
    centre = np.array([0.5, 0.55, 0.5])
    vel = [(s.v + rng.normal(0.0, 0.5, s.v.shape) - 5.0 * (s.x - centre)).astype(np.float32) for s in batch]

    def make(**over):
        b = pkg.Batch([pkg.make_params(*s.grid, s.n, s.h, device=local, **s.params(**over)) for s in batch])
        for i, s in enumerate(batch):
            b.set_particles(i, s.x, vel[i], s.mass)
        b.init_volumes()
        return b

    tgt = make(E=2e5, theta_c=2e-2, theta_s=5e-3)
    tgt.step(dt, steps)
    xt = [tgt.get_particles(i, ("x",))["x"].astype(np.float64) for i in range(len(batch))]
    tgt.close()
    b = make()
    t_fwd, t_fa = [], []
    g = None
    for _ in range(3):  # the first round warms up
        for i, s in enumerate(batch):
            b.set_particles(i, s.x, vel[i], s.mass)
        b.init_volumes()
        b.synchronize()
        t0 = time.perf_counter()
        b.step(dt, steps)
        b.synchronize()
        t_fwd.append(time.perf_counter() - t0)
        for i, s in enumerate(batch):
            b.set_particles(i, s.x, vel[i], s.mass)
        b.init_volumes()
        b.synchronize()
        t0 = time.perf_counter()
        b.adjoint_record(dt, steps, every)
        b.synchronize()
        t_rec = time.perf_counter() - t0
        gx, loss = [], []
        for i, s in enumerate(batch):
            x = b.get_particles(i, ("x",))["x"].astype(np.float64)
            loss.append(float(np.mean(np.sum((x - xt[i]) ** 2, axis=1))))
            gx.append((2.0 * (x - xt[i]) / s.n).astype(np.float32))
        gxa = np.concatenate(gx)
        t0 = time.perf_counter()
        g = b.adjoint_backward(gxa)
        t_fa.append(t_rec + time.perf_counter() - t0)
    n = b.n
    b.close()
    fwd, fa = min(t_fwd[1:]), min(t_fa[1:])
    return {"value": n * steps / fa, "unit": "particle-steps/s (forward + adjoint)", "ms_forward": fwd * 1e3,
            "ms_forward_adjoint": fa * 1e3, "ratio_vs_forward": fa / fwd, "scenes": len(batch), "particles": n,
            "steps": steps, "checkpoint_every": every, "loss_mean": float(np.mean(loss)),
            "grad_E_range": [float(np.min(g["E"])), float(np.max(g["E"]))],
            "grad_theta_c_range": [float(np.min(g["theta_c"])), float(np.max(g["theta_c"]))],
            "grad_theta_s_range": [float(np.min(g["theta_s"])), float(np.max(g["theta_s"]))],
            "finite": bool(all(np.all(np.isfinite(g[k])) for k in ("v0", "E", "theta_c", "theta_s"))),
            "workload": "uneven_snowballs (seed 1): 32 scenes, log-uniform 16k-131k particles, 64^3-96^3, "
                        "per-particle velocity noise N(0, 0.5) plus an inward radial 5 (x - c) / s (each ball "
                        "compressed ~5%, past the compression clamp), target rollout at E = 2e5, "
                        "theta = (2e-2, 5e-3), FP32"}


def workload_config(sc, ws):
    """The workload as both arms report it."""
    return {"workload": sc.name, "particles_per_gpu": sc.n, "grid": list(sc.grid), "dx": sc.h, "dt": sc.dt,
            "material": {k: v for k, v in sc.material.items()},
            "bc": f"sticky walls, {sc.bc_width} cells" if sc.bc else "none",
            "parallelism": f"{ws} independent replica(s)",
            "l2": f"inputs larger than L2: {2 * 7 * 16 * sc.n / 1e6:.0f} MB of particle planes per step"}


def run_ours(args):
    import torch

    ws, rank, local = dist_init("nccl")
    torch.cuda.set_device(local)
    pkg = graft.load_package()
    pkg.build()
    sc = make_scene(args.workload, seed=rank)
    params = pkg.make_params(*sc.grid, sc.n, sc.h, device=local, **sc.params())
    sim = pkg.Simulation(params)
    stream = torch.cuda.ExternalStream(sim.stream(), device=local)

    def reset():
        """The workload's initial state: every timed pass starts at step 0."""
        sim.set_particles(sc.x, sc.v, sc.mass)
        sim.init_volumes()

    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clocks:
        # keep the GPU busy for ~1 s so the clock record reflects load, then
        # start over from the initial state: W warm-up steps, K timed steps
        reset()
        t_soak = time.perf_counter()
        while time.perf_counter() - t_soak < 1.0:
            sim.step(sc.dt, 50)
            sim.synchronize()
        reset()
        sim.step(sc.dt, args.warmup)
        sim.synchronize()
        barrier(ws)
        torch.cuda.synchronize()
        sim.synchronize()
        l0 = sim.launch_count()
        ev0.record(stream)
        sim.step(sc.dt, args.steps)
        ev1.record(stream)
        ev1.synchronize()
        torch.cuda.synchronize()
        launches = sim.launch_count() - l0
        barrier(ws)
    ms = ev0.elapsed_time(ev1)
    ms_max = max_over_ranks(ws, ms, device=torch.device("cuda", local))
    value = ws * sc.n * args.steps / (ms_max / 1e3)
    assert sim.flags() & ~pkg.FLAG_OUT_OF_DOMAIN == 0, f"device flags {sim.flags()}"
    clock_summary = clocks.summary()

    # grid occupancy at the end of the timed steps, for the per-cell byte terms
    grid = sim.get_grid()
    active_cells = int(np.count_nonzero(grid["mass"]))

    # roofline pass: the same steps again with per-kernel events
    reset()
    sim.step(sc.dt, args.warmup)
    sim.set_kernel_timing(True)
    sim.step(sc.dt, args.steps)
    kt = sim.kernel_timing()
    sim.set_kernel_timing(False)
    dom = max(KERNEL_BYTES, key=lambda k: kt[k][1])
    n_launch, tot_ms = kt[dom]
    avg_s = tot_ms / max(n_launch, 1) / 1e3
    bpp, bpc = KERNEL_BYTES[dom]
    algo_bytes = bpp * sc.n + bpc * active_cells
    peak, peak_src = measured_peak_hbm()
    achieved = algo_bytes / avg_s / 1e9
    step_ms = ms / args.steps
    step_bytes = STEP_BYTES_PER_PARTICLE * sc.n + STEP_BYTES_PER_CELL * active_cells

    # end to end through the C ABI with host buffers: state in, step, state out
    fields = ("x", "v", "B", "FE", "Jp", "mass", "volume")
    shapes = {"x": (sc.n, 3), "v": (sc.n, 3), "B": (sc.n, 9), "FE": (sc.n, 9), "Jp": (sc.n,), "mass": (sc.n,),
              "volume": (sc.n,)}
    pinned = {k: torch.empty(shapes[k], dtype=torch.float32, pin_memory=True).numpy() for k in fields}
    reset()
    sim.step(sc.dt, args.warmup)
    sim.get_particles(fields, out=pinned)
    pageable = {k: a.copy() for k, a in pinned.items()}
    e2e_steps = max(1, args.e2e_steps)

    def e2e_pass(host, mapped):
        """Every step: the whole state in from host memory, one step, the whole
        state back out, then the host waits for it.  RD_HOST on page-locked
        arrays: the pack and unpack kernels read and write them in place over
        the CPU-GPU link; on pageable arrays: copies through the device staging
        buffer; mapped: the page-locked arrays passed as RD_DEVICE pointers."""
        sim.synchronize()
        barrier(ws)
        io0 = sim.io_bytes()
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            sim.set_particles(host["x"], host["v"], host["mass"], B=host["B"], FE=host["FE"], Jp=host["Jp"],
                              volume=host["volume"], sync=False, mapped=mapped)
            sim.step(sc.dt, 1)
            sim.get_particles(fields, out=host, mapped=mapped)
            if mapped:
                sim.synchronize()
        el = time.perf_counter() - t0
        io1 = sim.io_bytes()
        moved = ((io1[0] - io0[0]) // e2e_steps, (io1[1] - io0[1]) // e2e_steps)
        return max_over_ranks(ws, el, device=torch.device("cuda", local)), moved

    e2e_s, e2e_moved = e2e_pass(pinned, False)
    e2e_mapped_s, _ = e2e_pass(pinned, True)
    e2e_pageable_s, pageable_moved = e2e_pass(pageable, False)
    io_bytes = sum(int(np.prod(shapes[k])) * 4 for k in fields)
    e2e_value = ws * sc.n * e2e_steps / e2e_s
    e2e_mapped = ws * sc.n * e2e_steps / e2e_mapped_s
    e2e_pageable = ws * sc.n * e2e_steps / e2e_pageable_s
    del pinned, pageable
    # the host link's own rate: the floor of an e2e step is its bytes in and out
    # at that rate (in and out follow each other within a step)
    link = measure_link(local) if args.link else None
    e2e_ms = e2e_s / e2e_steps * 1e3
    link_keys = {}
    if link:
        floor_ms = (io_bytes / link["h2d"] + io_bytes / link["d2h"]) / 1e9 * 1e3
        link_keys = {"link_gbs_h2d": link["h2d"], "link_gbs_d2h": link["d2h"], "link_floor_ms": floor_ms,
                     "ms_per_step": e2e_ms, "link_frac": floor_ms / e2e_ms,
                     "link_method": "one cudaMemcpyAsync of 1 GiB each way between page-locked host memory "
                                    "and the device, CUDA events, best of 3"}

    # instruction ceiling of the dominant kernel: warp instructions per launch
    # (one ncu capture, scaled by particle count) over what the SMs can issue
    # in the event-timed launch at the sampled SM clock (4 schedulers per SM)
    kname = {"p2g": "k_p2g", "g2p2g": "k_g2p2g"}[dom]
    inst, inst_src = captured_issue(kname, sc.name, sc.n)
    issue = None
    if inst is not None:
        sms = torch.cuda.get_device_properties(local).multi_processor_count
        mhz = clock_summary.get("sm_mhz") or clock_summary.get("sm_max_mhz") or 2070.0
        slots = sms * 4 * mhz * 1e6 * avg_s
        issue = {"warp_instructions_per_launch": inst, "per_particle": inst / sc.n, "sms": sms, "sm_mhz": mhz,
                 "frac": inst / slots, "hbm_frac_at_full_issue": achieved / peak * slots / inst, "source": inst_src}

    out = {
        "metric": "particle-steps/s", "value": value, "unit": "particle-steps/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": workload_config(sc, ws),
        "e2e": {"value": e2e_value, "unit": "particle-steps/s", "h2d_bytes_per_step": io_bytes,
                "d2h_bytes_per_step": io_bytes, "steps": e2e_steps, **link_keys,
                "path": "rd_set_particles(RD_HOST) + rd_step + rd_get_particles(RD_HOST) on page-locked host "
                        "arrays: the pack / unpack kernels read and write them in place over NVLink-C2C",
                "bytes_in_place_per_step": e2e_moved[0], "bytes_staged_per_step": e2e_moved[1],
                "mapped_value": e2e_mapped,
                "mapped_path": "the same page-locked arrays passed as RD_DEVICE pointers (same kernels)",
                "pageable_value": e2e_pageable,
                "pageable_path": "pageable host arrays: cudaMemcpyAsync to and from the device staging buffer "
                                 "around the pack / unpack kernels",
                "pageable_bytes_staged_per_step": pageable_moved[1]},
        "roofline": {"bound": "hbm", "kernel": {"p2g": "k_p2g", "g2p2g": "k_g2p2g"}[dom],
                     "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_source": peak_src,
                     "traffic": captured_traffic({"p2g": "k_p2g", "g2p2g": "k_g2p2g"}[dom], sc.name, sc.n),
                     "algorithmic_bytes_per_launch": algo_bytes, "avg_launch_us": avg_s * 1e6,
                     "active_cells": active_cells, "issue": issue},
        "step_roofline": {"achieved": step_bytes / (step_ms / 1e3) / 1e9, "unit": "GB/s",
                          "frac": step_bytes / (step_ms / 1e3) / 1e9 / peak,
                          "bytes_per_step": step_bytes},
        "kernels_ms_per_step": {k: v[1] / max(v[0], 1) for k, v in kt.items() if v[0]},
        "gpu_launches": launches,
        "clocks": clock_summary,
    }
    if args.snowball:
        out["snowball"] = measure_snowball(pkg, local, max(args.warmup, 3))
    if args.implicit and rank == 0:
        out["implicit"] = measure_implicit(pkg, local)
    if args.next_rows and rank == 0:
        try:
            out["next_rows"] = measure_next_rows(pkg, local)
        except Exception as e:  # a secondary measurement must not lose the headline line
            out["next_rows"] = {"error": f"{type(e).__name__}: {e}"}
    batch_steps = args.steps if args.batch_steps < 0 else args.batch_steps
    if batch_steps > 0:
        out["batched_forward"] = measure_batched(pkg, local, batch_steps, max(args.warmup, 3), value)
    if args.adjoint:
        out["forward_adjoint"] = measure_adjoint(pkg, local)
        out["batched_forward_adjoint"] = measure_batched_adjoint(pkg, local)
    if rank == 0 and ws == 1 and args.cpu_baseline:
        v, kind, sample = cpu_baseline_single_core(sc)
        out["cpu_baseline"] = {"value": v, "unit": "particle-steps/s", "cores": 1, "kind": kind, "sample": sample,
                               "cpu_model": cpu_model()}
    if rank == 0:
        print(json.dumps(out), flush=True)
    sim.close()
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def _reference_worker(args_tuple):
    """One single-threaded reference instance stepping the FULL workload: init,
    `warmup` untimed steps, then timed steps until `steps` are done or
    `budget_s` has passed (at least one).  Returns (particle-steps/s, kind,
    steps done, seconds)."""
    name, seed, steps, warmup, budget_s, core = args_tuple
    pinned = pin_to_core(core) is not None
    orc = graft.load_oracle()
    sc = make_scene(name, seed=seed)
    sim, kind = oracle_for(orc, sc)
    sim.init()
    if warmup:
        sim.step(sc.dt, warmup)
    done, t0 = 0, time.perf_counter()
    while done < steps and (done == 0 or time.perf_counter() - t0 < budget_s):
        sim.step(sc.dt, 1)
        done += 1
    el = time.perf_counter() - t0
    return sc.n * done / el, kind, done, el, pinned


def run_reference(args):
    """The reference's own CPU step (the headless build of its
    LagrangeEulerView, else the C restatement) on every host core: one
    independent single-threaded instance per core, each stepping the whole
    workload, time-bounded so that the run ends within a few minutes."""
    import multiprocessing as mp

    ws, rank, _ = dist_init("gloo") if int(os.environ.get("WORLD_SIZE", "1")) > 1 else (1, 0, 0)
    if rank != 0:
        return
    orc = graft.load_oracle()
    orc.build_oracle()
    sc = make_scene(args.workload, seed=0)
    avail = sorted(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else list(range(os.cpu_count() or 1))
    cores = len(avail)
    per_worker = max(1, -(-args.steps // cores))
    warm = min(args.warmup, 1)
    budget_s = 60.0
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores) as pool:
        res = pool.map(_reference_worker,
                       [(args.workload, c, per_worker, warm, budget_s, avail[c]) for c in range(cores)])
    value = float(sum(r[0] for r in res))
    kind = res[0][1]
    steps_done = sum(r[2] for r in res)
    pinned = "each pinned to its own core" if all(r[4] for r in res) else "unpinned"
    walls = ("the reference has no grid walls: its step runs without them" if kind == "reference"
             else "with the workload's walls")
    out = {
        "metric": "particle-steps/s", "value": value, "unit": "particle-steps/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic", "impl": "reference",
        "config": workload_config(sc, ws),
        "cpu_baseline": {"value": value, "unit": "particle-steps/s", "cores": cores, "kind": kind,
                         "cpu_model": cpu_model(),
                         "sample": f"{cores} independent single-threaded instances ({pinned}), each stepping "
                                   f"all {sc.n} particles of the workload on its {sc.grid[0]}^3 grid after init "
                                   f"and {warm} untimed step ({walls}); {steps_done} full steps timed in total "
                                   f"(at most {per_worker} per instance, {budget_s:.0f} s bound)"},
        "e2e": {"value": value, "unit": "particle-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)


def run_only(args):
    import torch
    torch.cuda.set_device(0)
    pkg = graft.load_package()
    pkg.build()
    if args.only == "profile":
        sc = make_scene(args.workload, seed=0)
        sim = pkg.Simulation(pkg.make_params(*sc.grid, sc.n, sc.h, **sc.params()))
        sim.set_particles(sc.x, sc.v, sc.mass)
        sim.init_volumes()
        sim.step(sc.dt, args.warmup)
        sim.step(sc.dt, args.steps)
        sim.synchronize()
        out = {"workload": sc.name, "particles": sc.n, "steps": args.warmup + args.steps, "flags": sim.flags()}
        sim.close()
    elif args.only == "profile_batched":
        from rd_gb300 import scenes
        batch = scenes.uneven_snowballs(seed=0)
        b = pkg.Batch([pkg.make_params(*s.grid, s.n, s.h, **s.params()) for s in batch])
        for i, s in enumerate(batch):
            b.set_particles(i, s.x, s.v, s.mass)
        b.init_volumes()
        b.step(batch[0].dt, args.warmup)
        b.step(batch[0].dt, args.steps)
        b.synchronize()
        out = {"workload": "uneven_snowballs", "scenes": len(batch), "particles": b.n,
               "steps": args.warmup + args.steps, "flags": b.flags()}
        b.close()
    elif args.only == "snowball":
        out = measure_snowball(pkg, 0, max(args.warmup, 3))
    elif args.only == "implicit":
        out = measure_implicit(pkg, 0)
    elif args.only == "next_rows":
        out = measure_next_rows(pkg, 0)
    elif args.only == "batched":
        out = measure_batched(pkg, 0, args.steps, max(args.warmup, 3), float("nan"))
    elif args.only == "adjoint":
        out = measure_adjoint(pkg, 0)
    else:
        out = measure_batched_adjoint(pkg, 0)
    print(json.dumps({"only": args.only, **out}), flush=True)


def main():
    args = parse_args()
    if args.only:
        run_only(args)
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
