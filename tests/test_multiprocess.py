"""The N > 1 path of bench.py on the CPU: world size 2 over gloo, one process per
rank as torchrun would start them.  Replicas only: every rank steps its own
scene; the only exchange is the barrier and the max over ranks of the timed
region, and the reference arm runs on rank 0 alone."""
import contextlib
import io
import json
import multiprocessing as mp
import os
import socket
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, ws, port, q, reference):
    os.environ.update(WORLD_SIZE=str(ws), RANK=str(rank), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, REPO)
    import bench
    out = {"rank": rank}
    try:
        if reference:
            sys.argv = ["bench.py", "--impl", "reference", "--workload", "snowball", "--steps", "1", "--warmup", "0"]
            args = bench.parse_args()
            buf = io.StringIO()
            with contextlib.redirect_stdout(buf):
                bench.run_reference(args)
            out["stdout"] = buf.getvalue()
        else:
            ws_, rank_, local = bench.dist_init("gloo")
            bench.barrier(ws_)
            out["max"] = bench.max_over_ranks(ws_, 1.5 + rank_, device="cpu")
            # replicas: rank r steps the scene generated from seed r
            sc = bench.make_scene("snowball", seed=rank_)
            out["x0"] = [float(v) for v in sc.x[0]]
            import torch.distributed as dist
            dist.destroy_process_group()
    except Exception as e:  # reported to the parent
        out["error"] = repr(e)
    q.put(out)


def run_ranks(ws, reference=False, timeout=300):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, ws, port, q, reference)) for r in range(ws)]
    for p in procs:
        p.start()
    res = [q.get(timeout=timeout) for _ in procs]
    for p in procs:
        p.join(timeout=60)
    return sorted(res, key=lambda r: r["rank"])


def test_two_ranks_barrier_and_max_over_ranks():
    res = run_ranks(2)
    assert all("error" not in r for r in res), res
    assert [r["max"] for r in res] == [2.5, 2.5]
    assert res[0]["x0"] != res[1]["x0"]  # independent replicas


def test_reference_arm_runs_on_rank_zero_only(orc):
    if not orc.ref_available():
        pytest.skip("the reference is not built here")
    res = run_ranks(2, reference=True, timeout=600)
    assert all("error" not in r for r in res), res
    assert res[1]["stdout"] == ""
    line = json.loads(res[0]["stdout"].strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["value"] > 0 and line["n_gpus"] == 2
