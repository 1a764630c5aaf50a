"""Multi-process host logic of bench.py's replica mode on CPU (gloo, world size 2).

N > 1 runs N independent boxes, one per rank, with no collective on the data
path: the only communication is the barrier around the timed region and the
max-time / sum-of-units reductions that give the whole-job rate.  The
reference arm runs on rank 0 alone; the other ranks exit without work.
"""
from __future__ import annotations

import multiprocessing as mp
import os
import socket
import sys

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(ws), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, REPO)
    import torch.distributed as dist

    import bench
    ws_, r, local = bench.dist_init("gloo")
    bench.barrier(ws_)
    # rank r processed (r + 1) * 1000 units in (10 + r) ms
    value, ms_max = bench.whole_job_rate(ws_, (r + 1) * 1000.0, 10.0 + r)
    q.put((r, ws_, local, value, ms_max, bench.replica_seed(r)))
    dist.destroy_process_group()


def _reference_rank(rank, ws, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(ws), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, REPO)
    import argparse
    import contextlib
    import io

    import bench
    out = io.StringIO()
    with contextlib.redirect_stdout(out):
        rc = bench.run_reference(argparse.Namespace(n=16, warmup=1, steps=1, gpus=ws))
    q.put((rank, rc, out.getvalue()))


def _run(target, ws):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=target, args=(r, ws, port, q)) for r in range(ws)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in range(ws)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    return sorted(out)


def test_whole_job_rate_over_two_gloo_ranks():
    out = _run(_rank, 2)
    assert [o[0] for o in out] == [0, 1]
    for r, ws, local, value, ms_max, seed in out:
        assert ws == 2 and local == r
        assert ms_max == 11.0                      # the slowest rank's time
        assert value == 3000.0 / 11.0e-3           # all ranks' units over it
        assert seed == 2 + r                       # every replica its own box
    assert out[0][5] != out[1][5]


def test_reference_arm_runs_on_rank_zero_only():
    import json
    out = _run(_reference_rank, 2)
    (r0, rc0, text0), (r1, rc1, text1) = out
    assert rc0 == 0 and rc1 == 0
    assert text1 == ""                             # rank 1 exits without work
    line = json.loads(text0.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0
