"""The N > 1 path of bench.py on CPU: replicas over a world_size-2 `gloo`
process group. Each replica evaluates its own copy of the workload (a net
does not shard), and the bench takes the MAX of the timed regions and the
SUM of the interactions over ranks; only rank 0 runs the CPU reference arm."""
from __future__ import annotations

import importlib.util
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _load_bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank: int, ws: int, port: int, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(ws), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    bench = _load_bench()
    ws_, rank_, local_ = bench.dist_env()
    d = bench.Dist(ws_, rank_, local_, use_cuda=False)
    try:
        d.barrier()
        secs = d.max(1.0 + rank)           # slowest replica's timed region
        itrs = d.sum(1000.0 * (rank + 1))  # interactions of all replicas
        ref = bench.bench_reference(None, None, None, None, ws_, rank_, None) if rank_ != 0 else "rank0"
        out.put((rank_, secs, itrs, ref))
    finally:
        d.close()


def test_replicas_reduce_over_gloo():
    ws, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, ws, port, q)) for r in range(ws)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in range(ws))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [g[1] for g in got] == [2.0, 2.0]        # max over ranks
    assert [g[2] for g in got] == [3000.0, 3000.0]  # sum over ranks
    assert got[1][3] is None                        # the reference arm runs on rank 0 only
