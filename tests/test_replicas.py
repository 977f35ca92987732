"""bench.py's multi-GPU mode runs independent replicas (the path has no exchange step);
its host logic -- barrier and max-over-ranks timing -- is tested here with two gloo ranks
on the CPU."""
import importlib.util
import os
import socket
from pathlib import Path

import pytest
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parent.parent


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _load_bench():
    spec = importlib.util.spec_from_file_location("bench_mod", ROOT / "bench.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    bench = _load_bench()
    r, w, local = bench.dist_env()
    d = bench.Dist(w, "gloo")
    d.barrier()
    mx = d.max(10.0 * (rank + 1))
    d.barrier()
    d.close()
    q.put((r, w, local, mx))


@pytest.mark.parametrize("world", [2])
def test_replica_barrier_and_max(world):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[0] for o in out] == list(range(world))
    assert all(o[1] == world and o[3] == 10.0 * world for o in out)


def test_single_process_defaults(monkeypatch):
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    bench = _load_bench()
    assert bench.dist_env() == (0, 1, 0)
    d = bench.Dist(1, "gloo")
    d.barrier()
    assert d.max(3.5) == 3.5
