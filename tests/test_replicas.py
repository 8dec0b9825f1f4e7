"""Replica path (qsft_gb300/replicas.py) with world_size 2 on CPU (gloo): sharding,
result gathering in request order, the timing reductions, and a rank that fails
before a collective (the other rank gets an error, not a hang)."""
import os
import socket

import pytest
import torch.multiprocessing as mp

from qsft_gb300.replicas import shard


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _env(rank, world, port):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})


def _worker_gather(rank, world, port, n, out):
    _env(rank, world, port)
    from qsft_gb300 import replicas as R
    r, w, _ = R.init_from_env(backend="gloo", timeout_s=30)
    assert (r, w) == (rank, world)
    requests = [("req", i) for i in range(n)]
    res = R.run_sharded(requests, lambda mine: [(name, i, rank) for name, i in mine])
    mx = R.max_over_ranks(float(rank + 1))
    sm = R.sum_over_ranks(1.0)
    R.barrier()
    if rank == 0:
        out.put((res, mx, sm))
    R.shutdown()


def _worker_fail(rank, world, port, out):
    _env(rank, world, port)
    from qsft_gb300 import replicas as R
    R.init_from_env(backend="gloo", timeout_s=5)
    if rank == 1:
        os._exit(3)          # dies between steps, before the next collective
    try:
        R.max_over_ranks(1.0)
        out.put("no error")
    except Exception as e:  # noqa: BLE001 -- any error is the expected outcome
        out.put(f"error: {type(e).__name__}")


def test_shard_covers_every_request_once():
    for n in (0, 1, 5, 16, 17):
        for world in (1, 2, 3, 8):
            got = sorted(i for r in range(world) for i in shard(n, r, world))
            assert got == list(range(n))
    with pytest.raises(ValueError):
        shard(4, 2, 2)


@pytest.mark.parametrize("n", [0, 1, 7, 16])
def test_two_ranks_gather_in_request_order(n):
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    mp.start_processes(_worker_gather, args=(2, port, n, out), nprocs=2, join=True, start_method="spawn")
    res, mx, sm = out.get(timeout=60)
    assert [x[:2] for x in res] == [("req", i) for i in range(n)]
    assert all(x[2] == i % 2 for i, x in enumerate(res))   # served by rank i % 2
    assert mx == 2.0 and sm == 2.0


def test_dead_rank_makes_an_error_not_a_hang():
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker_fail, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    msg = out.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
    assert msg.startswith("error"), msg
