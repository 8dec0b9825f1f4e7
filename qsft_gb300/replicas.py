"""Multi-GPU serving as independent replicas: one process per GPU.

Every request is an independent sparse transform: the q-SFT path has no data
exchange between transforms, and within one transform the peeling loop couples
all subsampling groups at every iteration, so splitting a transform over GPUs
would put a collective into every peeling iteration for no gain at these sizes.
N GPUs therefore run N replicas.  Requests are dealt round-robin by index; each
rank runs its share through the single-GPU path; rank 0 gathers the results in
request order.  The only collectives are for timing (a barrier, the maximum of
the per-rank times) and the final gather -- none on the data path.

Processes are launched one per GPU (``torch.distributed.run``); rank, world size
and rendezvous come from the environment (RANK, WORLD_SIZE, LOCAL_RANK,
MASTER_ADDR, MASTER_PORT).  The same code runs under gloo on CPU for tests.
"""
import datetime
import os

import torch
import torch.distributed as dist

__all__ = ["init_from_env", "shard", "barrier", "max_over_ranks", "sum_over_ranks", "gather_in_order",
           "run_sharded", "shutdown"]


def init_from_env(backend=None, timeout_s=300.0):
    """(rank, world, local_rank) from the environment; with WORLD_SIZE > 1 the
    process group is created (nccl when CUDA is available, else gloo) with the
    given timeout, so that a rank that died turns the others' next collective
    into an error instead of a hang."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", str(rank)))
    if world > 1 and not dist.is_initialized():
        if backend is None:
            backend = "nccl" if torch.cuda.is_available() else "gloo"
        kw = {}
        if backend == "nccl":
            torch.cuda.set_device(local)
            kw["device_id"] = torch.device("cuda", local)
        dist.init_process_group(backend, rank=rank, world_size=world,
                                timeout=datetime.timedelta(seconds=timeout_s), **kw)
    return rank, world, local


def _active():
    return dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1


def shard(n, rank, world):
    """Indices of the requests rank `rank` of `world` serves: i % world == rank."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("need 0 <= rank < world")
    return list(range(rank, n, world))


def _device():
    if dist.get_backend() == "nccl":
        return torch.device("cuda", torch.cuda.current_device())
    return torch.device("cpu")


def barrier():
    if _active():
        dist.barrier()


def max_over_ranks(x):
    """max of a float over the ranks (x itself with one rank)."""
    if not _active():
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=_device())
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(x):
    if not _active():
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=_device())
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def gather_in_order(local_results, n, rank, world):
    """Rank 0: the list of all n results in request order (rank r's i-th result
    is request r + i*world); other ranks: None."""
    local_results = list(local_results)
    if len(local_results) != len(shard(n, rank, world)):
        raise ValueError("one local result per request of this rank's shard")
    if world == 1 or not _active():
        return local_results
    parts = [None] * world if rank == 0 else None
    dist.gather_object(local_results, parts, dst=0)
    if rank != 0:
        return None
    out = [None] * n
    for r, part in enumerate(parts):
        for i, res in zip(shard(n, r, world), part):
            out[i] = res
    return out


def run_sharded(requests, serve_fn):
    """Serve `requests` over all ranks: each rank calls serve_fn on its shard
    (a list of requests -> a list of results); rank 0 returns every result in
    request order, other ranks None."""
    rank = dist.get_rank() if _active() else 0
    world = dist.get_world_size() if _active() else 1
    mine = [requests[i] for i in shard(len(requests), rank, world)]
    return gather_in_order(serve_fn(mine) if mine else [], len(requests), rank, world)


def shutdown():
    if dist.is_available() and dist.is_initialized():
        dist.destroy_process_group()
