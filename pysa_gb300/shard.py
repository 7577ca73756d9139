"""Several GPUs: replicas only.

Reads of one instance, and instances of a batch, are independent Markov
chains (the exchange of pysa/utils.py:26-58 stays inside a read), so a run
over N GPUs is N runs over disjoint sets of reads with no exchange between
GPUs, one process per GPU.  This module holds that host-side logic: which
reads a rank runs, the concatenation of the ranks' result rows in read
order, the whole-job time (slowest rank) and the combination of per-read
log-partition estimates (pysa/ais.py:59-76).  Collectives go through
torch.distributed (NCCL between GPUs; gloo on the host for tests); none sits
on the data path of a sweep.
"""
from __future__ import annotations

import numpy as np


def read_range(num_reads: int, rank: int, world: int) -> tuple[int, int]:
    """[start, stop) of the reads rank runs: contiguous, sizes differing by
    at most one, earlier ranks taking the extra ones."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank must be in [0, world)")
    base, extra = divmod(int(num_reads), int(world))
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def gather_rows(rows: list, group=None) -> list:
    """Every rank's result rows (lists of per-read dicts), concatenated in
    rank order, on every rank."""
    import torch.distributed as dist
    if not dist.is_available() or not dist.is_initialized():
        return list(rows)
    out = [None] * dist.get_world_size(group)
    dist.all_gather_object(out, list(rows), group=group)
    return [r for part in out for r in part]


def slowest(seconds: float, group=None) -> float:
    """Whole-job time: the largest of the ranks' times."""
    import torch
    import torch.distributed as dist
    if not dist.is_available() or not dist.is_initialized():
        return float(seconds)
    backend = dist.get_backend(group)
    dev = "cuda" if backend == "nccl" else "cpu"
    t = torch.tensor([float(seconds)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())


def combined_logz(rows: list) -> float:
    """log-mean-exp of the rows' log_Zf (pysa/ais.py:59-76) over all reads
    of all ranks."""
    from .ais import combine_logZf
    return combine_logZf({"log_Zf": np.asarray([r["log_Zf"] for r in rows])})


def metropolis_update_sharded(solver, num_reads: int, *, seed: int,
                              group=None, **kwargs) -> list:
    """Solver.metropolis_update over num_reads reads split across the ranks
    of `group`: this rank runs its read_range with seed + rank (independent
    streams) on its own GPU; returns every rank's rows in read order."""
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized():
        rank, world = dist.get_rank(group), dist.get_world_size(group)
    else:
        rank, world = 0, 1
    start, stop = read_range(num_reads, rank, world)
    kwargs = dict(kwargs, return_dataframe=False)
    rows = solver.metropolis_update(num_reads=stop - start,
                                    seed=int(seed) + rank, **kwargs) \
        if stop > start else []
    return gather_rows(list(rows), group=group)
