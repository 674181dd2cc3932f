"""Several GB300s, one process each: the batch path shards, the single CPD replicates.

A single CPD has no exchange step worth a collective at these sizes, so
``bench.py --gpus N`` runs N independent replicas and only the timings meet
(the maximum over ranks).  A batch of independent CPDs (the workload of Tensor
Fox's ``rank``/``stats`` sweeps, TensorFox.py:820-1039) is partitioned into
contiguous slices, one per rank; each rank solves its slice with ``cpd_batch``
and the results are gathered, in the original order, on every rank.  No other
collective takes part.  Ranks talk through ``torch.distributed`` (NCCL between
GPUs, gloo on CPU).
"""
import torch
import torch.distributed as dist


def shard_bounds(n, rank, world):
    """Contiguous slice [start, stop) of n items for ``rank`` of ``world``.

    Sizes differ by at most one and the slices cover 0..n-1 in order."""
    if world < 1 or not 0 <= rank < world or n < 0:
        raise ValueError("bad shard request")
    base, extra = divmod(n, world)
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def gather_ordered(local, group=None):
    """Every rank's list of results concatenated in rank order, on every rank."""
    world = dist.get_world_size(group)
    parts = [None] * world
    dist.all_gather_object(parts, local, group=group)
    out = []
    for p in parts:
        out.extend(p)
    return out


def max_over_ranks(values, device=None, group=None):
    """Element-wise maximum over ranks of a list of floats (timings)."""
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return [float(v) for v in t.cpu()]


def cpd_batch_distributed(tensors, ranks, options=None, group=None, solve=None):
    """``cpd_batch`` over the ranks of ``group``: rank r solves its contiguous
    slice of the problems and every rank returns the full, ordered result list.

    ``solve`` defaults to :func:`tensorfox_gb300.cpd_batch`; it receives
    ``(tensors, ranks, options)`` for the local slice."""
    if solve is None:
        from .batch import cpd_batch as solve
    n = len(tensors)
    if isinstance(ranks, int):
        ranks = [ranks] * n
    if not dist.is_initialized():
        return solve(list(tensors), list(ranks), options)
    start, stop = shard_bounds(n, dist.get_rank(group), dist.get_world_size(group))
    local = solve(list(tensors[start:stop]), list(ranks[start:stop]), options) if stop > start else []
    return gather_ordered(list(local), group)
