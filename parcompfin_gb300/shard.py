"""Sharding of pricing work across ranks (one process per GPU).

The reference splits its work over MPI ranks in two ways, both kept here:
  * contracts shard with no communication at all (one request is priced by
    exactly one rank);
  * one contract's Monte Carlo paths shard by contiguous Philox ranges, and
    the per-rank moment sums are added (src/mc_eur_mpi.cpp:20-36 reduces the
    payoff sum to rank 0). Moment sums are exact to add, so a sharded price
    equals the unsharded one up to FP64 summation order.
On one GPU these functions reduce to the identity. Collectives are only used
to gather results on the host side, never inside a pricing kernel.
"""
from __future__ import annotations


def contract_slice(n: int, rank: int, world: int) -> range:
    """Contracts [lo, hi) priced by `rank`: contiguous, sizes differ by <= 1."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank/world")
    base, extra = divmod(n, world)
    lo = rank * base + min(rank, extra)
    return range(lo, lo + base + (1 if rank < extra else 0))


def path_split(N: int, rank: int, world: int) -> tuple[int, int]:
    """(first path, path count) of `rank`'s share of an N-path contract.

    Shares start on a multiple of 4 paths (one Philox block feeds a quad of
    European paths), so the union of the shares draws exactly the normals of
    the unsharded run."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank/world")
    quads = (N + 3) // 4
    lo_q = contract_slice(quads, rank, world)
    first = lo_q.start * 4
    last = min(N, lo_q.stop * 4)
    return first, max(0, last - first)


def combine_moments(parts):
    """Add per-rank moment sums [sum y, sum y^2, sum g, sum g^2, sum y g]."""
    out = [0.0] * 5
    for p in parts:
        for k in range(5):
            out[k] += p[k]
    return out


def gather_results(local: list, world: int, group=None) -> list:
    """All ranks' result lists, concatenated in rank order (torch.distributed)."""
    if world == 1:
        return list(local)
    import torch.distributed as dist
    bucket = [None] * world
    dist.all_gather_object(bucket, list(local), group=group)
    out = []
    for b in bucket:
        out.extend(b)
    return out
