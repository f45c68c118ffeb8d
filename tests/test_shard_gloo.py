"""Multi-rank host logic on CPU (gloo, world size 2): contract sharding,
path sharding of one contract, and the gather of results. The oracle's FP64
twin stands in for each rank's kernel, so no GPU is needed."""
import ctypes as C
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_contract_slices_partition():
    from parcompfin_gb300.shard import contract_slice
    for n in (0, 1, 7, 1024, 1025):
        for w in (1, 2, 3, 8):
            seen = []
            for r in range(w):
                seen.extend(contract_slice(n, r, w))
            assert seen == list(range(n))


def test_path_split_partitions_quads():
    from parcompfin_gb300.shard import path_split
    for N in (1, 5, 1000, 1001, 123457):
        for w in (1, 2, 3, 8):
            parts = [path_split(N, r, w) for r in range(w)]
            assert sum(c for _, c in parts) == N
            for f, c in parts:
                assert f % 4 == 0
            starts = [f for f, c in parts if c]
            assert starts == sorted(starts)


def _worker(rank, world, port, q):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from oracle import loader
        from parcompfin_gb300.shard import contract_slice, gather_results
        orc = loader.load()
        contracts = [(100.0, 90.0 + 2 * k, .03, .25, 1.0, 20000, 1 if k % 2 else -1)
                     for k in range(9)]
        mine = []
        for i in contract_slice(len(contracts), rank, world):
            S0, E, r, sg, T, N, pf = contracts[i]
            s = (C.c_double * 5)()
            orc.twin_mc_eur(S0, E, r, sg, T, N, pf, 7, i, s)  # stream = contract id
            mine.append((i, s[0]))
        allres = gather_results(mine, world)
        if rank == 0:
            q.put(allres)
    finally:
        dist.destroy_process_group()


def test_gloo_two_ranks_contract_sharding():
    import multiprocessing as mp
    import socket
    pytest.importorskip("torch.distributed")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    # Every contract priced exactly once, in order, with the same sums as a
    # single-rank run.
    assert [i for i, _ in res] == list(range(9))
    sys.path.insert(0, ROOT)
    from oracle import loader
    orc = loader.load()
    for i, v in res:
        s = (C.c_double * 5)()
        pf = 1 if i % 2 else -1
        orc.twin_mc_eur(100.0, 90.0 + 2 * i, .03, .25, 1.0, 20000, pf, 7, i, s)
        assert v == pytest.approx(s[0], rel=1e-12)  # the twin's OpenMP sum order varies


def test_path_sharded_moments_add_up(orc):
    """Summing the moment sums of disjoint path ranges reproduces the whole."""
    from parcompfin_gb300.shard import combine_moments, path_split
    N = 10_001
    whole = (C.c_double * 5)()
    orc.twin_mc_eur(100, 100, .05, .2, 1, N, 1, 3, 0, whole)
    # A rank's share [f, f + c) is the quads f/4 .. ; the twin prices a prefix,
    # so recover each share as a difference of prefixes.
    parts = []
    for r in range(3):
        f, c = path_split(N, r, 3)
        hi = (C.c_double * 5)()
        lo = (C.c_double * 5)()
        orc.twin_mc_eur(100, 100, .05, .2, 1, f + c, 1, 3, 0, hi)
        if f:
            orc.twin_mc_eur(100, 100, .05, .2, 1, f, 1, 3, 0, lo)
        parts.append([hi[k] - lo[k] for k in range(5)])
    tot = combine_moments(parts)
    for k in range(5):
        assert tot[k] == pytest.approx(whole[k], rel=1e-12)
