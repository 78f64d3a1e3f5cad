"""Multi-rank host logic on the CPU: one batch of spectra split across ranks
by the prefix sum of its candidate counts (hfx_gb300.shard.partition), each
rank searching its range, and the per-spectrum top-N rows gathered in batch
order on rank 0 (hfx_gb300.shard.gather).  World size 2 over gloo, with the
oracle standing in for each rank's GPU search: the gathered result must
equal one rank's search of the whole batch, row for row and bit for bit."""
import os
import socket

import numpy as np
import pytest

from hfx_gb300 import shard, synth

torch = pytest.importorskip("torch")


def test_partition_balances_pairs():
    rng = np.random.default_rng(3)
    for n, world in [(1, 1), (10, 2), (100, 3), (1000, 8), (5, 8)]:
        c = rng.integers(0, 5000, n)
        rr = shard.partition(c, world)
        assert len(rr) == world
        assert rr[0][0] == 0 and rr[-1][1] == n
        for (a, b), (c2, _) in zip(rr, rr[1:]):
            assert a <= b == c2
        if n >= 100:
            loads = [int(c[a:b].sum()) for a, b in rr]
            # no rank exceeds its share by more than one spectrum's candidates
            assert max(loads) <= c.sum() / world + c.max()
    assert shard.partition([0, 0, 0, 0], 2) == [(0, 2), (2, 4)]
    assert shard.partition([], 3) == [(0, 0), (0, 0), (0, 0)]
    with pytest.raises(ValueError):
        shard.partition([1, -1], 2)


def _db(O, prot):
    mt = O.mass_table(True, synth.static_mods())
    d = {k: v for k, v in synth.DIGEST.items() if k != "mono"}
    r, tc, tn = O.digest(prot.seq, prot.seg, mt, **d)
    return O.pack_ions(prot.seq), mt, r, tc, tn, O.sort_idx(r)


def _rank(rank, world, port, q):
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, os.path.join(root, "oracle"))
    import torch.distributed as dist
    import oracle as O
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        prot, sp, _ = synth.workload("tiny", n_spectra=40)
        db = _db(O, prot)
        # candidate counts of every spectrum (stage b), the same on every rank
        _, _, _, _, nc = O.search(*db, sp, topn=10)
        ranges = shard.partition(nc, world)
        lo, hi = ranges[rank]
        part = {"score": np.zeros((0, 10), np.float32), "key": np.zeros((0, 10), np.uint64),
                "pep": np.zeros((0, 10), np.uint32), "ncand": np.zeros(0, np.int64)}
        if hi > lo:
            s, _, k, p, n = O.search(*db, sp.subset(np.arange(lo, hi)), topn=10)
            part = {"score": s, "key": k, "pep": p, "ncand": n.astype(np.int64)}
        got = shard.gather(part, ranges, rank, world)
        if rank == 0:
            s, _, k, p, n = O.search(*db, sp, topn=10)
            ok = (np.array_equal(got["key"], k) and np.array_equal(got["score"].view(np.uint32), s.view(np.uint32))
                  and np.array_equal(got["pep"], p) and np.array_equal(got["ncand"], n.astype(np.int64)))
            loads = [int(nc[a:b].sum()) for a, b in ranges]
            q.put((ok, loads, ranges))
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_ranks_gather_equals_one_rank(oracle):
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    ok, loads, ranges = q.get(timeout=300)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert ok
    assert ranges[0][1] == ranges[1][0] and ranges[0][1] > 0
    assert min(loads) > 0
