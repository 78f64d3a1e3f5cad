"""Spectra across ranks: one batch split by candidate counts, results gathered.

Spectra are independent in the reference's search (`searchForMatches`,
Sequence/Search.hs:98-124, maps over spectra; its multi-GPU item is an
unimplemented TODO), and the peptide index (~40 MB at 20,000 proteins) is
small enough to replicate.  So a batch is sharded with no exchange on the
data path: each rank takes a contiguous run of spectra whose candidate
counts (the window sizes of stage b) add up to about 1/world of the batch's
pairs, searches it on its own GPU, and the per-spectrum top-N rows are
concatenated in batch order on rank 0.  The only collective is the final
gather of the results (host objects), which torch.distributed carries over
gloo or NCCL alike.
"""
from __future__ import annotations

import numpy as np


def partition(ncand, world: int) -> list[tuple[int, int]]:
    """Contiguous [lo, hi) spectrum ranges, one per rank, balanced by the
    prefix sum of the candidate counts: rank r ends at the first spectrum
    where the running pair count reaches (r + 1) / world of the total.
    Ranges may be empty (more ranks than spectra with candidates)."""
    if world < 1:
        raise ValueError("world must be >= 1")
    c = np.asarray(ncand, dtype=np.int64)
    if c.ndim != 1 or (c < 0).any():
        raise ValueError("ncand must be a 1-D array of non-negative counts")
    n = len(c)
    cum = np.cumsum(c)
    total = int(cum[-1]) if n else 0
    cuts = [0]
    for r in range(1, world):
        if total == 0:
            cut = (n * r) // world
        else:
            # first index whose inclusive prefix reaches the r-th share
            cut = int(np.searchsorted(cum, (total * r + world - 1) // world, side="left")) + 1
        cuts.append(min(max(cut, cuts[-1]), n))
    cuts.append(n)
    return [(cuts[r], cuts[r + 1]) for r in range(world)]


def gather(part: dict, ranges, rank: int, world: int, group=None):
    """Concatenate the ranks' result arrays (dict name -> array of one row per
    spectrum of the rank's range) in batch order on rank 0; other ranks get
    None.  Uses torch.distributed's object gather (host memory)."""
    if world == 1:
        return {k: np.asarray(v) for k, v in part.items()}
    import torch.distributed as dist
    lo, hi = ranges[rank]
    for k, v in part.items():
        if len(v) != hi - lo:
            raise ValueError(f"rank {rank}: {k} has {len(v)} rows for range [{lo}, {hi})")
    got = [None] * world if rank == 0 else None
    dist.gather_object({k: np.asarray(v) for k, v in part.items()}, got, dst=0, group=group)
    if rank != 0:
        return None
    return {k: np.concatenate([g[k] for g in got], axis=0) for k in part}
