"""Sharding windows across ranks (one process per GPU).

Windows are independent, so a multi-GPU run splits the work with no
collective on the data path: the locations of one pair are cut into
contiguous ranges of whole strips (the reference's only cross-window read,
the next window's first surface value, conv_ampl_demean.cu:89, stays inside a
strip), and the pairs of a stack are dealt to ranks whole, largest first.
Each rank correlates its share on its own GPU; the results are gathered to
the first rank in location order at the end (a host-side gather of 104-byte
records, not part of the correlation).
"""
from __future__ import annotations

import numpy as np


def strip_ranges(nlocs: int, strip_len: int, world: int):
    """[(w0, w1)] per rank: contiguous windows, whole strips, balanced by strips."""
    if world < 1:
        raise ValueError("world must be >= 1")
    sl = strip_len if strip_len > 0 else 1
    nstrips = (nlocs + sl - 1) // sl
    out = []
    for r in range(world):
        s0 = (nstrips * r) // world
        s1 = (nstrips * (r + 1)) // world
        out.append((min(s0 * sl, nlocs), min(s1 * sl, nlocs)))
    return out


def deal_pairs(window_counts, world: int):
    """Indices of the pairs each rank correlates: largest pair first to the
    least-loaded rank (longest-processing-time order), ties to the lower rank."""
    load = [0] * world
    owner = [[] for _ in range(world)]
    for i in sorted(range(len(window_counts)), key=lambda k: (-window_counts[k], k)):
        r = min(range(world), key=lambda q: (load[q], q))
        owner[r].append(i)
        load[r] += window_counts[i]
    return [sorted(o) for o in owner]


def gather_results(local: np.ndarray, ranges, group=None, dst: int = 0):
    """Collect every rank's result records (a structured array for its range
    of `ranges`) on rank `dst`, in location order; other ranks get None."""
    import torch
    import torch.distributed as dist
    rank, world = dist.get_rank(group), dist.get_world_size(group)
    itemsize = local.dtype.itemsize
    buf = torch.from_numpy(np.frombuffer(local.tobytes(), dtype=np.uint8).copy())
    sizes = [(w1 - w0) * itemsize for (w0, w1) in ranges]
    if rank == dst:
        parts = [torch.empty(n, dtype=torch.uint8) for n in sizes]
        for r in range(world):
            if r == dst:
                parts[r].copy_(buf)
            else:
                dist.recv(parts[r], src=r, group=group)
        flat = torch.cat(parts).numpy()
        return np.frombuffer(flat.tobytes(), dtype=local.dtype)
    dist.send(buf, dst=dst, group=group)
    return None
