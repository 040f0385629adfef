"""Sharding of a batched ensemble across ranks (one GPU each).

The boxes of an ensemble are independent (each has its own clock and dt), so
an ensemble partitions across GPUs with no exchange on the data path: every
rank advances its own share of the boxes through its own mhdgpu_batch, and the
only collective is an optional host-side gather of per-box diagnostics.  The
shares are balanced by cells (the work per step is proportional to them):
boxes in decreasing size go to the least-loaded rank, ties to the lower rank,
so every rank computes the same partition from the box sizes alone.
"""
from __future__ import annotations


def partition_boxes(dims, nparts: int):
    """dims: [(nx, ny, nz), ...].  Returns nparts lists of box indices (each in
    increasing order) whose cell counts are balanced greedily."""
    if nparts < 1:
        raise ValueError("nparts must be >= 1")
    cells = [int(d[0]) * int(d[1]) * int(d[2]) for d in dims]
    order = sorted(range(len(dims)), key=lambda i: (-cells[i], i))
    load = [0] * nparts
    parts = [[] for _ in range(nparts)]
    for i in order:
        r = min(range(nparts), key=lambda p: (load[p], p))
        parts[r].append(i)
        load[r] += cells[i]
    return [sorted(p) for p in parts]


def shard_cells(dims, parts):
    return [sum(int(dims[i][0]) * int(dims[i][1]) * int(dims[i][2]) for i in p) for p in parts]


def gather_box_records(records: dict, world: int):
    """All-gather {box index: record} dicts from every rank over the default
    torch.distributed process group (gloo or nccl) and merge them; with one
    rank, returns the input."""
    if world == 1:
        return dict(records)
    import torch.distributed as dist
    out = [None] * world
    dist.all_gather_object(out, records)
    merged = {}
    for part in out:
        merged.update(part)
    return merged
