"""CPU tests of the ensemble's sharding across ranks (mhd-gpu_gb300/shard.py):
the partition is complete, balanced and the same on every rank, and a
two-rank gloo run that advances each rank's share (on the oracle, no GPU)
and gathers per-box records equals the single-process run."""
import hashlib
import os
import socket

import numpy as np
import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def test_partition_complete_balanced_deterministic():
    import ics
    import shard
    ens = ics.ensemble(64, seed=0, sizes=(32, 48, 64, 96, 128))
    dims = [e["dims"] for e in ens]
    biggest = max(d[0] * d[1] * d[2] for d in dims)
    for n in (1, 2, 3, 4, 8):
        parts = shard.partition_boxes(dims, n)
        assert sorted(i for p in parts for i in p) == list(range(64))
        loads = shard.shard_cells(dims, parts)
        assert max(loads) - min(loads) <= biggest
        assert parts == shard.partition_boxes(list(dims), n)
    with pytest.raises(ValueError):
        shard.partition_boxes(dims, 0)


def _box_record(oracle_mod, e, steps):
    O = oracle_mod.oracle("f32")
    u, b = e["u"].copy(), e["b"].copy()
    O.run(u, b, *e["dims"], cfl_number=0.7, max_steps=steps)
    tot = np.asarray(u, dtype=np.float64).reshape(-1, 5).sum(0)
    return {"sha": hashlib.sha256(u.tobytes() + b.tobytes()).hexdigest(), "mass": float(tot[0]),
            "energy": float(tot[4])}


def _rank_main(rank, world, port, q):
    import sys
    repo = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    for sub in ("mhd-gpu_gb300", "oracle"):
        sys.path.insert(0, os.path.join(repo, sub))
    import torch.distributed as dist
    import ics
    import oracle as O
    import shard
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ens = ics.ensemble(6, seed=3, sizes=(8, 12, 16))
        parts = shard.partition_boxes([e["dims"] for e in ens], world)
        mine = {i: _box_record(O, ens[i], 2) for i in parts[rank]}
        merged = shard.gather_box_records(mine, world)
        if rank == 0:
            q.put(merged)
    finally:
        dist.destroy_process_group()


def test_two_rank_gloo_shard_equals_single_process(oracle_lib):
    import multiprocessing as mp
    import ics
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    merged = q.get(timeout=180)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    ens = ics.ensemble(6, seed=3, sizes=(8, 12, 16))
    ref = {i: _box_record(oracle_lib, e, 2) for i, e in enumerate(ens)}
    assert merged == ref
