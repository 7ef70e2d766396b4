"""The multi-GPU path on CPU: replicas over LP shards.

LPs are independent, so `bench.py --gpus N` gives each rank one contiguous
shard (`simplexprojects_gb300.shard`) and solves it alone: no collective on
the data path.  Here two `gloo` ranks each generate and solve (with the CPU
oracle, no GPU) only their shard; the gathered results must be exactly those
of one process solving the whole batch, and the shards must partition it.
"""
import json
import os
import socket

import numpy as np
import pytest


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, count, out_path):
    import torch.distributed as dist
    import simplexprojects_gb300 as sp
    from oracle import ref
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                            world_size=world)
    lo, n = sp.shard(count, 0, rank, world)
    batch = sp.generate(0, n, seed=sp.DEFAULT_SEED, first=lo)
    r = ref.solve_batch(batch, "fp64", threads=2)
    mine = dict(lo=lo, n=n, status=r.status.tolist(), objective=r.objective.tolist(),
                pivots=r.pivots.tolist())
    gathered = [None] * world
    dist.all_gather_object(gathered, mine)  # the test's check only, not the solve
    if rank == 0:
        with open(out_path, "w") as f:
            json.dump(gathered, f)
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("world", [2])
def test_two_rank_shards_match_single_process(built, tmp_path, world):
    import torch.multiprocessing as mp
    import simplexprojects_gb300 as sp
    from oracle import ref
    count = 301  # not a multiple of the world size: the last shard is shorter
    out = tmp_path / "gathered.json"
    os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
    mp.spawn(_rank_main, args=(world, _free_port(), count, str(out)), nprocs=world, join=True)
    parts = json.loads(out.read_text())
    assert [p["lo"] for p in parts] == [0, 151]
    assert sum(p["n"] for p in parts) == count
    whole = ref.solve_batch(sp.generate(0, count, seed=sp.DEFAULT_SEED), "fp64", threads=2)
    status = np.concatenate([np.array(p["status"], np.int32) for p in parts])
    obj = np.concatenate([np.array(p["objective"]) for p in parts])
    piv = np.concatenate([np.array(p["pivots"], np.int32) for p in parts])
    assert np.array_equal(status, whole.status)
    assert np.array_equal(obj.view(np.uint64), whole.objective.view(np.uint64))
    assert np.array_equal(piv, whole.pivots)


def test_shard_partitions():
    import simplexprojects_gb300 as sp
    for count in (0, 1, 7, 10_000):
        for world in (1, 2, 3, 8):
            spans = [sp.shard(count, 40, r, world) for r in range(world)]
            covered = [i for lo, n in spans for i in range(lo, lo + n)]
            assert covered == list(range(40, 40 + count))
