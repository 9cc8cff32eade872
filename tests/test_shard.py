"""Splitting a batch over ranks (ghcm_gb300.batch.shard_instances /
solve_sharded), on the CPU.

Instances are independent, so N GPUs each solve a share with no collective on
the data path, and rank 0 gathers the per-instance results. Here two `gloo`
ranks stand in for two GPUs and the oracle FIM stands in for each rank's
batch solve; the test checks that every instance is solved exactly once and
that rank 0 ends up with all of them.
"""
from __future__ import annotations

import os
import socket

import numpy as np
import pytest

from ghcm_gb300.batch import shard_instances, solve_sharded


def test_shards_cover_every_instance_once_and_balance_cells():
    rng = np.random.default_rng(0)
    cells = [int(s) ** 2 for s in rng.integers(64, 1025, size=512)]
    for world in (1, 2, 3, 4, 8):
        shards = shard_instances(cells, world)
        flat = sorted(i for s in shards for i in s)
        assert flat == list(range(len(cells)))
        loads = [sum(cells[i] for i in s) for s in shards]
        # LPT bound: no rank exceeds the mean by more than the largest instance
        assert max(loads) - sum(loads) / world <= max(cells)
        assert shard_instances(cells, world) == shards  # deterministic


def test_shards_edge_cases():
    assert shard_instances([], 2) == [[], []]
    assert shard_instances([5], 3) == [[0], [], []]
    assert shard_instances([4, 4, 4, 4], 2) == [[0, 2], [1, 3]]
    with pytest.raises(ValueError):
        shard_instances([1], 0)


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _instances():
    from ghcm_gb300 import fields

    return fields.batched_mix(6, seed=17, side_min=32, side_max=64)


def _rank_main(rank: int, world: int, port: int, out_dir: str) -> None:
    import pickle

    import torch.distributed as dist

    from ghcm_gb300 import fields
    from oracle.oracle import Oracle

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        insts = _instances()
        oracle = Oracle()

        def solve(indices):
            return {i: (rank, oracle.fim(fields.cost_from_speed(insts[i].speed), insts[i].seeds, 1e-5)[0])
                    for i in indices}

        merged = solve_sharded([i.speed.size for i in insts], solve, rank, world)
        if rank == 0:
            with open(os.path.join(out_dir, "merged.pkl"), "wb") as f:
                pickle.dump(merged, f)
        else:
            assert merged is None
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_solve_disjoint_shares(tmp_path, oracle_lib):
    import pickle

    import torch.multiprocessing as mp

    from ghcm_gb300 import fields
    from oracle.oracle import rel_diff

    world = 2
    mp.start_processes(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True,
                       start_method="spawn")
    merged = pickle.loads((tmp_path / "merged.pkl").read_bytes())
    insts = _instances()
    assert sorted(merged) == list(range(len(insts)))
    shards = shard_instances([i.speed.size for i in insts], world)
    for i, inst in enumerate(insts):
        rank, field = merged[i]
        assert i in shards[rank]
        ref = oracle_lib.fim(fields.cost_from_speed(inst.speed), inst.seeds, 1e-5)[0]
        assert rel_diff(field, ref) == 0.0
