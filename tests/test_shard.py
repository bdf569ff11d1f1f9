"""Multi-GPU sharding of batched work (host logic, no GPU): the bytes-balanced
partition every rank computes independently, and a world-size-2 gloo run of
the sharded path in which each rank sorts only its own segments (with the
CPU oracle standing in for its GPU) and the union equals the unsharded
result."""

import os

import numpy as np
import pytest

from _oracle import raw_keys


def lpt(weights, world):
    """Independent restatement of the greedy rule for the check."""
    order = sorted(range(len(weights)), key=lambda i: (-int(weights[i]), i))
    load = [0] * world
    owner = [0] * len(weights)
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        owner[i] = r
        load[r] += int(weights[i])
    return owner, load


@pytest.mark.parametrize("world", [1, 2, 3, 8])
def test_partition_matches_rule_and_bounds(gb, world):
    rng = np.random.default_rng(world)
    sizes = np.floor(np.exp2(rng.uniform(8, 20, 4096))).astype(np.uint64)
    off = np.concatenate([[0], np.cumsum(sizes)]).astype(np.uint64)
    owner, load = gb.partition_segments(off, world, 4, 4)
    ref_owner, ref_load = lpt(sizes * 8, world)
    assert owner.tolist() == ref_owner and load.tolist() == ref_load
    assert owner.min() >= 0 and owner.max() < world
    total, biggest = int((sizes * 8).sum()), int(sizes.max() * 8)
    assert int(load.max()) <= total // world + biggest  # list-schedule bound
    assert int(load.sum()) == total


def test_partition_edge_cases(gb):
    owner, load = gb.partition_weights([], 4)
    assert len(owner) == 0 and load.tolist() == [0, 0, 0, 0]
    owner, load = gb.partition_weights([5, 5, 5, 5], 2)
    assert owner.tolist() == [0, 1, 0, 1] and load.tolist() == [10, 10]
    owner, _ = gb.partition_weights([1, 100, 1], 5)
    assert owner.tolist() == [1, 0, 2]
    with pytest.raises(gb.GbsortError):
        gb.partition_weights([1], 0)
    with pytest.raises(gb.GbsortError):
        gb.partition_segments(np.array([0, 5, 3], dtype=np.uint64), 2, 4)


def _rank_main(rank, world, port, result_path):
    import sys

    here = os.path.dirname(os.path.abspath(__file__))
    sys.path.insert(0, here)
    sys.path.insert(0, os.path.join(os.path.dirname(here), "cuda-fast-sort_gb300"))
    import torch
    import torch.distributed as dist

    import _oracle
    import gbsort

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    oracle = _oracle.load()
    rng = np.random.default_rng(1234)  # same layout on every rank
    sizes = np.floor(np.exp2(rng.uniform(4, 14, 300))).astype(np.uint64)
    off = np.concatenate([[0], np.cumsum(sizes)]).astype(np.uint64)
    n = int(off[-1])
    keys = raw_keys("u32", n, seed=77)
    owner, load = gbsort.partition_segments(off, world, 4, 0)
    # every rank derived the same owners: compare through the process group
    mine_t = torch.from_numpy(owner.astype(np.int64))
    gathered = [torch.empty_like(mine_t) for _ in range(world)]
    dist.all_gather(gathered, mine_t)
    agree = all(torch.equal(g, gathered[0]) for g in gathered)
    # each rank sorts only its own segments, compacted into its own batch
    sub_off, idx = gbsort.shard_offsets(off, owner, rank)
    local = np.concatenate([keys[int(off[i]):int(off[i + 1])] for i in idx]) if len(idx) else keys[:0]
    out = local.copy()
    for s in range(len(idx)):
        b, e = int(sub_off[s]), int(sub_off[s + 1])
        out[b:e] = oracle.sort("u32", local[b:e], False)
    # results travel to rank 0 only for the check
    obj = [None] * world
    dist.all_gather_object(obj, (rank, idx.tolist(), out.tolist()))
    if rank == 0:
        full = keys.copy()
        covered = np.zeros(len(sizes), dtype=np.int64)
        for r, ridx, rout in obj:
            rsub = np.concatenate([[0], np.cumsum(sizes[ridx])]).astype(np.int64)
            rout = np.asarray(rout, dtype=np.uint32)
            for j, i in enumerate(ridx):
                full[int(off[i]):int(off[i + 1])] = rout[rsub[j]:rsub[j + 1]]
                covered[i] += 1
        expect = keys.copy()
        for i in range(len(sizes)):
            expect[int(off[i]):int(off[i + 1])] = np.sort(keys[int(off[i]):int(off[i + 1])])
        ok = agree and bool((covered == 1).all()) and np.array_equal(full, expect)
        with open(result_path, "w") as f:
            f.write("ok" if ok else f"fail agree={agree} covered={covered.min()}..{covered.max()}")
    dist.barrier()
    dist.destroy_process_group()


def test_sharded_batch_world2_gloo(tmp_path):
    torch = pytest.importorskip("torch")
    import socket

    import torch.multiprocessing as mp

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    result = str(tmp_path / "result.txt")
    mp.start_processes(_rank_main, args=(2, port, result), nprocs=2, join=True, start_method="spawn")
    assert open(result).read() == "ok"
