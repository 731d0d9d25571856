"""The multi-process path on CPU: two gloo ranks split a batch by system
(pascal_btdma_gb300.shard), each solves its shard, and the gathered shards
equal the whole batch solved at once; the job time is the slowest rank's.
The per-rank solve here is the oracle (no GPU): the test covers the host
logic -- partition, shard gather / scatter, the max-over-ranks reduction --
that bench.py and a multi-GPU caller use around the GPU solve."""
import json
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

M, NSYS, NROW, NSEG = 3, 37, 12, 2


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch
    import torch.distributed as dist

    from oracle import oracle as O
    from pascal_btdma_gb300 import shard, synth

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        w = synth.dominant(M, NSYS, NROW, seed=12, delta=1.5)
        first, count = shard.shard_of(NSYS, world, rank)
        part = [shard.take_shard(x, NSYS, first, count) for x in w.arrays]
        O.solve_noncyclic(M, count, NROW, NSEG, *part)
        x_local = torch.from_numpy(part[3])
        gathered = [None] * world
        dist.all_gather_object(gathered, (first, count, x_local.numpy()))
        slowest = shard.max_over_ranks(1.0 + rank)
        if rank == 0:
            full = w.D.copy()
            O.solve_noncyclic(M, NSYS, NROW, NSEG, w.A.copy(), w.B.copy(), w.C.copy(), full)
            x = np.zeros_like(full)
            covered = 0
            for f, c, xs in gathered:
                shard.put_shard(x, xs, NSYS, f, c)
                covered += c
            json.dump({"equal": bool(np.array_equal(x, full)), "covered": covered,
                       "shards": [[f, c] for f, c, _ in gathered], "slowest": slowest},
                      open(os.path.join(out_dir, "result.json"), "w"))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_shard_by_system(tmp_path):
    pytest.importorskip("torch.distributed")
    port = _free_port()
    mp.start_processes(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    res = json.load(open(tmp_path / "result.json"))
    assert res["equal"]
    assert res["covered"] == NSYS
    assert res["shards"] == [[0, 19], [19, 18]]  # remainder to the low rank, like partition_1d
    assert res["slowest"] == 2.0


@pytest.mark.parametrize("nsys,world", [(37, 2), (8, 3), (2, 4), (65536, 8)])
def test_shards_tile_the_batch(nsys, world):
    from pascal_btdma_gb300 import shard

    spans = [shard.shard_of(nsys, world, r) for r in range(world)]
    assert sum(c for _, c in spans) == nsys
    pos = 0
    for f, c in spans:
        if c:
            assert f == pos
        pos += c
    counts = [c for _, c in spans]
    assert max(counts) - min(counts) <= 1 and counts == sorted(counts, reverse=True)


def test_take_put_roundtrip():
    from pascal_btdma_gb300 import shard

    nsys, planes = 10, 6
    x = np.arange(nsys * planes, dtype=np.float64)
    y = np.zeros_like(x)
    for f, c in [(0, 4), (4, 3), (7, 3)]:
        s = shard.take_shard(x, nsys, f, c)
        assert s.shape == (planes * c,)
        shard.put_shard(y, s, nsys, f, c)
    assert np.array_equal(x, y)
