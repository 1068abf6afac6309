"""The multi-rank host path on CPU: two gloo ranks split a mixed set of picture pairs and
combine per-frame values into the same per-sequence means as one process."""
import os
import socket

import pytest

from ivpsnr_gb300.shard import kbns_sum, sequence_means, shard_units

AREAS = [4096 * 2048] * 3 * 8 + [1920 * 1080] * 6 * 8 + [2048 * 1088] * 3 * 8


def test_shards_are_disjoint_complete_and_balanced():
    for world in (1, 2, 3, 4, 8):
        parts = [shard_units(AREAS, r, world) for r in range(world)]
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(AREAS)))
        loads = [sum(AREAS[i] for i in p) for p in parts]
        assert max(loads) - min(loads) <= max(AREAS)
    assert shard_units(AREAS, 1, 2) == shard_units(AREAS, 1, 2)
    with pytest.raises(ValueError):
        shard_units(AREAS, 2, 2)


def test_kbns_matches_reference_semantics():
    vals = [1e16, 1.0, -1e16, 1.0]
    assert kbns_sum(vals) == 2.0
    plain = 0.0
    for v in vals:
        plain += v
    assert plain == 1.0


def _frame_values(f):
    # deterministic per-frame values with a spread that makes summation order matter
    return {"ivpsnr": 30.0 + (f * 7919 % 97) / 13.0 + 1e-13 * f, "psnr_pic": 1e8 if f == 3 else 25.0 + f / 7.0}


def _worker(rank, world, port, out_dir):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        mine = shard_units(AREAS, rank, world)
        local = {f: _frame_values(f) for f in mine}
        means = sequence_means(local)
        gathered = [None] * world
        dist.all_gather_object(gathered, mine)
        with open(os.path.join(out_dir, "r%d.txt" % rank), "w") as fh:
            fh.write(repr((means, gathered)))
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_gloo_ranks_reproduce_single_process_means(tmp_path):
    import torch.multiprocessing as mp
    world = 2
    mp.start_processes(_worker, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True,
                       start_method="spawn")
    single = sequence_means({f: _frame_values(f) for f in range(len(AREAS))})
    results = [eval(open(tmp_path / ("r%d.txt" % r)).read()) for r in range(world)]
    for means, gathered in results:
        assert means == single  # bit-identical: frame-ordered compensated sums
        assert sorted(i for p in gathered for i in p) == list(range(len(AREAS)))
    assert not set(results[0][1][0]) & set(results[0][1][1])
