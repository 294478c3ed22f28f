"""The replicas-only multi-GPU form on CPU: two gloo ranks shard the views
with no overlap and reduce timing (max) and samples (sum); plus the tile
autotuner's JSON cache."""
import json
import os

import pytest

from aloha_gb300 import autotune
from aloha_gb300.replicas import shard_views


def test_shards_partition_the_views():
    for n in (1, 7, 256):
        for world in (1, 2, 3, 8):
            got = sorted(v for r in range(world) for v in shard_views(n, r, world))
            assert got == list(range(n))
    with pytest.raises(ValueError):
        shard_views(4, 2, 2)


def _worker(rank, world, port, out_dir):
    import torch.distributed as dist

    from aloha_gb300.replicas import max_over_ranks, shard_views, sum_over_ranks
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    views = shard_views(10, rank, world)
    elapsed = 1.0 + rank          # pretend rank r took r + 1 seconds
    samples = 100 * len(views)
    res = {"views": views, "max": max_over_ranks(elapsed), "sum": sum_over_ranks(samples)}
    with open(os.path.join(out_dir, f"r{rank}.json"), "w") as f:
        json.dump(res, f)
    dist.destroy_process_group()


def test_two_gloo_ranks_reduce_time_and_samples(tmp_path):
    torch = pytest.importorskip("torch")
    import socket
    import torch.multiprocessing as mp
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    mp.start_processes(_worker, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    r = [json.load(open(tmp_path / f"r{k}.json")) for k in range(2)]
    assert sorted(r[0]["views"] + r[1]["views"]) == list(range(10))
    assert r[0]["max"] == r[1]["max"] == 2.0
    assert r[0]["sum"] == r[1]["sum"] == 1000.0
    del torch


class _FakeBatch:
    def __init__(self):
        self.sweeps = 0
        self.config = None
        self.stage = 0
        self.steps = 1

    def autotune(self, stream=None, reps=2):
        self.sweeps += 1
        self.stage = 0
        self.steps = 2
        return 32, 4, 1.5

    def set_config(self, w, h, c):
        self.config = (w, h)

    def set_staging(self, stage):
        self.stage = stage

    def staging(self):
        return self.stage

    def set_unroll(self, steps):
        self.steps = steps

    def unroll(self):
        return self.steps


def test_autotune_cache(tmp_path):
    path = str(tmp_path / "tune.json")
    key = autotune.batch_key("NVIDIA GB300", [(1024, 1024)] * 64 + [(512, 512)] * 32, 12, 12, 256)
    assert "1024x1024*64" in key and "512x512*32" in key
    b = _FakeBatch()
    first = autotune.tune(b, key, path=path)
    assert first["cached"] is False and b.sweeps == 1
    b2 = _FakeBatch()
    second = autotune.tune(b2, key, path=path)
    assert second["cached"] is True and b2.sweeps == 0 and b2.config == (32, 4)
    assert b2.stage == 0 and b2.steps == 2
    assert json.load(open(path))[key]["tile_w"] == 32
    assert json.load(open(path))[key]["staging"] == 0 and json.load(open(path))[key]["unroll"] == 2
