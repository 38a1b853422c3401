"""Multi-rank host logic on the CPU (gloo, world size 2): the probe sharding a
multi-GPU scan uses (contiguous ranges, disjoint, covering every probe, sizes
within one) and the bench's barrier + max-over-ranks timing reduction."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from conftest import ROOT


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, shape, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import sys
    sys.path.insert(0, ROOT)
    import bench
    import temgymcore_gb300 as t
    sg = t.ScanGrid(z=0.0, pixel_size=(1e-9, 1e-9), shape=shape, rotation=17.0)
    start, stop, pos = t.scan_shard(sg, rank, world)
    ranges = [None] * world
    dist.all_gather_object(ranges, (start, stop, pos.tolist()))
    bench._barrier(world)
    slowest = bench._max_over_ranks(1.0 + rank, world)
    if rank == 0:
        np.save(os.path.join(out_dir, "ranges.npy"), np.array([(a, b) for a, b, _ in ranges]))
        np.save(os.path.join(out_dir, "pos.npy"), np.concatenate([np.array(p).reshape(-1, 2) for _, _, p in ranges]))
        np.save(os.path.join(out_dir, "slowest.npy"), np.array([slowest]))
    dist.destroy_process_group()


@pytest.mark.parametrize("shape", [(5, 7), (64, 64), (1, 3)])
def test_two_rank_scan_sharding_and_timing_reduction(shape, tmp_path):
    world = 2
    mp.spawn(_worker, args=(world, _free_port(), shape, str(tmp_path)), nprocs=world, join=True)
    ranges = np.load(tmp_path / "ranges.npy")
    n = shape[0] * shape[1]
    assert ranges[0][0] == 0 and ranges[-1][1] == n
    assert all(ranges[i][1] == ranges[i + 1][0] for i in range(world - 1))
    sizes = ranges[:, 1] - ranges[:, 0]
    assert sizes.max() - sizes.min() <= 1
    import temgymcore_gb300 as t
    sg = t.ScanGrid(z=0.0, pixel_size=(1e-9, 1e-9), shape=shape, rotation=17.0)
    np.testing.assert_array_equal(np.load(tmp_path / "pos.npy"), t.scan_positions(sg))
    assert float(np.load(tmp_path / "slowest.npy")[0]) == 2.0
