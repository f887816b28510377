"""The sharded (z-slab) path's host logic with two ranks on CPU (gloo):
slab ranges from lolaCudaSlab cover the volume without overlap, each rank
fills its slab (with the oracle: there is no GPU here) and rank 0 gathers the
slabs with a gloo collective and checks the reassembled volume against the
unsharded one.  No data-path collective exists in the GPU path itself: this
exercises the partition and reassembly around it."""
from __future__ import annotations

import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank: int, world: int, port: int, result_path: str):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from conftest import small_spec
    from oracle import oracle
    from rabbitct_gb300 import synth
    from rabbitct_gb300.lolacuda import slab
    scan = synth.make_scan(small_spec(nproj=5, width=64, height=48, seed=51))
    n = 24
    vs = 256.0 / n
    o = synth.origin_index(n, vs)
    b, c = slab(n, rank, world, 8)
    idx = np.arange(b * n * n, (b + c) * n * n, dtype=np.int64)
    mine = oracle.bunny_points(n, vs, o, scan.matrices, scan.images, idx)
    counts = [None] * world
    dist.all_gather_object(counts, (b, c))
    gathered = [None] * world
    dist.all_gather_object(gathered, mine)
    if rank == 0:
        covered = sorted(counts)
        ok_cover = covered[0][0] == 0 and all(covered[i][0] + covered[i][1] == covered[i + 1][0]
                                             for i in range(world - 1))
        ok_cover = ok_cover and covered[-1][0] + covered[-1][1] == n
        vol = np.concatenate([g for _, g in sorted(zip(counts, gathered), key=lambda t: t[0])])
        whole = oracle.bunny_f64(n, vs, o, scan.matrices, scan.images).reshape(-1)
        np.save(result_path, np.array([ok_cover, np.array_equal(vol, whole)]))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_slab_partition_and_reassembly(tmp_path):
    from rabbitct_gb300 import build as b
    b.build_lolacuda()
    out = str(tmp_path / "result.npy")
    mp.start_processes(_worker, args=(2, _free_port(), out), nprocs=2, start_method="spawn")
    assert np.load(out).tolist() == [True, True]


@pytest.mark.parametrize("n,ranks,align", [(1024, 8, 8), (512, 3, 8), (100, 4, 8), (7, 3, 1),
                                            (64, 1, 8), (16, 5, 8)])
def test_slab_ranges_cover_volume(n, ranks, align):
    from rabbitct_gb300.lolacuda import slab
    got = [slab(n, r, ranks, align) for r in range(ranks)]
    pos = 0
    for b, c in got:
        assert b == pos and c >= 0
        assert b % align == 0
        pos += c
    assert pos == n
