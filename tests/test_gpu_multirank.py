"""The z-slab multi-GPU path with two ranks, on the GPU.

Two processes (gloo for the host-side exchange) each reconstruct their own
slab of one volume with the CUDA library (lolaCudaSlab, a slab plan, every
projection) and rank 0 gathers the slabs on the host: the reassembled volume
must equal one whole-volume plan bit for bit (slabs start on tile
boundaries) and the FP64 oracle within the FP32 bar.  The ranks meet only at
host barriers and gathers; no kernel of one rank waits on another, so both
may share the one GPU of this host (CUDA_VISIBLE_DEVICES=0 for both).

Also bench.py's own two-rank launch (torchrun, slabs, max over ranks): it must
print one JSON line for two GPUs' worth of ranks."""
from __future__ import annotations

import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = Path(__file__).resolve().parent.parent


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank: int, world: int, port: int, result_path: str):
    sys.path.insert(0, str(ROOT))
    sys.path.insert(0, str(ROOT / "tests"))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), CUDA_VISIBLE_DEVICES="0")
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from conftest import small_spec
    from rabbitct_gb300 import synth
    from rabbitct_gb300.lolacuda import Plan, slab
    scan = synth.make_scan(small_spec(nproj=9, seed=52))
    n = 64
    vs = 256.0 / n
    o = synth.origin_index(n, vs)
    b, c = slab(n, rank, world, 16)
    with Plan(n, vs, o, scan.width, scan.height, storage="f32", batch=4, slab=(b, c)) as p:
        p.backproject_host(scan.images, scan.matrices)
        mine = p.download()
    parts = [None] * world
    dist.all_gather_object(parts, (b, c, mine))
    if rank == 0:
        from oracle import oracle
        from rabbitct_gb300 import metrics
        parts.sort(key=lambda t: t[0])
        cover = parts[0][0] == 0 and all(parts[i][0] + parts[i][1] == parts[i + 1][0]
                                         for i in range(world - 1))
        cover = cover and parts[-1][0] + parts[-1][1] == n
        vol = np.concatenate([v for _, _, v in parts])
        with Plan(n, vs, o, scan.width, scan.height, storage="f32", batch=4) as p:
            p.backproject_host(scan.images, scan.matrices)
            whole = p.download()
        ref = oracle.bunny_f64(n, vs, o, scan.matrices, scan.images)
        e = metrics.errors(vol, ref)["rel_rmse"]
        np.save(result_path, np.array([cover, np.array_equal(vol, whole), e <= 1e-5]))
    dist.barrier()
    dist.destroy_process_group()


def test_two_ranks_reconstruct_slabs_on_the_gpu(tmp_path):
    from rabbitct_gb300 import build as b
    b.build_lolacuda()
    out = str(tmp_path / "result.npy")
    mp.start_processes(_worker, args=(2, _free_port(), out), nprocs=2, start_method="spawn")
    assert np.load(out).tolist() == [True, True, True]


def test_bench_two_rank_launch(tmp_path):
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="0")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()), "bench.py",
           "--gpus", "2", "--steps", "1", "--warmup", "1", "--problem-size", "256",
           "--projections", "32", "--no-cpu", "--no-batch64", "--no-probes", "--autotune", "0",
           "--e2e-steps", "1"]
    proc = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=900)
    assert proc.returncode == 0, proc.stdout[-2000:] + proc.stderr[-4000:]
    lines = [ln for ln in proc.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, proc.stdout[-2000:]
    d = json.loads(lines[0])
    assert d["n_gpus"] == 2 and d["scaling"] == "strong" and d["value"] > 0
    assert d["e2e"]["value"] > 0 and d["config"]["N"] == 256
