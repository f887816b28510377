"""Batched uneven reconstructions (lolaCudaBatchCreate / Run) against one
plan per job: the batch's persistent pass computes every tile with the same
arithmetic as the per-plan pass, so volumes must agree bit for bit; and
against the FP64 oracle within the storage's bar."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import small_spec
from oracle import oracle
from rabbitct_gb300 import metrics, synth

pytestmark = pytest.mark.gpu

JOBS = [  # (N, width, height, projections, seed)
    (24, 64, 48, 7, 61), (40, 96, 80, 12, 62), (33, 80, 64, 3, 63), (64, 160, 128, 9, 64),
    (48, 128, 96, 5, 65),
]
BAR = {"f32": 1e-5, "f16qx": 1e-3, "tex16": 1e-3, "f16": 1e-3}


@pytest.fixture(scope="module")
def scans():
    from rabbitct_gb300 import build as b
    b.build_lolacuda()
    out = []
    for n, w, h, p, seed in JOBS:
        scan = synth.make_scan(small_spec(nproj=p, width=w, height=h, seed=seed))
        vs = 256.0 / n
        out.append((n, vs, synth.origin_index(n, vs), scan))
    return out


@pytest.mark.parametrize("mode", [0, 1])  # LOLA_BATCH_BRANCHES, LOLA_BATCH_PERSISTENT
@pytest.mark.parametrize("storage", ["f32", "f16qx", "tex16", "f16"])
def test_batch_matches_plans_and_oracle(scans, storage, mode):
    from rabbitct_gb300.lolacuda import Batch, DeviceBuffer, Plan
    bufs, jobs = [], []
    for n, vs, o, scan in scans:
        d_img = DeviceBuffer.from_array(scan.images)
        d_vol = DeviceBuffer.from_array(np.zeros((n, n, n), np.float32))
        bufs.append((d_img, d_vol))
        jobs.append(dict(n=n, voxel_size=vs, origin_index=o, width=scan.width,
                         height=scan.height, d_images=d_img.ptr, matrices=scan.matrices,
                         d_volume=d_vol.ptr))
    # the persistent pass computes the default 16 x 4 tiles; the branches and
    # the plans use the same shape so every voxel sees the same tile origin
    with Batch(jobs, storage=storage, batch=4, batch_mode=mode, batch_branches=3,
               batch_tune=0, voxels_per_thread=16, rows_per_block=4) as bt:
        info = bt.info()
        waves = [-(-p // 4) for _, _, _, p, _ in JOBS]
        assert info.jobs == len(JOBS) and info.waves == max(waves)
        assert info.launchesPerRun == (2 * max(waves) if mode == 1 else 2 * sum(waves))
        bt.run()
        bt.synchronize()
        first = [v.to_array((n, n, n), np.float32) for (_, v), (n, *_rest) in zip(bufs, scans)]
        bt.run()  # a replay accumulates again
        bt.synchronize()
        second = [v.to_array((n, n, n), np.float32) for (_, v), (n, *_rest) in zip(bufs, scans)]
    for (n, vs, o, scan), got, again in zip(scans, first, second):
        with Plan(n, vs, o, scan.width, scan.height, storage=storage, batch=4,
                  voxels_per_thread=16, rows_per_block=4) as plan:
            plan.backproject_host(scan.images, scan.matrices)
            want = plan.download()
        assert np.array_equal(got, want), (n, storage)
        ref = oracle.bunny_f64(n, vs, o, scan.matrices, scan.images)
        assert metrics.errors(got, ref)["rel_rmse"] <= BAR[storage]
        assert metrics.errors(again, 2.0 * ref)["rel_rmse"] <= BAR[storage]
    for d_img, d_vol in bufs:
        d_img.free()
        d_vol.free()


def test_tuned_batch_matches_oracle(scans):
    """With per-class tile-shape tuning the shapes may differ from a plan's, so
    the check is against the FP64 oracle."""
    from rabbitct_gb300.lolacuda import Batch, DeviceBuffer
    bufs, jobs = [], []
    for n, vs, o, scan in scans:
        d_img = DeviceBuffer.from_array(scan.images)
        d_vol = DeviceBuffer.from_array(np.zeros((n, n, n), np.float32))
        bufs.append((d_img, d_vol))
        jobs.append(dict(n=n, voxel_size=vs, origin_index=o, width=scan.width,
                         height=scan.height, d_images=d_img.ptr, matrices=scan.matrices,
                         d_volume=d_vol.ptr))
    with Batch(jobs, storage="f32", batch=4, batch_tune=1) as bt:
        bt.run()
        bt.synchronize()
    for (n, vs, o, scan), (d_img, d_vol) in zip(scans, bufs):
        got = d_vol.to_array((n, n, n), np.float32)
        ref = oracle.bunny_f64(n, vs, o, scan.matrices, scan.images)
        assert metrics.errors(got, ref)["rel_rmse"] <= 1e-5
        d_img.free()
        d_vol.free()


def test_autotune_picks_a_measured_candidate(scans):
    from rabbitct_gb300.lolacuda import DeviceBuffer, Plan, autotune
    n, vs, o, scan = scans[3]
    d_img = DeviceBuffer.from_array(scan.images)
    cfg, tried = autotune(n, vs, o, scan.width, scan.height, d_img.ptr, scan.matrices,
                          storage="f16qx")
    ran = [t for t in tried if t[3] > 0]
    assert len(ran) >= 10
    best = min(ran, key=lambda t: t[3])
    assert (cfg.voxelsPerThread, cfg.rowsPerBlock) == best[0]
    assert cfg.batch == best[1] and cfg.staging == best[2] and cfg.storage == 8
    with Plan(n, vs, o, scan.width, scan.height, cfg=cfg) as plan:
        plan.backproject_device(d_img.ptr, scan.width * scan.height, scan.matrices)
        plan.synchronize()
        vol = plan.download()
    d_img.free()
    ref = oracle.bunny_f64(n, vs, o, scan.matrices, scan.images)
    assert metrics.errors(vol, ref)["rel_rmse"] <= 1e-3


@pytest.mark.parametrize("storage", ["f16qx", "f32"])
def test_persistent_batch_of_more_jobs_than_the_wave_parameters_hold(storage):
    """130 small jobs, more than a wave's kernel parameters carry (128): the
    persistent pass then reads the jobs from the device job table (mixed
    layouts by loads).  Same volumes as one plan per job."""
    from rabbitct_gb300 import build as b
    b.build_lolacuda()
    from rabbitct_gb300.lolacuda import Batch, DeviceBuffer, Plan
    cases = []
    for j in range(130):
        n = 8 + (j % 3) * 4
        scan = synth.make_scan(small_spec(nproj=2 + j % 3, width=24, height=20, seed=400 + j))
        vs = 256.0 / n
        cases.append((n, vs, synth.origin_index(n, vs), scan))
    bufs, jobs = [], []
    for n, vs, o, scan in cases:
        d_img = DeviceBuffer.from_array(scan.images)
        d_vol = DeviceBuffer.from_array(np.zeros((n, n, n), np.float32))
        bufs.append((d_img, d_vol))
        jobs.append(dict(n=n, voxel_size=vs, origin_index=o, width=scan.width,
                         height=scan.height, d_images=d_img.ptr, matrices=scan.matrices,
                         d_volume=d_vol.ptr))
    with Batch(jobs, storage=storage, batch=4, batch_mode=1) as bt:
        bt.run()
        bt.synchronize()
        got = [v.to_array((n, n, n), np.float32) for (_, v), (n, *_r) in zip(bufs, cases)]
    for (n, vs, o, scan), g in zip(cases, got):
        with Plan(n, vs, o, scan.width, scan.height, storage=storage, batch=4) as plan:
            plan.backproject_host(scan.images, scan.matrices)
            assert np.array_equal(g, plan.download()), (n, storage)
    for d_img, d_vol in bufs:
        d_img.free()
        d_vol.free()
