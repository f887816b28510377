"""Accuracy at the benchmark's full size: N=512 and N=1024 volumes from 496
projections of 1248x960, every storage and accumulation variant, against the
FP64 LolaBunny oracle evaluated at 20 000 sampled voxels (the full FP64 volume
is out of reach on the host).  Also against the FP32-accumulating LolaBunny,
which is what the reference itself computes.

Bars: FP32 storage relative RMSE <= 1e-5, FP16 <= 1e-3, BF16 <= 4e-3.
Run with -s to print the table."""
from __future__ import annotations

import numpy as np
import pytest

from oracle import oracle
from rabbitct_gb300 import metrics, synth

pytestmark = pytest.mark.gpu

VARIANTS = [("f32", "plain", 1e-5), ("f32", "kahan", 1e-5), ("f32q", "plain", 1e-5),
            ("tex32", "plain", 1e-5), ("f16q", "plain", 1e-3), ("f16q", "kahan", 1e-3),
            ("f16qx", "plain", 1e-3), ("tex16", "plain", 1e-3), ("bf16q", "plain", 4e-3)]


@pytest.fixture(scope="module")
def workload():
    from rabbitct_gb300 import build as b
    b.build_lolacuda()
    from rabbitct_gb300.lolacuda import DeviceBuffer
    scan = synth.make_scan(synth.ScanSpec(nproj=496))
    d_img = DeviceBuffer.from_array(scan.images)
    yield scan, d_img
    d_img.free()


@pytest.mark.parametrize("n", [512, 1024])
def test_full_size_accuracy(workload, n):
    from rabbitct_gb300.lolacuda import Plan
    scan, d_img = workload
    vs = synth.voxel_size(n)
    o = synth.origin_index(n, vs)
    idx = np.random.default_rng(n).choice(n ** 3, 20000, replace=False)
    ref64 = oracle.bunny_points(n, vs, o, scan.matrices, scan.images, idx)
    ref32 = oracle.bunny_points(n, vs, o, scan.matrices, scan.images, idx, fp32_accumulate=True)
    assert np.count_nonzero(ref64) > 5000   # most sampled voxels see the phantom
    rows = []
    failures = []
    for storage, accum, bar in VARIANTS:
        with Plan(n, vs, o, scan.width, scan.height, storage=storage, accumulation=accum,
                  batch=16) as plan:
            plan.backproject_device(d_img.ptr, scan.width * scan.height, scan.matrices)
            plan.synchronize()
            got = plan.download().reshape(-1)[idx]
        e64 = metrics.errors(got, ref64)
        e32 = metrics.errors(got, ref32)
        rows.append((storage, accum, e64, e32))
        if e64["rel_rmse"] > bar:
            failures.append((storage, accum, e64))
    print(f"\nN={n}: variant, vs FP64 oracle (rel RMSE, max abs, PSNR dB), "
          f"vs FP32-accumulating LolaBunny (rel RMSE)")
    for storage, accum, e64, e32 in rows:
        print(f"  {storage:6s} {accum:6s} rel_rmse={e64['rel_rmse']:.3e} "
              f"max_abs={e64['max_abs']:.3e} psnr={e64['psnr_db']:.1f}  "
              f"vs_bunny32={e32['rel_rmse']:.3e}")
    assert not failures, failures
