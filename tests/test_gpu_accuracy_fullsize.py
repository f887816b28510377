"""Accuracy at the benchmark's full size: 496 projections of 1248x960, against
the FP64 LolaBunny oracle evaluated at 20 000 sampled voxels (the full FP64
volume is out of reach on the host), and against the FP32-accumulating
LolaBunny restatement, which is what the reference itself computes
(src/LolaBunny.c:44-75: FP64 coordinates, FP32 `+=`).

  - every storage and accumulation variant at N=512 and N=1024 (pass size 16);
  - the drop-in as the runner drives it (src/rabbitRunner.c:183-287): one
    projection per backprojection call (-b 1), with and without the scan's
    geometry at prepare (-a), at N=256 and N=512, default configuration;
  - the 16-bit storages at N=512 over pass sizes 4, 8, 16 and 32, plain and
    Kahan accumulation.

Bars (relative RMSE): FP32 storage <= 1e-5 against the FP64 oracle and
<= 1e-5 against the FP32-accumulating LolaBunny; FP16 <= 1e-3 and BF16
<= 4e-3 against the FP64 oracle (the 16-bit pass-size sweep holds every
variant to 1e-3).  Run with -s to print the tables (max-abs, RMSE, PSNR)."""
from __future__ import annotations

import numpy as np
import pytest

from oracle import oracle
from rabbitct_gb300 import metrics, synth

pytestmark = pytest.mark.gpu

VARIANTS = [("f32", "plain", 1e-5), ("f32", "kahan", 1e-5), ("f32q", "plain", 1e-5),
            ("f32q", "kahan", 1e-5), ("tex32", "plain", 1e-5), ("f16q", "plain", 1e-3),
            ("f16q", "kahan", 1e-3), ("f16qx", "plain", 1e-3), ("f16qx", "kahan", 1e-3),
            ("tex16", "plain", 1e-3), ("bf16q", "plain", 4e-3), ("bf16q", "kahan", 4e-3)]
FP32_STORAGES = ("f32", "f32q", "tex32", "f32qx")
SAMPLES = 20000


@pytest.fixture(scope="module")
def workload():
    from rabbitct_gb300 import build as b
    b.build_lolacuda()
    from rabbitct_gb300.lolacuda import DeviceBuffer
    scan = synth.make_scan(synth.ScanSpec(nproj=496))
    d_img = DeviceBuffer.from_array(scan.images)
    yield scan, d_img
    d_img.free()


_refs = {}


def _references(scan, n):
    """(sampled voxel indices, FP64 oracle, FP32-accumulating LolaBunny) at N."""
    if n not in _refs:
        vs = synth.voxel_size(n)
        o = synth.origin_index(n, vs)
        idx = np.random.default_rng(n).choice(n ** 3, SAMPLES, replace=False)
        ref64 = oracle.bunny_points(n, vs, o, scan.matrices, scan.images, idx)
        ref32 = oracle.bunny_points(n, vs, o, scan.matrices, scan.images, idx,
                                    fp32_accumulate=True)
        assert np.count_nonzero(ref64) > SAMPLES // 4  # most sampled voxels see the phantom
        _refs[n] = (idx, ref64, ref32)
    return _refs[n]


def _plan_points(scan, d_img, n, idx, storage, accum, batch):
    from rabbitct_gb300.lolacuda import Plan
    vs = synth.voxel_size(n)
    o = synth.origin_index(n, vs)
    with Plan(n, vs, o, scan.width, scan.height, storage=storage, accumulation=accum,
              batch=batch) as plan:
        plan.backproject_device(d_img.ptr, scan.width * scan.height, scan.matrices)
        plan.synchronize()
        return plan.download().reshape(-1)[idx]


def _row(label, e64, e32=None):
    s = (f"  {label:28s} rel_rmse={e64['rel_rmse']:.3e} rmse={e64['rmse']:.3e} "
         f"max_abs={e64['max_abs']:.3e} psnr={e64['psnr_db']:.1f}")
    if e32 is not None:
        s += f"  vs_bunny32={e32['rel_rmse']:.3e}"
    return s


@pytest.mark.parametrize("n", [512, 1024])
def test_full_size_accuracy(workload, n):
    scan, d_img = workload
    idx, ref64, ref32 = _references(scan, n)
    rows, failures = [], []
    for storage, accum, bar in VARIANTS:
        got = _plan_points(scan, d_img, n, idx, storage, accum, 16)
        e64 = metrics.errors(got, ref64)
        e32 = metrics.errors(got, ref32)
        rows.append(_row(f"{storage} {accum}", e64, e32))
        if e64["rel_rmse"] > bar:
            failures.append((storage, accum, "vs FP64", e64))
        # the spec bar of the FP32 path: LolaBunny itself within 1e-5
        if storage in FP32_STORAGES and e32["rel_rmse"] > 1e-5:
            failures.append((storage, accum, "vs FP32 LolaBunny", e32))
    print(f"\nN={n}: variant vs FP64 oracle (rel RMSE, RMSE, max abs, PSNR dB), "
          f"vs FP32-accumulating LolaBunny (rel RMSE)")
    print("\n".join(rows))
    assert not failures, failures


@pytest.mark.parametrize("n", [256, 512])
@pytest.mark.parametrize("with_geometry", [True, False], ids=["with_a", "without_a"])
def test_dropin_one_projection_per_call(workload, n, with_geometry):
    """The module API driven like rabbitRunner -b 1 (with or without -a), the
    library's default configuration (FP32 storage), full detector, 496 views:
    LolaBunny's FP32 result within 1e-5 and the FP64 oracle within 1e-5."""
    from rabbitct_gb300._native import config, load_lolacuda
    from rabbitct_gb300.lolacuda import module_functions
    from rabbitct_gb300.runner import run_module
    scan, _ = workload
    idx, ref64, ref32 = _references(scan, n)
    lib = load_lolacuda()
    assert lib.lolaCudaSetConfig(config(exit_on_error=0))
    vs = synth.voxel_size(n)
    o = synth.origin_index(n, vs)
    r = run_module(module_functions(lib, "lolaCuda"), n, vs, o, scan.matrices, scan.images,
                   batch=1, with_geometry=with_geometry)
    got = r.volume.reshape(-1)[idx]
    assert np.isfinite(r.volume).all()
    e64 = metrics.errors(got, ref64)
    e32 = metrics.errors(got, ref32)
    print("\n" + _row(f"N={n} -b 1 {'-a' if with_geometry else 'no -a'}", e64, e32))
    assert e32["rel_rmse"] <= 1e-5, e32
    assert e64["rel_rmse"] <= 1e-5, e64


def test_16bit_storage_pass_sizes(workload):
    """N=512, projections stored in FP16 (quads, mixed quads) and BF16 (quads),
    FP32 interpolation and accumulation, pass sizes 4..32, plain and Kahan."""
    scan, d_img = workload
    n = 512
    idx, ref64, _ = _references(scan, n)
    rows, failures = [], []
    for storage in ("f16q", "f16qx", "bf16q"):
        for batch in (4, 8, 16, 32):
            for accum in ("plain", "kahan"):
                got = _plan_points(scan, d_img, n, idx, storage, accum, batch)
                e64 = metrics.errors(got, ref64)
                rows.append(_row(f"{storage} b={batch} {accum}", e64))
                if not (e64["rel_rmse"] <= 1e-3):
                    failures.append((storage, batch, accum, e64))
    print(f"\nN={n}: 16-bit storage, pass size, accumulation vs FP64 oracle")
    print("\n".join(rows))
    assert not failures, failures
