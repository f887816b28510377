"""GPU test of lolaCudaBackprojectNoAlloc, the entry point for callers that
cannot allocate device memory at run time (an acquisition loop that reserved
its memory at start-up and must not stall on cudaMalloc/cudaFree, or a host
framework that owns the device memory pool).

It calls the entry point through the C ABI twice in a row, on different
scans, storage types and sizes, and checks each result against the existing
plan entry point (lolaCudaPlanBackprojectDevice) within the FP32 tolerance the
other parity tests use.  The second call runs on scratch the first call left
behind, so stale contents would show up there.  The file name sorts last so a
run that stops at the first failure has run every other test before it.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from conftest import small_spec
from rabbitct_gb300 import metrics, synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib():
    from rabbitct_gb300 import build as b
    b.build_lolacuda()
    from rabbitct_gb300._native import load_lolacuda
    return load_lolacuda()


def _plan_volume(scan, n, vs, o, storage):
    from rabbitct_gb300.lolacuda import DeviceBuffer, Plan
    d_img = DeviceBuffer.from_array(scan.images)
    with Plan(n, vs, o, scan.width, scan.height, storage=storage, batch=8) as plan:
        plan.backproject_device(d_img.ptr, scan.width * scan.height, scan.matrices)
        plan.synchronize()
        vol = plan.download()
    d_img.free()
    return vol


def _no_alloc_volume(lib, scan, n, vs, o, storage):
    from rabbitct_gb300._native import LolaCudaGeometry, check, config
    from rabbitct_gb300.lolacuda import DeviceBuffer
    g = LolaCudaGeometry(n, scan.width, scan.height, vs, o)
    cfg = config(storage=storage, batch=8)
    d_img = DeviceBuffer.from_array(scan.images)
    d_vol = DeviceBuffer.from_array(np.zeros((n, n, n), np.float32))
    mats = np.ascontiguousarray(scan.matrices)
    check(lib.lolaCudaBackprojectNoAlloc(C.byref(g), C.byref(cfg), d_vol.ptr, d_img.ptr,
                                         scan.width * scan.height, mats.ctypes.data,
                                         scan.nproj, None), "no-alloc backprojection")
    check(lib.lolaCudaDeviceSynchronize(), "synchronize")
    vol = d_vol.to_array((n, n, n), np.float32)
    d_img.free()
    d_vol.free()
    return vol


def test_no_alloc_matches_plan_on_two_calls(lib):
    cases = [
        (synth.make_scan(small_spec(nproj=12, seed=31)), 48, "f32"),
        (synth.make_scan(small_spec(nproj=10, width=128, height=96, seed=32)), 40, "f16q"),
    ]
    for scan, n, storage in cases:
        vs = 256.0 / n
        o = synth.origin_index(n, vs)
        got = _no_alloc_volume(lib, scan, n, vs, o, storage)
        want = _plan_volume(scan, n, vs, o, storage)
        e = metrics.errors(got, want)
        assert e["rel_rmse"] <= 1e-5, (storage, e)
        assert np.isfinite(got).all()


def test_no_alloc_rejects_oversized_projection(lib):
    from rabbitct_gb300._native import LolaCudaGeometry, config, last_error
    # a 1600x1400 FP32-quad projection packs to about 42 MB > 32 MiB of scratch
    g = LolaCudaGeometry(64, 1600, 1400, 4.0, synth.origin_index(64, 4.0))
    cfg = config(storage="f32q")
    mats = np.zeros((1, 12), np.float64)
    ok = lib.lolaCudaBackprojectNoAlloc(C.byref(g), C.byref(cfg), C.c_void_p(16),
                                        C.c_void_p(16), 1600 * 1400, mats.ctypes.data, 1, None)
    assert ok == 0
    assert "scratch" in last_error()
