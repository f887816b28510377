"""GPU test of lolaCudaBackprojectNoAlloc, the entry point for callers that
cannot allocate device memory at run time (an acquisition loop that reserved
its memory at start-up and must not stall on cudaMalloc/cudaFree, or a host
framework that owns the device memory pool).

It calls the entry point through the C ABI twice in a row, on different
scans, storage types and sizes, and checks each result against the existing
plan entry point (lolaCudaPlanBackprojectDevice) with the same pass size:
the same kernels and pass partition, so the volumes must be equal bit for
bit.  Each result is also checked against the FP64 LolaBunny oracle with the
bars of the other parity tests.  The second call runs on scratch the first
call left behind, so stale contents would show up there.  The cases cover a
detector width whose padded pitch is not a multiple of 32 pixels, a mixed
storage (run by loads only), and a z-slab of the volume.  The file name sorts
last so a run that stops at the first failure has run every other test
before it.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from conftest import small_spec
from oracle import oracle
from rabbitct_gb300 import metrics, synth

pytestmark = pytest.mark.gpu

BAR = {"f32": 1e-5, "f32q": 1e-5, "f16q": 1e-3, "f16qx": 1e-3, "bf16": 4e-3}


@pytest.fixture(scope="module")
def lib():
    from rabbitct_gb300 import build as b
    b.build_lolacuda()
    from rabbitct_gb300._native import load_lolacuda
    return load_lolacuda()


def _plan_volume(scan, n, vs, o, storage, slab=None):
    from rabbitct_gb300.lolacuda import DeviceBuffer, Plan
    d_img = DeviceBuffer.from_array(scan.images)
    with Plan(n, vs, o, scan.width, scan.height, storage=storage, batch=8, slab=slab) as plan:
        plan.backproject_device(d_img.ptr, scan.width * scan.height, scan.matrices)
        plan.synchronize()
        vol = plan.download()
    d_img.free()
    return vol


def _no_alloc_volume(lib, scan, n, vs, o, storage, slab=(0, 0)):
    from rabbitct_gb300._native import LolaCudaGeometry, check, config
    from rabbitct_gb300.lolacuda import DeviceBuffer
    g = LolaCudaGeometry(n, scan.width, scan.height, vs, o, slab[0], slab[1])
    depth = slab[1] or n
    cfg = config(storage=storage, batch=8)
    d_img = DeviceBuffer.from_array(scan.images)
    d_vol = DeviceBuffer.from_array(np.zeros((depth, n, n), np.float32))
    mats = np.ascontiguousarray(scan.matrices)
    check(lib.lolaCudaBackprojectNoAlloc(C.byref(g), C.byref(cfg), d_vol.ptr, d_img.ptr,
                                         scan.width * scan.height, mats.ctypes.data,
                                         scan.nproj, None), "no-alloc backprojection")
    check(lib.lolaCudaDeviceSynchronize(), "synchronize")
    vol = d_vol.to_array((depth, n, n), np.float32)
    d_img.free()
    d_vol.free()
    return vol


CASES = [
    # (scan, N, storage): FP32 taps; FP16 quads on another detector; a width whose
    # padded pitch (150 + 128) is not a multiple of 32; f16qx, run as f16q
    (dict(nproj=12, seed=31), 48, "f32"),
    (dict(nproj=10, width=128, height=96, seed=32), 40, "f16q"),
    (dict(nproj=11, width=150, height=118, seed=33), 36, "f32q"),
    (dict(nproj=9, width=150, height=118, seed=34), 40, "f16qx"),
]


def test_no_alloc_matches_plan_on_two_calls(lib):
    for kw, n, storage in CASES:
        scan = synth.make_scan(small_spec(**kw))
        vs = 256.0 / n
        o = synth.origin_index(n, vs)
        first = _no_alloc_volume(lib, scan, n, vs, o, storage)
        second = _no_alloc_volume(lib, scan, n, vs, o, storage)
        want = _plan_volume(scan, n, vs, o, storage)
        assert np.isfinite(first).all()
        assert np.array_equal(first, want), (storage, metrics.errors(first, want))
        assert np.array_equal(second, want), (storage, metrics.errors(second, want))
        ref = oracle.bunny_f64(n, vs, o, scan.matrices, scan.images)
        e = metrics.errors(first, ref)
        assert e["rel_rmse"] <= BAR[storage], (storage, e)


def test_no_alloc_slab_matches_plan_slab(lib):
    """A z-slab geometry writes N x N x sliceCount voxels, the slab of the
    whole-volume result (slabs start at multiples of the tile depth)."""
    scan = synth.make_scan(small_spec(nproj=10, seed=35))
    n = 48
    vs = 256.0 / n
    o = synth.origin_index(n, vs)
    whole = _plan_volume(scan, n, vs, o, "f32")
    got = _no_alloc_volume(lib, scan, n, vs, o, "f32", slab=(16, 16))
    assert got.shape == (16, n, n)
    assert np.array_equal(got, whole[16:32])
    assert np.array_equal(got, _plan_volume(scan, n, vs, o, "f32", slab=(16, 16)))


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


def test_no_alloc_rejects_bad_slab_and_texture_storage(lib):
    from rabbitct_gb300._native import LolaCudaGeometry, config, last_error
    mats = np.zeros((1, 12), np.float64)
    g = LolaCudaGeometry(32, 64, 48, 8.0, synth.origin_index(32, 8.0), 24, 16)
    ok = lib.lolaCudaBackprojectNoAlloc(C.byref(g), C.byref(config(storage="f32")),
                                        C.c_void_p(16), C.c_void_p(16), 64 * 48,
                                        mats.ctypes.data, 1, None)
    assert ok == 0 and "slab" in last_error()
    g = LolaCudaGeometry(32, 64, 48, 8.0, synth.origin_index(32, 8.0))
    ok = lib.lolaCudaBackprojectNoAlloc(C.byref(g), C.byref(config(storage="tex16")),
                                        C.c_void_p(16), C.c_void_p(16), 64 * 48,
                                        mats.ctypes.data, 1, None)
    assert ok == 0 and "texture" in last_error()
