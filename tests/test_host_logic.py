"""Host-side behaviour of the C library that needs no GPU: configuration
validation, environment overrides, and the module API's error convention
(return 0 and a message instead of exit when exitOnError is 0)."""
from __future__ import annotations

import ctypes as C
import os

import numpy as np
import pytest


@pytest.fixture(scope="module")
def lib():
    from rabbitct_gb300 import build as b
    b.build_lolacuda()
    from rabbitct_gb300._native import load_lolacuda
    return load_lolacuda()


def test_config_validation(lib):
    from rabbitct_gb300._native import LolaCudaConfig, config
    good = config(storage="f16q", batch=8, exit_on_error=0)
    assert lib.lolaCudaSetConfig(C.byref(good)) == 1
    got = LolaCudaConfig()
    lib.lolaCudaGetConfig(C.byref(got))
    assert (got.storage, got.batch) == (4, 8)
    for field, value in (("storage", 99), ("batch", 0), ("batch", 65), ("accumulation", 7),
                         ("voxelsPerThread", 3)):
        bad = config(exit_on_error=0)
        setattr(bad, field, value)
        assert lib.lolaCudaSetConfig(C.byref(bad)) == 0
        assert lib.lolaCudaLastError()


def test_edge_batch_validation(lib):
    """The edge batch is 0 (twice the batch) or batch..64."""
    from rabbitct_gb300._native import config
    for batch, edge, ok in ((16, 0, True), (16, 16, True), (16, 32, True), (16, 15, False),
                            (16, 64, True), (16, 65, False), (32, 0, True), (1, 1, True)):
        c = config(batch=batch, edge_batch=edge, exit_on_error=0)
        assert lib.lolaCudaSetConfig(C.byref(c)) == int(ok), (batch, edge)
        if not ok:
            assert b"edge batch" in lib.lolaCudaLastError()


def test_environment_overrides(lib, monkeypatch):
    from rabbitct_gb300._native import LolaCudaConfig
    monkeypatch.setenv("LOLACUDA_STORAGE", "bf16q")
    monkeypatch.setenv("LOLACUDA_ACCUM", "kahan")
    monkeypatch.setenv("LOLACUDA_BATCH", "4")
    monkeypatch.setenv("LOLACUDA_EXIT", "0")
    monkeypatch.setenv("LOLACUDA_EDGE_BATCH", "12")
    c = LolaCudaConfig()
    lib.lolaCudaDefaultConfig(C.byref(c))
    assert (c.storage, c.accumulation, c.batch, c.exitOnError, c.edgeBatch) == (5, 1, 4, 0, 12)


def test_module_api_errors_without_prepare(lib):
    from rabbitct_gb300._native import config
    from rabbitct_gb300.lolacuda import GlobalData, module_functions
    assert lib.lolaCudaSetConfig(C.byref(config(exit_on_error=0)))
    prepare, iterate, finish = module_functions(lib, "lolaCuda")
    gd = GlobalData(16, 1.0, -7.5, 32, 24, 1)
    assert iterate(gd.ref) == 0
    assert "before prepare" in lib.lolaCudaLastError().decode()
    assert finish(gd.ref) == 0


def test_prepare_rejects_null_volume(lib):
    from rabbitct_gb300._native import RabbitCtGlobalData, config
    from rabbitct_gb300.lolacuda import module_functions
    assert lib.lolaCudaSetConfig(C.byref(config(exit_on_error=0)))
    prepare, _, _ = module_functions(lib, "lolaCuda")
    d = RabbitCtGlobalData()
    d.problemSize, d.imageWidth, d.imageHeight = 16, 32, 24
    d.voxelSize, d.O_Index = 1.0, -7.5
    assert prepare(C.byref(d)) == 0
    assert "volumeData" in lib.lolaCudaLastError().decode()


def test_plan_create_reports_bad_device(lib):
    from rabbitct_gb300._native import LolaCudaGeometry, config
    g = LolaCudaGeometry(16, 32, 24, 1.0, -7.5)
    cfg = config(device=999)
    h = C.c_void_p()
    assert lib.lolaCudaPlanCreate(C.byref(g), C.byref(cfg), C.byref(h)) == 0
    assert not h.value
    assert lib.lolaCudaLastError()


def test_plan_create_rejects_bad_geometry(lib):
    from rabbitct_gb300._native import LolaCudaGeometry, config
    h = C.c_void_p()
    for g in (LolaCudaGeometry(0, 32, 24, 1.0, 0.0), LolaCudaGeometry(16, 32, 24, 0.0, 0.0),
              LolaCudaGeometry(4096, 32, 24, 1.0, 0.0)):
        assert lib.lolaCudaPlanCreate(C.byref(g), C.byref(config()), C.byref(h)) == 0


def test_no_alloc_validates_before_touching_the_device(lib):
    from rabbitct_gb300._native import LolaCudaGeometry, config
    g = LolaCudaGeometry(16, 32, 24, 1.0, -7.5)
    m = np.zeros((1, 12))
    assert lib.lolaCudaBackprojectNoAlloc(None, None, None, None, 0, None, 1, None) == 0
    assert lib.lolaCudaBackprojectNoAlloc(C.byref(g), C.byref(config()), None, None, 0,
                                          m.ctypes.data, -1, None) == 0
    bad = config()
    bad.storage = 6  # texture layouts need texture objects: not offered here
    assert lib.lolaCudaBackprojectNoAlloc(C.byref(g), C.byref(bad), C.c_void_p(16),
                                          C.c_void_p(16), 32 * 24, m.ctypes.data, 1, None) == 0
    # zero projections: nothing to do, success without device work
    assert lib.lolaCudaBackprojectNoAlloc(C.byref(g), C.byref(config()), None, None, 0,
                                          m.ctypes.data, 0, None) == 1


def test_runner_rejects_batch_not_dividing_projections():
    from rabbitct_gb300.runner import run_module
    imgs = np.zeros((5, 4, 4), np.float32)
    with pytest.raises(ValueError):
        run_module((None, None, None), 8, 1.0, -3.5, np.zeros((5, 12)), imgs, batch=2)
