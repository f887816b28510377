"""The .rct format, the synthetic scan generator and the error metrics."""
from __future__ import annotations

import math

import numpy as np
import pytest

from rabbitct_gb300 import metrics, rct, synth


def test_rct_roundtrip(tmp_path):
    rng = np.random.default_rng(3)
    imgs = rng.standard_normal((3, 5, 7)).astype(np.float32)
    mats = rng.standard_normal((3, 12))
    p = tmp_path / "x.rct"
    rct.write_rct(p, imgs, mats, (123.5, -4.0))
    assert p.stat().st_size == 20 + 3 * (96 + 4 * 35)
    with rct.RctReader(p) as r:
        assert (r.header.width, r.header.height, r.header.count) == (7, 5, 3)
        assert r.header.hus == (123.5, -4.0)
        m = np.zeros(12)
        im = np.zeros((5, 7), np.float32)
        for k in range(3):
            assert r.read_image(m, im) == k + 1  # 1-based ids, file order
            assert np.array_equal(m, mats[k]) and np.array_equal(im, imgs[k])
        with pytest.raises(EOFError):
            r.read_image(m, im)
    g = tmp_path / "g.rct"
    rct.write_geometry(g, mats, 7, 5)
    h, m2 = rct.read_geometry(g)
    assert h.count == 3 and np.array_equal(m2, mats)


def test_voxel_size_and_origin_follow_runner():
    assert [synth.voxel_size(n) for n in (128, 256, 512, 1024)] == [2.0, 1.0, 0.5, 0.25]
    # -0.5f * vs * ((float)N - 1.0f) in float32
    assert synth.origin_index(512, 0.5) == float(np.float32(-0.25) * np.float32(511.0))
    assert synth.origin_index(128, 2.0) == -127.0


def test_generator_is_deterministic_and_geometric():
    spec = synth.ScanSpec(nproj=6, width=96, height=80, pitch=0.308 * 13, seed=4)
    a, b = synth.make_scan(spec), synth.make_scan(spec)
    assert np.array_equal(a.images, b.images) and np.array_equal(a.matrices, b.matrices)
    for p in range(spec.nproj):
        P = a.matrices[p].reshape(4, 3).T  # column-major a[col*3+row]
        u, v, w = P @ np.array([0.0, 0.0, 0.0, 1.0])
        assert w == pytest.approx(spec.sod)  # isocentre depth
        assert abs(u / w - (spec.width - 1) / 2) <= spec.pp_jitter + 1e-9
        assert abs(v / w - (spec.height - 1) / 2) <= spec.pp_jitter + 1e-9
    assert a.images.max() > 1.0  # ellipsoid line integrals present
    other = synth.make_scan(synth.ScanSpec(nproj=6, width=96, height=80, pitch=0.308 * 13,
                                           seed=5))
    assert not np.array_equal(a.images, other.images)


def test_error_metrics():
    ref = np.array([1.0, 2.0, 3.0, 4.0])
    test = ref + np.array([0.0, 0.1, -0.1, 0.0])
    e = metrics.errors(test, ref)
    assert e["max_abs"] == pytest.approx(0.1)
    assert e["rmse"] == pytest.approx(math.sqrt(0.02 / 4))
    assert e["rel_rmse"] == pytest.approx(e["rmse"] / math.sqrt(30 / 4))
    assert e["psnr_db"] == pytest.approx(20 * math.log10(4.0 / e["rmse"]))
    assert metrics.errors(ref, ref)["psnr_db"] == math.inf


def test_hu_conversion_semantics():
    vol = np.array([-1.0, 0.0, 0.001, 0.0015, 1.0], np.float32)
    hu = metrics.to_hu(vol, (1000.0, 0.0))
    assert hu.tolist() == [0.0, 0.0, 1.0, 2.0, 1000.0]   # floor(x + 0.5); v <= 0 -> 0
    assert metrics.to_hu(np.array([10.0], np.float32), (1000.0, 0.0))[0] == 4095.0
