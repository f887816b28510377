"""Device geometry analysis (lolaCudaComputeLineRanges / lolaCudaComputeShadow)
against the oracle restatements of computeLineRanges and
computeShadowOfProjection, which tests/test_oracle_golden.py pins to the
reference itself.  Bit-exact tables are required."""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np
import pytest

from conftest import small_spec
from oracle import oracle
from rabbitct_gb300 import synth

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"


@pytest.fixture(scope="module")
def lib():
    from rabbitct_gb300 import build as b
    b.build_lolacuda()
    from rabbitct_gb300._native import load_lolacuda
    return load_lolacuda()


def device_ranges(lib, n, vs, o, mats, w, h, vector_size, signed):
    from rabbitct_gb300._native import check
    from rabbitct_gb300.lolacuda import GlobalData
    gd = GlobalData(n, vs, o, w, h, 1, geometry=mats)
    out = np.zeros((mats.shape[0], n * n, 2), np.int16)
    ptrs = (C.c_void_p * mats.shape[0])(*[out[v].ctypes.data for v in range(mats.shape[0])])
    check(lib.lolaCudaComputeLineRanges(gd.ref, ptrs, vector_size, int(signed)), "ranges")
    return out


@pytest.mark.parametrize("name", ["bunny_n32", "bunny_n40_halffov"])
def test_line_ranges_match_reference_fixture(lib, name):
    g = dict(np.load(GOLDEN / f"{name}.npz"))
    n, vs, o = int(g["n"]), float(g["voxel_size"]), float(g["origin_index"])
    h, w = g["images"].shape[1:]
    got = device_ranges(lib, n, vs, o, g["matrices"], w, h, int(g["ranges_vector_size"]), False)
    assert np.array_equal(got, g["ranges"])


@pytest.mark.parametrize("n", [128, 256])
@pytest.mark.parametrize("vector_size", [4, 8, 16])
@pytest.mark.parametrize("signed", [False, True])
def test_line_ranges_full_detector(lib, n, vector_size, signed):
    spec = synth.ScanSpec(nproj=6, seed=12)
    mats = synth.matrices(spec)
    vs = synth.voxel_size(n)
    o = synth.origin_index(n, vs)
    want = oracle.line_ranges(n, vs, o, mats, spec.width, spec.height, vector_size, signed)
    got = device_ranges(lib, n, vs, o, mats, spec.width, spec.height, vector_size, signed)
    assert np.array_equal(got, want)


def test_line_ranges_source_inside_volume(lib):
    """Source inside the volume: some rows have w <= 0 and take the full scan."""
    spec = small_spec(nproj=4, width=96, height=80, seed=13)
    spec.sod = 100.0
    spec.sid = 160.0
    mats = synth.matrices(spec)
    n = 48
    vs = 256.0 / n
    o = synth.origin_index(n, vs)
    for signed in (False, True):
        want = oracle.line_ranges(n, vs, o, mats, spec.width, spec.height, 4, signed)
        got = device_ranges(lib, n, vs, o, mats, spec.width, spec.height, 4, signed)
        assert np.array_equal(got, want)


def test_shadow_matches_oracle(lib):
    from rabbitct_gb300.lolacuda import GlobalData
    spec = synth.ScanSpec(nproj=9, seed=14)
    mats = synth.matrices(spec)
    for n in (128, 512):
        vs = synth.voxel_size(n)
        o = synth.origin_index(n, vs)
        gd = GlobalData(n, vs, o, spec.width, spec.height, 1, geometry=mats)
        sh = np.zeros(4, np.int32)
        assert lib.lolaCudaComputeShadow(gd.ref, sh.ctypes.data) == 1
        assert tuple(sh) == oracle.shadow(n, vs, o, mats, spec.width, spec.height)
