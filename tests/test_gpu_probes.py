"""The roofline probes on the GPU: they run, return rates, and the texture
request probe shows the cost of a request that straddles detector rows (one
data-stage wavefront per row touched), which the pass kernel's lane layout
is built around."""
from __future__ import annotations

import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib():
    from rabbitct_gb300 import build as b
    b.build_lolacuda()
    from rabbitct_gb300._native import load_lolacuda
    return load_lolacuda()


def test_issue_and_gather_probes(lib):
    from rabbitct_gb300._native import STORAGE
    assert lib.lolaCudaProbeIssueRate() > 1e12
    for name in ("f32", "f32q", "f16qx"):
        peak = lib.lolaCudaProbeGatherPeak(STORAGE[name])
        l2 = lib.lolaCudaProbeGatherRate(STORAGE[name], 1248, 960)
        assert peak > 1e11 and l2 > 1e11, name
    assert lib.lolaCudaProbeGatherPeak(99) < 0


def test_texture_requests_over_more_rows_cost_more(lib):
    r1, r2, r8 = (lib.lolaCudaProbeTextureRows(r) for r in (1, 2, 8))
    assert r1 > 1.5 * r2 > 0
    assert r2 > 1.5 * r8 > 0
    assert lib.lolaCudaProbeTextureRows(3) < 0
