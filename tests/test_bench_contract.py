"""bench.py's measurement contract on the host (no GPU): the default workload
is the N=1024, 496-projection scan; the roofline object is shaped as the
contract asks (bound hbm, GB/s against the measured HBM bandwidth, DRAM
traffic from the committed ncu capture) with the gather/issue ceiling nested;
and the issue-slot model covers every storage layout."""
from __future__ import annotations

import json
import sys
import types
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


@pytest.fixture(scope="module")
def bench():
    sys.path.insert(0, str(ROOT))
    import bench as b
    return b


def _args(b, *argv):
    old = sys.argv
    sys.argv = ["bench.py", *argv]
    try:
        return b.parse_args()
    finally:
        sys.argv = old


def test_default_workload(bench):
    a = _args(bench)
    assert (a.n, a.nproj, a.width, a.height) == (1024, 496, 1248, 960)
    assert a.storage == "f16qx" and a.gpus == 1 and a.warmup >= 3
    assert a.impl == "lolacuda"


def test_roofline_shape(bench):
    a = _args(bench)
    # one pass launch of the bench workload: 12 ms, 12.4e9 computed updates
    st = types.SimpleNamespace(tilePassesFast=378_000, tilePassesSlow=0,
                               tilePassesSkipped=147_000, tilePassesPaired=365_000,
                               passes=1, passMs=12.0)
    probes = {"issue_inst_per_s": 3.9e13, "gather": {"f16qx": 1.8e12},
              "gather_peak": {"f16qx": 2.6e12}}
    r = bench.roofline(a, None, "f16qx", st, probes)
    assert r["bound"] == "hbm" and r["unit"] == "GB/s"
    peaks = ROOT / "MEASURED_PEAKS.json"
    peak = json.loads(peaks.read_text())["hbm_gbs"] if peaks.exists() else 6800.0
    assert r["peak"] == pytest.approx(peak)
    alg = r["algorithmic_bytes_per_launch"]
    assert alg > 8 * 1024 ** 3  # the volume read and written once
    assert r["achieved"] == pytest.approx(alg / 12e-3 / 1e9)
    assert r["frac"] == pytest.approx(r["achieved"] / r["peak"])
    # f16qx at 16x4 tiles, batch 16, N=1024 has a committed DRAM capture
    assert r["traffic"] is not None and r["traffic"] >= alg
    c = r["ceiling"]
    assert c["unit"] == "Gupdate/s" and c["bound"] in ("gather", "issue")
    assert c["peak"] == pytest.approx(min(c["peak_gather"], c["peak_issue"]))
    assert c["peak_gather"] >= c["gather_l2_random"]
    assert 0 < c["paired_fraction"] <= 1
    # the committed f16qx capture gives the kernel's wavefronts per texture
    # request: the locality-matched gather ceiling is the probe's rate over it
    wpr = c["ncu_pipes"]["tex_wf_per_request"]
    assert wpr >= 1.0
    assert c["peak_gather_locality"] == pytest.approx(c["peak_gather"] / wpr)
    assert c["frac_of_locality_gather"] == pytest.approx(c["achieved"] / c["peak_gather_locality"])


def test_traffic_only_for_captured_configurations(bench):
    assert bench.dram_traffic("f16qx", 16, 4, 16, 1024)[0] is not None
    assert bench.dram_traffic("f32q", 16, 4, 32, 1024)[0] is not None
    assert bench.dram_traffic("f16qx", 8, 8, 16, 1024) == (None, None)
    assert bench.dram_traffic("f16qx", 16, 4, 16, 512) == (None, None)


@pytest.mark.parametrize("storage", ["f32", "f16", "bf16", "f32q", "f16q", "bf16q", "tex32",
                                     "tex16", "f16qx", "f32qx"])
def test_issue_model_covers_every_layout(bench, storage):
    paired = bench.instr_per_update(storage, 1.0)
    single = bench.instr_per_update(storage, 0.0)
    assert 5 < paired < single < 40
