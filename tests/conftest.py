"""Shared test setup.

Markers: `gpu` — needs a CUDA device (runs the CUDA path through the C ABI).
Everything else runs on CPU: the oracle against the reference and the golden
fixtures, host logic, file formats, and the C-ABI library's exports.
"""
from __future__ import annotations

import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session", autouse=True)
def _native_libs():
    """Builds the in-tree libraries once per session if they are missing."""
    from rabbitct_gb300 import build as b
    from oracle import oracle
    b.build_synth()
    if not oracle.LIB.exists():
        oracle.build()
    yield


def small_spec(**kw):
    """A reduced detector whose pixels are scaled so that it covers the same
    field of view as the 1248x960 detector (pitch * width kept constant)."""
    from rabbitct_gb300 import synth
    width = kw.pop("width", 160)
    height = kw.pop("height", 128)
    base = dict(nproj=12, width=width, height=height, pitch=0.308 * 1248 / width, seed=11)
    base.update(kw)
    return synth.ScanSpec(**base)
