"""The drop-in as a maintainer would build it: the reference runner compiled
from its own sources with a registry that has a LolaCUDA row
(oracle/registry_lolacuda.c), linked to liblolacuda.so (oracle/ref.mk, target
`lolacuda`).  Needs the reference source tree, so it runs where that tree is
and is skipped elsewhere.

On a host without a GPU the runner must reach LolaCUDA's prepare through the
registry and stop there with the module's error convention (message and
non-zero exit, src/error.h:21-31), while the reference's own modules in the
same binary still reconstruct.  On a GPU host the same binary reconstructs
through LolaCUDA and must agree with LolaBunny."""
from __future__ import annotations

import os
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from oracle import refpath
from rabbitct_gb300 import rct, synth

ROOT = Path(__file__).resolve().parent.parent
REF = refpath.reference_root()
RUNNER = ROOT / "oracle" / "_ref" / "rabbitRunnerLolaCUDA"


@pytest.fixture(scope="module")
def runner():
    if not (REF / "src" / "rabbitRunner.c").exists() or shutil.which("gcc") is None:
        pytest.skip("reference sources or gcc not available")
    from rabbitct_gb300 import build as b
    b.build_lolacuda()
    subprocess.run(["make", "-C", str(ROOT), "-f", "oracle/ref.mk", f"REF={REF}", "lolacuda"],
                   check=True, capture_output=True)
    return RUNNER


@pytest.fixture(scope="module")
def scan_file(tmp_path_factory):
    scan = synth.make_scan(synth.ScanSpec(nproj=4, seed=5))
    path = tmp_path_factory.mktemp("rct") / "scan.rct"
    rct.write_rct(path, scan.images, scan.matrices, scan.hus)
    return path


def _run(runner, module, scan_file, out, cwd):
    env = dict(os.environ, OMP_NUM_THREADS="4")
    return subprocess.run([str(runner), "-m", module, "-s", "128", "-b", "2", "-i",
                           str(scan_file), "-o", str(out)], capture_output=True, text=True,
                          cwd=cwd, env=env, timeout=600)


def test_registry_lists_lolacuda(runner, tmp_path):
    p = subprocess.run([str(runner), "-m", "NoSuchModule", "-s", "128", "-i", "x.rct"],
                       capture_output=True, text=True, cwd=tmp_path, timeout=60)
    assert "LolaCUDA" in p.stdout and "LolaBunny" in p.stdout


def test_reference_modules_still_run(runner, scan_file, tmp_path):
    p = _run(runner, "LolaBunny", scan_file, tmp_path / "bunny.vol", tmp_path)
    assert p.returncode == 0, p.stdout + p.stderr
    vol = np.fromfile(tmp_path / "bunny.vol", np.float32)
    assert vol.size == 128 ** 3 and np.abs(vol).max() > 0


def test_lolacuda_through_the_runner(runner, scan_file, tmp_path):
    """No GPU: prepare fails loudly.  With a GPU: the volume agrees with the
    same binary's LolaBunny within the FP32 bar."""
    p = _run(runner, "LolaCUDA", scan_file, tmp_path / "cuda.vol", tmp_path)
    if not _has_gpu():
        assert p.returncode != 0
        assert "LolaCUDA prepare" in (p.stdout + p.stderr)
        return
    assert p.returncode == 0, p.stdout + p.stderr
    q = _run(runner, "LolaBunny", scan_file, tmp_path / "bunny.vol", tmp_path)
    assert q.returncode == 0
    got = np.fromfile(tmp_path / "cuda.vol", np.float32)
    want = np.fromfile(tmp_path / "bunny.vol", np.float32)
    rel = np.sqrt(np.mean((got.astype(np.float64) - want) ** 2)) / np.sqrt(np.mean(
        want.astype(np.float64) ** 2))
    assert rel <= 1e-5


def _has_gpu() -> bool:
    smi = shutil.which("nvidia-smi")
    return smi is not None and subprocess.run([smi, "-L"], capture_output=True).returncode == 0
