"""The oracle against golden fixtures made by the reference itself
(tests/golden/make_golden.py) and, where the reference was built here
(oracle/_ref), against the live reference.  CPU only.

The reference compiles with -ffast-math -march=native, so its compiler may
contract a multiply-add into an FMA that the oracle (built without
contraction) rounds twice: the FP32-accumulating oracle must agree with
LolaBunny to within 2 ulp per voxel (in practice all but a few voxels are
bit-identical)."""
from __future__ import annotations

import hashlib
import json
import os
import subprocess
from pathlib import Path

import numpy as np
import pytest

from oracle import oracle
from rabbitct_gb300 import metrics, rct, synth

GOLDEN = Path(__file__).resolve().parent / "golden"
CASES = ["bunny_n32", "bunny_n40_halffov"]


def load(name):
    return dict(np.load(GOLDEN / f"{name}.npz"))


@pytest.mark.parametrize("name", CASES)
def test_bunny_f32_oracle_matches_reference_to_2ulp(name):
    g = load(name)
    n, vs, o = int(g["n"]), float(g["voxel_size"]), float(g["origin_index"])
    v = oracle.bunny_f32(n, vs, o, g["matrices"], g["images"])
    np.testing.assert_array_max_ulp(v, g["bunny"], maxulp=2)


@pytest.mark.parametrize("name", CASES)
def test_bunny_f64_oracle_close_to_reference(name):
    g = load(name)
    n, vs, o = int(g["n"]), float(g["voxel_size"]), float(g["origin_index"])
    v = oracle.bunny_f64(n, vs, o, g["matrices"], g["images"])
    e = metrics.errors(g["bunny"], v)
    assert e["rel_rmse"] < 1e-6, e


@pytest.mark.parametrize("name", CASES)
def test_line_ranges_equal_reference(name):
    g = load(name)
    n, vs, o = int(g["n"]), float(g["voxel_size"]), float(g["origin_index"])
    h, w = g["images"].shape[1:]
    r = oracle.line_ranges(n, vs, o, g["matrices"], w, h, int(g["ranges_vector_size"]),
                           signed_hit=False)
    assert np.array_equal(r, g["ranges"])


@pytest.mark.parametrize("name", CASES)
def test_shadow_equals_reference(name):
    g = load(name)
    n, vs, o = int(g["n"]), float(g["voxel_size"]), float(g["origin_index"])
    h, w = g["images"].shape[1:]
    assert tuple(oracle.shadow(n, vs, o, g["matrices"], w, h)) == tuple(g["shadow"])


@pytest.mark.parametrize("name", CASES)
def test_opt_port_matches_reference_opt(name):
    g = load(name)
    n, vs, o = int(g["n"]), float(g["voxel_size"]), float(g["origin_index"])
    h, w = g["images"].shape[1:]
    ob = oracle.OptBaseline(n, vs, o, g["matrices"], w, h,
                            vector_size=int(g["ranges_vector_size"]))
    vol = np.zeros((n, n, n), np.float32)
    for i in range(g["images"].shape[0]):
        ob.backproject(vol, np.array([i + 1]), g["images"][i:i + 1])
    e = metrics.errors(vol, g["opt"])
    assert e["rel_rmse"] < 1e-6, e


def test_asm_port_matches_reference_asm():
    """The LolaASM restatement (oracle_asm.c) against the reference's own
    LolaASM (src/LolaASM.c:84-211 and its SIMD row kernel) on the same inputs,
    with the reference build's vector width.  They differ only in how the
    reciprocal is refined (see oracle_asm.c)."""
    g = load("bunny_n32")
    a = np.load(GOLDEN / "bunny_n32_asm.npz")
    n, vs, o = int(g["n"]), float(g["voxel_size"]), float(g["origin_index"])
    h, w = g["images"].shape[1:]
    ab = oracle.AsmBaseline(n, vs, o, g["matrices"], w, h,
                            vector_size=int(a["asm_vector_size"]))
    vol = np.zeros((n, n, n), np.float32)
    for i in range(g["images"].shape[0]):
        ab.backproject(vol, np.array([i + 1]), g["images"][i:i + 1])
    # compared on voxels inside their row's range for every view: outside it
    # the reference's row kernel still runs up to a vector width of voxels,
    # some of whose taps lie past its padded buffer (its top pad is one row
    # short), so their values are whatever memory follows the buffer
    inside = np.ones((n * n, n), bool)
    x = np.arange(n)
    for p in range(ab.ranges.shape[0]):
        lo = ab.ranges[p, :, 0].astype(int)[:, None]
        hi = ab.ranges[p, :, 1].astype(int)[:, None]
        inside &= (x >= lo) & (x < hi)
    inside = inside.reshape(n, n, n)
    assert inside.sum() > n ** 3 // 4
    e = metrics.errors(vol[inside], a["asm"][inside])
    assert e["rel_rmse"] < 1e-6, e


def test_signed_hit_ranges_cover_bunny_support():
    """With the signed hit test every voxel LolaBunny gives a non-zero
    contribution lies inside its row's range; the reference's unsigned test
    misses the u or v in (-2, -1] band (its documented clipping gap)."""
    g = load("bunny_n40_halffov")
    n, vs, o = int(g["n"]), float(g["voxel_size"]), float(g["origin_index"])
    h, w = g["images"].shape[1:]
    signed = oracle.line_ranges(n, vs, o, g["matrices"], w, h, 1, signed_hit=True)
    for p in range(g["matrices"].shape[0]):
        contrib = oracle.bunny_f64(n, vs, o, g["matrices"][p:p + 1], g["images"][p:p + 1])
        rows = contrib.reshape(n * n, n)
        for r in np.flatnonzero(np.any(rows != 0, axis=1)):
            xs = np.flatnonzero(rows[r] != 0)
            lo, hi = signed[p, r]
            assert lo <= xs.min() and xs.max() < hi


def test_runner_fixture_inputs_reproduce():
    info = json.loads((GOLDEN / "runner_n128.json").read_text())
    spec = synth.ScanSpec(**info["spec"])
    scan = synth.make_scan(spec)
    assert hashlib.sha256(scan.images.tobytes()).hexdigest() == info["images_sha256"]
    assert np.array_equal(scan.matrices, np.array(info["matrices"]))


def test_bunny_oracle_matches_reference_runner_n128():
    """The reference runner (rabbitRunner -m LolaBunny -s 128 -c ... -o ...
    on a .rct file) against the FP32-accumulating oracle.  With -c the runner
    converts the volume to HU in place (src/rabbitRunner.c:362) before -o
    writes it (:426-430), so the stored volume is in HU."""
    info = json.loads((GOLDEN / "runner_n128.json").read_text())
    scan = synth.make_scan(synth.ScanSpec(**info["spec"]))
    n = info["n"]
    vs = synth.voxel_size(n)
    o = synth.origin_index(n, vs)
    v = oracle.bunny_f32(n, vs, o, scan.matrices, scan.images)
    hu = metrics.to_hu(v, info["hus"])
    sample = hu.reshape(-1)[::info["sample_stride"]]
    want = np.array(info["volume_sample"], np.float32)
    diff = np.abs(sample - want)
    assert diff.max() <= 1.0
    assert np.count_nonzero(diff) <= max(1, sample.size // 10000)
    assert float(hu.astype(np.float64).sum()) == pytest.approx(info["volume_sum"], rel=1e-6)


def test_hu_metrics_match_runner_verification():
    """metrics.hu_quality restates src/rabbitRunner.c:320-384; compare with the
    numbers the reference runner printed for the same volumes."""
    info = json.loads((GOLDEN / "runner_n128.json").read_text())
    scan = synth.make_scan(synth.ScanSpec(**info["spec"]))
    n = info["n"]
    vs = synth.voxel_size(n)
    o = synth.origin_index(n, vs)
    bunny = oracle.bunny_f32(n, vs, o, scan.matrices, scan.images)
    v64 = oracle.bunny_f64(n, vs, o, scan.matrices, scan.images)
    hu_ref = metrics.to_hu(v64.astype(np.float32), info["hus"]).astype(np.uint16)
    assert hashlib.sha256(hu_ref.tobytes()).hexdigest() == info["hu_reference_sha256"]
    q = metrics.hu_quality(bunny, hu_ref, info["hus"])
    printed = info["runner_quality"]
    assert q["rmse_hu"] == pytest.approx(printed["rmse_hu"], rel=1e-5)
    assert q["max_abs_hu"] == printed["max_abs_hu"]
    assert q["psnr_db"] == pytest.approx(printed["psnr_db"], abs=0.05)


# ---- live reference (only where oracle/_ref was built from the sources) -------

needs_ref = pytest.mark.skipif(not oracle.ref_available(),
                               reason="reference not built here (needs its source tree)")


@needs_ref
def test_live_reference_bunny_random_scan():
    from rabbitct_gb300.lolacuda import module_functions
    from rabbitct_gb300.runner import run_module
    from conftest import small_spec
    scan = synth.make_scan(small_spec(nproj=4, width=96, height=72, seed=909))
    n = 24
    vs = 256.0 / n
    o = synth.origin_index(n, vs)
    r = run_module(module_functions(oracle.ref_lib(), "lolaBunny"), n, vs, o, scan.matrices,
                   scan.images, batch=4)
    np.testing.assert_array_max_ulp(r.volume,
                                    oracle.bunny_f32(n, vs, o, scan.matrices, scan.images),
                                    maxulp=2)


@needs_ref
def test_live_reference_runner_reads_our_rct(tmp_path):
    """Our .rct writer is read by the reference's own ctFileReader (runner)."""
    from conftest import small_spec
    spec = synth.ScanSpec(nproj=2, seed=77)
    scan = synth.make_scan(spec)
    p = tmp_path / "s.rct"
    rct.write_rct(p, scan.images, scan.matrices, scan.hus)
    out = tmp_path / "v.vol"
    proc = subprocess.run([str(oracle.REF_RUNNER), "-m", "LolaBunny", "-s", "128", "-i", str(p),
                           "-o", str(out)], capture_output=True, text=True, cwd=tmp_path,
                          env=dict(os.environ, OMP_NUM_THREADS="2"))
    assert proc.returncode == 0, proc.stdout + proc.stderr
    assert "2 projections with size 1248 X 960" in proc.stdout
    vs = synth.voxel_size(128)
    o = synth.origin_index(128, vs)
    v = np.fromfile(out, np.float32).reshape(128, 128, 128)
    np.testing.assert_array_max_ulp(v, oracle.bunny_f32(128, vs, o, scan.matrices, scan.images),
                                    maxulp=2)


def _parse_rctd(raw: bytes, n: int) -> dict:
    """result.rctd as the reference runner writes it (src/rabbitRunner.c:396-404)."""
    head = np.frombuffer(raw[:12], np.int32)
    k = int(head[2])
    off = 12 + 8 * k
    out = {"magic": int(head[0]), "size": int(head[1]), "images": k,
           "runtime": np.frombuffer(raw[12:off], np.uint64),
           "slice": np.frombuffer(raw[off:off + 4 * n * n], np.float32).reshape(n, n)}
    off += 4 * n * n
    out["mse"], out["max"] = np.frombuffer(raw[off:off + 16], np.float64)
    out["hist"] = np.frombuffer(raw[off + 16:off + 60], np.uint32)
    out["magic_end"] = int(np.frombuffer(raw[off + 60:off + 64], np.int32)[0])
    assert len(raw) == off + 64
    return out


def test_runner_output_files_follow_hu_restatement():
    """The reference runner's -p PGM and result.rctd for the N=128 run: both
    slices are metrics.to_hu of the raw FP32 middle slice (the HU formula the
    device writers use), and the file's metrics are the ones it printed."""
    info = json.loads((GOLDEN / "runner_n128.json").read_text())
    z = np.load(GOLDEN / "runner_n128_outputs.npz")
    n = info["n"]
    hu = metrics.to_hu(z["raw_mid_slice"], info["hus"])
    pgm = z["pgm"].tobytes()
    head = f"P5\n{n} {n}\n4095\n".encode()
    assert pgm.startswith(head)
    assert np.array_equal(np.frombuffer(pgm[len(head):], ">u2").reshape(n, n), hu)
    r = _parse_rctd(z["rctd"].tobytes(), n)
    assert (r["magic"], r["size"], r["images"], r["magic_end"]) == (591984, n, 4, 489195)
    assert np.array_equal(r["slice"], hu)
    assert np.array_equal(r["slice"], z["hu_mid_slice"])
    printed = info["runner_quality"]
    assert r["mse"] == pytest.approx(printed["mse_hu2"], rel=1e-5)
    assert r["max"] == printed["max_abs_hu"]
    assert int(r["hist"].sum()) == n ** 3
