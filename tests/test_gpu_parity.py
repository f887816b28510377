"""Parity of the CUDA path (through the C ABI) with the FP64 LolaBunny oracle.

Bars (the FP64 oracle is the reference of every comparison):
  FP32 storage (plain, quad or texture), plain or Kahan accumulation
                                     relative RMSE <= 1e-5 (and <= 1e-5 vs the
                                     FP32-accumulating LolaBunny restatement)
  FP16 storage (plain, quad or texture) relative RMSE <= 1e-3
  BF16 storage (plain or quad)       relative RMSE <= 4e-3 (8-bit mantissa)
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import small_spec
from oracle import oracle
from rabbitct_gb300 import metrics, synth

pytestmark = pytest.mark.gpu

BAR = {"f32": 1e-5, "f32q": 1e-5, "f16": 1e-3, "f16q": 1e-3, "bf16": 4e-3, "bf16q": 4e-3,
       "tex32": 1e-5, "tex16": 1e-3, "f16qx": 1e-3, "f32qx": 1e-5}


@pytest.fixture(scope="module")
def lib():
    from rabbitct_gb300 import build as b
    b.build_lolacuda()
    from rabbitct_gb300._native import load_lolacuda
    return load_lolacuda()


def _scan(**kw):
    return synth.make_scan(small_spec(**kw))


def _geom(n):
    vs = 256.0 / n
    return vs, synth.origin_index(n, vs)


_cache = {}


def _oracle64(scan, n, vs, o):
    key = (id(scan), n)
    if key not in _cache:
        _cache[key] = oracle.bunny_f64(n, vs, o, scan.matrices, scan.images)
    return _cache[key]


@pytest.fixture(scope="module")
def scan12():
    return _scan()


@pytest.mark.parametrize("storage", ["f32", "f32q", "f16", "f16q", "bf16", "bf16q", "tex32",
                                     "tex16", "f16qx", "f32qx"])
@pytest.mark.parametrize("accum", ["plain", "kahan"])
def test_storage_accum_vs_oracle(lib, scan12, storage, accum):
    from rabbitct_gb300.lolacuda import Plan
    n = 48
    vs, o = _geom(n)
    ref = _oracle64(scan12, n, vs, o)
    with Plan(n, vs, o, scan12.width, scan12.height, storage=storage, accumulation=accum,
              batch=5) as plan:
        plan.backproject_host(scan12.images, scan12.matrices)
        vol = plan.download()
    e = metrics.errors(vol, ref)
    assert e["rel_rmse"] <= BAR[storage], e


@pytest.mark.parametrize("vpt,rows", [(8, 8), (8, 4), (16, 8), (16, 4), (4, 8)])
@pytest.mark.parametrize("n", [32, 40, 64])
def test_shapes_and_ragged_sizes(lib, scan12, vpt, rows, n):
    """Tile shapes, and N that is not a multiple of the tile (ragged edges)."""
    from rabbitct_gb300.lolacuda import Plan
    vs, o = _geom(n)
    ref = _oracle64(scan12, n, vs, o)
    ref32 = oracle.bunny_f32(n, vs, o, scan12.matrices, scan12.images)
    with Plan(n, vs, o, scan12.width, scan12.height, storage="f32", batch=7,
              voxels_per_thread=vpt, rows_per_block=rows) as plan:
        plan.backproject_host(scan12.images, scan12.matrices)
        vol = plan.download()
    assert metrics.errors(vol, ref)["rel_rmse"] <= 1e-5
    assert metrics.errors(vol, ref32)["rel_rmse"] <= 1e-5


@pytest.mark.parametrize("batch", [1, 2, 12, 32])
def test_batch_sizes_device_path(lib, scan12, batch):
    """Projections resident in device memory, any pass size."""
    from rabbitct_gb300.lolacuda import DeviceBuffer, Plan
    n = 32
    vs, o = _geom(n)
    ref = _oracle64(scan12, n, vs, o)
    d = DeviceBuffer.from_array(scan12.images)
    with Plan(n, vs, o, scan12.width, scan12.height, storage="f32", batch=batch,
              collect_stats=1) as plan:
        plan.backproject_device(d.ptr, scan12.width * scan12.height, scan12.matrices)
        plan.synchronize()
        vol = plan.download()
        st = plan.stats()
    d.free()
    assert metrics.errors(vol, ref)["rel_rmse"] <= 1e-5
    assert st.projections == 12
    assert st.passes == -(-12 // batch)


def test_accumulates_into_initial_volume(lib, scan12):
    from rabbitct_gb300.lolacuda import Plan
    n = 32
    vs, o = _geom(n)
    rng = np.random.default_rng(0)
    init = rng.standard_normal((n, n, n)).astype(np.float32) * 1e-4
    ref = oracle.bunny_f64(n, vs, o, scan12.matrices, scan12.images,
                           vol=init.astype(np.float64).copy())
    with Plan(n, vs, o, scan12.width, scan12.height) as plan:
        plan.upload(init)
        plan.backproject_host(scan12.images, scan12.matrices)
        vol = plan.download()
    assert metrics.errors(vol, ref)["rel_rmse"] <= 1e-5


@pytest.mark.parametrize("vpt,rows", [(8, 8), (16, 4)])
def test_truncation_border_semantics(lib, vpt, rows):
    """A detector much smaller than the volume's shadow: many voxels project
    to u or v in (-2, 0), where LolaBunny's truncation gives negative weights,
    and many tiles reach past the 64-pixel zero margin (clamped path) or miss
    the detector (skipped)."""
    from rabbitct_gb300.lolacuda import Plan
    spec = small_spec(width=64, height=48, nproj=9, seed=21)
    spec.pitch = 0.308 * 1248 / 64 * 0.25   # a quarter of the field of view
    scan = synth.make_scan(spec)
    n = 48
    vs, o = _geom(n)
    ref = oracle.bunny_f64(n, vs, o, scan.matrices, scan.images)
    with Plan(n, vs, o, spec.width, spec.height, batch=9, collect_stats=1,
              voxels_per_thread=vpt, rows_per_block=rows) as plan:
        plan.backproject_host(scan.images, scan.matrices)
        vol = plan.download()
        st = plan.stats()
    assert metrics.errors(vol, ref)["rel_rmse"] <= 1e-5
    assert st.tilePassesSkipped > 0 and st.tilePassesSlow > 0


def test_fast_path_exercised(lib):
    """Full-size detector, N=128: interior tiles run unclamped."""
    from rabbitct_gb300.lolacuda import Plan
    spec = synth.ScanSpec(nproj=4, seed=2)
    scan = synth.make_scan(spec)
    n = 128
    vs = synth.voxel_size(n)
    o = synth.origin_index(n, vs)
    ref = oracle.bunny_f64(n, vs, o, scan.matrices, scan.images)
    with Plan(n, vs, o, spec.width, spec.height, batch=4, collect_stats=1) as plan:
        plan.backproject_host(scan.images, scan.matrices)
        vol = plan.download()
        st = plan.stats()
    assert metrics.errors(vol, ref)["rel_rmse"] <= 1e-5
    assert st.tilePassesFast > 0


@pytest.mark.parametrize("storage", ["f32q", "f32qx"])
def test_fp32_quads_equal_plain_fp32(lib, storage):
    """FP32 quads hold the exact FP32 taps (f32q column by column, read by one
    16-byte load; f32qx row by row, by a load or one texel), and the paired
    path's column-pair interpolation rounds as the plain layout's pairwise
    one: the volumes are identical.
    Full-size detector, N=128, 16 x 4 and 8 x 8 tiles: paired, one-voxel and
    clamped tiles all occur."""
    from rabbitct_gb300.lolacuda import Plan
    spec = synth.ScanSpec(nproj=6, seed=3)
    scan = synth.make_scan(spec)
    n = 128
    vs = synth.voxel_size(n)
    o = synth.origin_index(n, vs)
    for vpt, rows in ((16, 4), (8, 8)):
        vols, stats = [], []
        for st_name in ("f32", storage):
            with Plan(n, vs, o, spec.width, spec.height, storage=st_name, batch=6,
                      voxels_per_thread=vpt, rows_per_block=rows, collect_stats=1) as plan:
                plan.backproject_host(scan.images, scan.matrices)
                vols.append(plan.download())
                stats.append(plan.stats())
        assert stats[1].tilePassesPaired > 0 and stats[1].tilePassesSlow > 0
        assert np.array_equal(vols[1], vols[0]), (vpt, rows)


@pytest.mark.parametrize("n", [128, 640])
def test_mixed_fp16_quads_equal_load_only_quads(lib, n):
    """f16qx (column-ordered quads, every voxel through the texture unit,
    4 x 2 voxels per warp quarter) and f16q (row-ordered quads, loads only,
    rows of 8 lanes) hold the same FP16 terms, and the texture's point fetch
    widens them exactly: the volumes are identical."""
    from rabbitct_gb300.lolacuda import Plan
    spec = synth.ScanSpec(nproj=4, seed=4)
    scan = synth.make_scan(spec)
    vs = synth.voxel_size(n)
    o = synth.origin_index(n, vs)
    vols = []
    for storage in ("f16q", "f16qx"):
        with Plan(n, vs, o, spec.width, spec.height, storage=storage, batch=4,
                  collect_stats=1) as plan:
            plan.backproject_host(scan.images, scan.matrices)
            vols.append(plan.download())
            assert plan.stats().tilePassesPaired > 0
    assert np.array_equal(vols[1], vols[0])


@pytest.mark.parametrize("batch_call", [1, 3])
@pytest.mark.parametrize("with_geometry", [True, False])
def test_module_api_like_runner(lib, scan12, batch_call, with_geometry):
    """prepare / backprojection / finish driven like src/rabbitRunner.c."""
    from rabbitct_gb300._native import config
    from rabbitct_gb300.lolacuda import module_functions
    from rabbitct_gb300.runner import run_module
    n = 40
    vs, o = _geom(n)
    ref = _oracle64(scan12, n, vs, o)
    assert lib.lolaCudaSetConfig(config(storage="f32", batch=5, exit_on_error=0))
    r = run_module(module_functions(lib, "lolaCuda"), n, vs, o, scan12.matrices, scan12.images,
                   batch=batch_call, with_geometry=with_geometry)
    assert metrics.errors(r.volume, ref)["rel_rmse"] <= 1e-5


def _staging_scan():
    """Full-size detector and a 64 mm cube of 0.5 mm voxels: tile footprints
    are small enough to be staged in shared memory."""
    return synth.make_scan(synth.ScanSpec(nproj=10, seed=41))


@pytest.mark.parametrize("storage", ["f32", "f16", "bf16", "f32q", "f16q", "bf16q", "f16qx",
                                     "f32qx"])
@pytest.mark.parametrize("accum", ["plain", "kahan"])
def test_staged_pass_matches_oracle_and_load_path(lib, storage, accum):
    from rabbitct_gb300.lolacuda import Plan
    scan = _staging_scan()
    n, vs = 96, 0.5
    o = synth.origin_index(n, vs)
    ref = oracle.bunny_f64(n, vs, o, scan.matrices, scan.images)
    vols = {}
    for staging in (1, 0):
        with Plan(n, vs, o, scan.width, scan.height, storage=storage, accumulation=accum,
                  batch=5, staging=staging, collect_stats=1, voxels_per_thread=8,
                  rows_per_block=8) as plan:
            plan.backproject_host(scan.images, scan.matrices)
            vols[staging] = plan.download()
            st = plan.stats()
        if staging and storage not in ("f32q", "f32qx"):
            assert st.stagedPasses == 2 and st.tilePassesStaged > 0, (st.stagedPasses,
                                                                      st.tilePassesStaged)
        elif staging:
            # 16-byte pixels: this footprint does not fit a 24 KB stage, the
            # pass runs on the load path
            assert st.stagedPasses == 0
        else:
            assert st.stagedPasses == 0 and st.tilePassesStaged == 0
    assert metrics.errors(vols[1], ref)["rel_rmse"] <= BAR[storage]
    # same arithmetic on the same taps: the two gather paths agree exactly
    assert np.array_equal(vols[1], vols[0])


def test_staged_pass_ragged_volume_and_rows(lib):
    from rabbitct_gb300.lolacuda import Plan
    scan = _staging_scan()
    n, vs = 100, 0.5
    o = synth.origin_index(n, vs)
    ref = oracle.bunny_f64(n, vs, o, scan.matrices, scan.images)
    with Plan(n, vs, o, scan.width, scan.height, storage="f32", batch=10, rows_per_block=4,
              voxels_per_thread=8, collect_stats=1, staging=1) as plan:
        plan.backproject_host(scan.images, scan.matrices)
        vol = plan.download()
        st = plan.stats()
    assert st.tilePassesStaged > 0
    assert metrics.errors(vol, ref)["rel_rmse"] <= 1e-5


@pytest.mark.parametrize("convert", [False, True])
def test_device_verification_matches_runner_metrics(lib, convert):
    """lolaCudaPlanVerify against metrics.hu_quality (the restatement of the
    runner's -c block pinned to the reference runner's own printout)."""
    from rabbitct_gb300.lolacuda import Plan
    spec = synth.ScanSpec(nproj=6, seed=43)
    scan = synth.make_scan(spec)
    n = 128
    vs = synth.voxel_size(n)
    o = synth.origin_index(n, vs)
    ref64 = oracle.bunny_f64(n, vs, o, scan.matrices, scan.images)
    # a reference volume a few HU away so every histogram bin is populated
    hu_ref = metrics.to_hu(ref64.astype(np.float32), scan.hus)
    noise = np.random.default_rng(1).integers(-12, 13, hu_ref.shape)
    hu_ref = np.clip(hu_ref + noise, 0, 4095).astype(np.uint16)
    with Plan(n, vs, o, scan.width, scan.height) as plan:
        plan.backproject_host(scan.images, scan.matrices)
        vol = plan.download()
        q = plan.verify(hu_ref, scan.hus, convert_in_place=convert)
        after = plan.download()
    want = metrics.hu_quality(vol, hu_ref, scan.hus)
    assert q["histogram"] == want["histogram"]
    assert q["max_abs_hu"] == want["max_abs_hu"]
    assert q["mse_hu2"] == pytest.approx(want["mse_hu2"], rel=1e-9)
    assert q["psnr_db"] == pytest.approx(want["psnr_db"], rel=1e-9)
    if convert:
        assert np.array_equal(after, metrics.to_hu(vol, scan.hus))
    else:
        assert np.array_equal(after, vol)


def test_slabs_reassemble_unsharded_volume(lib):
    """Three tile-aligned z-slabs (as three GPUs would hold them) equal the
    unsharded volume bit for bit; an unaligned split agrees to rounding."""
    from rabbitct_gb300._native import config
    from rabbitct_gb300.lolacuda import Plan, slab
    scan = synth.make_scan(small_spec(nproj=8, seed=44))
    n = 64
    vs, o = _geom(n)
    with Plan(n, vs, o, scan.width, scan.height, batch=8) as plan:
        plan.backproject_host(scan.images, scan.matrices)
        whole = plan.download()
    tile = config().voxelsPerThread  # slabs on tile boundaries: identical tiles
    for align, exact in ((tile, True), (1, False)):
        parts = []
        for r in range(3):
            b, c = slab(n, r, 3, align)
            with Plan(n, vs, o, scan.width, scan.height, batch=8, slab=(b, c)) as plan:
                plan.backproject_host(scan.images, scan.matrices)
                parts.append(plan.download())
        joined = np.concatenate(parts)
        if exact:
            assert np.array_equal(joined, whole)
        else:
            assert metrics.errors(joined, whole)["rel_rmse"] < 1e-6


@pytest.mark.parametrize("batch", [3, 16])
def test_reconstruct_from_rct_file(lib, tmp_path, batch):
    """lolaCudaReconstructFile on a .rct written with the reference's format:
    same volume as the plan path, within the FP32 bar of the oracle."""
    from rabbitct_gb300 import rct
    from rabbitct_gb300.lolacuda import Plan, reconstruct_file
    scan = synth.make_scan(small_spec(nproj=11, seed=71))
    path = tmp_path / "scan.rct"
    rct.write_rct(path, scan.images, scan.matrices, scan.hus)
    n = 40
    vs, o = _geom(n)
    vol, rep = reconstruct_file(path, n, vs, o, batch=batch)
    assert rep["projections"] == 11 and rep["hus"] == pytest.approx(scan.hus)
    # the file is read in the plan's passes: edge batch (2 x batch) first and
    # last, the last one full: 5 + 6 at batch 3, all 11 at once at batch 16
    cuts = [0, 5, 11] if batch == 3 else [0, 11]
    with Plan(n, vs, o, scan.width, scan.height, batch=min(32, 2 * batch)) as plan:
        for a, b in zip(cuts[:-1], cuts[1:]):
            plan.backproject_host(scan.images[a:b], scan.matrices[a:b])
        want = plan.download()
    assert np.array_equal(vol, want)
    ref = oracle.bunny_f64(n, vs, o, scan.matrices, scan.images)
    assert metrics.errors(vol, ref)["rel_rmse"] <= 1e-5


def test_reconstruct_file_reports_truncation(lib, tmp_path):
    from rabbitct_gb300 import rct
    from rabbitct_gb300._native import LolaCudaError
    from rabbitct_gb300.lolacuda import reconstruct_file
    scan = synth.make_scan(small_spec(nproj=4, seed=72))
    path = tmp_path / "cut.rct"
    rct.write_rct(path, scan.images, scan.matrices, scan.hus)
    data = path.read_bytes()
    path.write_bytes(data[:len(data) - 1000])
    with pytest.raises(LolaCudaError, match="truncated"):
        reconstruct_file(path, 24, 256.0 / 24, synth.origin_index(24, 256.0 / 24))


def test_runner_output_writers_match_reference_files(lib, tmp_path):
    """lolaCudaPlanWriteSlicePgm / lolaCudaPlanWriteResult on a volume whose
    middle slice is the reference runner's raw slice: the PGM equals the
    runner's file byte for byte, result.rctd has its layout and HU slice, and
    its metrics equal the restatement over the whole volume."""
    import json
    from pathlib import Path

    from rabbitct_gb300.lolacuda import Plan
    golden = Path(__file__).resolve().parent / "golden"
    info = json.loads((golden / "runner_n128.json").read_text())
    z = np.load(golden / "runner_n128_outputs.npz")
    n, hus = info["n"], info["hus"]
    rng = np.random.default_rng(17)
    vol = rng.uniform(-0.002, float(z["raw_mid_slice"].max()), (n, n, n)).astype(np.float32)
    vol[n // 2 - 1] = z["raw_mid_slice"]
    hu_ref = metrics.to_hu(vol, hus) + rng.integers(-12, 13, vol.shape)
    hu_ref = np.clip(hu_ref, 0, 4095).astype(np.uint16)
    vs, o = _geom(n)
    with Plan(n, vs, o, 64, 48) as plan:
        plan.upload(vol)
        plan.write_pgm(tmp_path / "slice.pgm", hus)
        q = plan.write_result(tmp_path / "result.rctd", hu_ref, hus, 4, 4 * 19437 + 3)
    assert (tmp_path / "slice.pgm").read_bytes() == z["pgm"].tobytes()
    got, ref = (tmp_path / "result.rctd").read_bytes(), z["rctd"].tobytes()
    assert len(got) == len(ref)
    assert got[:12] == ref[:12]                                   # magic, size, images
    assert got[12:44] == np.full(4, 19437, np.uint64).tobytes()   # mean time per image
    assert got[44:44 + 4 * n * n] == ref[44:44 + 4 * n * n]       # HU slice
    assert got[-4:] == ref[-4:]
    want = metrics.hu_quality(vol, hu_ref, hus)
    off = 44 + 4 * n * n
    mse, mx = np.frombuffer(got[off:off + 16], np.float64)
    hist = np.frombuffer(got[off + 16:off + 60], np.uint32)
    assert mse == want["mse_hu2"] and mx == want["max_abs_hu"]    # integer sums: exact
    assert hist.tolist() == want["histogram"] == q["histogram"]


@pytest.mark.parametrize("with_geometry", [True, False])
def test_run_scan_matches_module_loop(lib, scan12, with_geometry):
    """lolaCudaRunScan (the runner's loop in C) gives exactly the volume of the
    same module calls made one by one, and reports its phase times."""
    import ctypes as C

    from rabbitct_gb300._native import LolaCudaScanTiming, check, config
    from rabbitct_gb300.lolacuda import GlobalData, module_functions
    from rabbitct_gb300.runner import run_module
    n = 40
    vs, o = _geom(n)
    assert lib.lolaCudaSetConfig(config(batch=5, exit_on_error=0))
    want = run_module(module_functions(lib, "lolaCuda"), n, vs, o, scan12.matrices,
                      scan12.images, batch=3, with_geometry=with_geometry).volume
    imgs = np.ascontiguousarray(scan12.images, np.float32)
    mats = np.ascontiguousarray(scan12.matrices, np.float64)
    vol = np.zeros((n, n, n), np.float32)
    gd = GlobalData(n, vs, o, scan12.width, scan12.height, 1, volume=vol,
                    geometry=mats if with_geometry else None)
    t = LolaCudaScanTiming()
    check(lib.lolaCudaRunScan(gd.ref, imgs.ctypes.data, scan12.width * scan12.height,
                              mats.ctypes.data, mats.shape[0], 3, C.byref(t)), "run scan")
    assert np.array_equal(vol, want)
    assert 0 < t.callSeconds <= t.totalSeconds and t.prepareSeconds > 0
