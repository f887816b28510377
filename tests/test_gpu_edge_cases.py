"""Edge cases of the backprojection against the FP64 LolaBunny oracle: tiny
and odd volume and detector sizes, a source inside the volume (w changes sign
across it, so tiles take the clamped path with negative w), a ragged last
pass at the largest batch, calls without projections, the largest volume that
fits (N=2048) and one that does not."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import small_spec
from oracle import oracle
from rabbitct_gb300 import metrics, synth

pytestmark = pytest.mark.gpu

BAR = {"f32": 1e-5, "f32q": 1e-5, "f16qx": 1e-3, "tex16": 1e-3}


@pytest.fixture(scope="module")
def lib():
    from rabbitct_gb300 import build as b
    b.build_lolacuda()
    from rabbitct_gb300._native import load_lolacuda
    return load_lolacuda()


def _geom(n):
    vs = 256.0 / n
    return vs, synth.origin_index(n, vs)


def _close(got, ref, bar):
    """Relative RMSE within the bar, or, where the oracle is all but zero (a
    volume outside every view), absolute agreement."""
    scale = float(np.abs(ref).max())
    if scale < 1e-12:
        assert float(np.abs(got).max()) < 1e-12
        return
    assert metrics.errors(got, ref)["rel_rmse"] <= bar


@pytest.mark.parametrize("storage", ["f32", "f32q", "f16qx", "tex16"])
@pytest.mark.parametrize("n,w,h", [(1, 1, 1), (2, 3, 2), (3, 7, 5), (5, 16, 9), (17, 33, 20)])
def test_tiny_and_odd_sizes(lib, storage, n, w, h):
    from rabbitct_gb300.lolacuda import Plan
    scan = synth.make_scan(small_spec(nproj=5, width=w, height=h, seed=90 + n))
    vs, o = _geom(n)
    ref = oracle.bunny_f64(n, vs, o, scan.matrices, scan.images)
    with Plan(n, vs, o, w, h, storage=storage, batch=3) as plan:
        plan.backproject_host(scan.images, scan.matrices)
        got = plan.download()
    _close(got, ref, BAR[storage])


def _w_of_voxels(n, vs, o, m):
    """w = a2 x + a5 y + a8 z + a11 of every voxel (src/LolaBunny.c:58-64)."""
    c = o + vs * np.arange(n, dtype=np.float64)
    z, y, x = np.meshgrid(c, c, c, indexing="ij")
    return m[2] * x + m[5] * y + m[8] * z + m[11]


@pytest.mark.parametrize("storage", ["f32", "f16qx"])
def test_source_inside_the_volume(lib, storage):
    """Source 40 mm from the centre of a 256 mm cube: voxels behind it have
    w < 0 (LolaBunny backprojects them through the mirrored ray, weight
    1/w^2 > 0).  Voxels within one voxel of the source plane, where 1/w^2
    explodes and the FP32 reciprocal of a tiny w cannot match FP64, are left
    out of the comparison."""
    from rabbitct_gb300.lolacuda import Plan
    spec = small_spec(nproj=6, width=96, height=80, seed=97)
    spec.sod = 40.0
    scan = synth.make_scan(spec)
    n = 32
    vs, o = _geom(n)
    ref = oracle.bunny_f64(n, vs, o, scan.matrices, scan.images)
    with Plan(n, vs, o, spec.width, spec.height, storage=storage, batch=6,
              collect_stats=1) as plan:
        plan.backproject_host(scan.images, scan.matrices)
        got = plan.download()
        st = plan.stats()
    keep = np.ones(got.shape, bool)
    behind = np.zeros(got.shape, bool)
    for m in scan.matrices:
        wv = _w_of_voxels(n, vs, o, m)
        # a voxel step changes w by at most |a2|+|a5|+|a8| times the voxel size
        step = (abs(m[2]) + abs(m[5]) + abs(m[8])) * vs
        keep &= np.abs(wv) > step
        behind |= wv < 0
    assert behind.any() and keep.mean() > 0.5
    assert st.tilePassesSlow > 0
    _close(got[keep], ref[keep], BAR[storage])


def test_ragged_last_pass_at_largest_batch(lib):
    from rabbitct_gb300.lolacuda import Plan
    scan = synth.make_scan(small_spec(nproj=33, width=64, height=48, seed=98))
    n = 24
    vs, o = _geom(n)
    ref = oracle.bunny_f64(n, vs, o, scan.matrices, scan.images)
    with Plan(n, vs, o, scan.width, scan.height, batch=32) as plan:
        plan.backproject_host(scan.images, scan.matrices)
        got = plan.download()
        st = plan.stats()
    assert st.passes == 2 and st.projections == 33
    _close(got, ref, 1e-5)


def test_calls_without_projections(lib):
    """An empty host or device call and a module call of zero projections
    leave the volume as it was."""
    from rabbitct_gb300._native import check, config
    from rabbitct_gb300.lolacuda import GlobalData, Plan, module_functions
    scan = synth.make_scan(small_spec(nproj=2, width=64, height=48, seed=99))
    n = 16
    vs, o = _geom(n)
    init = np.random.default_rng(3).standard_normal((n, n, n)).astype(np.float32)
    with Plan(n, vs, o, scan.width, scan.height) as plan:
        plan.upload(init)
        plan.backproject_host(scan.images[:0], scan.matrices[:0])
        plan.backproject_device(0, 0, scan.matrices[:0], count=0)
        assert np.array_equal(plan.download(), init)
    assert lib.lolaCudaSetConfig(config(exit_on_error=0))
    prepare, iterate, finish = module_functions(lib, "lolaCuda")
    vol = init.copy()
    gd = GlobalData(n, vs, o, scan.width, scan.height, 1, volume=vol)
    check(prepare(gd.ref), "prepare")
    gd.data.numberOfProjections = 0
    check(iterate(gd.ref), "backprojection")
    check(finish(gd.ref), "finish")
    assert np.array_equal(vol, init)


def test_largest_volume_n2048(lib):
    """N=2048: a 32 GiB volume, 8.6e9 voxels (past 32-bit voxel indices), one
    pass of two full-detector projections; three slices copied back and
    sampled against the oracle."""
    from rabbitct_gb300._native import check
    from rabbitct_gb300.lolacuda import Plan
    scan = synth.make_scan(synth.ScanSpec(nproj=2, seed=31))
    n = 2048
    vs = synth.voxel_size(n)
    o = synth.origin_index(n, vs)
    rng = np.random.default_rng(8)
    area = n * n
    with Plan(n, vs, o, scan.width, scan.height, storage="f32q", batch=2) as plan:
        plan.zero()
        plan.backproject_host(scan.images, scan.matrices)
        plan.synchronize()
        got, idx = [], []
        for z in (0, n // 2 + 7, n - 1):
            sl = np.empty(area, np.float32)
            check(lib.lolaCudaCopyToHost(sl.ctypes.data, plan.volume_ptr + 4 * z * area,
                                         sl.nbytes), "slice")
            pick = rng.choice(area, 700, replace=False)
            got.append(sl[pick])
            idx.append(z * area + pick.astype(np.int64))
    got = np.concatenate(got)
    idx = np.concatenate(idx)
    assert idx.max() > 2 ** 32
    ref = oracle.bunny_points(n, vs, o, scan.matrices, scan.images, idx)
    assert np.count_nonzero(ref) > 300
    _close(got, ref, 1e-5)


def test_volume_too_large_is_an_error(lib):
    """A 2 TiB volume cannot be allocated: plan creation reports it."""
    from rabbitct_gb300._native import LolaCudaError
    from rabbitct_gb300.lolacuda import Plan
    n = 8192
    vs, o = _geom(n)
    with pytest.raises(LolaCudaError):
        Plan(n, vs, o, 64, 48)
