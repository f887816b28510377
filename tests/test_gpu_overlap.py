"""Volume transfers overlapped with passes (asynchronous chunked upload before
the first pass, streamed-out download after the last one) give exactly the
volume of the synchronous path: the chunked pass launches cover the tiles of a
whole pass, so every voxel sees the same operations in the same order."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import small_spec
from rabbitct_gb300 import synth

pytestmark = pytest.mark.gpu

N = 416  # 416^3 FP32 = 288 MB: the transfers split into 8 z-chunks


@pytest.fixture(scope="module")
def lib():
    from rabbitct_gb300 import build as b
    b.build_lolacuda()
    from rabbitct_gb300._native import load_lolacuda
    return load_lolacuda()


@pytest.fixture(scope="module")
def scan7():
    return synth.make_scan(small_spec(nproj=7, seed=81))


def _geom(n):
    vs = 256.0 / n
    return vs, synth.origin_index(n, vs)


def _initial(depth, n, seed=5):
    rng = np.random.default_rng(seed)
    return (rng.standard_normal((depth, n, n)) * 1e-3).astype(np.float32)


def _sync_result(scan, n, init, slab, splits=(), **kw):
    """The synchronous path; `splits` are the projection indices where a new
    pass starts beyond those the batch makes (each host call closes a pass)."""
    from rabbitct_gb300.lolacuda import Plan
    vs, o = _geom(n)
    cuts = [0, *splits, scan.images.shape[0]]
    with Plan(n, vs, o, scan.width, scan.height, slab=slab, **kw) as p:
        p.upload(init)
        for a, b in zip(cuts[:-1], cuts[1:]):
            p.backproject_host(scan.images[a:b], scan.matrices[a:b])
        return p.download()


@pytest.mark.parametrize("slab", [None, (13, 301)])
@pytest.mark.parametrize("vpt,rows", [(8, 4), (16, 8)])
def test_overlapped_transfers_bit_identical(lib, scan7, slab, vpt, rows):
    """Two passes (4 + 3 projections): the first waits for the upload chunk by
    chunk, the second streams the volume out; an unaligned, ragged slab too."""
    from rabbitct_gb300.lolacuda import Plan
    depth = N if slab is None else slab[1]
    init = _initial(depth, N)
    kw = dict(batch=4, voxels_per_thread=vpt, rows_per_block=rows, storage="f16qx")
    want = _sync_result(scan7, N, init, slab, **kw)
    vs, o = _geom(N)
    out = np.full_like(init, np.nan)
    with Plan(N, vs, o, scan7.width, scan7.height, slab=slab, **kw) as p:
        p.upload_async(init.copy())
        p.backproject_host(scan7.images[:4], scan7.matrices[:4])
        p.stream_out(out)
        p.backproject_host(scan7.images[4:], scan7.matrices[4:])
        p.synchronize()
        st = p.stats()
    assert np.array_equal(out, want)
    assert st.overlappedPasses == 2 and st.chunkLaunches > 2 * 4


def test_single_pass_overlaps_both_transfers(lib, scan7):
    """One pass that waits for the upload and streams the result out."""
    from rabbitct_gb300.lolacuda import Plan
    init = _initial(N, N, seed=6)
    want = _sync_result(scan7, N, init, None, batch=7)
    vs, o = _geom(N)
    out = np.empty_like(init)
    with Plan(N, vs, o, scan7.width, scan7.height, batch=7) as p:
        p.upload_async(init.copy())
        p.stream_out(out)
        p.backproject_host(scan7.images, scan7.matrices)
        p.synchronize()
        st = p.stats()
    assert np.array_equal(out, want)
    assert st.overlappedPasses == 1


def test_first_pass_after_upload_takes_the_edge_batch(lib, scan7):
    """After an asynchronous upload the first host-staged pass takes the edge
    batch (4 here), the rest the batch (2): passes of 4, 2 and 1."""
    from rabbitct_gb300.lolacuda import Plan
    init = _initial(N, N, seed=9)
    want = _sync_result(scan7, N, init, None, splits=(4, 6), batch=4)
    vs, o = _geom(N)
    with Plan(N, vs, o, scan7.width, scan7.height, batch=2, edge_batch=4,
              collect_stats=1) as p:
        p.upload_async(init.copy())
        p.backproject_host(scan7.images, scan7.matrices)
        out = p.download()
        st = p.stats()
    assert st.passes == 3 and st.overlappedPasses == 1
    assert np.array_equal(out, want)


def test_stream_out_belongs_to_the_calls_last_pass(lib, scan7):
    """A stream-out request made before a call of several passes delivers the
    volume after the call's last pass.  From host images that last pass takes
    the edge batch (4; batch 2: passes of 2, 1 and 4); from device images the
    passes are batch-sized (3, 3, 1)."""
    from rabbitct_gb300.lolacuda import DeviceBuffer, Plan
    init = _initial(N, N, seed=10)
    vs, o = _geom(N)
    want = _sync_result(scan7, N, init, None, splits=(2, 3), batch=4)
    out = np.full_like(init, np.nan)
    with Plan(N, vs, o, scan7.width, scan7.height, batch=2, edge_batch=4,
              collect_stats=1) as p:
        p.upload(init)
        p.stream_out(out)
        p.backproject_host(scan7.images, scan7.matrices)
        p.synchronize()
        st = p.stats()
    assert st.passes == 3 and st.overlappedPasses == 1
    assert np.array_equal(out, want)
    want = _sync_result(scan7, N, init, None, batch=3)
    out = np.full_like(init, np.nan)
    d_img = DeviceBuffer.from_array(np.ascontiguousarray(scan7.images, np.float32))
    try:
        with Plan(N, vs, o, scan7.width, scan7.height, batch=3, collect_stats=1) as p:
            p.upload(init)
            p.stream_out(out)
            p.backproject_device(d_img.ptr, scan7.width * scan7.height, scan7.matrices)
            p.synchronize()
            st = p.stats()
    finally:
        d_img.free()
    assert st.passes == 3 and st.overlappedPasses == 1
    assert np.array_equal(out, want)


def test_edge_batch_is_validated(lib):
    from rabbitct_gb300._native import LolaCudaError
    from rabbitct_gb300.lolacuda import Plan
    vs, o = _geom(16)
    for edge in (3, 65):
        with pytest.raises(LolaCudaError, match="edge batch"):
            Plan(16, vs, o, 64, 48, batch=4, edge_batch=edge)


def test_transfers_order_against_other_volume_work(lib, scan7):
    """An asynchronous upload followed by a zeroing, and a stream-out request
    with no pass before synchronize (a plain copy of the volume)."""
    from rabbitct_gb300.lolacuda import Plan
    vs, o = _geom(N)
    want = _sync_result(scan7, N, np.zeros((N, N, N), np.float32), None, batch=4)
    with Plan(N, vs, o, scan7.width, scan7.height, batch=4) as p:
        p.upload_async(_initial(N, N, seed=7))
        p.zero()                       # must land after the upload
        p.backproject_host(scan7.images, scan7.matrices)
        out = np.empty((N, N, N), np.float32)
        p.stream_out(out)              # no pass follows: copied at synchronize
        p.synchronize()
        assert np.array_equal(out, want)
        again = p.download()
    assert np.array_equal(again, want)


@pytest.mark.parametrize("edge", [0, 3])
@pytest.mark.parametrize("pinned", [True, False])
@pytest.mark.parametrize("with_geometry", [True, False])
def test_module_api_overlap_matches_plan(lib, scan7, with_geometry, pinned, edge):
    """prepare uploads asynchronously; into a page-locked volume the scan's
    last call (with -a) or finish's closing pass (without) streams the volume
    out, a pageable one is copied in finish.

    Passes of 7 projections at batch 3: with the default edge batch (6) the
    first pass takes 6 where the scan length is unknown (6 + 1) and the last
    pass takes 6 where it is known (1 + 6); with edge batch 3, 3 + 3 + 1."""
    import ctypes as C

    from rabbitct_gb300._native import config
    from rabbitct_gb300.lolacuda import module_functions
    from rabbitct_gb300.runner import run_module
    init = _initial(N, N, seed=8)
    splits = (3, 6) if edge == 3 else (1,) if with_geometry else (6,)
    want = _sync_result(scan7, N, init, None, splits=splits, batch=6)
    vs, o = _geom(N)
    host = None
    if pinned:
        host = lib.lolaCudaHostAlloc(init.nbytes)
        assert host
        vol = np.ctypeslib.as_array((C.c_float * init.size).from_address(host))
        vol = vol.reshape(init.shape)
        vol[...] = init
    else:
        vol = init.copy()
    try:
        assert lib.lolaCudaSetConfig(config(storage="f32", batch=3, edge_batch=edge,
                                            exit_on_error=0))
        r = run_module(module_functions(lib, "lolaCuda"), N, vs, o, scan7.matrices,
                       scan7.images, batch=1, with_geometry=with_geometry, volume=vol)
        assert np.array_equal(r.volume, want)
    finally:
        if host:
            lib.lolaCudaHostFree(host)


@pytest.mark.parametrize("pinned", [True, False])
def test_deferred_upload_reaches_the_volume_without_a_pass(lib, pinned):
    """From page-locked memory the asynchronous upload is issued with the
    next pass; with none, by synchronize or by any other use of the volume
    (from pageable memory it is issued at once).  A second upload before
    either replaces the first."""
    import ctypes as C

    from rabbitct_gb300.lolacuda import Plan
    vs, o = _geom(64)
    shape, nbytes = (64, 64, 64), 4 * 64 ** 3
    bufs = []

    def host_array():
        if not pinned:
            return np.empty(shape, np.float32)
        ptr = lib.lolaCudaHostAlloc(nbytes)
        assert ptr
        bufs.append(ptr)
        return np.ctypeslib.as_array((C.c_float * (nbytes // 4)).from_address(ptr)).reshape(shape)

    try:
        a, b, out = host_array(), host_array(), host_array()
        a[...] = _initial(64, 64, seed=11)
        b[...] = _initial(64, 64, seed=12)
        with Plan(64, vs, o, 96, 80, batch=4) as p:
            p.upload_async(a)
            p.synchronize()
            assert np.array_equal(p.download(), a)
            p.upload_async(a)
            p.upload_async(b)
            assert np.array_equal(p.download(), b)   # download issues it first
            p.upload_async(a)
            out[...] = np.nan
            p.stream_out(out)                        # no pass: copied at synchronize
            p.synchronize()
            assert np.array_equal(out, a)
    finally:
        for ptr in bufs:
            lib.lolaCudaHostFree(ptr)
