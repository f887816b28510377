"""Python front end of LolaCUDA: the plan API and RabbitCtGlobalData helpers.

Everything calls liblolacuda.so through its C ABI (include/lolaCuda.h); there
is no Python or CPU implementation of the backprojection in this package.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _native
from ._native import (LolaCudaConfig, LolaCudaGeometry, LolaCudaStats, Projection,
                      RabbitCtGlobalData, check, config, load_lolacuda)

__all__ = ["Plan", "Batch", "DeviceBuffer", "GlobalData", "module_functions", "config", "slab",
           "autotune"]


def slab(n: int, rank: int, ranks: int, align: int = 8) -> tuple[int, int]:
    """(sliceBegin, sliceCount) of `rank` among `ranks` (lolaCudaSlab)."""
    b, c = C.c_int32(), C.c_int32()
    check(load_lolacuda().lolaCudaSlab(n, rank, ranks, align, C.byref(b), C.byref(c)), "slab")
    return b.value, c.value


class DeviceBuffer:
    """A cudaMalloc'ed buffer owned by Python (via lolaCudaDeviceAlloc)."""

    def __init__(self, nbytes: int):
        self.lib = load_lolacuda()
        self.nbytes = int(nbytes)
        self.ptr = self.lib.lolaCudaDeviceAlloc(self.nbytes)
        if not self.ptr:
            raise _native.LolaCudaError(f"device alloc: {_native.last_error()}")

    @classmethod
    def from_array(cls, a: np.ndarray) -> "DeviceBuffer":
        a = np.ascontiguousarray(a)
        buf = cls(a.nbytes)
        check(buf.lib.lolaCudaCopyToDevice(buf.ptr, a.ctypes.data, a.nbytes), "copy to device")
        return buf

    def to_array(self, shape, dtype) -> np.ndarray:
        out = np.empty(shape, dtype)
        assert out.nbytes <= self.nbytes
        check(self.lib.lolaCudaCopyToHost(out.ctypes.data, self.ptr, out.nbytes), "copy to host")
        return out

    def free(self) -> None:
        if self.ptr:
            self.lib.lolaCudaDeviceFree(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class Plan:
    """One reconstruction volume on the device plus its projection ring."""

    def __init__(self, n: int, voxel_size: float, origin_index: float, width: int, height: int,
                 cfg: LolaCudaConfig | None = None, slab: tuple[int, int] | None = None,
                 **cfg_kw):
        self.lib = load_lolacuda()
        self.n, self.width, self.height = int(n), int(width), int(height)
        self.slab = (0, self.n) if slab is None else (int(slab[0]), int(slab[1]))
        g = LolaCudaGeometry(self.n, self.width, self.height, voxel_size, origin_index,
                             self.slab[0], self.slab[1])
        self.cfg = cfg if cfg is not None else config(**cfg_kw)
        self._hold: list[np.ndarray] = []  # host buffers of transfers in flight
        h = C.c_void_p()
        check(self.lib.lolaCudaPlanCreate(C.byref(g), C.byref(self.cfg), C.byref(h)),
              "plan create")
        self.handle = h

    @property
    def volume_ptr(self) -> int:
        return self.lib.lolaCudaPlanVolume(self.handle)

    @property
    def stream(self) -> int:
        return self.lib.lolaCudaPlanStream(self.handle)

    def zero(self) -> None:
        check(self.lib.lolaCudaPlanZeroVolume(self.handle), "zero volume")

    def upload(self, vol: np.ndarray) -> None:
        vol = np.ascontiguousarray(vol, np.float32)
        assert vol.size == self.n * self.n * self.slab[1]
        check(self.lib.lolaCudaPlanUploadVolume(self.handle, vol.ctypes.data), "upload volume")

    def upload_async(self, vol: np.ndarray) -> None:
        """A chunked upload that the next pass overlaps: its copies are issued
        with that pass, after the projections it reads (or by any other use
        of the volume, or synchronize()); `vol` is kept alive (and must stay
        unchanged) until synchronize()."""
        assert vol.dtype == np.float32 and vol.flags.c_contiguous
        assert vol.size == self.n * self.n * self.slab[1]
        self._hold.append(vol)
        check(self.lib.lolaCudaPlanUploadVolumeAsync(self.handle, vol.ctypes.data),
              "upload volume async")

    def stream_out(self, out: np.ndarray) -> np.ndarray:
        """The volume lands in `out` after the last pass of the next
        backproject call (or at synchronize()), chunk by chunk as that pass
        finishes; complete after synchronize()."""
        assert out.dtype == np.float32 and out.flags.c_contiguous
        assert out.size == self.n * self.n * self.slab[1]
        self._hold.append(out)
        check(self.lib.lolaCudaPlanStreamVolumeOut(self.handle, out.ctypes.data), "stream out")
        return out

    def download(self, out: np.ndarray | None = None) -> np.ndarray:
        """The plan's volume (its slab: sliceCount x N x N), z slowest."""
        if out is None:
            out = np.empty((self.slab[1], self.n, self.n), np.float32)
        check(self.lib.lolaCudaPlanDownloadVolume(self.handle, out.ctypes.data), "download")
        return out

    def backproject_device(self, d_images: int, image_stride: int, matrices: np.ndarray,
                           count: int | None = None) -> None:
        m = np.ascontiguousarray(matrices, np.float64).reshape(-1, 12)
        count = m.shape[0] if count is None else count
        check(self.lib.lolaCudaPlanBackprojectDevice(self.handle, d_images, image_stride,
                                                     m.ctypes.data, count), "backproject")

    def backproject_host(self, images: np.ndarray, matrices: np.ndarray) -> None:
        imgs = np.ascontiguousarray(images, np.float32)
        m = np.ascontiguousarray(matrices, np.float64).reshape(-1, 12)
        assert imgs.shape[0] == m.shape[0]
        stride = self.width * self.height
        check(self.lib.lolaCudaPlanBackprojectHost(self.handle, imgs.ctypes.data, stride,
                                                   m.ctypes.data, m.shape[0]), "backproject")

    def synchronize(self) -> None:
        check(self.lib.lolaCudaPlanSynchronize(self.handle), "synchronize")
        self._hold.clear()

    def timer_start(self) -> None:
        check(self.lib.lolaCudaPlanTimerStart(self.handle), "timer start")

    def timer_stop(self) -> float:
        """Milliseconds since timer_start, measured by CUDA events on the plan stream."""
        ms = C.c_double()
        check(self.lib.lolaCudaPlanTimerStop(self.handle, C.byref(ms)), "timer stop")
        return ms.value

    def verify(self, reference_hu: np.ndarray, hus, convert_in_place: bool = False) -> dict:
        """The runner's -c verification on the device (see lolaCudaPlanVerify)."""
        from ._native import LolaCudaQuality
        ref = np.ascontiguousarray(reference_hu, np.uint16)
        assert ref.size == self.n * self.n * self.slab[1]
        h = np.asarray(hus, np.float32)
        q = LolaCudaQuality()
        check(self.lib.lolaCudaPlanVerify(self.handle, ref.ctypes.data, h.ctypes.data,
                                          int(convert_in_place), C.byref(q)), "verify")
        return {"rmse_hu": q.rmse, "mse_hu2": q.mse, "max_abs_hu": q.maxAbs,
                "psnr_db": q.psnr, "histogram": list(q.histogram)}

    def write_pgm(self, path, hus) -> None:
        """The runner's -p slice (N/2-1, HU, 16-bit PGM) from the device volume."""
        h = np.asarray(hus, np.float32)
        check(self.lib.lolaCudaPlanWriteSlicePgm(self.handle, os.fsencode(path), h.ctypes.data),
              "write pgm")

    def write_result(self, path, reference_hu: np.ndarray, hus, number_of_images: int,
                     total_usec: int) -> dict:
        """The runner's -c result.rctd; converts the device volume to HU."""
        from ._native import LolaCudaQuality
        ref = np.ascontiguousarray(reference_hu, np.uint16)
        assert ref.size == self.n ** 3
        h = np.asarray(hus, np.float32)
        q = LolaCudaQuality()
        check(self.lib.lolaCudaPlanWriteResult(self.handle, os.fsencode(path), ref.ctypes.data,
                                               h.ctypes.data, int(number_of_images),
                                               int(total_usec), C.byref(q)), "write result")
        return {"rmse_hu": q.rmse, "mse_hu2": q.mse, "max_abs_hu": q.maxAbs,
                "psnr_db": q.psnr, "histogram": list(q.histogram)}

    def stats(self) -> LolaCudaStats:
        s = LolaCudaStats()
        check(self.lib.lolaCudaPlanGetStats(self.handle, C.byref(s)), "stats")
        return s

    def reset_stats(self) -> None:
        check(self.lib.lolaCudaPlanResetStats(self.handle), "reset stats")

    def close(self) -> None:
        if getattr(self, "handle", None):
            self.lib.lolaCudaPlanDestroy(self.handle)  # waits for its streams
            self.handle = None
            self._hold.clear()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def reconstruct_file(path, n: int, voxel_size: float, origin_index: float,
                     volume: np.ndarray | None = None, cfg: LolaCudaConfig | None = None,
                     **cfg_kw):
    """lolaCudaReconstructFile: (volume, report dict)."""
    from ._native import LolaCudaFileReport
    lib = load_lolacuda()
    vol = np.zeros((n, n, n), np.float32) if volume is None else volume
    assert vol.dtype == np.float32 and vol.flags["C_CONTIGUOUS"] and vol.size == n ** 3
    c = cfg if cfg is not None else config(**cfg_kw)
    rep = LolaCudaFileReport()
    check(lib.lolaCudaReconstructFile(str(path).encode(), n, voxel_size, origin_index,
                                      C.byref(c), vol.ctypes.data, C.byref(rep)),
          "reconstruct file")
    return vol, {"seconds": rep.seconds, "read_seconds": rep.readSeconds,
                 "projections": rep.projections, "gups": rep.gups, "hus": tuple(rep.hus)}


def autotune(n: int, voxel_size: float, origin_index: float, width: int, height: int,
             d_images: int, matrices: np.ndarray, cfg: LolaCudaConfig | None = None,
             slab: tuple[int, int] | None = None, **cfg_kw):
    """lolaCudaAutotune: returns (tuned config, list of (shape, batch, staging, ms))."""
    from ._native import LolaCudaTuneReport
    lib = load_lolacuda()
    c = cfg if cfg is not None else config(**cfg_kw)
    b, k = (0, 0) if slab is None else slab
    g = LolaCudaGeometry(n, width, height, voxel_size, origin_index, b, k)
    m = np.ascontiguousarray(matrices, np.float64).reshape(-1, 12)
    rep = LolaCudaTuneReport()
    check(lib.lolaCudaAutotune(C.byref(g), d_images, width * height, m.ctypes.data, m.shape[0],
                               C.byref(c), C.byref(rep)), "autotune")
    tried = [((t.voxelsPerThread, t.rowsPerBlock), t.batch, t.staging, t.ms)
             for t in rep.tried[:rep.candidates]]
    return c, tried


class Batch:
    """Uneven reconstructions run together (lolaCudaBatchCreate / Run).

    jobs: dicts with keys n, voxel_size, origin_index, width, height,
    d_images (device pointer), matrices (projections x 12) and d_volume
    (device pointer to N^3 floats)."""

    def __init__(self, jobs: list[dict], cfg: LolaCudaConfig | None = None, **cfg_kw):
        from ._native import LolaCudaJob
        self.lib = load_lolacuda()
        arr = (LolaCudaJob * len(jobs))()
        self._mats = []
        for i, j in enumerate(jobs):
            m = np.ascontiguousarray(j["matrices"], np.float64).reshape(-1, 12)
            self._mats.append(m)
            arr[i].geometry = LolaCudaGeometry(j["n"], j["width"], j["height"], j["voxel_size"],
                                               j["origin_index"], 0, 0)
            arr[i].projections = m.shape[0]
            arr[i].d_images = j["d_images"]
            arr[i].h_matrices = m.ctypes.data
            arr[i].d_volume = j["d_volume"]
        self.cfg = cfg if cfg is not None else config(**cfg_kw)
        h = C.c_void_p()
        check(self.lib.lolaCudaBatchCreate(arr, len(jobs), C.byref(self.cfg), C.byref(h)),
              "batch create")
        self.handle = h

    def run(self) -> None:
        check(self.lib.lolaCudaBatchRun(self.handle), "batch run")

    def synchronize(self) -> None:
        check(self.lib.lolaCudaBatchSynchronize(self.handle), "batch synchronize")

    def info(self):
        from ._native import LolaCudaBatchInfo
        i = LolaCudaBatchInfo()
        check(self.lib.lolaCudaBatchGetInfo(self.handle, C.byref(i)), "batch info")
        return i

    def close(self) -> None:
        if getattr(self, "handle", None):
            self.lib.lolaCudaBatchDestroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class GlobalData:
    """A RabbitCtGlobalData whose buffers are numpy arrays kept alive here."""

    def __init__(self, n: int, voxel_size: float, origin_index: float, width: int, height: int,
                 batch: int, volume: np.ndarray | None = None,
                 geometry: np.ndarray | None = None):
        self.volume = (np.zeros((n, n, n), np.float32) if volume is None else volume)
        assert self.volume.dtype == np.float32 and self.volume.flags["C_CONTIGUOUS"]
        self.geometry = None if geometry is None else np.ascontiguousarray(geometry, np.float64)
        self.mats = np.zeros((batch, 12), np.float64)
        self.images = np.zeros((batch, height, width), np.float32)
        self.projs = (Projection * batch)()
        for i in range(batch):
            self.projs[i].id = 0
            self.projs[i].matrix = self.mats[i].ctypes.data_as(C.POINTER(C.c_double))
            self.projs[i].image = self.images[i].ctypes.data_as(C.POINTER(C.c_float))
        d = RabbitCtGlobalData()
        d.problemSize, d.imageWidth, d.imageHeight = n, width, height
        d.voxelSize, d.O_Index = voxel_size, origin_index
        d.volumeData = self.volume.ctypes.data_as(C.POINTER(C.c_float))
        d.numberOfProjections = 0 if self.geometry is None else self.geometry.shape[0]
        d.globalGeometry = (None if self.geometry is None
                            else self.geometry.ctypes.data_as(C.POINTER(C.c_double)))
        d.projectionBuffer = self.projs
        d.clipFilename = None
        self.data = d

    @property
    def ref(self):
        return C.byref(self.data)


def module_functions(lib: C.CDLL, prefix: str):
    """(prepare, backprojection, finish) of a RabbitCT module in `lib`, e.g.
    prefix 'lolaCuda' or, for the reference build, 'lolaBunny'."""
    fns = []
    for suffix in ("Prepare", "Backprojection", "Finish"):
        f = getattr(lib, prefix + suffix)
        f.restype = C.c_int
        f.argtypes = [C.POINTER(RabbitCtGlobalData)]
        fns.append(f)
    return tuple(fns)
