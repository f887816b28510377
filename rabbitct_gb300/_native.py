"""ctypes bindings of liblolacuda.so (include/lolaCuda.h) and librctsynth.so.

The CUDA library must be present: every entry point here raises if it is
missing instead of falling back to anything else.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

_LIB_DIR = Path(__file__).resolve().parent / "_lib"


class LolaCudaError(RuntimeError):
    pass


# ---- RabbitCT data contract (src/rabbitCt.h:9-27 of the reference) ----------

class Projection(C.Structure):
    _fields_ = [("id", C.c_int),
                ("matrix", C.POINTER(C.c_double)),
                ("image", C.POINTER(C.c_float))]


class RabbitCtGlobalData(C.Structure):
    _fields_ = [("problemSize", C.c_uint32),
                ("imageWidth", C.c_uint32),
                ("imageHeight", C.c_uint32),
                ("voxelSize", C.c_float),
                ("O_Index", C.c_float),
                ("volumeData", C.POINTER(C.c_float)),
                ("numberOfProjections", C.c_uint32),
                ("globalGeometry", C.POINTER(C.c_double)),
                ("projectionBuffer", C.POINTER(Projection)),
                ("clipFilename", C.c_char_p)]


class LolaCudaConfig(C.Structure):
    _fields_ = [("storage", C.c_int32),
                ("accumulation", C.c_int32),
                ("batch", C.c_int32),
                ("voxelsPerThread", C.c_int32),
                ("rowsPerBlock", C.c_int32),
                ("syncEachCall", C.c_int32),
                ("exitOnError", C.c_int32),
                ("collectStats", C.c_int32),
                ("device", C.c_int32),
                ("staging", C.c_int32),
                ("batchMode", C.c_int32),
                ("batchBranches", C.c_int32),
                ("batchTune", C.c_int32),
                ("edgeBatch", C.c_int32),
                ("reserved", C.c_int32 * 2)]


class LolaCudaGeometry(C.Structure):
    _fields_ = [("problemSize", C.c_int32),
                ("imageWidth", C.c_int32),
                ("imageHeight", C.c_int32),
                ("voxelSize", C.c_float),
                ("originIndex", C.c_float),
                ("sliceBegin", C.c_int32),
                ("sliceCount", C.c_int32)]


class LolaCudaQuality(C.Structure):
    _fields_ = [("mse", C.c_double), ("rmse", C.c_double), ("maxAbs", C.c_double),
                ("psnr", C.c_double), ("histogram", C.c_uint64 * 11)]


class LolaCudaJob(C.Structure):
    _fields_ = [("geometry", LolaCudaGeometry), ("projections", C.c_int32),
                ("reserved", C.c_int32), ("d_images", C.c_void_p),
                ("h_matrices", C.c_void_p), ("d_volume", C.c_void_p)]


class LolaCudaBatchInfo(C.Structure):
    _fields_ = [("jobs", C.c_int32), ("waves", C.c_int32), ("blocks", C.c_int32),
                ("launchesPerRun", C.c_int32), ("voxelUpdates", C.c_double),
                ("ringBytes", C.c_size_t)]


class LolaCudaTuneCandidate(C.Structure):
    _fields_ = [("voxelsPerThread", C.c_int32), ("rowsPerBlock", C.c_int32),
                ("batch", C.c_int32), ("staging", C.c_int32), ("ms", C.c_double)]


class LolaCudaTuneReport(C.Structure):
    _fields_ = [("candidates", C.c_int32), ("best", C.c_int32),
                ("tried", LolaCudaTuneCandidate * 64)]


class LolaCudaFileReport(C.Structure):
    _fields_ = [("seconds", C.c_double), ("readSeconds", C.c_double),
                ("projections", C.c_int64), ("gups", C.c_double), ("hus", C.c_float * 2)]


class LolaCudaScanTiming(C.Structure):
    _fields_ = [("prepareSeconds", C.c_double),
                ("callSeconds", C.c_double),
                ("finishSeconds", C.c_double),
                ("totalSeconds", C.c_double)]


class LolaCudaStats(C.Structure):
    _fields_ = [("passes", C.c_int64),
                ("packs", C.c_int64),
                ("projections", C.c_int64),
                ("passMs", C.c_double),
                ("tilePassesFast", C.c_int64),
                ("tilePassesSlow", C.c_int64),
                ("tilePassesSkipped", C.c_int64),
                ("tilePassesStaged", C.c_int64),
                ("stagedPasses", C.c_int64),
                ("overlappedPasses", C.c_int64),
                ("chunkLaunches", C.c_int64),
                ("tilePassesPaired", C.c_int64)]


STORAGE = {"f32": 0, "f16": 1, "bf16": 2, "f32q": 3, "f16q": 4, "bf16q": 5, "tex32": 6,
           "tex16": 7, "f16qx": 8, "f32qx": 9}
ACCUM = {"plain": 0, "kahan": 1}
MAX_BATCH = 64

# every symbol include/lolaCuda.h declares: (name, restype, argtypes)
_P = C.c_void_p
_SIGNATURES = [
    ("lolaCudaPrepare", C.c_int, [C.POINTER(RabbitCtGlobalData)]),
    ("lolaCudaBackprojection", C.c_int, [C.POINTER(RabbitCtGlobalData)]),
    ("lolaCudaFinish", C.c_int, [C.POINTER(RabbitCtGlobalData)]),
    ("lolaCudaDefaultConfig", None, [C.POINTER(LolaCudaConfig)]),
    ("lolaCudaSetConfig", C.c_int, [C.POINTER(LolaCudaConfig)]),
    ("lolaCudaGetConfig", C.c_int, [C.POINTER(LolaCudaConfig)]),
    ("lolaCudaLastError", C.c_char_p, []),
    ("lolaCudaPlanCreate", C.c_int, [C.POINTER(LolaCudaGeometry), C.POINTER(LolaCudaConfig),
                                      C.POINTER(_P)]),
    ("lolaCudaPlanDestroy", C.c_int, [_P]),
    ("lolaCudaPlanVolume", _P, [_P]),
    ("lolaCudaPlanStream", _P, [_P]),
    ("lolaCudaPlanZeroVolume", C.c_int, [_P]),
    ("lolaCudaPlanUploadVolume", C.c_int, [_P, _P]),
    ("lolaCudaPlanDownloadVolume", C.c_int, [_P, _P]),
    ("lolaCudaPlanUploadVolumeAsync", C.c_int, [_P, _P]),
    ("lolaCudaPlanStreamVolumeOut", C.c_int, [_P, _P]),
    ("lolaCudaPlanBackprojectDevice", C.c_int, [_P, _P, C.c_size_t, _P, C.c_int]),
    ("lolaCudaPlanBackprojectHost", C.c_int, [_P, _P, C.c_size_t, _P, C.c_int]),
    ("lolaCudaPlanSynchronize", C.c_int, [_P]),
    ("lolaCudaPlanTimerStart", C.c_int, [_P]),
    ("lolaCudaPlanTimerStop", C.c_int, [_P, C.POINTER(C.c_double)]),
    ("lolaCudaPlanGetStats", C.c_int, [_P, C.POINTER(LolaCudaStats)]),
    ("lolaCudaPlanResetStats", C.c_int, [_P]),
    ("lolaCudaDeviceAlloc", _P, [C.c_size_t]),
    ("lolaCudaDeviceFree", C.c_int, [_P]),
    ("lolaCudaCopyToDevice", C.c_int, [_P, _P, C.c_size_t]),
    ("lolaCudaCopyToHost", C.c_int, [_P, _P, C.c_size_t]),
    ("lolaCudaDeviceSynchronize", C.c_int, []),
    ("lolaCudaBackprojectNoAlloc", C.c_int, [C.POINTER(LolaCudaGeometry),
                                             C.POINTER(LolaCudaConfig), _P, _P, C.c_size_t,
                                             _P, C.c_int, _P]),
    ("lolaCudaComputeLineRanges", C.c_int, [C.POINTER(RabbitCtGlobalData), _P, C.c_int,
                                            C.c_int]),
    ("lolaCudaComputeShadow", C.c_int, [C.POINTER(RabbitCtGlobalData), _P]),
    ("lolaCudaVerifyVolume", C.c_int, [_P, C.c_size_t, _P, _P, C.c_int, _P,
                                       C.POINTER(LolaCudaQuality)]),
    ("lolaCudaPlanVerify", C.c_int, [_P, _P, _P, C.c_int, C.POINTER(LolaCudaQuality)]),
    ("lolaCudaPlanWriteSlicePgm", C.c_int, [_P, C.c_char_p, _P]),
    ("lolaCudaPlanWriteResult", C.c_int, [_P, C.c_char_p, _P, _P, C.c_uint32, C.c_uint64,
                                          C.POINTER(LolaCudaQuality)]),
    ("lolaCudaSlab", C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int32),
                               C.POINTER(C.c_int32)]),
    ("lolaCudaBatchCreate", C.c_int, [_P, C.c_int, C.POINTER(LolaCudaConfig), C.POINTER(_P)]),
    ("lolaCudaBatchRun", C.c_int, [_P]),
    ("lolaCudaBatchSynchronize", C.c_int, [_P]),
    ("lolaCudaBatchStream", _P, [_P]),
    ("lolaCudaBatchGetInfo", C.c_int, [_P, C.POINTER(LolaCudaBatchInfo)]),
    ("lolaCudaBatchDestroy", C.c_int, [_P]),
    ("lolaCudaAutotune", C.c_int, [C.POINTER(LolaCudaGeometry), _P, C.c_size_t, _P, C.c_int,
                                   C.POINTER(LolaCudaConfig), C.POINTER(LolaCudaTuneReport)]),
    ("lolaCudaReadRctHeader", C.c_int, [C.c_char_p, _P, _P, _P, _P]),
    ("lolaCudaRunScan", C.c_int, [C.POINTER(RabbitCtGlobalData), _P, C.c_size_t, _P, C.c_int,
                                  C.c_int, C.POINTER(LolaCudaScanTiming)]),
    ("lolaCudaReconstructFile", C.c_int, [C.c_char_p, C.c_int, C.c_float, C.c_float,
                                          C.POINTER(LolaCudaConfig), _P,
                                          C.POINTER(LolaCudaFileReport)]),
    ("lolaCudaHostAlloc", _P, [C.c_size_t]),
    ("lolaCudaHostFree", C.c_int, [_P]),
    ("lolaCudaProbeIssueRate", C.c_double, []),
    ("lolaCudaProbeGatherRate", C.c_double, [C.c_int, C.c_int, C.c_int]),
    ("lolaCudaProbeGatherPeak", C.c_double, [C.c_int]),
    ("lolaCudaProbeTextureRows", C.c_double, [C.c_int]),
    ("lolaCudaDeviceInfo", C.c_int, [C.POINTER(C.c_int), C.POINTER(C.c_int), C.c_char_p,
                                     C.c_int]),
]

_lola = None
_synth = None


def lib_path() -> Path:
    return _LIB_DIR / "liblolacuda.so"


def load_lolacuda() -> C.CDLL:
    """Loads liblolacuda.so; raises if it was not built (no fallback)."""
    global _lola
    if _lola is None:
        path = lib_path()
        if not path.exists():
            raise LolaCudaError(f"{path} is missing: build it with "
                                "`python -c 'import __graft_entry__ as g; g.build()'`")
        lib = C.CDLL(str(path))
        for name, res, args in _SIGNATURES:
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lola = lib
    return _lola


def last_error() -> str:
    msg = load_lolacuda().lolaCudaLastError()
    return msg.decode() if msg else ""


def check(ok: int, what: str) -> None:
    if not ok:
        raise LolaCudaError(f"{what}: {last_error()}")


def load_synth() -> C.CDLL:
    global _synth
    if _synth is None:
        path = _LIB_DIR / "librctsynth.so"
        if not path.exists():
            raise LolaCudaError(f"{path} is missing: run rabbitct_gb300.build.build_all()")
        lib = C.CDLL(str(path))
        lib.rctSynthMatrices.restype = None
        lib.rctSynthMatrices.argtypes = [_P, _P]
        lib.rctSynthPhantom.restype = C.c_int
        lib.rctSynthPhantom.argtypes = [C.c_uint64, C.c_int, C.c_double, _P]
        lib.rctSynthProjections.restype = None
        lib.rctSynthProjections.argtypes = [_P, _P, C.c_int, C.c_double, C.c_uint64, _P]
        _synth = lib
    return _synth


def ptr(a: np.ndarray) -> int:
    assert a.flags["C_CONTIGUOUS"], "array must be C-contiguous"
    return a.ctypes.data


def config(storage: str | None = None, accumulation: str | None = None,
           batch: int | None = None, voxels_per_thread: int | None = None,
           rows_per_block: int | None = None, sync_each_call: int | None = None,
           exit_on_error: int = 0, collect_stats: int | None = None, device: int | None = None,
           staging: int | None = None, batch_mode: int | None = None,
           batch_branches: int | None = None, batch_tune: int | None = None,
           edge_batch: int | None = None) -> LolaCudaConfig:
    """A LolaCudaConfig from the library's defaults (which honour the
    LOLACUDA_* environment overrides) with the given fields replaced.
    exit_on_error defaults to 0 here: Python callers want exceptions."""
    c = LolaCudaConfig()
    load_lolacuda().lolaCudaDefaultConfig(C.byref(c))
    if storage is not None:
        c.storage = STORAGE[storage]
    if accumulation is not None:
        c.accumulation = ACCUM[accumulation]
    for name, value in (("batch", batch), ("voxelsPerThread", voxels_per_thread),
                        ("rowsPerBlock", rows_per_block), ("syncEachCall", sync_each_call),
                        ("exitOnError", exit_on_error), ("collectStats", collect_stats),
                        ("device", device), ("staging", staging), ("batchMode", batch_mode),
                        ("batchBranches", batch_branches), ("batchTune", batch_tune),
                        ("edgeBatch", edge_batch)):
        if value is not None:
            setattr(c, name, value)
    return c
