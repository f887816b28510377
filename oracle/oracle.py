"""ORACLE — test infrastructure only.

ctypes front end of oracle/liboracle.so (the CPU restatements in oracle.c,
oracle_opt.c and oracle_asm.c) and of oracle/_ref/libref.so (the reference built from its own
sources by oracle/ref.mk, present only where the reference tree is).  Only
tests/, __graft_entry__.smoke() and bench.py's CPU-baseline arm import this.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "liboracle.so"
REF_LIB = HERE / "_ref" / "libref.so"
REF_RUNNER = HERE / "_ref" / "rabbitRunner"

_P = C.c_void_p
_lib = None


def build() -> None:
    subprocess.run(["make", "-C", str(HERE)], check=True, capture_output=True)


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB.exists():
            build()
        L = C.CDLL(str(LIB))
        geo = [C.c_int, C.c_float, C.c_float, C.c_int, C.c_int, C.c_int, _P]
        L.oracleBunnyF64.argtypes = geo + [_P, _P]
        L.oracleBunnyF64.restype = None
        L.oracleBunnyF32.argtypes = geo + [_P, _P]
        L.oracleBunnyF32.restype = None
        L.oracleShadow.argtypes = geo + [_P]
        L.oracleShadow.restype = None
        L.oracleLineRanges.argtypes = geo + [C.c_int, C.c_int, _P]
        L.oracleLineRanges.restype = None
        L.oracleOptPadding.argtypes = [_P, C.c_int, C.c_int, _P]
        L.oracleOptPadding.restype = C.c_int
        L.oracleOptBackproject.argtypes = [C.c_int, C.c_float, C.c_float, C.c_int, _P, _P, _P,
                                           C.c_int, C.c_int, _P, _P]
        L.oracleOptBackproject.restype = None
        L.oracleAsmPadding.argtypes = [_P, C.c_int, C.c_int, C.c_int, _P, _P]
        L.oracleAsmPadding.restype = C.c_int
        L.oracleAsmBackproject.argtypes = [C.c_int, C.c_float, C.c_float, C.c_int, _P, _P, _P,
                                           C.c_int, C.c_int, _P, C.c_int, _P]
        L.oracleAsmBackproject.restype = None
        L.oracleBunnyPoints.argtypes = geo + [_P, C.c_int, _P, C.c_int, _P]
        L.oracleBunnyPoints.restype = None
        L.oracleThreads.argtypes = []
        L.oracleThreads.restype = C.c_int
        _lib = L
    return _lib


def _geo(n, vs, o, mats, images):
    mats = np.ascontiguousarray(mats, np.float64).reshape(-1, 12)
    images = np.ascontiguousarray(images, np.float32)
    nproj, h, w = images.shape
    assert mats.shape[0] == nproj
    return mats, images, [n, vs, o, w, h, nproj, mats.ctypes.data]


def bunny_f64(n, vs, o, mats, images, vol=None) -> np.ndarray:
    """LolaBunny's method with FP64 accumulation (the error baseline)."""
    mats, images, g = _geo(n, vs, o, mats, images)
    out = np.zeros((n, n, n), np.float64) if vol is None else vol
    lib().oracleBunnyF64(*g, images.ctypes.data, out.ctypes.data)
    return out


def bunny_f32(n, vs, o, mats, images, vol=None) -> np.ndarray:
    """LolaBunny's method accumulating into FP32 exactly as the reference does."""
    mats, images, g = _geo(n, vs, o, mats, images)
    out = np.zeros((n, n, n), np.float32) if vol is None else vol
    lib().oracleBunnyF32(*g, images.ctypes.data, out.ctypes.data)
    return out


def bunny_points(n, vs, o, mats, images, index, fp32_accumulate=False) -> np.ndarray:
    """LolaBunny at the flattened voxel indices `index` (FP64 sums, or FP32
    accumulation like the reference)."""
    mats, images, g = _geo(n, vs, o, mats, images)
    idx = np.ascontiguousarray(index, np.int64)
    out = np.zeros(idx.size, np.float64)
    lib().oracleBunnyPoints(*g, images.ctypes.data, idx.size, idx.ctypes.data,
                            int(fp32_accumulate), out.ctypes.data)
    return out


def shadow(n, vs, o, mats, w, h) -> tuple[int, int, int, int]:
    mats = np.ascontiguousarray(mats, np.float64).reshape(-1, 12)
    s = np.zeros(4, np.int32)
    lib().oracleShadow(n, vs, o, w, h, mats.shape[0], mats.ctypes.data, s.ctypes.data)
    return tuple(int(x) for x in s)


def line_ranges(n, vs, o, mats, w, h, vector_size=8, signed_hit=False) -> np.ndarray:
    """(nproj, N*N, 2) int16 {start, stop} per row z*N + y."""
    mats = np.ascontiguousarray(mats, np.float64).reshape(-1, 12)
    out = np.zeros((mats.shape[0], n * n, 2), np.int16)
    lib().oracleLineRanges(n, vs, o, w, h, mats.shape[0], mats.ctypes.data, vector_size,
                           int(signed_hit), out.ctypes.data)
    return out


class OptBaseline:
    """The LolaOPT port (oracle_opt.c) set up like lolaOptPrepare
    (src/LolaOPT.c:23-84): line ranges over all views, padding from the shadow."""

    def __init__(self, n, vs, o, mats, w, h, vector_size=4):
        self.n, self.vs, self.o, self.w, self.h = n, vs, o, w, h
        self.mats = np.ascontiguousarray(mats, np.float64).reshape(-1, 12)
        self.ranges = line_ranges(n, vs, o, self.mats, w, h, vector_size, signed_hit=False)
        sh = np.array(shadow(n, vs, o, self.mats, w, h), np.int32)
        pad = np.zeros(4, np.int32)
        self.line = lib().oracleOptPadding(sh.ctypes.data, w, h, pad.ctypes.data)
        self.pad = pad
        self.rows = int(pad[2] + h + pad[3])
        self.start = int(pad[2] * self.line + pad[0])
        self._bufs: list[np.ndarray] = []

    def backproject(self, vol: np.ndarray, ids, images) -> None:
        """One module call: views with 1-based `ids` and their images.  The
        copy into the zero-padded buffers is part of the call, as in
        src/LolaOPT.c:110-117."""
        while len(self._bufs) < len(ids):
            self._bufs.append(np.zeros((self.rows, self.line), np.float32))
        ptrs = (C.c_void_p * len(ids))()
        r0, c0 = int(self.pad[2]), int(self.pad[0])
        for i, img in enumerate(images):
            self._bufs[i][r0:r0 + self.h, c0:c0 + self.w] = img
            ptrs[i] = self._bufs[i].ctypes.data
        idarr = np.ascontiguousarray(ids, np.int32)
        mats = np.ascontiguousarray(self.mats[idarr - 1])
        lib().oracleOptBackproject(self.n, self.vs, self.o, len(ids), idarr.ctypes.data,
                                   mats.ctypes.data, ptrs, self.start, self.line,
                                   self.ranges.ctypes.data, vol.ctypes.data)


class AsmBaseline:
    """The LolaASM restatement (oracle_asm.c) set up like lolaAsmPrepare
    (src/LolaASM.c:26-70): line ranges over all views widened to the vector
    width, padding from the shadow rounded up to it.  Each call copies its
    views into zero-padded buffers (src/LolaASM.c:113-122) and backprojects
    them, y-blocked by 8 with the call's views inside each block."""

    def __init__(self, n, vs, o, mats, w, h, vector_size=4, ranges=None):
        self.n, self.vs, self.o, self.w, self.h = n, vs, o, w, h
        self.vec = vector_size
        self.mats = np.ascontiguousarray(mats, np.float64).reshape(-1, 12)
        # the same table LolaOPT uses (computeLineRanges with this vector size)
        self.ranges = (line_ranges(n, vs, o, self.mats, w, h, vector_size, signed_hit=False)
                       if ranges is None else ranges)
        sh = np.array(shadow(n, vs, o, self.mats, w, h), np.int32)
        pad = np.zeros(4, np.int32)
        rows = C.c_int(0)
        self.line = lib().oracleAsmPadding(sh.ctypes.data, w, h, vector_size, pad.ctypes.data,
                                           C.addressof(rows))
        self.pad = pad
        self.rows = rows.value
        self.start = int(pad[2] * self.line + pad[0])
        self._bufs: list[np.ndarray] = []

    def backproject(self, vol: np.ndarray, ids, images) -> None:
        # two zero rows past the padded image: LolaASM's top pad, abs(Vmax) - H
        # (src/LolaASM.c:48), leaves no row for the second tap of a voxel that
        # projects into the last padded row, and its row kernel also runs over
        # voxels outside a row's range; the reference reads whatever follows
        # its buffer there, this restatement reads zeros
        while len(self._bufs) < len(ids):
            self._bufs.append(np.zeros((self.rows + 2, self.line), np.float32))
        ptrs = (C.c_void_p * len(ids))()
        r0, c0 = int(self.pad[2]), int(self.pad[0])
        for i, img in enumerate(images):
            self._bufs[i][r0:r0 + self.h, c0:c0 + self.w] = img
            ptrs[i] = self._bufs[i].ctypes.data
        idarr = np.ascontiguousarray(ids, np.int32)
        mats = np.ascontiguousarray(self.mats[idarr - 1])
        lib().oracleAsmBackproject(self.n, self.vs, self.o, len(ids), idarr.ctypes.data,
                                   mats.ctypes.data, ptrs, self.start, self.line,
                                   self.ranges.ctypes.data, self.vec, vol.ctypes.data)


def threads() -> int:
    return lib().oracleThreads()


# ---- the reference itself (only where oracle/_ref was built) ------------------

def ref_available() -> bool:
    return REF_LIB.exists()


_ref = None


def ref_lib() -> C.CDLL:
    global _ref
    if _ref is None:
        if not REF_LIB.exists():
            raise FileNotFoundError(f"{REF_LIB} not built (needs the reference sources)")
        _ref = C.CDLL(str(REF_LIB))
    return _ref


def env_threads(n: int | None):
    """Context helper: OMP_NUM_THREADS for child processes."""
    env = dict(os.environ)
    if n is not None:
        env["OMP_NUM_THREADS"] = str(n)
    return env
