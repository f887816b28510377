"""Seeded synthetic scans with the RabbitCT dataset's shapes and formats.

The rabbit dataset itself (496 x 1248x960 float32, reference README.md:100-107)
is not available, so every workload is synthesised: circular C-arm geometry
(SOD 780 mm, SID 1200 mm, 0.308 mm pitch, 200 degree arc by default) and
analytic line integrals through seeded random ellipsoids plus Gaussian noise.
See csrc/rct_synth.c for the model.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _native


class _Geom(C.Structure):
    _fields_ = [("nproj", C.c_int32), ("width", C.c_int32), ("height", C.c_int32),
                ("reserved", C.c_int32), ("sod", C.c_double), ("sid", C.c_double),
                ("pitch", C.c_double), ("arcDeg", C.c_double), ("startDeg", C.c_double),
                ("ppJitter", C.c_double), ("seed", C.c_uint64)]


class _Ellipsoid(C.Structure):
    _fields_ = [("center", C.c_double * 3), ("axes", C.c_double * 3),
                ("rot", C.c_double * 9), ("density", C.c_double)]


# reference src/rabbitRunner.c:61-84 (voxel size per problem size)
_REFERENCE_VOXEL_SIZE = {128: 2.0, 256: 1.0, 512: 0.5, 1024: 0.25}


def voxel_size(n: int) -> float:
    """Voxel edge in mm: the reference's table for 128..1024, else a 256 mm cube."""
    return float(np.float32(_REFERENCE_VOXEL_SIZE.get(n, 256.0 / n)))


def origin_index(n: int, vs: float) -> float:
    """O_Index = -0.5f * voxelSize * ((float)N - 1.0f) in float32, left to right
    (src/rabbitRunner.c:189)."""
    f = np.float32
    return float((f(-0.5) * f(vs)) * (f(n) - f(1.0)))


@dataclass
class ScanSpec:
    nproj: int = 496
    width: int = 1248
    height: int = 960
    sod: float = 780.0
    sid: float = 1200.0
    pitch: float = 0.308
    arc_deg: float = 200.0
    start_deg: float = 0.0
    pp_jitter: float = 2.0
    seed: int = 1
    n_ellipsoids: int = 10
    phantom_radius: float = 128.0
    noise_sigma: float = 0.01
    noise_seed: int = 7


@dataclass
class Scan:
    spec: ScanSpec
    matrices: np.ndarray            # (nproj, 12) float64
    images: np.ndarray              # (nproj, H, W) float32
    hus: tuple = field(default=(1.0, 0.0))

    @property
    def width(self) -> int:
        return self.spec.width

    @property
    def height(self) -> int:
        return self.spec.height

    @property
    def nproj(self) -> int:
        return self.spec.nproj


def _geom(spec: ScanSpec) -> _Geom:
    g = _Geom()
    g.nproj, g.width, g.height = spec.nproj, spec.width, spec.height
    g.sod, g.sid, g.pitch = spec.sod, spec.sid, spec.pitch
    g.arcDeg, g.startDeg, g.ppJitter = spec.arc_deg, spec.start_deg, spec.pp_jitter
    g.seed = spec.seed
    return g


def matrices(spec: ScanSpec) -> np.ndarray:
    lib = _native.load_synth()
    out = np.empty((spec.nproj, 12), np.float64)
    g = _geom(spec)
    lib.rctSynthMatrices(C.addressof(g), out.ctypes.data)
    return out


def projections(spec: ScanSpec, out: np.ndarray | None = None) -> np.ndarray:
    lib = _native.load_synth()
    ell = (_Ellipsoid * max(1, spec.n_ellipsoids))()
    n = lib.rctSynthPhantom(spec.seed, spec.n_ellipsoids, spec.phantom_radius, C.addressof(ell))
    if n != spec.n_ellipsoids:
        raise ValueError("ellipsoid count outside 0..64")
    if out is None:
        out = np.empty((spec.nproj, spec.height, spec.width), np.float32)
    assert out.shape == (spec.nproj, spec.height, spec.width) and out.dtype == np.float32
    g = _geom(spec)
    lib.rctSynthProjections(C.addressof(g), C.addressof(ell), spec.n_ellipsoids,
                            spec.noise_sigma, spec.noise_seed, out.ctypes.data)
    return out


def make_scan(spec: ScanSpec) -> Scan:
    mats = matrices(spec)
    imgs = projections(spec)
    # HU factors so that the brightest expected voxel maps near 3000 HU
    peak = float(np.abs(imgs).max()) or 1.0
    scale = 3000.0 * spec.sod ** 2 / (spec.nproj * peak)
    return Scan(spec, mats, imgs, (float(np.float32(scale)), 0.0))
