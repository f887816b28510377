"""RabbitCT `.rct` file format (reference src/ctFileReader.c, ctFileReader_types.h).

Layout, little-endian, no padding:
  header   uint32 imageDimension[2]; uint32 numberOfImages; float32 HUScalingFactors[2]
           (20 bytes, src/ctFileReader_types.h:11-15)
  records  per projection: 12 float64 matrix (column-major 3x4), then
           width*height float32 image (src/ctFileReader.c:47-61)
A geometry file (-a) is the same header followed by numberOfImages * 12
float64 (src/ctFileReader.c:36-45).
"""
from __future__ import annotations

from dataclasses import dataclass
from pathlib import Path

import numpy as np

HEADER_DTYPE = np.dtype([("imageDimension", "<u4", (2,)), ("numberOfImages", "<u4"),
                         ("HUScalingFactors", "<f4", (2,))])
assert HEADER_DTYPE.itemsize == 20


@dataclass
class RctHeader:
    width: int
    height: int
    count: int
    hus: tuple[float, float]


def _header_bytes(width: int, height: int, count: int, hus) -> bytes:
    h = np.zeros((), HEADER_DTYPE)
    h["imageDimension"] = (width, height)
    h["numberOfImages"] = count
    h["HUScalingFactors"] = hus
    return h.tobytes()


def write_rct(path, images: np.ndarray, matrices: np.ndarray, hus=(1.0, 0.0)) -> None:
    """images: (n, H, W) float32; matrices: (n, 12) float64."""
    images = np.ascontiguousarray(images, dtype="<f4")
    matrices = np.ascontiguousarray(matrices, dtype="<f8")
    n, H, W = images.shape
    assert matrices.shape == (n, 12)
    with open(path, "wb") as f:
        f.write(_header_bytes(W, H, n, hus))
        for p in range(n):
            f.write(matrices[p].tobytes())
            f.write(images[p].tobytes())


def write_geometry(path, matrices: np.ndarray, width: int, height: int, hus=(1.0, 0.0)) -> None:
    matrices = np.ascontiguousarray(matrices, dtype="<f8")
    with open(path, "wb") as f:
        f.write(_header_bytes(width, height, matrices.shape[0], hus))
        f.write(matrices.tobytes())


def read_header(path) -> RctHeader:
    raw = np.fromfile(path, dtype=HEADER_DTYPE, count=1)
    if raw.size != 1:
        raise ValueError(f"{path}: no RabbitCT header")
    h = raw[0]
    return RctHeader(int(h["imageDimension"][0]), int(h["imageDimension"][1]),
                     int(h["numberOfImages"]), (float(h["HUScalingFactors"][0]),
                                                float(h["HUScalingFactors"][1])))


class RctReader:
    """Sequential reader with the reference's 1-based image ids
    (src/ctFileReader.c:10,47-61)."""

    def __init__(self, path):
        self.path = Path(path)
        self.header = read_header(self.path)
        self._f = open(self.path, "rb")
        self._f.seek(HEADER_DTYPE.itemsize)
        self.current = 0
        self.image_size = self.header.width * self.header.height

    def read_image(self, matrix_out: np.ndarray, image_out: np.ndarray) -> int:
        m = self._f.read(96)
        img = self._f.read(4 * self.image_size)
        if len(m) != 96 or len(img) != 4 * self.image_size:
            raise EOFError(f"{self.path}: read past the last projection")
        self.current += 1
        matrix_out[...] = np.frombuffer(m, "<f8")
        image_out.reshape(-1)[...] = np.frombuffer(img, "<f4")
        return self.current

    def close(self) -> None:
        self._f.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def read_geometry(path) -> tuple[RctHeader, np.ndarray]:
    h = read_header(path)
    m = np.fromfile(path, dtype="<f8", offset=HEADER_DTYPE.itemsize, count=12 * h.count)
    if m.size != 12 * h.count:
        raise ValueError(f"{path}: truncated geometry")
    return h, m.reshape(h.count, 12)
