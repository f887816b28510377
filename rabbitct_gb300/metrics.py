"""Error metrics for reconstructed volumes.

`errors` compares against a reference volume (normally the FP64 oracle):
max-abs, RMSE, relative RMSE = RMSE / RMS(reference), PSNR = 20 log10(max|ref| / RMSE).
`hu_quality` restates the runner's verification (reference
src/rabbitRunner.c:320-384): voxels are mapped to Hounsfield units with the
file's scaling factors (round(hus0 * v + hus1) for v > 0, else 0, clamped to
4095) and compared with a uint16 HU reference volume.
"""
from __future__ import annotations

import math

import numpy as np


def errors(test: np.ndarray, ref: np.ndarray) -> dict:
    t = np.asarray(test, np.float64).ravel()
    r = np.asarray(ref, np.float64).ravel()
    d = t - r
    mse = float(np.mean(d * d))
    rmse = math.sqrt(mse)
    rms_ref = math.sqrt(float(np.mean(r * r)))
    peak = float(np.max(np.abs(r))) if r.size else 0.0
    return {
        "max_abs": float(np.max(np.abs(d))) if d.size else 0.0,
        "rmse": rmse,
        "rel_rmse": rmse / rms_ref if rms_ref > 0 else (0.0 if rmse == 0 else math.inf),
        "psnr_db": (20.0 * math.log10(peak / rmse)) if rmse > 0 and peak > 0 else math.inf,
    }


def to_hu(vol: np.ndarray, hus) -> np.ndarray:
    """float32 volume -> HU as the runner forms it (src/rabbitRunner.c:346-355)."""
    v = np.asarray(vol, np.float32)
    s0, s1 = np.float32(hus[0]), np.float32(hus[1])
    hu = np.where(v > 0, np.floor(s0 * v + s1 + np.float32(0.5)), np.float32(0.0))
    return np.minimum(hu, np.float32(4095.0)).astype(np.float32)


def hu_quality(vol: np.ndarray, ref_hu: np.ndarray, hus) -> dict:
    hu = to_hu(vol, hus).ravel()
    err = hu - np.asarray(ref_hu, np.float32).ravel()
    abs_err = np.abs(err)
    mse = float(np.mean(err.astype(np.float64) ** 2))
    hist = np.bincount(np.minimum(np.floor(abs_err).astype(np.int64), 10), minlength=11)
    return {
        "rmse_hu": math.sqrt(mse),
        "mse_hu2": mse,
        "max_abs_hu": float(abs_err.max()) if abs_err.size else 0.0,
        "psnr_db": (10.0 * math.log10(4095.0 ** 2 / mse)) if mse > 1e-8 else math.inf,
        "histogram": hist.tolist(),
    }
