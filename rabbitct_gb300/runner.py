"""Python mirror of rabbitRunner's driver loop (reference src/rabbitRunner.c:183-287).

`run_module` drives any RabbitCT module (LolaCUDA, or a reference module
loaded from a build of the reference) through prepare / backprojection /
finish exactly as the runner does:
  - numberOfProjections = total and globalGeometry set only "with -a"
    (:209-217), then prepare (:222-232);
  - numberOfProjections = b, buffers reused for every call, 1-based ids in
    file order (:256-278);
  - each backprojection call timed on its own (PROFILE, :41-59, :279-280);
  - finish untimed (:287).
The reported `total_s` is the runner's "Total" (:436-440); `e2e_s` also
covers prepare and finish.
"""
from __future__ import annotations

import time
from dataclasses import dataclass

import numpy as np

from .lolacuda import GlobalData


@dataclass
class RunResult:
    volume: np.ndarray
    total_s: float       # sum of timed backprojection calls, like the runner's "Total"
    prepare_s: float
    finish_s: float
    e2e_s: float         # prepare + all calls + finish


def run_module(fns, n: int, voxel_size: float, origin_index: float, matrices: np.ndarray,
               images: np.ndarray, batch: int = 1, with_geometry: bool = True,
               volume: np.ndarray | None = None,
               clip_filename: str | None = None) -> RunResult:
    prepare, iterate, finish = fns
    nproj, height, width = images.shape
    if nproj % batch != 0:
        # the runner would read past the end of the file and exit
        # (src/rabbitRunner.c:267-283, src/ctFileReader.c:51-54)
        raise ValueError(f"batch {batch} does not divide {nproj} projections")
    gd = GlobalData(n, voxel_size, origin_index, width, height, batch, volume=volume,
                    geometry=matrices if with_geometry else None)
    # -C: line-range cache file of the reference's clipping modules
    clip = None if clip_filename is None else clip_filename.encode()
    gd.data.clipFilename = clip
    t0 = time.perf_counter()
    if not prepare(gd.ref):
        raise RuntimeError("prepare failed")
    t1 = time.perf_counter()
    gd.data.numberOfProjections = batch
    total = 0.0
    next_id = 0
    for _ in range(nproj // batch):
        for i in range(batch):
            gd.mats[i] = matrices[next_id]
            gd.images[i] = images[next_id]
            next_id += 1
            gd.projs[i].id = next_id
        c0 = time.perf_counter()
        if not iterate(gd.ref):
            raise RuntimeError("backprojection failed")
        total += time.perf_counter() - c0
    t2 = time.perf_counter()
    if not finish(gd.ref):
        raise RuntimeError("finish failed")
    t3 = time.perf_counter()
    return RunResult(gd.volume, total, t1 - t0, t3 - t2, t3 - t0)
