#!/usr/bin/env python3
"""LolaCUDA benchmark: GUPS of cone-beam backprojection on GB300.

Workload (one step = one full reconstruction): N=1024 volume (0.25 mm voxels,
4 GiB FP32 resident in HBM), 496 synthetic projections of 1248x960 (seeded
ellipsoid phantom, circular 200 degree scan) — the RabbitCT dataset's shapes.
GUPS = N^3 * projections / time (RabbitCT's convention: every voxel counts for
every projection, clipped or not).

Lines printed (rank 0, one JSON object):
  value   device-resident throughput of the FP16-stored path (projections
          already in HBM when the timed region starts; CUDA events on the
          plan's stream); tile shape, batch and staging are picked by the
          autotuner on the first 64 projections before the timed region
  fp32_path, fp32_quads  the plain FP32 path (four FP32 taps per update) and
          FP32 storage as 2x2 quads (the same results), measured the same way
  e2e     the same metric through the RabbitCT module API (prepare, one
          backprojection call per projection from pinned host buffers,
          finish with the volume copied back), wall clock around the calls,
          median of --e2e-steps
  roofline  the pass kernel against the measured HBM copy bandwidth
          (MEASURED_PEAKS.json), from one instrumented reconstruction after
          the (uninstrumented) timed steps: algorithmic bytes per launch /
          launch time (CUDA events around every pass),
          and the DRAM bytes of one launch from the committed ncu capture of
          the same configuration; `ceiling` holds the bound the kernel meets,
          the gather and FP32-issue rates measured by probe kernels on the
          same GPU
  clocks  SM clocks and throttle reasons sampled during the timed region
  cpu_baseline  the reference's two fastest CPU methods, LolaASM and LolaOPT,
          as restated under oracle/ (oracle_asm.c, oracle_opt.c; pinned to the
          reference's own build by tests/test_oracle_golden.py), on the host
          cores, on a bounded sample of the same workload (warm repeat); the
          faster one is `value`, both are in `methods`
  batch64  the batched uneven workload (64 reconstructions of N 128-384,
          180-496 projections, three detector sizes) in its two graph-captured
          schedules, against the same jobs through sequential plain FP32 plans
          (skip with --no-batch64)
`--impl reference` times the same two CPU methods alone (the reference's own
build cannot travel to this host) on the same workload, reporting the faster.
`--workload batch64` prints that workload alone as the line.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

import numpy as np  # noqa: E402

METRIC = "GUPS (1e9 voxel updates/s) N=512,1024: FP16-stored vs FP32 path, RMSE vs FP64"

# Issue slots per computed voxel update of the pass kernel's two implemented
# sequences (hand count of the source, FP32/INT/memory instructions):
#  - one voxel at a time (slow tiles, and fast tiles that touch negative
#    detector coordinates): 3 FMA for u,v,w; 1 reciprocal; 2 FMA for the pixel
#    coordinates; 2 truncations; 2 fraction subtractions; 6 for the two-level
#    bilinear lerp; 2 for 1/w^2 and the weighted accumulate = 18, plus the
#    stored index's FMA on the load path;
#  - two voxels per packed f32x2 instruction (paired tiles): per pair 3 steps,
#    2 coordinates, 6 floor/fraction, 1 index, 6 lerp, 2 weight+accumulate =
#    20 packed + 2 reciprocals, i.e. 11 per voxel;
# plus, per voxel and either way, its fetch: 2 index integer ops, 1 address,
# the gathers (4 plain or 1 quad) and 4 widenings of 16-bit taps on the load
# path; 2 coordinate adds and 1 texture gather for the 2D texture layouts
# (tex32, tex16); 1 index op and 1 texel fetch by index for the mixed layouts'
# linear textures (LOLA_MIXED_TEX_LINEAR).  Mixed layouts fetch
# MIXED_TEX_FRACTION of their voxels through the texture unit
# (LOLA_F16QX_TEX_MASK = 0xFFFF for f16qx: all of them; LOLA_MIXED_TEX_MASK =
# 0xAAAA for f32qx, in lolacuda_internal.h).  The 16-bit quad
# layouts store bilinear terms, so their interpolation is 3 FMAs instead of 6
# operations (3 issue slots less per voxel, 1.5 on the paired path).  FP32
# quads (f32q) are stored column by column and interpolated per voxel on the
# paired path: 2 packed + 2 scalar instead of 3 packed per voxel (+1), in
# exchange for the register moves the pairwise form needs (moves are not
# counted for either form).
MIXED_TEX_FRACTION = {"f16qx": 1.0, "f32qx": 0.5}  # LOLA_F16QX_TEX_MASK, LOLA_MIXED_TEX_MASK
_TERM_LAYOUTS = ("f16q", "bf16q", "f16qx")
_COLUMN_LAYOUTS = ("f32q",)
_LOAD_FETCH = {"f32": 7, "f16": 11, "bf16": 11, "f32q": 4, "f16q": 8, "bf16q": 8}
_TEX_FETCH = 3         # 2D texture: two coordinate adds + the gather
_TEX_LINEAR_FETCH = 2  # linear texture: the index op + the fetch


def _fetch_cost(storage):
    """(issue slots of a voxel's fetch, fraction of voxels on the load path)."""
    if storage in ("tex32", "tex16"):
        return _TEX_FETCH, 0.0
    if storage in ("f16qx", "f32qx"):
        load = _LOAD_FETCH["f16q" if storage == "f16qx" else "f32q"]
        t = MIXED_TEX_FRACTION[storage]
        return t * _TEX_LINEAR_FETCH + (1 - t) * load, 1 - t
    return _LOAD_FETCH[storage], 1.0


def instr_per_update(storage, paired_fraction):
    fetch, load_frac = _fetch_cost(storage)
    terms = storage in _TERM_LAYOUTS
    one = (15 if terms else 18) + load_frac + fetch
    two = (9.5 if terms else 12 if storage in _COLUMN_LAYOUTS else 11) + fetch
    return paired_fraction * two + (1 - paired_fraction) * one


STORAGE_IDS = {"f32": 0, "f16": 1, "bf16": 2, "f32q": 3, "f16q": 4, "bf16q": 5, "tex32": 6,
               "tex16": 7, "f16qx": 8, "f32qx": 9}


def parse_args():
    ap = argparse.ArgumentParser(description=__doc__,
                                 formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="lolacuda", choices=["lolacuda", "reference"])
    ap.add_argument("--workload", default="n1024", choices=["n1024", "batch64"],
                    help="n1024: one N=1024 reconstruction (headline); batch64: 64 uneven "
                         "reconstructions in one graph-captured persistent run")
    ap.add_argument("--jobs", type=int, default=64, help="batch64: number of reconstructions")
    # long aliases: under torchrun, whose own parser prefix-matches --n*
    ap.add_argument("--n", "--problem-size", dest="n", type=int, default=1024)
    ap.add_argument("--nproj", "--projections", dest="nproj", type=int, default=496)
    ap.add_argument("--width", type=int, default=1248)
    ap.add_argument("--height", type=int, default=960)
    ap.add_argument("--storage", default="f16qx", choices=list(STORAGE_IDS))
    ap.add_argument("--fp32-storage", default="f32", choices=list(STORAGE_IDS),
                    help="the plain FP32 path (four FP32 taps per update)")
    ap.add_argument("--fp32-quad-storage", default="f32q", choices=list(STORAGE_IDS) + ["none"],
                    help="FP32 storage as 2x2 quads: the same exact FP32 taps and results as the "
                         "plain path, one 16-byte load per update (none: skip)")
    ap.add_argument("--batch", type=int, default=16)
    ap.add_argument("--vpt", type=int, default=16)
    ap.add_argument("--rows", type=int, default=4)
    ap.add_argument("--autotune", type=int, default=1,
                    help="1: pick tile shape / batch / staging with lolaCudaAutotune on the "
                         "first 64 projections before timing (untimed)")
    ap.add_argument("--staging", type=int, default=None,
                    help="1/0: force shared-memory staging on/off (default: library default)")
    ap.add_argument("--e2e-steps", type=int, default=4)
    ap.add_argument("--cpu-views", type=int, default=8,
                    help="projections in the bounded CPU-baseline sample")
    ap.add_argument("--shard", default="slabs", choices=["slabs", "replicas"],
                    help="N>1: z-slabs of one volume per GPU (strong scaling) or one "
                         "whole reconstruction per GPU (weak scaling)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-fp32", action="store_true")
    ap.add_argument("--no-probes", action="store_true")
    ap.add_argument("--no-batch64", action="store_true",
                    help="skip the 64-reconstruction batch that the default run adds as "
                         "line['batch64']")
    return ap.parse_args()


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class Dist:
    """Host-side barrier and max-reduction across ranks (gloo); no data-path
    collective: every rank reconstructs its own volume."""

    def __init__(self, rank, world):
        self.rank, self.world = rank, world
        self.pg = None
        if world > 1:
            import torch.distributed as dist
            dist.init_process_group("gloo")
            self.dist = dist

    def barrier(self):
        if self.world > 1:
            self.dist.barrier()

    def max(self, x: float) -> float:
        if self.world == 1:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.world > 1:
            self.dist.destroy_process_group()


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.thread.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def make_workload(args):
    from rabbitct_gb300 import synth
    spec = synth.ScanSpec(nproj=args.nproj, width=args.width, height=args.height)
    scan = synth.make_scan(spec)
    vs = synth.voxel_size(args.n)
    o = synth.origin_index(args.n, vs)
    return scan, vs, o


# ---------------------------------------------------------------------------
# CPU baseline: the reference's CPU methods on the host cores (bounded sample)
# ---------------------------------------------------------------------------

CPU_METHODS = {
    "asm": ("LolaASM", "oracle/oracle_asm.c, the portable-vector restatement of LolaASM "
                       "(src/LolaASM.c + its SIMD row kernel)"),
    "opt": ("LolaOPT", "oracle/oracle_opt.c, the port of LolaOPT (src/LolaOPT.c)"),
}


def cpu_baseline(args, scan, vs, o, repeats=1) -> dict:
    """The reference's two fastest CPU methods, LolaASM and LolaOPT (as
    restated under oracle/), on a bounded sample of the workload: every
    `nproj // views`-th projection, one module call per projection (the
    runner's -b 1 of run-bench.sh), the volume zero-filled before the timed
    calls like the runner's (src/memoryUtils.c:59-63).  Returns the faster
    method as `value`, both in `methods`."""
    from oracle import oracle
    views = max(1, min(args.cpu_views, scan.nproj))
    stride = max(1, scan.nproj // views)
    sel = np.arange(0, stride * views, stride)[:views]
    mats = scan.matrices[sel]
    imgs = scan.images[sel]
    n = args.n
    # prepare (untimed, like src/rabbitRunner.c:222-232): ranges + padding,
    # one line-range table for both methods (vector width 4, NEON's)
    ob = oracle.OptBaseline(n, vs, o, mats, scan.width, scan.height, vector_size=4)
    ab = oracle.AsmBaseline(n, vs, o, mats, scan.width, scan.height, vector_size=4,
                            ranges=ob.ranges)
    per = {"asm": [], "opt": []}
    for _ in range(repeats):
        for name, mod in (("asm", ab), ("opt", ob)):
            vol = np.empty((n, n, n), np.float32)
            vol.fill(0.0)
            t = 0.0
            for i in range(views):
                t0 = time.perf_counter()
                # one runner call with -b 1; ids index the sampled views' ranges
                mod.backproject(vol, np.array([i + 1]), imgs[i:i + 1])
                t += time.perf_counter() - t0
            per[name].append(n ** 3 * views / t / 1e9)
            del vol
    med = {k: statistics.median(v) for k, v in per.items()}
    best = max(med, key=med.get)
    cores = oracle.threads()
    return {"value": med[best], "unit": "GUPS", "cores": cores, "kind": "port",
            "method": CPU_METHODS[best][0],
            "sample": (f"{CPU_METHODS[best][0]} ({CPU_METHODS[best][1]}), {views} of "
                       f"{scan.nproj} projections at N={n}, one call per projection, OpenMP "
                       f"over {cores} threads; the faster of LolaASM and LolaOPT"),
            "methods": {CPU_METHODS[k][0]: {"value": med[k], "per_repeat": per[k]}
                        for k in per},
            "per_repeat": per[best]}


def run_reference(args, rank, world):
    if rank != 0:
        return 0
    scan, vs, o = make_workload(args)
    from oracle import oracle
    oracle.lib()
    warm = max(0, args.warmup)
    # each step: one bounded sample of the workload through each CPU method
    res = cpu_baseline(args, scan, vs, o, repeats=warm + args.steps)
    timed = {m: statistics.median(v["per_repeat"][warm:]) for m, v in res["methods"].items()}
    best = max(timed, key=timed.get)
    value = timed[best]
    views = min(args.cpu_views, scan.nproj)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "GUPS",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": args.n ** 3 * views / value / 1e6,
        "higher_is_better": True, "scaling": "strong" if args.shard == "slabs" else "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded ellipsoid phantom, RabbitCT shapes)",
        "config": workload_config(args, "f32"),
        "cpu_baseline": {"value": value, "unit": "GUPS", "cores": res["cores"], "kind": "port",
                         "method": best,
                         "sample": res["sample"].replace(res["method"], best, 1),
                         "methods": timed},
        "e2e": {"value": value, "unit": "GUPS", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "note": ("the reference's own compiled modules cannot run on this host (its sources "
                 "are not here and binaries built elsewhere do not travel); its two fastest "
                 "CPU methods run as restatements pinned to its build (tests/golden), and "
                 "the faster is reported"),
    }
    print(json.dumps(line), flush=True)
    return 0


def workload_config(args, storage):
    return {"workload": (f"cone-beam backprojection, N={args.n}^3 FP32 volume, {args.nproj} "
                         f"projections of {args.width}x{args.height}"),
            "N": args.n, "projections": args.nproj,
            "detector": f"{args.width}x{args.height}", "storage": storage,
            "batch": args.batch, "voxels_per_thread": args.vpt, "rows_per_block": args.rows,
            "l2": "inputs larger than L2 (volume and projections each exceed 129 MB)",
            "parallelism": ("z-slabs of one volume, one per GPU, no collective"
                            if args.shard == "slabs" else
                            "replicas (one full reconstruction per GPU)")}


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------

def my_slab(args, dist):
    """z-slab of this rank: all of the volume unless sharding by slabs."""
    from rabbitct_gb300.lolacuda import slab
    if args.shard == "slabs" and dist.world > 1:
        # aligned to 16 slices, a multiple of every tile depth (4, 8, 16): the
        # slabs stay on tile boundaries whatever shape each rank's autotuner
        # picks, so ranks agree on them and the union equals one whole volume
        return slab(args.n, dist.rank, dist.world, 16)
    return (0, args.n)


def total_updates(args, scan, dist) -> float:
    """Voxel updates of one step over all ranks."""
    per = float(args.n) ** 3 * scan.nproj
    return per if args.shard == "slabs" else per * dist.world


def tuned_config(args, dist, scan, vs, o, d_images, storage):
    """The configuration a run uses: autotuned on the first 64 projections
    (untimed) or taken from the command line."""
    from rabbitct_gb300.lolacuda import autotune, config
    base = config(storage=storage, batch=args.batch, voxels_per_thread=args.vpt,
                  rows_per_block=args.rows, staging=args.staging)
    if not args.autotune:
        return base, None
    cfg, tried = autotune(args.n, vs, o, scan.width, scan.height, d_images.ptr,
                          scan.matrices[:64], cfg=base, slab=my_slab(args, dist))
    return cfg, tried


def time_device(args, dist, lib_mod, scan, vs, o, d_images, storage, clocks=None):
    from rabbitct_gb300.lolacuda import Plan
    W, H = scan.width, scan.height
    cfg, tried = tuned_config(args, dist, scan, vs, o, d_images, storage)
    # the timed steps run uninstrumented; the per-launch times and the tile
    # counters of the roofline come from one more reconstruction afterwards
    # with statistics on (events around every pass, counters in the kernel)
    cfg.collectStats = 0
    with Plan(args.n, vs, o, W, H, cfg=cfg, slab=my_slab(args, dist)) as p:
        for _ in range(args.warmup):
            p.zero()
            p.backproject_device(d_images.ptr, W * H, scan.matrices)
        p.synchronize()
        p.reset_stats()
        dist.barrier()
        p.synchronize()
        if clocks is not None:
            clocks.start()
        p.timer_start()
        for _ in range(args.steps):
            p.zero()
            p.backproject_device(d_images.ptr, W * H, scan.matrices)
        ms = p.timer_stop()
        clk = clocks.stop() if clocks is not None else None
        p.synchronize()
        dist.barrier()
        launches = p.stats()
    cfg.collectStats = 1
    with Plan(args.n, vs, o, W, H, cfg=cfg, slab=my_slab(args, dist)) as p:
        p.backproject_device(d_images.ptr, W * H, scan.matrices)
        p.synchronize()
        p.reset_stats()
        p.zero()
        p.backproject_device(d_images.ptr, W * H, scan.matrices)
        p.synchronize()
        st = p.stats()
    ms_max = dist.max(ms)
    updates = total_updates(args, scan, dist) * args.steps
    chosen = {"storage": storage, "voxels_per_thread": cfg.voxelsPerThread,
              "rows_per_block": cfg.rowsPerBlock, "batch": cfg.batch, "staging": cfg.staging,
              "autotuned": bool(args.autotune),
              "candidates_timed": 0 if tried is None else sum(1 for t in tried if t[3] > 0)}
    return {"ms": ms_max, "gups": updates / (ms_max * 1e-3) / 1e9, "stats": st, "clocks": clk,
            "cfg": cfg, "chosen": chosen, "launches": launches.passes + launches.packs}


def roofline(args, lib, storage, st, probes, cfg=None) -> dict:
    """The pass kernel's roofline.  Top level, against the measured HBM copy
    bandwidth: algorithmic bytes per launch (the volume read and written once
    per pass plus one read of the stored projections) / the launch's CUDA-event
    time, and the launch's DRAM traffic from the committed ncu capture.  The
    kernel is not bound by HBM: `ceiling` holds the bound it meets, the
    gather and issue rates measured on this GPU by the probe kernels, in
    computed voxel updates per second."""
    rows = cfg.rowsPerBlock if cfg is not None else args.rows
    vpt = cfg.voxelsPerThread if cfg is not None else args.vpt
    batch = cfg.batch if cfg is not None else args.batch
    tile = 32 * rows * vpt
    computed = (st.tilePassesFast + st.tilePassesSlow) * tile
    launches = max(1, st.passes)
    avg_ms = st.passMs / launches
    per_launch = computed / launches
    elem = {"f32": 4, "f16": 2, "bf16": 2, "f32q": 16, "f16q": 8, "bf16q": 8, "tex32": 4,
            "tex16": 2, "f16qx": 8, "f32qx": 16}[storage]
    vol_bytes = 8.0 * args.n ** 3
    proj_bytes = batch * (args.width + 128) * (args.height + 128) * elem
    hbm_gbs = (vol_bytes + proj_bytes) / (avg_ms * 1e-3) / 1e9
    peaks = {}
    mp = ROOT / "MEASURED_PEAKS.json"
    if mp.exists():
        peaks = json.loads(mp.read_text())
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    out = {"bound": "hbm", "achieved": hbm_gbs, "peak": hbm_peak, "unit": "GB/s",
           "frac": hbm_gbs / hbm_peak,
           "peak_source": ("MEASURED_PEAKS.json (hbm_gbs), of measured" if "hbm_gbs" in peaks
                           else "fallback 6800 GB/s"),
           "algorithmic_bytes_per_launch": vol_bytes + proj_bytes,
           "kernel": "passKernel", "avg_launch_ms": avg_ms}
    out["traffic"], out["traffic_source"] = dram_traffic(storage, vpt, rows, batch, args.n)
    achieved = per_launch / (avg_ms * 1e-3) / 1e9  # Gupdate/s while the kernel runs
    computed_pairs = max(1, st.tilePassesFast + st.tilePassesSlow)
    ceil = {"unit": "Gupdate/s", "achieved": achieved, "updates_per_launch": per_launch,
            "skipped_fraction": st.tilePassesSkipped / max(1, st.tilePassesSkipped +
                                                            st.tilePassesFast +
                                                            st.tilePassesSlow),
            "paired_fraction": st.tilePassesPaired / computed_pairs}
    if probes:
        ipu = instr_per_update(storage, ceil["paired_fraction"])
        issue = probes["issue_inst_per_s"] / ipu / 1e9
        # the gather pipes' own rate (an L1-resident image): an upper bound
        # whatever the access pattern; the L2-resident random pattern beside it
        gather = probes["gather_peak"][storage] / 1e9
        gather_l2 = probes["gather"][storage] / 1e9
        bound, peak = ("issue", issue) if issue <= gather else ("gather", gather)
        ceil.update({"bound": bound, "peak": peak, "frac": achieved / peak,
                     "peak_issue": issue, "peak_gather": gather,
                     "gather_l2_random": gather_l2, "frac_of_l2_random": achieved / gather_l2,
                     "instr_per_update": round(ipu, 2),
                     "peak_source": "probe kernels on this GPU (lolaCudaProbeIssueRate; "
                                    "lolaCudaProbeGatherPeak: the layout's fetches inside an "
                                    "L1-resident image; lolaCudaProbeGatherRate: at random "
                                    "positions of an L2-resident projection)"})
    pipes = pipe_utilisation(storage)
    if pipes is not None:
        ceil["ncu_pipes"] = pipes
        wpr = pipes.get("tex_wf_per_request")
        if probes and isinstance(wpr, float) and wpr > 0:
            # the texture pipe's rate for the kernel's own access pattern: the
            # probe's requests take one data-stage wavefront each, the kernel's
            # wpr on average (detector rows straddled)
            ceil["peak_gather_locality"] = ceil["peak_gather"] / wpr
            ceil["frac_of_locality_gather"] = achieved / ceil["peak_gather_locality"]
    out["ceiling"] = ceil
    return out


TRAFFIC_FILE = ROOT / "profiles" / "passKernel_dram_n1024.txt"


def dram_traffic(storage, vpt, rows, batch, n):
    """dram__bytes_read.sum + dram__bytes_write.sum of one pass launch, from
    the committed ncu capture of the same configuration (lines
    `storage vpt rows batch n bytes`), or None when none matches."""
    if not TRAFFIC_FILE.exists():
        return None, None
    for line in TRAFFIC_FILE.read_text().splitlines():
        f = line.split()
        if len(f) != 6 or line.startswith("#"):
            continue
        if (f[0], int(f[1]), int(f[2]), int(f[3]), int(f[4])) == (storage, vpt, rows, batch, n):
            return float(f[5]), f"ncu capture, {TRAFFIC_FILE.relative_to(ROOT)}"
    return None, None


PIPES_FILE = ROOT / "profiles" / "passKernel_pipes.txt"


def pipe_utilisation(storage):
    """Hardware-pipe utilisation of the pass kernel for a storage layout, from
    the committed ncu capture of a small case (lines `storage key=value ...`,
    percentages of peak), or None."""
    if not PIPES_FILE.exists():
        return None
    for line in PIPES_FILE.read_text().splitlines():
        f = line.split()
        if not f or line.startswith("#") or f[0] != storage:
            continue
        out = {}
        for kv in f[1:]:
            k, _, v = kv.partition("=")
            try:
                out[k] = float(v)
            except ValueError:
                out[k] = v
        out["source"] = f"ncu capture, {PIPES_FILE.relative_to(ROOT)}"
        return out
    return None


def time_e2e_slab(args, dist, scan, vs, o, storage) -> dict:
    """N>1 with slabs: the plan API from pinned host buffers, each rank
    uploading every projection and reading its slab back."""
    import ctypes as C

    from rabbitct_gb300._native import load_lolacuda
    from rabbitct_gb300.lolacuda import Plan
    lib = load_lolacuda()
    n, W, H = args.n, scan.width, scan.height
    b, c = my_slab(args, dist)
    nbytes_img = 4 * W * H * scan.nproj
    hi = lib.lolaCudaHostAlloc(nbytes_img)
    hv = lib.lolaCudaHostAlloc(max(4, 4 * n * n * c))
    imgs = np.ctypeslib.as_array((C.c_float * (W * H * scan.nproj)).from_address(hi))
    imgs = imgs.reshape(scan.nproj, H, W)
    imgs[...] = scan.images
    vol = np.ctypeslib.as_array((C.c_float * max(1, n * n * c)).from_address(hv))
    times = []
    for step in range(1 + args.e2e_steps):
        dist.barrier()
        t0 = time.perf_counter()
        with Plan(n, vs, o, W, H, storage=storage, batch=args.batch, voxels_per_thread=args.vpt,
                  rows_per_block=args.rows, staging=args.staging, slab=(b, c)) as p:
            p.backproject_host(imgs, scan.matrices)
            p.download(vol[:n * n * c].reshape(c, n, n))
        dt = time.perf_counter() - t0
        dist.barrier()
        if step > 0:
            times.append(dist.max(dt))
    lib.lolaCudaHostFree(hi)
    lib.lolaCudaHostFree(hv)
    t = statistics.median(times)
    return {"value": total_updates(args, scan, dist) / t / 1e9, "unit": "GUPS", "seconds": t,
            "h2d_bytes_per_step": nbytes_img, "d2h_bytes_per_step": 4 * n * n * c,
            "path": "plan API per z-slab, pinned host"}


def host_link_gbs(lib, h_buf, nbytes) -> dict:
    """Pinned host <-> device copy bandwidth of this machine (GB/s), median of 3
    synchronous copies of `nbytes` each way: the e2e figure moves 6.7 GB in and
    4.3 GB out per step, and the host link is shared with other tenants."""
    d = lib.lolaCudaDeviceAlloc(nbytes)
    if not d:
        return None
    out = {}
    for name, fn, args_ in (("h2d", lib.lolaCudaCopyToDevice, (d, h_buf, nbytes)),
                            ("d2h", lib.lolaCudaCopyToHost, (h_buf, d, nbytes))):
        ts = []
        for _ in range(3):
            t0 = time.perf_counter()
            fn(*args_)
            ts.append(time.perf_counter() - t0)
        out[name] = nbytes / statistics.median(ts) / 1e9
    lib.lolaCudaDeviceFree(d)
    return out


def time_e2e(args, dist, scan, vs, o, storage) -> dict:
    """Module API (prepare / backprojection per projection / finish) with
    pinned host buffers, as rabbitRunner drives a module with -b 1 -a."""
    if args.shard == "slabs" and dist.world > 1:
        return time_e2e_slab(args, dist, scan, vs, o, storage)
    import ctypes as C

    from rabbitct_gb300._native import LolaCudaScanTiming, check, config, load_lolacuda
    from rabbitct_gb300.lolacuda import GlobalData
    lib = load_lolacuda()
    n, W, H = args.n, scan.width, scan.height
    nbytes_vol = 4 * n ** 3
    nbytes_img = 4 * W * H * scan.nproj
    hv = lib.lolaCudaHostAlloc(nbytes_vol)
    hi = lib.lolaCudaHostAlloc(nbytes_img)
    if not hv or not hi:
        raise RuntimeError("pinned host allocation failed")
    vol = np.ctypeslib.as_array((C.c_float * (n ** 3)).from_address(hv)).reshape(n, n, n)
    imgs = np.ctypeslib.as_array((C.c_float * (W * H * scan.nproj)).from_address(hi))
    imgs = imgs.reshape(scan.nproj, H, W)
    imgs[...] = scan.images
    mats = np.ascontiguousarray(scan.matrices)
    # the timer below spans prepare to finish, so calls need not wait for their
    # passes (syncEachCall 0): uploads of the next batch overlap the running
    # pass and no work escapes the timed region (finish synchronizes)
    check(lib.lolaCudaSetConfig(config(storage=storage, batch=args.batch,
                                       voxels_per_thread=args.vpt, rows_per_block=args.rows,
                                       exit_on_error=0, staging=args.staging,
                                       sync_each_call=0)), "config")
    link = host_link_gbs(lib, hv, min(nbytes_vol, 1 << 30))
    times, phases = [], []
    for step in range(1 + args.e2e_steps):
        vol.fill(0.0)  # the runner hands over a zeroed volume (src/rabbitRunner.c:192)
        gd = GlobalData(n, vs, o, W, H, 1, volume=vol, geometry=mats)
        timing = LolaCudaScanTiming()
        dist.barrier()
        # the runner's loop in C (lolaCudaRunScan): prepare, one backprojection
        # call per projection from the pinned images (-b 1, ids 1..496, -a),
        # finish; wall clock from prepare to the volume back in host memory
        check(lib.lolaCudaRunScan(gd.ref, hi, W * H, mats.ctypes.data, scan.nproj, 1,
                                  C.byref(timing)), "run scan")
        dt = timing.totalSeconds
        dist.barrier()
        if step > 0:
            times.append(dist.max(dt))
            phases.append((timing.prepareSeconds, timing.callSeconds, timing.finishSeconds))
    checksum = float(np.float64(vol[n // 2].sum()))
    lib.lolaCudaHostFree(hv)
    lib.lolaCudaHostFree(hi)
    t = statistics.median(times)
    gups = total_updates(args, scan, dist) / t / 1e9
    return {"value": gups, "unit": "GUPS", "seconds": t,
            "h2d_bytes_per_step": nbytes_vol + nbytes_img,
            "d2h_bytes_per_step": nbytes_vol,
            "path": "module API driven by a C loop (lolaCudaRunScan): -b 1 -a calls, pinned "
                    "host, syncEachCall 0; volume upload and download overlapped with the first "
                    "and last pass",
            "checksum_mid_slice": checksum,
            "host_link_gbs": link,
            "phases_ms": {"prepare": 1e3 * statistics.median(p[0] for p in phases),
                          "calls": 1e3 * statistics.median(p[1] for p in phases),
                          "finish": 1e3 * statistics.median(p[2] for p in phases)}}


def run_gpu(args, rank, world, local):
    if world > 1 and "CUDA_VISIBLE_DEVICES" not in os.environ:
        os.environ["CUDA_VISIBLE_DEVICES"] = str(local)
    dist = Dist(rank, world)
    from rabbitct_gb300 import build as b
    b.build_lolacuda()
    b.build_synth()
    from rabbitct_gb300._native import load_lolacuda
    from rabbitct_gb300.lolacuda import DeviceBuffer
    lib = load_lolacuda()
    scan, vs, o = make_workload(args)
    d_images = DeviceBuffer.from_array(scan.images)

    probes = None
    if not args.no_probes:
        used = {args.storage, args.fp32_storage, args.fp32_quad_storage} - {"none"}
        probes = {"issue_inst_per_s": lib.lolaCudaProbeIssueRate(),
                  "gather": {s: lib.lolaCudaProbeGatherRate(STORAGE_IDS[s], scan.width,
                                                            scan.height) for s in used},
                  "gather_peak": {s: lib.lolaCudaProbeGatherPeak(STORAGE_IDS[s])
                                  for s in used},
                  # lane fetches/s of 8-lane texture requests over 1, 2 or 8
                  # detector rows: one data-stage wavefront per row touched
                  "texture_rows": {str(r): lib.lolaCudaProbeTextureRows(r) for r in (1, 2, 8)}}

    clocks = ClockSampler(0)
    head = time_device(args, dist, lib, scan, vs, o, d_images, args.storage, clocks)
    fp32 = fp32q = None
    if not args.no_fp32 and args.fp32_storage != args.storage:
        fp32 = time_device(args, dist, lib, scan, vs, o, d_images, args.fp32_storage)
    if not args.no_fp32 and args.fp32_quad_storage not in ("none", args.storage):
        fp32q = time_device(args, dist, lib, scan, vs, o, d_images, args.fp32_quad_storage)
    d_images.free()
    if args.autotune:
        args.vpt = head["cfg"].voxelsPerThread
        args.rows = head["cfg"].rowsPerBlock
        args.batch = head["cfg"].batch
        args.staging = head["cfg"].staging
    e2e = None if args.no_e2e else time_e2e(args, dist, scan, vs, o, args.storage)

    if rank != 0:
        dist.close()
        return 0
    st = head["stats"]
    line = {
        "metric": METRIC, "value": head["gups"], "unit": "GUPS", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": head["ms"] / args.steps, "higher_is_better": True,
        "scaling": "strong" if args.shard == "slabs" else "weak", "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded ellipsoid phantom, RabbitCT shapes)",
        "config": workload_config(args, args.storage),
        "gpu_launches": int(head["launches"]),
        "clocks": head["clocks"],
        "roofline": roofline(args, lib, args.storage, st, probes, head["cfg"]),
        "tuned": head["chosen"],
    }
    if fp32 is not None:
        line["fp32_path"] = {"value": fp32["gups"], "unit": "GUPS",
                             "storage": args.fp32_storage,
                             "ms_per_step": fp32["ms"] / args.steps,
                             "roofline": roofline(args, lib, args.fp32_storage, fp32["stats"],
                                                  probes, fp32["cfg"]),
                             "tuned": fp32["chosen"]}
        line["fp16_over_fp32"] = head["gups"] / fp32["gups"]
    if fp32q is not None:
        line["fp32_quads"] = {"value": fp32q["gups"], "unit": "GUPS",
                              "storage": args.fp32_quad_storage,
                              "ms_per_step": fp32q["ms"] / args.steps,
                              "roofline": roofline(args, lib, args.fp32_quad_storage,
                                                   fp32q["stats"], probes, fp32q["cfg"]),
                              "tuned": fp32q["chosen"]}
        line["fp16_over_fp32_quads"] = head["gups"] / fp32q["gups"]
    if e2e is not None:
        line["e2e"] = e2e
    if probes:
        line["probes"] = probes
    if world == 1 and not args.no_batch64:
        # the batched uneven workload, measured in the same run (its own metric)
        line["batch64"] = batch64(args)
    if world == 1 and not args.no_cpu:
        # a warm-up repeat, then the timed one, like the reference arm's steps
        cb = cpu_baseline(args, scan, vs, o, repeats=2)
        last = {m: v["per_repeat"][-1] for m, v in cb["methods"].items()}
        best = max(last, key=last.get)
        line["cpu_baseline"] = {"value": last[best], "unit": "GUPS", "cores": cb["cores"],
                                "kind": "port", "method": best,
                                "sample": cb["sample"].replace(cb["method"], best, 1),
                                "methods": last}
    print(json.dumps(line), flush=True)
    dist.close()
    return 0


# ---------------------------------------------------------------------------
# Batched uneven workload: 64 reconstructions
# ---------------------------------------------------------------------------

BATCH_METRIC = ("aggregate GUPS, 64 uneven reconstructions (N in {128,192,256,384}, "
                "180-496 projections, detectors 620x480 / 960x768 / 1248x960)")


def batch_specs(count: int, seed: int = 2024):
    """Seeded job list: N, projection count, detector, arc and SOD per job; each
    job its own ellipsoid phantom (seed)."""
    rng = np.random.default_rng(seed)
    dets = [(620, 480), (960, 768), (1248, 960)]
    out = []
    for j in range(count):
        n = int(rng.choice([128, 192, 256, 384]))
        nproj = int(rng.integers(180, 497))
        w, h = dets[int(rng.integers(0, 3))]
        sod = float(rng.uniform(600.0, 900.0))
        from rabbitct_gb300 import synth
        spec = synth.ScanSpec(nproj=nproj, width=w, height=h, pitch=0.308 * 1248 / w,
                              sod=sod, sid=sod * 1200.0 / 780.0,
                              arc_deg=float(rng.uniform(180.0, 360.0)), seed=1000 + j,
                              noise_seed=5000 + j)
        out.append((n, spec))
    return out


def batch64(args) -> dict:
    """The batched uneven workload (BATCH_METRIC): 64 seeded reconstructions of
    uneven size, detector and projection count, each with its own phantom and
    geometry, FP16-stored (args.storage) with FP32 arithmetic, as one
    graph-captured batch per schedule (parallel graph branches of per-job
    passes, and one persistent pass per wave), against the same 64 run one
    after another through plain FP32 plans.  Aggregate GUPS = sum of N^3 x
    projections over the jobs / wall time of one replay (steps replays, after
    warm-up replays, synchronised on each side)."""
    from rabbitct_gb300 import build as b
    b.build_lolacuda()
    b.build_synth()
    from rabbitct_gb300 import synth
    from rabbitct_gb300.lolacuda import Batch, DeviceBuffer, Plan
    specs = batch_specs(args.jobs)
    t_gen = time.perf_counter()
    jobs, bufs = [], []
    for n, spec in specs:
        scan = synth.make_scan(spec)
        vs = synth.voxel_size(n)
        o = synth.origin_index(n, vs)
        d_img = DeviceBuffer.from_array(scan.images)
        d_vol = DeviceBuffer.from_array(np.zeros((n, n, n), np.float32))
        bufs.append((d_img, d_vol, n, vs, o, spec, scan.matrices))
        jobs.append(dict(n=n, voxel_size=vs, origin_index=o, width=spec.width,
                         height=spec.height, d_images=d_img.ptr, matrices=scan.matrices,
                         d_volume=d_vol.ptr))
        del scan
    t_gen = time.perf_counter() - t_gen
    updates = sum(float(n) ** 3 * spec.nproj for n, spec in specs)
    out = {"metric": BATCH_METRIC, "unit": "GUPS", "steps": args.steps, "warmup": args.warmup,
           "storage": args.storage, "batch": args.batch, "jobs": len(specs),
           "voxel_updates": updates, "generation_s": t_gen, "schedules": {}}
    launches = 0
    for name, mode in (("branches", 0), ("persistent", 1)):
        with Batch(jobs, storage=args.storage, batch=args.batch, batch_mode=mode) as bt:
            info = bt.info()
            for _ in range(args.warmup):
                bt.run()
            bt.synchronize()
            t0 = time.perf_counter()
            for _ in range(args.steps):
                bt.run()
            bt.synchronize()
            t = (time.perf_counter() - t0) / args.steps
        out["schedules"][name] = {"value": updates / t / 1e9, "ms_per_step": t * 1e3,
                                  "launches_per_run": info.launchesPerRun,
                                  "waves": info.waves, "persistent_blocks": info.blocks,
                                  "ring_bytes": info.ringBytes}
        launches += info.launchesPerRun * args.steps
    # the same reconstructions one after another through the plain FP32 path
    plans = [Plan(n, vs, o, spec.width, spec.height, storage="f32", batch=args.batch)
             for (_, _, n, vs, o, spec, _) in bufs]
    for _ in range(max(1, args.warmup - 2)):
        for p, (d_img, _, n, vs, o, spec, mats) in zip(plans, bufs):
            p.backproject_device(d_img.ptr, spec.width * spec.height, mats)
            p.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        for p, (d_img, _, n, vs, o, spec, mats) in zip(plans, bufs):
            p.backproject_device(d_img.ptr, spec.width * spec.height, mats)
            p.synchronize()
    t_seq = (time.perf_counter() - t0) / args.steps
    for p in plans:
        p.close()
    for d_img, d_vol, *_ in bufs:
        d_img.free()
        d_vol.free()
    best = max(out["schedules"], key=lambda k: out["schedules"][k]["value"])
    out["value"] = out["schedules"][best]["value"]
    out["schedule"] = best
    out["gpu_launches"] = launches
    out["sequential_fp32"] = {"value": updates / t_seq / 1e9, "unit": "GUPS",
                              "ms_per_step": t_seq * 1e3,
                              "path": "one plan per job, FP32 storage, synchronised"}
    out["batch_over_sequential"] = {k: v["value"] / out["sequential_fp32"]["value"]
                                    for k, v in out["schedules"].items()}
    return out


def run_batch(args, rank, world, local):
    if rank != 0:
        return 0
    r = batch64(args)
    line = {"metric": BATCH_METRIC, "value": r["value"], "unit": "GUPS", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": r["schedules"][r["schedule"]]["ms_per_step"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (64 seeded phantoms and geometries)",
            "config": {"workload": (f"{r['jobs']} uneven reconstructions, graph-captured "
                                    f"({r['schedule']} schedule)"),
                       "storage": args.storage, "batch": args.batch,
                       "voxel_updates": r["voxel_updates"], "generation_s": r["generation_s"]},
            "gpu_launches": r["gpu_launches"], "schedules": r["schedules"],
            "sequential_fp32": r["sequential_fp32"],
            "batch_over_sequential": r["batch_over_sequential"]}
    print(json.dumps(line), flush=True)
    return 0


def main():
    args = parse_args()
    rank, world, local = dist_info()
    if args.impl == "reference":
        return run_reference(args, rank, world)
    if args.workload == "batch64":
        return run_batch(args, rank, world, local)
    return run_gpu(args, rank, world, local)


if __name__ == "__main__":
    sys.exit(main())
