"""Generates the golden fixtures from the reference RabbitCT itself.

Needs the reference source tree ($RABBITCT_REFERENCE, or oracle/refpath.py's default):
it builds the unmodified reference into oracle/_ref (oracle/ref.mk) and runs

  - LolaBunny and LolaOPT through their module API (src/LolaBunny.c,
    src/LolaOPT.c), driven like src/rabbitRunner.c drives them;
  - LolaASM (src/LolaASM.c with its SIMD row kernel) the same way on the
    full-field case, in a process of its own (`--asm-case NAME` writes
    NAME_asm.npz from NAME.npz's inputs);
  - computeLineRanges and computeShadowOfProjection (src/analyseGeometry.c);
  - the reference runner binary end to end on a .rct file (N=128, the
    runner's smallest size), including its -c verification printout, its
    result.rctd file and its -p PGM slice.

Outputs (committed): tests/golden/*.npz and runner_n128.json.  Inputs are
synthetic scans from rabbitct_gb300.synth; small cases store the images
themselves, the full-detector case stores the generator spec and a SHA-256 of
the images so a change of the generator is detected instead of silently
changing the inputs.

    python tests/golden/make_golden.py
    python tests/golden/make_golden.py --asm-case bunny_n32   # one LolaASM fixture
"""
from __future__ import annotations

import ctypes as C
import hashlib
import json
import os
import re
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

from oracle import oracle, refpath  # noqa: E402
from rabbitct_gb300 import rct, synth  # noqa: E402
from rabbitct_gb300.lolacuda import GlobalData, module_functions  # noqa: E402
from rabbitct_gb300.runner import run_module  # noqa: E402

REF = refpath.reference_root()


class OutShadow(C.Structure):
    _fields_ = [("Umin", C.c_int), ("Umax", C.c_int), ("Vmin", C.c_int), ("Vmax", C.c_int)]


def small_spec(nproj, width, height, seed, fov=1.0):
    return synth.ScanSpec(nproj=nproj, width=width, height=height,
                          pitch=0.308 * 1248 / width * fov, seed=seed)


def reference_line_ranges(lib, n, vs, o, mats, w, h, tmp):
    """computeLineRanges via LolaOPT's prepare, which writes the -C cache file."""
    prepare = lib.lolaOptPrepare
    prepare.argtypes = [C.c_void_p]
    gd = GlobalData(n, vs, o, w, h, 1, geometry=mats)
    clip = os.path.join(tmp, f"ranges_{n}_{w}x{h}.rct").encode()
    gd.data.clipFilename = clip
    prepare(C.addressof(gd.data))
    vec = 8 if os.uname().machine == "x86_64" else 4
    return np.fromfile(clip.decode(), np.int16).reshape(mats.shape[0], n * n, 2), vec


def reference_shadow(lib, n, vs, o, mats, w, h):
    fn = lib.computeShadowOfProjection
    fn.argtypes = [C.c_void_p, C.POINTER(OutShadow)]
    gd = GlobalData(n, vs, o, w, h, 1, geometry=mats)
    sh = OutShadow()
    fn(C.addressof(gd.data), C.byref(sh))
    return np.array([sh.Umin, sh.Umax, sh.Vmin, sh.Vmax], np.int32)


def small_case(lib, name, n, spec, tmp):
    scan = synth.make_scan(spec)
    vs = 256.0 / n
    o = synth.origin_index(n, vs)
    bunny = run_module(module_functions(lib, "lolaBunny"), n, vs, o, scan.matrices,
                       scan.images, batch=2).volume
    opt = run_module(module_functions(lib, "lolaOpt"), n, vs, o, scan.matrices, scan.images,
                     batch=1, clip_filename=os.path.join(tmp, f"opt_{name}.rct")).volume
    ranges, vec = reference_line_ranges(lib, n, vs, o, scan.matrices, spec.width, spec.height,
                                        tmp)
    shadow = reference_shadow(lib, n, vs, o, scan.matrices, spec.width, spec.height)
    np.savez_compressed(HERE / f"{name}.npz", n=n, voxel_size=vs, origin_index=o,
                        matrices=scan.matrices, images=scan.images, bunny=bunny, opt=opt,
                        ranges=ranges, ranges_vector_size=vec, shadow=shadow)
    print(f"{name}: N={n} det={spec.width}x{spec.height} views={spec.nproj}")


def runner_case(tmp):
    """The reference runner end to end on a .rct file (N=128, full detector)."""
    spec = synth.ScanSpec(nproj=4, seed=5)
    scan = synth.make_scan(spec)
    n = 128
    path = os.path.join(tmp, "scan.rct")
    geo = os.path.join(tmp, "geo.rct")
    rct.write_rct(path, scan.images, scan.matrices, scan.hus)
    rct.write_geometry(geo, scan.matrices, spec.width, spec.height, scan.hus)
    out = os.path.join(tmp, "bunny.vol")
    # -c needs a uint16 HU reference volume: use the FP64 oracle's HU volume
    vs = synth.voxel_size(n)
    o = synth.origin_index(n, vs)
    v64 = oracle.bunny_f64(n, vs, o, scan.matrices, scan.images)
    from rabbitct_gb300 import metrics
    hu_ref = metrics.to_hu(v64.astype(np.float32), scan.hus).astype(np.uint16)
    refvol = os.path.join(tmp, "ref.vol")
    hu_ref.tofile(refvol)
    env = dict(os.environ, OMP_NUM_THREADS="4")
    pgm = os.path.join(tmp, "slice.pgm")
    proc = subprocess.run([str(oracle.REF_RUNNER), "-m", "LolaBunny", "-s", str(n), "-b", "2",
                           "-i", path, "-o", out, "-c", refvol, "-p", pgm], capture_output=True,
                          text=True, cwd=tmp, env=env, check=True)
    vol = np.fromfile(out, np.float32).reshape(n, n, n)
    # the runner's optional outputs: -p slice (written from the FP32 volume)
    # and result.rctd (written by -c into the working directory); the raw
    # middle slice they come from needs a second run without -c (LolaBunny is
    # deterministic), because -c converts the volume to HU before -o
    raw_out = os.path.join(tmp, "bunny_raw.vol")
    subprocess.run([str(oracle.REF_RUNNER), "-m", "LolaBunny", "-s", str(n), "-b", "2",
                    "-i", path, "-o", raw_out], capture_output=True, text=True, cwd=tmp,
                   env=env, check=True)
    raw = np.fromfile(raw_out, np.float32).reshape(n, n, n)
    rctd = np.fromfile(os.path.join(tmp, "result.rctd"), np.uint8)
    np.savez_compressed(HERE / "runner_n128_outputs.npz",
                        raw_mid_slice=raw[n // 2 - 1].copy(),
                        pgm=np.fromfile(pgm, np.uint8), rctd=rctd,
                        hu_mid_slice=vol[n // 2 - 1].copy())
    def grab(pat):
        m = re.search(pat, proc.stdout)
        return float(m.group(1)) if m else None
    printed = {"rmse_hu": grab(r"Root Mean Squared Error: ([-\d.eE+]+) HU"),
               "mse_hu2": grab(r"Mean Squared Error: ([-\d.eE+]+) HU\^2"),
               "max_abs_hu": grab(r"Max. Absolute Error: ([-\d.eE+]+) HU"),
               "psnr_db": grab(r"PSNR: ([-\d.eE+]+) db")}
    stride = 97
    info = {
        "spec": spec.__dict__, "n": n, "hus": list(scan.hus),
        "images_sha256": hashlib.sha256(scan.images.tobytes()).hexdigest(),
        "matrices": scan.matrices.tolist(),
        "volume_sum": float(vol.astype(np.float64).sum()),
        "volume_sumsq": float((vol.astype(np.float64) ** 2).sum()),
        "sample_stride": stride,
        "volume_sample": vol.reshape(-1)[::stride].astype(float).tolist(),
        "runner_quality": printed,
        "hu_reference_sha256": hashlib.sha256(hu_ref.tobytes()).hexdigest(),
    }
    (HERE / "runner_n128.json").write_text(json.dumps(info))
    print("runner_n128:", printed)


def asm_case(name):
    """The reference's LolaASM on a small case's inputs -> {name}_asm.npz.  One
    process per case: lolaAsmBackprojection keeps its padded buffers in static
    state sized by the first call (src/LolaASM.c:92-105), never reset."""
    lib = oracle.ref_lib()
    g = np.load(HERE / f"{name}.npz")
    n, vs, o = int(g["n"]), float(g["voxel_size"]), float(g["origin_index"])
    with tempfile.TemporaryDirectory() as tmp:
        vol = run_module(module_functions(lib, "lolaAsm"), n, vs, o, g["matrices"], g["images"],
                         batch=1, clip_filename=os.path.join(tmp, f"asm_{name}.rct")).volume
    vec = 8 if os.uname().machine == "x86_64" else 4
    np.savez_compressed(HERE / f"{name}_asm.npz", asm=vol, asm_vector_size=vec)
    print(f"{name}_asm: LolaASM, vector size {vec}")


def main():
    if len(sys.argv) == 3 and sys.argv[1] == "--asm-case":
        asm_case(sys.argv[2])
        return
    if not (REF / "src" / "LolaBunny.c").exists():
        sys.exit(f"reference sources not found under {REF}")
    subprocess.run(["make", "-C", str(ROOT), "-f", "oracle/ref.mk", f"REF={REF}"], check=True,
                   capture_output=True)
    oracle.build()
    lib = oracle.ref_lib()
    with tempfile.TemporaryDirectory() as tmp:
        small_case(lib, "bunny_n32", 32, small_spec(6, 64, 48, seed=101), tmp)
        small_case(lib, "bunny_n40_halffov", 40, small_spec(6, 80, 64, seed=102, fov=0.5), tmp)
        runner_case(tmp)
    # bunny_n40_halffov only for LolaOPT: its volume's shadow lies inside the
    # detector, so LolaASM's pads (abs(Umax) - W, src/LolaASM.c:45-48) come out
    # negative and its run ends in a segmentation fault
    subprocess.run([sys.executable, __file__, "--asm-case", "bunny_n32"], check=True)


if __name__ == "__main__":
    main()
