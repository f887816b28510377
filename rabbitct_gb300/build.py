"""In-tree build of the native libraries (no cmake, no pip install).

Products (git-ignored, rebuilt on every machine):
  rabbitct_gb300/_lib/liblolacuda.so   CUDA kernels (sm_103a) + C host code
  rabbitct_gb300/_lib/librctsynth.so   synthetic scan generator (host C)

The CUDA translation units are compiled in parallel, one per storage layout,
for ``-gencode arch=compute_103a,code=sm_103a`` only.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
LIB = PKG / "_lib"
OBJ = PKG / "_build"
REPO = PKG.parent
INCLUDE = REPO / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_SOURCES = [
    "bp_f32.cu", "bp_f16.cu", "bp_bf16.cu", "bp_f32q.cu", "bp_f16q.cu", "bp_bf16q.cu",
    "bp_tex32.cu", "bp_tex16.cu", "bp_f16qx.cu", "bp_f32qx.cu",
    "lolacuda_dispatch.cu", "lolacuda_probe.cu", "lolacuda_noalloc.cu",
    "lolacuda_geometry.cu", "lolacuda_verify.cu", "lolacuda_batch.cu",
]
C_SOURCES = ["lolacuda_host.c", "lolacuda_file.c", "lolacuda_result.c"]


def _cuda_home() -> Path:
    env = os.environ.get("CUDA_HOME") or os.environ.get("CUDA_PATH")
    if env:
        return Path(env)
    nvcc = shutil.which("nvcc")
    if nvcc:
        return Path(nvcc).resolve().parent.parent
    return Path("/usr/local/cuda")


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"command failed ({proc.returncode}): {' '.join(cmd)}\n"
                           f"{proc.stdout}\n{proc.stderr}")


class _BuildLock:
    """Serialises builds of this tree across processes (one process per GPU
    may start at once, each checking the library), so that no two compile
    into the same outputs."""

    def __enter__(self):
        import fcntl
        OBJ.mkdir(parents=True, exist_ok=True)
        self._f = open(OBJ / ".build.lock", "w")
        fcntl.flock(self._f, fcntl.LOCK_EX)
        return self

    def __exit__(self, *exc):
        import fcntl
        fcntl.flock(self._f, fcntl.LOCK_UN)
        self._f.close()


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def _build_synth(force: bool = False) -> Path:
    LIB.mkdir(exist_ok=True)
    out = LIB / "librctsynth.so"
    src = CSRC / "rct_synth.c"
    if force or _stale(out, [src]):
        tmp = out.with_suffix(".so.tmp")
        _run(["gcc", "-O2", "-fno-fast-math", "-ffp-contract=off", "-std=c99", "-fopenmp",
              "-fPIC", "-shared", "-o", str(tmp), str(src), "-lm"])
        os.replace(tmp, out)
    return out


def _build_lolacuda(force: bool = False, jobs: int | None = None, variant: str = "",
                    variant_flags: tuple[str, ...] = ()) -> Path:
    LIB.mkdir(exist_ok=True)
    obj_dir = OBJ if not variant else PKG / f"_build_{variant}"
    obj_dir.mkdir(exist_ok=True)
    cuda = _cuda_home()
    nvcc = str(cuda / "bin" / "nvcc")
    out = LIB / (f"liblolacuda_{variant}.so" if variant else "liblolacuda.so")
    headers = [CSRC / "bp_kernels.cuh", CSRC / "bp_staged.cuh", CSRC / "bp_batch.cuh",
               CSRC / "lolacuda_internal.h",
               INCLUDE / "lolaCuda.h"]
    common_inc = ["-I" + str(INCLUDE), "-I" + str(CSRC)]

    # extra nvcc flags for tuning builds, e.g. LOLACUDA_NVCC_FLAGS=-DLOLA_MIN_BLOCKS=5
    extra = os.environ.get("LOLACUDA_NVCC_FLAGS", "").split() + list(variant_flags)

    def compile_cu(name: str) -> Path:
        src = CSRC / name
        obj = obj_dir / (name + ".o")
        if force or _stale(obj, [src] + headers):
            _run([nvcc, *ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC",
                  *extra, *common_inc, "-c", str(src), "-o", str(obj)])
        return obj

    # the host code sees the same tuning defines as the kernels
    defines = [f for f in extra if f.startswith("-D")]

    def compile_c(name: str) -> Path:
        src = CSRC / name
        obj = obj_dir / (name + ".o")
        if force or _stale(obj, [src] + headers):
            # no contraction: host arithmetic rounds alike on x86 and Arm
            _run(["gcc", "-O2", "-std=c99", "-fPIC", "-ffp-contract=off", "-Wall", "-Wextra",
                  "-Wno-unused-parameter",
                  *defines, *common_inc, "-I" + str(cuda / "include"), "-c", str(src), "-o",
                  str(obj)])
        return obj

    with ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 4)) as ex:
        futs = [ex.submit(compile_cu, n) for n in CU_SOURCES]
        futs += [ex.submit(compile_c, n) for n in C_SOURCES]
        objs = [f.result() for f in futs]
    if force or _stale(out, objs):
        # linked under another name and renamed: a process that has the old
        # library mapped keeps a whole file
        tmp = out.with_suffix(".so.tmp")
        _run([nvcc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-cudart", "static"])
        os.replace(tmp, out)
    return out


def _build_oracle(force: bool = False) -> Path:
    """Builds the oracle (test infrastructure) and, where the reference sources
    are present, the reference itself into oracle/_ref."""
    oracle = REPO / "oracle"
    if force:
        _run(["make", "-C", str(oracle), "clean"])
    _run(["make", "-C", str(oracle)])
    from oracle import refpath
    if refpath.present():
        _run(["make", "-C", str(REPO), "-f", "oracle/ref.mk",
              f"REF={refpath.reference_root()}"])
    return oracle / "liboracle.so"


def build_synth(force: bool = False) -> Path:
    """The synthetic-scan generator, librctsynth.so."""
    with _BuildLock():
        return _build_synth(force)


def build_lolacuda(force: bool = False, jobs: int | None = None) -> Path:
    """liblolacuda.so: every CUDA translation unit for sm_103a plus the C host
    code, compiled in parallel; only stale objects are rebuilt."""
    with _BuildLock():
        return _build_lolacuda(force, jobs)


# Test-only builds of the library, each with its own objects and file name.
#  stagetimeout: the staged pass's producer issues no tensor copies and every
#  mbarrier wait gives up after 200 000 clock cycles, so each wait runs out
#  and the kernel's error path (error flag, abandoned stages, normal return)
#  can be tested without a fault or a hang (tests/test_gpu_stage_timeout.py).
VARIANTS = {
    "stagetimeout": ("-DLOLA_STAGE_ISSUE_COPIES=0", "-DLOLA_STAGE_WAIT_CYCLES=200000ll"),
}


def build_lolacuda_variant(name: str, force: bool = False, jobs: int | None = None) -> Path:
    """A test-only build of liblolacuda (VARIANTS[name]) as
    _lib/liblolacuda_<name>.so; the product library is not touched."""
    with _BuildLock():
        return _build_lolacuda(force, jobs, variant=name, variant_flags=VARIANTS[name])


def build_oracle(force: bool = False) -> Path:
    """The oracle (test infrastructure) and, where the reference sources are
    present, the reference itself into oracle/_ref."""
    with _BuildLock():
        return _build_oracle(force)


def build_all(force: bool = False) -> None:
    with _BuildLock():
        _build_synth(force)
        _build_lolacuda(force)
        _build_oracle(force)


if __name__ == "__main__":
    import sys
    build_all(force="--force" in sys.argv)
    print("built", *sorted(p.name for p in LIB.glob("*.so")))
