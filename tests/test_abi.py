"""The C-ABI library: it loads without a GPU, exports every function that
include/lolaCuda.h declares, and its structs have the layout the ctypes
bindings (and, for RabbitCtGlobalData, the reference's rabbitCt.h) use."""
from __future__ import annotations

import ctypes as C
import re
import subprocess
from pathlib import Path

import pytest

from oracle import refpath

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "lolaCuda.h"
REF_HEADER = refpath.reference_root() / "src" / "rabbitCt.h"


@pytest.fixture(scope="module")
def lib():
    from rabbitct_gb300 import build as b
    b.build_lolacuda()
    from rabbitct_gb300._native import load_lolacuda
    return load_lolacuda()


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^[A-Za-z_][\w \*]*?\b(lolaCuda\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_header_declares_module_api():
    names = declared_functions()
    for n in ("lolaCudaPrepare", "lolaCudaBackprojection", "lolaCudaFinish"):
        assert n in names
    assert len(names) >= 25


def test_library_exports_every_declared_function(lib):
    out = subprocess.run(["nm", "-D", "--defined-only", str(ROOT / "rabbitct_gb300" / "_lib" /
                                                            "liblolacuda.so")],
                         capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r" T (\w+)$", out, flags=re.M))
    missing = [n for n in declared_functions() if n not in exported]
    assert not missing, missing
    for n in declared_functions():
        getattr(lib, n)  # resolvable through ctypes too


LAYOUT_PROGRAM = r"""
#include <stdio.h>
#include <stddef.h>
%s
#include "lolaCuda.h"
#define P(T) printf(#T " %%zu\n", sizeof(T))
#define O(T, f) printf(#T "." #f " %%zu\n", offsetof(T, f))
int main(void) {
  P(Projection); O(Projection, matrix); O(Projection, image);
  P(RabbitCtGlobalData); O(RabbitCtGlobalData, volumeData);
  O(RabbitCtGlobalData, numberOfProjections); O(RabbitCtGlobalData, globalGeometry);
  O(RabbitCtGlobalData, projectionBuffer); O(RabbitCtGlobalData, clipFilename);
  P(LolaCudaConfig); P(LolaCudaGeometry); P(LolaCudaStats);
  O(LolaCudaStats, passMs); O(LolaCudaStats, tilePassesSkipped);
  return 0;
}
"""


def c_layout(tmp_path, pre=""):
    src = tmp_path / "layout.c"
    src.write_text(LAYOUT_PROGRAM % pre)
    exe = tmp_path / "layout"
    inc = ["-I" + str(ROOT / "include")]
    if pre:
        inc.append("-I" + str(REF_HEADER.parent))
    subprocess.run(["gcc", "-std=c99", *inc, "-o", str(exe), str(src)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout
    return dict(line.rsplit(" ", 1) for line in out.strip().splitlines())


def test_struct_layouts_match_ctypes(tmp_path):
    from rabbitct_gb300 import _native as N
    lay = {k: int(v) for k, v in c_layout(tmp_path).items()}
    assert lay["Projection"] == C.sizeof(N.Projection)
    assert lay["Projection.image"] == N.Projection.image.offset
    assert lay["RabbitCtGlobalData"] == C.sizeof(N.RabbitCtGlobalData)
    for f in ("volumeData", "numberOfProjections", "globalGeometry", "projectionBuffer",
              "clipFilename"):
        assert lay[f"RabbitCtGlobalData.{f}"] == getattr(N.RabbitCtGlobalData, f).offset
    assert lay["LolaCudaConfig"] == C.sizeof(N.LolaCudaConfig)
    assert lay["LolaCudaGeometry"] == C.sizeof(N.LolaCudaGeometry)
    assert lay["LolaCudaStats"] == C.sizeof(N.LolaCudaStats)
    assert lay["LolaCudaStats.tilePassesSkipped"] == N.LolaCudaStats.tilePassesSkipped.offset


@pytest.mark.skipif(not REF_HEADER.exists(), reason="reference headers not present")
def test_coexists_with_reference_header(tmp_path):
    """A registry translation unit can include the reference's rabbitCt.h and
    lolaCuda.h together; the data contract is the reference's own."""
    ours = c_layout(tmp_path)
    both = c_layout(tmp_path, pre='#include "rabbitCt.h"')
    assert ours == both
