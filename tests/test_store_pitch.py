"""The stored projections' row pitch (lolaStorePitch, lolacuda_internal.h),
compiled on the host: the padded width rounded up to 32 pixels, plus 64 bytes
for the layouts read by index so that consecutive rows start 64 bytes apart
modulo 128; row starts stay 64-byte aligned (texture fetches from pitched
memory) and strides multiples of 16 bytes (tensor copies)."""
from __future__ import annotations

import subprocess
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
ELEM = {0: 4, 1: 2, 2: 2, 3: 16, 4: 8, 5: 8, 6: 4, 7: 2, 8: 8, 9: 16}  # LOLA_STORE_* bytes

PROGRAM = r"""
#include <stdio.h>
#include "lolacuda_internal.h"
int main(void) {
  static const int widths[] = {1, 31, 64, 96, 128, 150, 620, 960, 1248, 2048, 3001};
  static const int elem[] = {4, 2, 2, 16, 8, 8, 4, 2, 8, 16};
  for (unsigned w = 0; w < sizeof(widths) / sizeof(widths[0]); w++)
    for (int s = 0; s < 10; s++)
      printf("%d %d %d\n", widths[w], s, lolaStorePitch(widths[w], s, elem[s]));
  return 0;
}
"""


def test_store_pitch(tmp_path):
    src = tmp_path / "pitch.c"
    src.write_text(PROGRAM)
    exe = tmp_path / "pitch"
    inc = ["-I" + str(ROOT / "include"), "-I" + str(ROOT / "rabbitct_gb300" / "csrc"),
           "-I/usr/local/cuda/include"]
    subprocess.run(["gcc", "-std=c99", *inc, "-o", str(exe), str(src)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout
    rows = [tuple(map(int, ln.split())) for ln in out.splitlines()]
    assert len(rows) == 11 * 10
    for width, storage, pitch in rows:
        elem = ELEM[storage]
        base = (width + 128 + 31) // 32 * 32
        if storage in (6, 7):  # texture layouts over 2D pitched memory: no skew
            assert pitch == base
            continue
        assert pitch * elem == base * elem + 64, (width, storage, pitch)
        assert pitch >= width + 128
        assert (pitch * elem) % 64 == 0 and (pitch * elem) % 16 == 0
        if (base * elem) % 128 == 0:
            assert (pitch * elem) % 128 == 64
