"""Where the reference's source tree is, for the recipes that build or read it.

Test infrastructure only.  The reference tree is read only by the build recipe
of oracle/_ref (oracle/ref.mk), the golden-fixture generator and the CPU tests
that compare against the reference's own build.  Nothing on the CUDA path, in
smoke() or in bench.py reads it, and the GPU host has no copy of it.

The location is $RABBITCT_REFERENCE when set, else the tree's default
location in the build container; callers check `present()` and skip where it
is absent.
"""
from __future__ import annotations

import os
from pathlib import Path

_DEFAULT = "/root/reference"


def reference_root() -> Path:
    """The reference's source tree (it need not exist)."""
    return Path(os.environ.get("RABBITCT_REFERENCE") or _DEFAULT)


def present() -> bool:
    """True when the reference's sources can be read here."""
    return (reference_root() / "src" / "LolaBunny.c").exists()
