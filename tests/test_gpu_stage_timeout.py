"""The staged pass's bounded waits, made to run out on purpose without a fault
or a hang.

A test-only build of the library (rabbitct_gb300/build.py VARIANTS
"stagetimeout") compiles the staged pass with LOLA_STAGE_ISSUE_COPIES=0 and
LOLA_STAGE_WAIT_CYCLES=200000: its producer issues no tensor copies (none is
ever in flight), so every stage's full barrier stays incomplete and each
consumer warp's wait gives up after about 0.1 ms.  The kernel must then record
its error code, abandon the staged work and return normally; the host must
report "stage wait timed out" from the next synchronisation, and the CUDA
context must stay usable: a load-path plan in the same process afterwards
matches the FP64 oracle.

It runs in a child process, so the test build is never loaded next to the
product library of the other tests.
"""
from __future__ import annotations

import json
import subprocess
import sys
import textwrap
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parent.parent

CHILD = textwrap.dedent(r"""
    import json, sys
    sys.path.insert(0, sys.argv[1])
    from pathlib import Path
    from rabbitct_gb300 import build as b, _native, metrics, synth
    lib_file = b.build_lolacuda_variant("stagetimeout")
    _native.lib_path = lambda: Path(lib_file)   # this process loads the test build only
    from rabbitct_gb300._native import LolaCudaError
    from rabbitct_gb300.lolacuda import Plan
    from oracle import oracle
    scan = synth.make_scan(synth.ScanSpec(nproj=10, seed=41))
    n, vs = 96, 0.5
    o = synth.origin_index(n, vs)
    out = {}
    plan = Plan(n, vs, o, scan.width, scan.height, storage="f32", batch=5, staging=1,
                collect_stats=1, voxels_per_thread=8, rows_per_block=8)
    try:
        plan.backproject_host(scan.images, scan.matrices)
        plan.synchronize()
        out["error"] = None
    except LolaCudaError as e:
        out["error"] = str(e)
    st = plan.stats()
    out["staged_passes"] = int(st.stagedPasses)
    out["tiles_staged"] = int(st.tilePassesStaged)
    plan.close()
    ref = oracle.bunny_f64(n, vs, o, scan.matrices, scan.images)
    with Plan(n, vs, o, scan.width, scan.height, storage="f32", batch=5, staging=0) as p:
        p.backproject_host(scan.images, scan.matrices)
        vol = p.download()
    out["after_rel_rmse"] = metrics.errors(vol, ref)["rel_rmse"]
    print("RESULT " + json.dumps(out))
""")


def test_stage_wait_timeout_is_reported_and_context_survives():
    proc = subprocess.run([sys.executable, "-c", CHILD, str(ROOT)], capture_output=True,
                          text=True, timeout=600, cwd=ROOT)
    assert proc.returncode == 0, proc.stdout[-2000:] + proc.stderr[-4000:]
    line = [ln for ln in proc.stdout.splitlines() if ln.startswith("RESULT ")][-1]
    res = json.loads(line[len("RESULT "):])
    assert res["staged_passes"] >= 1 and res["tiles_staged"] > 0, res
    assert res["error"] is not None and "stage wait timed out" in res["error"], res
    assert res["after_rel_rmse"] <= 1e-5, res
