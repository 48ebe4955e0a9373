"""The driver-trace fixture (tests/golden/make_driver_trace.py): well formed,
and -- where the reference checkout is available (XPBD_REFERENCE_DIR) --
reproduced by running the reference's drivers again."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _load(d=GOLDEN):
    with open(os.path.join(d, "driver_trace.json")) as f:
        return json.load(f), np.load(os.path.join(d, "driver_trace.npz"))


def test_trace_is_well_formed():
    trace, arrays = _load()
    ev = trace["events"]
    assert ev[0]["op"] == "init" and len(ev[0]["sdf"]) == 2
    depth = 0
    for e in ev:
        depth += e["op"] == "callback_begin"
        depth -= e["op"] == "callback_end"
        assert depth in (0, 1)
    assert depth == 0
    reads = [e for e in ev if e["op"] == "call" and "positions_index" in e]
    assert [e["positions_index"] for e in reads] == list(range(len(arrays["positions"])))
    frames = sum(1 for e in ev if e["op"] == "call" and e["path"] == "solver.solve")
    assert frames == int(trace["argv"][trace["argv"].index("--frames") + 1])
    # every substep of every frame reported its convergence records
    subs = int(trace["argv"][trace["argv"].index("--substeps") + 1])
    assert sum(1 for e in ev if e["op"] == "callback_begin") == frames * subs
    assert any(p.endswith("convergence_data.csv") for p in trace["files_written"])


@pytest.mark.skipif(not os.path.isdir(os.environ.get("XPBD_REFERENCE_DIR", "") or "/nonexistent"),
                    reason="needs the reference checkout (XPBD_REFERENCE_DIR)")
def test_trace_regenerates(tmp_path):
    script = os.path.join(GOLDEN, "make_driver_trace.py")
    r = subprocess.run([sys.executable, script, "--out", str(tmp_path)], capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr
    new, new_arr = _load(str(tmp_path))
    old, old_arr = _load()
    assert new["events"] == old["events"]  # float reads carry their kind only, not their value
    np.testing.assert_array_equal(new_arr["positions"], old_arr["positions"])
    np.testing.assert_array_equal(new_arr["indices"], old_arr["indices"])
