"""GPU: the reference's drivers, replayed against the GB300 solver.

tests/golden/make_driver_trace.py ran the reference's ``run_neohookean_usd.py``
unmodified (with ``usd_export.py`` and ``convergence_report.py`` behind it)
on the reference's own solver, and logged every access those drivers made to
the solver object: the constructor arguments and SDF list
(``run_neohookean_usd.py:83-106``), the mesh fields the USD renderer keeps
and reads each frame (``usd_export.py:58-60``, ``utils/renderer.py:108-122``),
the convergence callback and what it reads during each substep
(``convergence_report.py:32-96,152-164``), the timing and configuration
attributes, and ``convergence_history`` (``:186-282``).

This test constructs the GB300 solver from the logged arguments and replays
the log in order.  Every read must exist and have the logged kind (for
scalars, the logged value: iteration counts, call counts, flags); every
callback must arrive for the same frame and substep with the same number of
records and the same record keys, and the reads the driver made inside it
are replayed inside it.  The positions the renderer reads after each frame
must match the reference's FP64 run within 1e-4 of the bounding-box
diagonal, and the surface triangles ``indices`` exactly.
"""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
POS_TOL = 1e-4


def _load():
    with open(os.path.join(GOLDEN, "driver_trace.json")) as f:
        trace = json.load(f)
    return trace, np.load(os.path.join(GOLDEN, "driver_trace.npz"))


def _nest(events):
    """Top-level events, each callback_begin carrying its inner events."""
    out, stack = [], []
    for e in events:
        if e["op"] == "callback_begin":
            node = dict(e, inner=[])
            (stack[-1]["inner"] if stack else out).append(node)
            stack.append(node)
        elif e["op"] == "callback_end":
            stack.pop()
        else:
            (stack[-1]["inner"] if stack else out).append(e)
    assert not stack
    return out


def _resolve(root, path):
    obj = root
    for name in path.split(".")[1:]:
        obj = getattr(obj, name)
    return obj


def _check(got, want, where):
    k = want["kind"]
    if k == "float":
        assert isinstance(got, (float, np.floating)) and not isinstance(got, bool), where
    elif k == "int":
        assert isinstance(got, (int, np.integer)) and not isinstance(got, bool), where
        assert int(got) == want["value"], "%s: %r != %r" % (where, got, want["value"])
    elif k == "bool":
        assert bool(got) == want["value"], where
    elif k == "str":
        assert got == want["value"], where
    elif k == "none":
        assert got is None, where
    elif k == "array":
        a = np.asarray(got)
        assert list(a.shape) == want["shape"], "%s: shape %s != %s" % (where, a.shape, want["shape"])
        # the FP64 shim's float arrays are FP32 here, as in the reference on the GPU
        assert a.dtype.kind == np.dtype(want["dtype"]).kind or (a.dtype.kind in "iu" and
                                                                np.dtype(want["dtype"]).kind in "iu"), where
    elif k == "tuple":
        assert len(got) == len(want["items"]), where
        for g, w in zip(got, want["items"]):
            _check(g, w, where)
    elif k == "list":
        assert len(got) == want["len"], "%s: len %d != %d" % (where, len(got), want["len"])
        if "keys" in want:
            assert sorted(got[0].keys()) == want["keys"], where
    elif k == "object":
        assert not isinstance(got, (int, float, str, bool, np.ndarray, list, tuple, dict)), where
    elif k == "callable":
        assert callable(got), where


def _sdfs(records):
    from xpbd_gpu.sdf import CubeSdf, PlaneSdf, SphereSdf
    out = []
    for r in records:
        if r["class"] == "PlaneSdf":
            out.append(PlaneSdf(point=r["point"], dir=r["dir"], fixed=r["fixed"]))
        elif r["class"] == "SphereSdf":
            out.append(SphereSdf(center=r["center"], radius=float(np.ravel(r["radius"])[0]), fixed=r["fixed"]))
        else:
            out.append(CubeSdf(center=r["center"], size=list(2.0 * np.asarray(r["half_size"])), fixed=r["fixed"]))
    return out


def test_reference_driver_trace_replays():
    from xpbd_gpu.mesh import TetMesh
    from xpbd_gpu.neohookean_solver import XPBDNeoHookeanSolver
    trace, arrays = _load()
    events = _nest(trace["events"])
    init = events[0]
    assert init["op"] == "init"
    kw = dict(init["kwargs"])
    kw.pop("rest_pose")
    kw["offset"] = tuple(kw["offset"])
    solver = XPBDNeoHookeanSolver(TetMesh(arrays["points"], arrays["tets"]), _sdfs(init["sdf"]), **kw)
    ref_pos = arrays["positions"]
    diag = float(np.linalg.norm(ref_pos[0].max(0) - ref_pos[0].min(0)))
    pending = []  # recorded callbacks still to be matched, in order
    seen = {"callbacks": 0, "positions": 0}

    def replay(ev, where):
        op = ev["op"]
        if op == "get":
            _check(_resolve(solver, ev["path"]), ev["value"], "%s %s" % (where, ev["path"]))
        elif op == "class_name":
            assert type(solver).__name__ == ev["value"]
        elif op == "set":
            assert ev["path"] == "solver.convergence_callback"
            solver.convergence_callback = on_substep
        elif op == "call":
            fn = _resolve(solver, ev["path"])
            got = fn()
            _check(got, ev["result"], "%s %s()" % (where, ev["path"]))
            if "positions_index" in ev:
                k = ev["positions_index"]
                err = float(np.abs(np.asarray(got, dtype=np.float64) - ref_pos[k]).max())
                assert err <= POS_TOL * diag, "positions read %d: %.3e of the diagonal" % (k, err / diag)
                seen["positions"] += 1
            if ev["path"].endswith("indices.to_numpy"):
                np.testing.assert_array_equal(np.asarray(got), arrays["indices"])
        elif op == "callback_begin":
            pending.append(ev)
        else:
            raise AssertionError("unknown event %r" % op)

    def on_substep(frame, substep, data):
        assert pending, "a convergence callback the drivers did not receive"
        ev = pending.pop(0)
        assert (frame, substep) == (ev["frame"], ev["substep"])
        _check(list(data), ev["records"], "callback f%d s%d" % (frame, substep))
        for inner in ev["inner"]:
            replay(inner, "in callback f%d s%d:" % (frame, substep))
        seen["callbacks"] += 1

    for i, ev in enumerate(events[1:]):
        if ev["op"] == "callback_begin":
            continue  # delivered by the solver during the preceding call
        if ev["op"] == "call" and ev["path"] == "solver.solve":
            # the callbacks this frame delivers, in the order the drivers saw them
            j = i + 2
            while j < len(events) and events[j]["op"] == "callback_begin":
                pending.append(events[j])
                j += 1
            _resolve(solver, ev["path"])()
            assert not pending, "callbacks the GB300 solver did not deliver: %d" % len(pending)
            continue
        replay(ev, "event %d:" % i)
    n_cb = sum(1 for e in trace["events"] if e["op"] == "callback_begin")
    assert seen["callbacks"] == n_cb
    assert seen["positions"] == len(ref_pos)
    solver.check_status()
