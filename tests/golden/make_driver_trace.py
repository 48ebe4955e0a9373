"""Record how the reference's own drivers use the solver -- TEST INFRASTRUCTURE.

Usage (only where the reference checkout is present):

    XPBD_REFERENCE_DIR=<reference checkout> python tests/golden/make_driver_trace.py

The reference is driven by ``run_neohookean_usd.py`` (construction
``:88-106``, the frame loop ``:146-161``, the reports ``:184-190``), which
calls ``usd_export.py`` (``add_solver_mesh`` / ``add_sdfs``, ``:58-92``) and
``convergence_report.py`` (``setup_convergence_callback`` ``:152-164``,
``save_substep_convergence`` ``:32-96``, ``print_convergence_analysis``
``:215-282``).  This script runs that driver file unmodified, with:

* the reference's own ``xpbd_gpu`` package under ``taichi_shim`` (FP64, the
  shim that also makes the golden vectors);
* test-only stand-ins for ``pxr`` and ``matplotlib`` (absent here), which
  accept every call and write nothing;
* the solver class wrapped so that every attribute read, attribute write,
  method call and callback invocation the drivers make is logged, with a
  summary of each value (type, shape, dtype, keys) and the positions the
  USD renderer reads after every frame.

The mesh is a small Kuhn grid registered with the shim's patcher under a
``.node`` name, so the driver's ``--model`` argument takes it unchanged.
Output: ``driver_trace.json`` (the event log and the driver's arguments) and
``driver_trace.npz`` (the mesh and the recorded positions) next to this
script.  ``tests/test_gpu_driver_trace.py`` replays the log against the GB300
solver.
"""
import argparse
import contextlib
import io
import json
import os
import runpy
import sys
import tempfile
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

MODEL = "kuhn_driver.node"
DRIVER_ARGS = ["--model", MODEL, "--frames", "3", "--dt", str(1.0 / 60), "--substeps", "2", "--iterations", "12",
               "--young", "1e5", "--poisson", "0.45", "--cheb-warmup", "4", "--monitor-convergence",
               "--plot-frames", "--plot-frame-ids", "1", "--export-csv", "--streaming"]


def summary(v):
    """A JSON description of a value the drivers read."""
    if isinstance(v, (bool, np.bool_)):
        return {"kind": "bool", "value": bool(v)}
    if isinstance(v, (int, np.integer)):
        return {"kind": "int", "value": int(v)}
    if isinstance(v, (float, np.floating)):
        return {"kind": "float"}
    if isinstance(v, str):
        return {"kind": "str", "value": v}
    if v is None:
        return {"kind": "none"}
    if isinstance(v, np.ndarray):
        return {"kind": "array", "shape": list(v.shape), "dtype": str(v.dtype)}
    if isinstance(v, tuple):
        return {"kind": "tuple", "items": [summary(x) for x in v]}
    if isinstance(v, list):
        out = {"kind": "list", "len": len(v)}
        if v and isinstance(v[0], dict):
            out["keys"] = sorted(v[0].keys())
        return out
    if isinstance(v, dict):
        return {"kind": "dict", "keys": sorted(v.keys())}
    if callable(v):
        return {"kind": "callable"}
    return {"kind": "object"}


class Log:
    def __init__(self):
        self.events = []
        self.positions = []
        self.indices = None


class Recorded:
    """Wraps an object the drivers reach through the solver and logs every access."""

    def __init__(self, target, path, log):
        object.__setattr__(self, "_t", target)
        object.__setattr__(self, "_p", path)
        object.__setattr__(self, "_log", log)

    @property
    def __class__(self):  # noqa: D401 - convergence_report.py:59 reads solver.__class__.__name__
        t = object.__getattribute__(self, "_t")
        log = object.__getattribute__(self, "_log")
        log.events.append({"op": "class_name", "path": object.__getattribute__(self, "_p"),
                           "value": type(t).__name__})
        return type(t)

    def __getattr__(self, name):
        t, p, log = self._t, self._p, self._log
        v = getattr(t, name)
        path = p + "." + name
        if isinstance(v, types.MethodType) or (callable(v) and not hasattr(v, "__dict__")):
            return RecordedCall(v, path, log)
        s = summary(v)
        log.events.append({"op": "get", "path": path, "value": s})
        if s["kind"] == "object":
            return Recorded(v, path, log)
        return v

    def __setattr__(self, name, value):
        t, p, log = self._t, self._p, self._log
        path = p + "." + name
        log.events.append({"op": "set", "path": path, "value": summary(value)})
        if name == "convergence_callback" and callable(value):
            def wrapped(frame, substep, data, _f=value):
                # what the callback reads from the solver is logged between begin and end
                log.events.append({"op": "callback_begin", "path": path, "frame": int(frame),
                                   "substep": int(substep), "records": summary(list(data))})
                r = _f(frame, substep, data)
                log.events.append({"op": "callback_end", "path": path})
                return r
            value = wrapped
        setattr(t, name, value)

    def __getitem__(self, k):
        return self._t[k]


class RecordedCall:
    def __init__(self, fn, path, log):
        self.fn, self.path, self.log = fn, path, log

    def __call__(self, *args, **kw):
        # logged before the call runs, so that callbacks it triggers follow it
        ev = {"op": "call", "path": self.path, "args": [summary(a) for a in args]}
        self.log.events.append(ev)
        r = self.fn(*args, **kw)
        ev["result"] = summary(r)
        if self.path.endswith("mesh.verts.x.to_numpy"):
            ev["positions_index"] = len(self.log.positions)
            self.log.positions.append(np.asarray(r, dtype=np.float64).copy())
        if self.path.endswith("indices.to_numpy"):
            self.log.indices = np.asarray(r).copy()
        return r


class _Anything:
    """Test-only stand-in for pxr / matplotlib objects: every attribute and call
    yields another stand-in."""

    def __init__(self, *a, **k):
        pass

    def __getattr__(self, name):
        return _Anything()

    def __call__(self, *a, **k):
        return _Anything()

    def __iter__(self):
        return iter(())


def install_stubs():
    pxr = types.ModuleType("pxr")
    pxr.Usd = _Anything()
    pxr.UsdGeom = _Anything()
    pxr.Sdf = _Anything()
    pxr.Gf = _Anything()
    pxr.Vt = _Anything()
    sys.modules["pxr"] = pxr
    mpl = types.ModuleType("matplotlib")
    plt = types.ModuleType("matplotlib.pyplot")
    plt.subplots = lambda *a, **k: (_Anything(), (_Anything(), _Anything()))
    for name in ("tight_layout", "savefig", "close", "figure", "plot", "show", "legend"):
        setattr(plt, name, lambda *a, **k: None)
    ticker = types.ModuleType("matplotlib.ticker")
    ticker.ScalarFormatter = _Anything
    ticker.MaxNLocator = _Anything
    mpl.pyplot, mpl.ticker = plt, ticker
    mpl.use = lambda *a, **k: None
    sys.modules["matplotlib"] = mpl
    sys.modules["matplotlib.pyplot"] = plt
    sys.modules["matplotlib.ticker"] = ticker


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("XPBD_REFERENCE_DIR"),
                    help="the reference checkout (or set XPBD_REFERENCE_DIR)")
    ap.add_argument("--out", default=HERE)
    args = ap.parse_args()
    if not args.ref:
        ap.error("give --ref or set XPBD_REFERENCE_DIR")
    ref = os.path.abspath(args.ref)
    from make_golden import kuhn_grid
    import taichi_shim
    # above the sphere (centre (0, -1, 0), radius 0.3) once the driver adds offset (0, 1, 0): in contact
    # within the first frames
    pts, tets = kuhn_grid(3, 2, 3, 0.1, (-0.15, -1.695, -0.15), 0.1, 21)
    taichi_shim.install("f64", meshes={MODEL: (pts, tets)})
    install_stubs()
    sys.path.insert(0, ref)
    import xpbd_gpu.neohookean_solver as nh  # the reference's module
    log = Log()
    cls = nh.XPBDNeoHookeanSolver

    def sdf_record(s):
        out = {"class": type(s).__name__, "fixed": bool(s.fixed)}
        for name in ("point", "dir", "center", "radius", "half_size"):
            if hasattr(s, name):
                out[name] = np.asarray(getattr(s, name)[None], dtype=np.float64).tolist()
        return out

    def constructed(*a, **kw):
        log.events.append({"op": "init", "args": [summary(x) for x in a],
                           "kwargs": {k: (v if isinstance(v, (int, float, str, bool, tuple)) or v is None
                                          else summary(v)) for k, v in kw.items() if k != "sdf"},
                           "sdf": [sdf_record(s) for s in kw.get("sdf", [])]})
        return Recorded(cls(*a, **kw), "solver", log)

    nh.XPBDNeoHookeanSolver = constructed
    out_stdout = io.StringIO()
    with tempfile.TemporaryDirectory() as tmp:
        cwd = os.getcwd()
        os.chdir(tmp)
        argv = sys.argv
        sys.argv = [os.path.join(ref, "run_neohookean_usd.py")] + DRIVER_ARGS
        try:
            with contextlib.redirect_stdout(out_stdout):
                runpy.run_path(os.path.join(ref, "run_neohookean_usd.py"), run_name="__main__")
            written = sorted(os.path.relpath(os.path.join(r, f), tmp)
                             for r, _, fs in os.walk(tmp) for f in fs)
        finally:
            sys.argv = argv
            os.chdir(cwd)
    lines = out_stdout.getvalue().splitlines()
    trace = {"driver": "run_neohookean_usd.py", "argv": DRIVER_ARGS, "events": log.events,
             "files_written": written,
             "stdout_markers": [ln for ln in lines if ln.startswith(("Solver per frame", "Total constraint",
                                                                      "NEO-HOOKEAN", "Method:"))]}
    with open(os.path.join(args.out, "driver_trace.json"), "w") as f:
        json.dump(trace, f, indent=1)
    np.savez_compressed(os.path.join(args.out, "driver_trace.npz"), points=pts, tets=tets,
                        positions=np.array(log.positions), indices=log.indices)
    print("%d events, %d position reads, %d files written by the drivers" % (
        len(log.events), len(log.positions), len(written)))


if __name__ == "__main__":
    main()
