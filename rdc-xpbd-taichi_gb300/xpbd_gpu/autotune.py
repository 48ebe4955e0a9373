"""Launch-configuration autotuner for the substep kernels.

The reference leaves launch shapes to Taichi: ``block_size`` is a constructor
argument that no kernel reads (``neohookean_solver.py:27``) and the
mesh-local layout is decided by the patcher (``xpbd_base.py:42``).  Here the
shape is chosen per mesh and per GPU by measurement:

* single body (``XPBDNeoHookeanSolver(..., scatter="auto")``): the Jacobi
  scatter variant -- vector ``red.global.add`` atomics, the deterministic
  vertex->tet CSR gather, or shared-memory patch tiles -- and, for tiles, the
  patch size (the CTA holds ``patch_tets / tets_per_thread`` threads), the
  tets per thread and the pipelined (persistent, bulk-copy) tile form;
* batch (``XPBDBatchedSolver(..., tets_per_thread="auto")``): tets per thread
  (CTA size 256 or 128) of the batched tile kernels.

Every candidate runs ``warmup`` substeps and then ``reps`` timed substeps,
each a replay of the candidate's one-substep CUDA graph, timed with CUDA
events on the solver's stream; the fastest candidate wins.  Single-body
candidates that share a device layout are timed on one solver, switched in
place; the batch is tuned in place and its state restored afterwards.
Choices are cached in a JSON file (``XPBD_AUTOTUNE_CACHE`` or
``~/.cache/xpbd_gb300/autotune.json``) keyed by the GPU, the library build
and the problem's shape, so a later construction of the same problem skips
the measurement.
"""
import json
import os
import threading

from xpbd_gpu import _native

# (scatter, patch_tets, tets_per_thread, patch_pipeline); grouped by device layout
SINGLE_CANDIDATES = (
    ("patch", 256, 2, 0), ("patch", 256, 1, 0), ("patch", 256, 4, 0), ("patch", 256, 2, 1), ("patch", 256, 1, 1),
    ("patch", 128, 2, 0), ("patch", 128, 1, 0),
    ("patch", 64, 2, 0), ("patch", 64, 1, 0),
    ("atomic", 0, 1, 0), ("gather", 0, 1, 0),
)
BATCH_CANDIDATES = (2, 1)

_lock = threading.Lock()


def cache_path():
    p = os.environ.get("XPBD_AUTOTUNE_CACHE")
    if p:
        return p
    return os.path.join(os.path.expanduser("~"), ".cache", "xpbd_gb300", "autotune.json")


def _load_cache(path):
    try:
        with open(path) as f:
            data = json.load(f)
        return data if isinstance(data, dict) else {}
    except (OSError, ValueError):
        return {}


def _store_cache(path, key, value):
    with _lock:
        data = _load_cache(path)
        data[key] = value
        d = os.path.dirname(path)
        if d:
            os.makedirs(d, exist_ok=True)
        tmp = "%s.%d.tmp" % (path, os.getpid())
        with open(tmp, "w") as f:
            json.dump(data, f, indent=1, sort_keys=True)
        os.replace(tmp, path)


def library_stamp():
    """Identifies the library build, so that a rebuilt kernel set is re-tuned."""
    try:
        st = os.stat(_native.LIB_PATH)
        return "%d-%d" % (st.st_size, st.st_mtime_ns)
    except OSError:
        return "unbuilt"


def device_stamp(device_index=None):
    import torch
    i = torch.cuda.current_device() if device_index is None else device_index
    p = torch.cuda.get_device_properties(i)
    return "%s/sm%d%d/%dSM" % (p.name, p.major, p.minor, p.multi_processor_count)


def problem_key(kind, device, library, **shape):
    """Cache key: a stable string of the kind, the GPU, the build and the shape."""
    items = ",".join("%s=%s" % (k, shape[k]) for k in sorted(shape))
    return "%s|%s|%s|%s" % (kind, device, library, items)


def pick(timings):
    """Index of the fastest finite timing (first one on a tie); timings is a list of ms or None."""
    best = None
    for i, t in enumerate(timings):
        if t is None or t != t:
            continue
        if best is None or t < timings[best]:
            best = i
    if best is None:
        raise RuntimeError("autotune: no candidate could be timed")
    return best


def single_candidates(per_tet_materials, max_patch_verts_ok=True):
    """Candidates valid for a body: patch tiles need uniform materials."""
    out = []
    for c in SINGLE_CANDIDATES:
        if c[0] == "patch" and (per_tet_materials or not max_patch_verts_ok):
            continue
        out.append(c)
    return out


def _time_graph_substeps(solver, sub_dt, warmup, reps):
    """ms per substep: `reps` replays of the solver's one-substep graph."""
    import torch
    lib, h, st = solver._lib, solver._handle, solver._stream()
    solver._sync()
    for _ in range(max(1, warmup)):
        _native.check(lib.xpbd_solve(h, float(sub_dt), float(sub_dt), 1, st))
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(reps):
        _native.check(lib.xpbd_solve(h, float(sub_dt), float(sub_dt), 1, st))
    b.record()
    b.synchronize()
    solver.check_status()
    return a.elapsed_time(b) / reps


def tune_single(solver_cls, ctor_args, warmup=2, reps=5, cache=True, log=None):
    """Pick (scatter, patch_tets, tets_per_thread, patch_pipeline) for one body.

    `ctor_args` are the keyword arguments of the solver being built; temporary
    solvers are constructed from them with each candidate layout.  Returns a
    dict with the choice, its ms per substep and the table of all timings."""
    from xpbd_gpu.xpbd_base import load_rest_pose
    mesh = load_rest_pose(ctor_args["rest_pose"])
    per_tet = ctor_args.get("tet_young_modulus") is not None
    nu = ctor_args.get("poisson_ratio", 0.495)
    precise = ctor_args.get("precise_hydro")
    precise = (nu >= 0.49) if precise is None else bool(precise)
    key = problem_key("single", device_stamp(), library_stamp(), tets=mesh.n_tets, verts=mesh.n_verts,
                      block=int(bool(ctor_args.get("block_neohookean_enable", False))), precise=int(precise),
                      per_tet=int(per_tet), cheb=int(bool(ctor_args.get("cheb_enable", True))),
                      monitor=int(bool(ctor_args.get("monitor_convergence", False))))
    path = cache_path() if cache is True else cache
    if path:
        hit = _load_cache(path).get(key)
        if hit:
            return dict(hit, cached=True)
    cands = single_candidates(per_tet)
    groups = {}
    for c in cands:
        layout = ("patch", c[1]) if c[0] == "patch" else ("csr", 0)
        groups.setdefault(layout, []).append(c)
    sub_dt = float(ctor_args.get("dt", 1e-2)) / max(1, int(ctor_args.get("substeps_num", 1)))
    sub_dt = min(sub_dt, float(ctor_args.get("frame_dt", sub_dt)))
    table = []
    for layout, members in groups.items():
        first = members[0]
        kw = dict(ctor_args)
        # candidates are timed at the fixed iteration count (stop mode off), so
        # that every replay does the same work
        kw.update(scatter="gather" if layout[0] == "csr" else "patch", patch_tets=first[1] or 256,
                  tets_per_thread=first[2], patch_pipeline=first[3], use_graph=True, monitor_convergence=False,
                  target_rel_residual=0.0, residual_floor=0.0)
        try:
            s = solver_cls(**kw)
        except (RuntimeError, ValueError) as e:
            for c in members:
                table.append(dict(scatter=c[0], patch_tets=c[1], tets_per_thread=c[2], patch_pipeline=c[3],
                                  ms=None, error=str(e)))
            continue
        for c in members:
            row = dict(scatter=c[0], patch_tets=c[1], tets_per_thread=c[2], patch_pipeline=c[3], ms=None)
            if c[0] == "patch" and s.scatter != "patch":
                row["error"] = "no patch size fits 256 vertices"
            elif c[0] == "patch" and s._patch_tets != c[1]:
                row["error"] = "patches of %d tets exceed 256 vertices" % c[1]
            else:
                s.scatter, s.tets_per_thread, s.patch_pipeline = c[0], c[2], c[3]
                row["ms"] = _time_graph_substeps(s, sub_dt, warmup, reps)
            table.append(row)
            if log:
                log(row)
        del s
    best = table[pick([r["ms"] for r in table])]
    out = dict(scatter=best["scatter"], patch_tets=best["patch_tets"] or 256,
               tets_per_thread=best["tets_per_thread"], patch_pipeline=best["patch_pipeline"],
               ms_per_substep=best["ms"], table=table, key=key)
    if path:
        _store_cache(path, key, out)
    return dict(out, cached=False)


def tune_batch(batch, warmup=2, reps=5, cache=True, log=None):
    """Pick tets per thread for a constructed XPBDBatchedSolver, timed in place
    on one-substep replays; the batch's state (positions, velocities,
    multipliers, Chebyshev rho_hat) is restored afterwards."""
    key = problem_key("batch", device_stamp(), library_stamp(), bodies=batch.n_bodies, tets=batch.n_tets,
                      verts=batch.n_verts, block=int(bool(batch.block_neohookean_enable)),
                      precise=int(bool(batch.precise_hydro)), per_tet=int(batch.per_tet_materials),
                      cheb=int(bool(batch.cheb_enable)))
    path = cache_path() if cache is True else cache
    if path:
        hit = _load_cache(path).get(key)
        if hit:
            return dict(hit, cached=True)
    snap = batch.snapshot()
    sub_dt = min(float(batch.dt) / max(1, int(batch.substeps_num)), float(batch.frame_dt) or 1.0)
    # timed at the fixed iteration count (stop mode off): every replay does the same work
    stop = (batch.target_rel_residual, batch.residual_floor)
    batch.target_rel_residual = batch.residual_floor = 0.0
    table = []
    for tpt in BATCH_CANDIDATES:
        batch.set_tets_per_thread(tpt)
        ms = batch.time_substeps(sub_dt, warmup, reps)
        row = dict(tets_per_thread=tpt, ms=ms)
        table.append(row)
        if log:
            log(row)
    batch.target_rel_residual, batch.residual_floor = stop
    batch.restore(snap)
    best = table[pick([r["ms"] for r in table])]
    out = dict(tets_per_thread=best["tets_per_thread"], ms_per_substep=best["ms"], table=table, key=key)
    if path:
        _store_cache(path, key, out)
    return dict(out, cached=False)
