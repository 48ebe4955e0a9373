"""Benchmark of the RDC-XPBD substep on GB300.

Workload (default ``c2``): a 64x64x64-cell Kuhn-split cube (1,572,864 tets,
274,625 vertices, jitter +-0.05 cell), E = 1e6 Pa, nu = 0.49, rho = 1000
kg/m^3, dt = 1/60 s, 10 substeps x 50 Jacobi iterations with residual-driven
Chebyshev (block 2x2 Neo-Hookean), dropped onto an SDF list of the plane
y = 0, 8 random spheres and an axis-aligned box.  One step = one frame =
786.4 M tet-iterations.  Inputs are synthetic (seeded numpy PCG64).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

The gb300 arm prints one JSON line with ``value`` in tet-iterations/s
(inputs resident on the device, CUDA-graph replay, L2 flushed between steps),
``e2e`` through the public API with host buffers (from_numpy -> solve ->
to_numpy per step), ``roofline`` of the projection kernel from CUDA events,
``cpu_baseline`` from the CPU oracle on a bounded sample, and ``clocks``.
The reference arm times the CPU restatement of the reference's algorithm.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "rdc-xpbd-taichi_gb300"))
sys.path.insert(0, ROOT)

METRIC = "tet-iterations/s & frames/s: batched+adjoint vs plain GPU at equal residual"
UNIT = "tet-iterations/s"
L2_FLUSH_BYTES = 512 << 20


# ---------------------------------------------------------------------------
# workloads
# ---------------------------------------------------------------------------

def workload(name, seed=0):
    """Mesh, SDF specs and solver kwargs of a named workload."""
    from xpbd_gpu.mesh import kuhn_grid
    if name == "c2":
        n = 64
        mesh = kuhn_grid(n, n, n, 1.0 / n, origin=(0.0, 1.25, 0.0), jitter=0.05, seed=seed)
        rng = np.random.default_rng(seed + 1)
        sdfs = [("plane", dict(point=[0.0, 0.0, 0.0], dir=[0.0, 1.0, 0.0], fixed=True))]
        for _ in range(8):
            sdfs.append(("sphere", dict(center=rng.uniform(0.0, 1.0, 3).tolist(),
                                        radius=float(rng.uniform(0.05, 0.2)), fixed=True)))
        sdfs.append(("cube", dict(center=[0.5, 0.15, 0.5], size=[0.4, 0.3, 0.4], fixed=True)))
        kw = dict(young_modulus=1e6, poisson_ratio=0.49, frame_dt=1.0 / 60, dt=1.0 / 60, substeps_num=10,
                  constraints_iter=50, cheb_enable=True, cheb_warmup=5, cheb_gamma=0.6666,
                  block_neohookean_enable=True, density=1000.0)
        desc = "64^3 Kuhn cube (1,572,864 tets, 274,625 verts), E=1e6, nu=0.49, 10 substeps x 50 it, plane+8 spheres+box"
        return mesh, sdfs, kw, desc
    if name == "c1":
        mesh = kuhn_grid(10, 10, 10, 0.1, origin=(0.0, 1.1, 0.0), jitter=0.1, seed=seed)
        sdfs = [("plane", dict(point=[0.0, 0.0, 0.0], dir=[0.0, 1.0, 0.0], fixed=True)),
                ("sphere", dict(center=[0.5, 0.3, 0.5], radius=0.3, fixed=True))]
        kw = dict(young_modulus=1e5, poisson_ratio=0.45, frame_dt=1.0 / 60, dt=1.0 / 60, substeps_num=5,
                  constraints_iter=20, cheb_enable=True, cheb_warmup=5, cheb_gamma=0.6666,
                  block_neohookean_enable=True, density=1000.0)
        desc = "10^3 Kuhn cube (6,000 tets, 1,331 verts), E=1e5, nu=0.45, 5 substeps x 20 it, plane+sphere"
        return mesh, sdfs, kw, desc
    raise ValueError("unknown workload %r" % name)


def product_sdfs(specs):
    from xpbd_gpu.sdf import CubeSdf, PlaneSdf, SphereSdf
    out = []
    for k, p in specs:
        if k == "plane":
            out.append(PlaneSdf(point=p["point"], dir=p["dir"], fixed=p["fixed"]))
        elif k == "sphere":
            out.append(SphereSdf(center=p["center"], radius=p["radius"], fixed=p["fixed"]))
        else:
            out.append(CubeSdf(center=p["center"], size=p["size"], fixed=p["fixed"]))
    return out


def tet_iterations_per_frame(mesh, kw):
    from xpbd_gpu.neohookean_solver import frame_chunks
    return mesh.n_tets * len(frame_chunks(kw["frame_dt"], kw["dt"])) * kw["substeps_num"] * kw["constraints_iter"]


# ---------------------------------------------------------------------------
# CPU baseline: the oracle on a bounded sample
# ---------------------------------------------------------------------------

def cpu_baseline(mesh, specs, kw, iters=3):
    """Time ``iters`` Jacobi iterations of one substep of the workload with the
    CPU oracle (float32); returns tet-iterations/s and the sample text."""
    from oracle.xpbd_oracle import OracleSdf, OracleSolver
    okw = dict(kw)
    okw.update(substeps_num=1, constraints_iter=iters, frame_dt=kw["dt"] / kw["substeps_num"],
               dt=kw["dt"] / kw["substeps_num"])
    o = OracleSolver(mesh.points, mesh.tets, [OracleSdf(k, **p) for k, p in specs], dtype=np.float32,
                     total_mass=1000.0, **{k: v for k, v in okw.items() if k != "density"})
    t0 = time.perf_counter()
    o.solve()
    el = time.perf_counter() - t0
    units = mesh.n_tets * iters
    return dict(value=units / el, unit=UNIT, cores=1, kind="port",
                sample="NumPy float32 oracle, 1 substep x %d iterations of the same mesh (%d tet-iterations, %.1f s)"
                % (iters, units, el))


# ---------------------------------------------------------------------------
# clocks
# ---------------------------------------------------------------------------

class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for nm, val in zip(names, f[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(smax)), "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------------------
# arms
# ---------------------------------------------------------------------------

def dist_info():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("LOCAL_RANK", 0)), int(os.environ.get("WORLD_SIZE", 1))


def run_reference(args):
    rank, _, world = dist_info()
    if rank != 0:
        return
    mesh, specs, kw, desc = workload(args.workload)
    vals = []
    for _ in range(args.warmup):
        cpu_baseline(mesh, specs, kw, iters=1)
    for _ in range(args.steps):
        vals.append(cpu_baseline(mesh, specs, kw, iters=args.ref_iters))
    v = float(np.mean([r["value"] for r in vals]))
    frame_units = tet_iterations_per_frame(mesh, kw)
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": frame_units / v * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": {"workload": desc},
            "cpu_baseline": dict(vals[-1], value=v),
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_gb300(args):
    import torch
    rank, local_rank, world = dist_info()
    torch.cuda.set_device(local_rank)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from xpbd_gpu import _native
    from xpbd_gpu.neohookean_solver import XPBDNeoHookeanSolver, frame_chunks

    mesh, specs, kw, desc = workload(args.workload)
    solver = XPBDNeoHookeanSolver(mesh, product_sdfs(specs), scatter=args.scatter, sweep_order=args.sweep_order,
                                  patch_pipeline=args.patch_pipeline, patch_reduce=args.patch_reduce, **kw)
    frame_units = tet_iterations_per_frame(mesh, kw)
    n_chunks = len(frame_chunks(kw["frame_dt"], kw["dt"]))
    per_iter = 3 + (1 if args.scatter == "gather" else 0)
    launches_per_frame = n_chunks * kw["substeps_num"] * (2 + kw["constraints_iter"] * per_iter)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    for _ in range(max(args.warmup, 3)):
        solver.solve()
    torch.cuda.synchronize()

    # timed region: K frames, device-resident inputs, L2 flushed between frames
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    barrier()
    torch.cuda.synchronize()
    with ClockSampler(torch.cuda.current_device()) as clk:
        for a, b in ev:
            flush.fill_(1.0)
            a.record(stream)
            solver.solve()
            b.record(stream)
        torch.cuda.synchronize()
    barrier()
    ms = [a.elapsed_time(b) for a, b in ev]
    total_ms = float(sum(ms))
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([total_ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    ms_per_step = total_ms / args.steps
    value = frame_units * args.steps * world / (total_ms * 1e-3)
    solver.check_status()

    # per-kernel durations: the same frames with direct launches bracketed by events
    solver.set_profiling(True)
    solver.read_profile(reset=True)
    for _ in range(args.profile_steps):
        flush.fill_(1.0)
        solver.solve()
    prof = solver.read_profile(reset=True)
    solver.set_profiling(False)

    # end to end through the public API with pinned host buffers
    x_host = torch.from_numpy(solver.mesh.verts.x.to_numpy()).pin_memory()
    v_host = torch.from_numpy(solver.mesh.verts.v.to_numpy()).pin_memory()
    e2e_ms = []
    for k in range(args.e2e_steps + 1):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        solver.mesh.verts.x.from_numpy(x_host)
        solver.mesh.verts.v.from_numpy(v_host)
        solver.solve()
        out = solver.mesh.verts.x.to_numpy()
        t1 = time.perf_counter()
        if k > 0:
            e2e_ms.append((t1 - t0) * 1e3)
    e2e_step = float(np.mean(e2e_ms))
    V, T = mesh.n_verts, mesh.n_tets
    assert out.shape == (V, 3)

    if rank != 0:
        return
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(peaks_path):
        peak = float(json.load(open(peaks_path))["hbm_gbs"])
        peak_src = "measured"
    else:
        peak, peak_src = 6800.0, "fallback"
    K = kw["constraints_iter"]
    n_proj = prof["project"]["launches"]
    # algorithmic bytes of one projection launch (per-unit figures of the
    # reference-semantics accounting): per tet 16 ids + 36 inv_Dm + 4 V0 +
    # 8 lambda read + 8 lambda write = 72 B; per vertex 16 gather + 16 scatter
    proj_bytes = 72.0 * T + 32.0 * V
    proj_ms = prof["project"]["ms"] / max(1, n_proj)
    achieved = proj_bytes / (proj_ms * 1e-3) / 1e9
    kernel_name = {"patch": "k_project_patch1 (tile, 256-tet patches, red.global.add.v4 per corner)",
                   "atomic": "k_project (one thread per tet, red.global.add.v4 per corner)",
                   "gather": "k_project (per-corner buffer + deterministic vertex gather)"}[args.scatter]
    # dram__bytes_read.sum + dram__bytes_write.sum of one launch of this kernel on this
    # workload, from the ncu captures summarised in profiles/k_project_*_c2_64cube.md
    traffic = {"patch": 89.4e6, "atomic": 115.2e6}.get(args.scatter)
    if args.patch_pipeline != 0 or args.patch_reduce != 0 or args.workload != "c2":
        traffic = None
    iter_bytes = 136.0 * T + 128.0 * V
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": desc, "step": "one frame (%d tet-iterations)" % frame_units,
                   "scatter": args.scatter, "sweep_order": args.sweep_order,
                   "patch_pipeline": args.patch_pipeline, "l2": "flushed between steps (%d MiB write)" % (L2_FLUSH_BYTES >> 20),
                   "parallelism": "replicas" if world > 1 else "single GPU", "graph": "one CUDA graph per frame"},
        "frames_per_s": 1e3 / ms_per_step * world,
        "gpu_launches": launches_per_frame * args.steps,
        "roofline": {"bound": "hbm", "kernel": kernel_name,
                     "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_source": peak_src, "traffic": traffic,
                     "bytes_per_launch": proj_bytes, "ms_per_launch": proj_ms},
        "iteration_roofline": {"bytes_per_iteration": iter_bytes,
                               "achieved_GBps": iter_bytes * K * n_chunks * kw["substeps_num"] / (ms_per_step * 1e-3) / 1e9,
                               "frac": iter_bytes * K * n_chunks * kw["substeps_num"] / (ms_per_step * 1e-3) / 1e9 / peak},
        "kernel_profile": {k: {"ms_per_launch": v["ms"] / max(1, v["launches"]), "launches": v["launches"],
                               "share": v["ms"] / max(1e-12, sum(x["ms"] for x in prof.values()))}
                           for k, v in prof.items() if v["launches"]},
        "e2e": {"value": frame_units / (e2e_step * 1e-3) * world, "unit": UNIT,
                "h2d_bytes_per_step": 2 * V * 12, "d2h_bytes_per_step": V * 12, "ms_per_step": e2e_step},
        "clocks": clk.summary(),
    }
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(mesh, specs, kw, iters=args.cpu_iters)
    print(json.dumps(line), flush=True)


def run_profile(args):
    """Frames with direct launches and no timing, for an external profiler."""
    import torch
    from xpbd_gpu.neohookean_solver import XPBDNeoHookeanSolver
    mesh, specs, kw, desc = workload(args.workload)
    solver = XPBDNeoHookeanSolver(mesh, product_sdfs(specs), scatter=args.scatter, sweep_order=args.sweep_order,
                                  patch_pipeline=args.patch_pipeline, patch_reduce=args.patch_reduce,
                                  use_graph=False, **kw)
    for _ in range(args.profile_frames):
        solver.solve()
    torch.cuda.synchronize()
    solver.check_status()
    print("profile mode: %d frame(s) of %s" % (args.profile_frames, desc))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="c2", choices=["c2", "c1"])
    ap.add_argument("--scatter", default="patch", choices=["atomic", "gather", "patch"])
    ap.add_argument("--sweep-order", type=int, default=1, choices=[0, 1])
    ap.add_argument("--patch-pipeline", type=int, default=0, choices=[0, 1])
    ap.add_argument("--patch-reduce", type=int, default=0, choices=[0, 1])
    ap.add_argument("--profile-steps", type=int, default=2)
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--cpu-iters", type=int, default=3)
    ap.add_argument("--ref-iters", type=int, default=2)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--mode", default="bench", choices=["bench", "profile"])
    ap.add_argument("--profile-frames", type=int, default=1)
    args = ap.parse_args()
    if args.mode == "profile":
        run_profile(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
