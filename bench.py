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


def workload_c3(seed=0, n_bodies=256, h=0.03):
    """256 Kuhn bodies with per-axis cell counts U{4..32}, E log-U[1e4, 1e7], nu U[0.30, 0.495],
    rho U[500, 2000], random rotation, non-overlapping placement (rejection sampling on bounding
    spheres) in a 16 x 4 x 16 m arena above the plane y = 0 and 32 random spheres."""
    from xpbd_gpu.batched import Body
    from xpbd_gpu.mesh import kuhn_grid, random_rotation
    rng = np.random.default_rng(seed)
    dims = rng.integers(4, 33, size=(n_bodies, 3))
    E = np.exp(rng.uniform(np.log(1e4), np.log(1e7), n_bodies))
    nu = rng.uniform(0.30, 0.495, n_bodies)
    rho = rng.uniform(500.0, 2000.0, n_bodies)
    radius = 0.5 * h * np.linalg.norm(dims, axis=1)
    order = np.argsort(-radius)
    centers = np.zeros((n_bodies, 3))
    placed = []
    for k in order:
        r = radius[k]
        for _ in range(20000):
            c = np.array([rng.uniform(r, 16.0 - r), rng.uniform(r + 0.9, 4.0 - r), rng.uniform(r, 16.0 - r)])
            if all(np.linalg.norm(c - centers[j]) > r + radius[j] for j in placed):
                break
        else:
            raise RuntimeError("could not place body %d" % k)
        centers[k] = c
        placed.append(k)
    bodies = []
    for k in range(n_bodies):
        nx, ny, nz = (int(v) for v in dims[k])
        mesh = kuhn_grid(nx, ny, nz, h, origin=(-0.5 * nx * h, -0.5 * ny * h, -0.5 * nz * h), jitter=0.1,
                         seed=seed * 1000 + k)
        bodies.append(Body(mesh, young_modulus=float(E[k]), poisson_ratio=float(nu[k]), density=float(rho[k]),
                           rotation=random_rotation(rng), offset=tuple(centers[k])))
    sdfs = [("plane", dict(point=[0.0, 0.0, 0.0], dir=[0.0, 1.0, 0.0], fixed=True))]
    for _ in range(32):
        sdfs.append(("sphere", dict(center=[float(rng.uniform(0, 16)), float(rng.uniform(-0.6, 0.0)),
                                            float(rng.uniform(0, 16))], radius=float(rng.uniform(0.3, 0.8)),
                                    fixed=True)))
    kw = dict(frame_dt=1.0 / 60, dt=1.0 / 60, substeps_num=5, constraints_iter=30, cheb_enable=True,
              cheb_warmup=5, cheb_gamma=0.6666, block_neohookean_enable=True)
    desc = ("256 uneven Kuhn bodies (cells U{4..32}^3, %d tets, %d verts), E log-U[1e4,1e7], nu U[0.30,0.495], "
            "rho U[500,2000], plane + 32 spheres, 5 substeps x 30 it" % (
                sum(6 * int(np.prod(d)) for d in dims), sum(int(np.prod(d + 1)) for d in dims)))
    return bodies, sdfs, kw, desc


def smooth_field(shape, sigma, rng):
    """Unit-variance Gaussian random field: Gaussian-filtered white noise on a grid."""
    from scipy.ndimage import gaussian_filter
    g = gaussian_filter(rng.normal(size=shape), sigma=sigma, mode="wrap")
    return (g - g.mean()) / g.std()


def workload_c4(seed=0, n=16, sigma=2.0):
    """16^3 Kuhn cube (edge 1/16 m) above the plane y = 0; per-tet log E = log 1e5 + 0.5 g with g a
    unit-variance Gaussian field (Gaussian filter of sigma cells on white noise), nu = 0.45."""
    from xpbd_gpu.mesh import kuhn_grid
    rng = np.random.default_rng(seed)
    mesh = kuhn_grid(n, n, n, 1.0 / n, origin=(0.0, 0.3, 0.0), jitter=0.1, seed=seed)
    g = smooth_field((n, n, n), sigma, rng)
    cell = g.ravel(order="F")  # cell (i, j, k), i fastest, as the Kuhn tets
    log_E = np.log(1e5) + 0.5 * np.repeat(cell, 6)
    specs = [("plane", dict(point=[0.0, 0.0, 0.0], dir=[0.0, 1.0, 0.0], fixed=True))]
    kw = dict(frame_dt=1.0 / 60, dt=1.0 / 60, substeps_num=5, constraints_iter=20, cheb_enable=True,
              cheb_warmup=5, cheb_gamma=0.6666, block_neohookean_enable=True, total_mass=1000.0)
    desc = ("16^3 Kuhn cube (24,576 tets, 4,913 verts), per-tet log E = log 1e5 + 0.5 g (Gaussian field, "
            "sigma %.1f cells), nu 0.45, 60 frames x 5 substeps x 20 it, MSE of final positions" % sigma)
    return mesh, specs, kw, log_E, desc


def run_c4(args):
    print(json.dumps(c4_block(args)), flush=True)


# the reference's four-way comparison: (label, block Neo-Hookean, dynamic Chebyshev)
MATRIX = [("NH", False, False), ("NH-DC", False, True), ("BNH", True, False), ("BNH-DC", True, True)]


def matrix_scene(args):
    """Scene, material and stepping of the reference's convergence comparison
    (scripts/compare_convergence_armadillo.bat:14-17 with the driver
    run_neohookean_usd.py:82-106): the mesh at scale 0.01 and offset (0, 1, 0),
    E 5e8, nu 0.4999, relaxation 1.2, dt 0.01 at 60 fps (two chunks per frame),
    1 substep of 200 iterations, Chebyshev warm-up 5 and gamma 0.666, the plane
    y = -2 and the fixed sphere at (0, -1, 0) of radius 0.3, monitoring on."""
    kw = dict(scale=args.matrix_scale, offset=(0.0, 1.0, 0.0), hydrostatic_relaxation=1.2,
              deviatoric_relaxation=1.2, frame_dt=1.0 / 60, dt=0.01, substeps_num=1, constraints_iter=200,
              young_modulus=5e8, poisson_ratio=0.4999, cheb_warmup=5, cheb_gamma=0.666, monitor_convergence=True)
    sdfs = [("plane", dict(point=[0.0, -2.0, 0.0], dir=[0.0, 1.0, 0.0], fixed=True)),
            ("sphere", dict(center=[0.0, -1.0, 0.0], radius=0.3, fixed=True))]
    return kw, sdfs


def run_matrix(args):
    """NH / NH-DC / BNH / BNH-DC on one mesh for `matrix_frame` + 1 frames: the
    convergence records of frame `matrix_frame` (r_hat, hydrostatic and
    deviatoric error per iteration, both chunks), the solver time per frame
    (monitoring on, as the driver runs it), and that frame against the C
    restatement in FP64 and FP32 started from the GPU state before it."""
    import torch
    from oracle.xpbd_oracle import OracleSdf
    from oracle.xpbd_oracle_c import COracle
    from xpbd_gpu.mesh import read_tetgen
    from xpbd_gpu.neohookean_solver import XPBDNeoHookeanSolver
    torch.cuda.set_device(0)
    mesh = read_tetgen(args.mesh)
    kw0, specs = matrix_scene(args)
    F = args.matrix_frame
    out = {"workload": "convergence matrix", "mesh": os.path.basename(args.mesh), "verts": mesh.n_verts,
           "tets": mesh.n_tets, "frames": F + 1, "recorded_frame": F,
           "scene": "scale %g, offset (0, 1, 0), E 5e8, nu 0.4999, relax 1.2, dt 0.01 at 60 fps, 1 substep x 200 it, "
                    "plane y=-2 + sphere (0,-1,0) r 0.3" % args.matrix_scale, "configs": {}}
    for label, block, cheb in MATRIX:
        kw = dict(kw0, block_neohookean_enable=block, cheb_enable=cheb)
        s = XPBDNeoHookeanSolver(rest_pose=mesh, sdf=product_sdfs(specs), **kw)
        recs = []

        def record(frame, substep, data, s=s, recs=recs):
            if frame == F:  # r_hat from the history rows (computed with the Chebyshev step only)
                rh = s.read_history(s.constraints_iter)[:, 0].tolist() if s.cheb_enable else None
                recs.append((rh, [dict(r) for r in data]))
        s.convergence_callback = record
        times = []
        for f in range(F + 1):
            if f == F:
                x_prev = s.mesh.verts.x.to_numpy().astype(np.float64)
                v_prev = s.mesh.verts.v.to_numpy().astype(np.float64)
                rho_prev = float(s.rho_hat)
            t0 = time.perf_counter()
            s.solve()
            times.append(time.perf_counter() - t0)
        s.check_status()
        x_gpu = s.mesh.verts.x.to_numpy().astype(np.float64)
        diag = float(np.linalg.norm(x_gpu.max(0) - x_gpu.min(0)))
        cfg = {"ms_per_frame": 1e3 * float(np.mean(times[1:])),
               "chunks": [{"r_hat": rh, "hydro_error": [r["hydro_error"] for r in c],
                           "dev_error": [r["dev_error"] for r in c]} for rh, c in recs]}
        # the recorded frame from the same state in the C restatement
        ok = dict(kw, block_neohookean_enable=block, cheb_enable=cheb)
        hist_len = 2 * 200
        for name, dt_ in (("fp64", np.float64), ("fp32", np.float32)):
            o = COracle(mesh.points, mesh.tets, [OracleSdf(k, **p) for k, p in specs], dtype=dt_, **ok)
            o.x[:] = x_prev
            o.v[:] = v_prev
            o.rho_hat.value = rho_prev
            hist = np.zeros(hist_len)
            o.solve(1, r_hat_hist=hist)
            cfg[name + "_max_dev_over_bbox_diag"] = float(np.abs(x_gpu - o.x).max()) / diag
            if name == "fp64":
                x64 = o.x.astype(np.float64).copy()
                cfg["fp64_r_hat"] = hist.tolist()
            else:
                cfg["fp32_vs_fp64_max_dev_over_bbox_diag"] = float(np.abs(o.x - x64).max()) / diag
        out["configs"][label] = cfg
        print("%s: %.2f ms/frame, vs FP64 %.2e (FP32 reference vs FP64 %.2e)" % (
            label, cfg["ms_per_frame"], cfg["fp64_max_dev_over_bbox_diag"],
            cfg["fp32_vs_fp64_max_dev_over_bbox_diag"]), file=sys.stderr, flush=True)
    print(json.dumps(out), flush=True)


def plain_forward_ms(sim, simulate, x0, v0, log_E, nu, frames, reps):
    """Mean device time of the forward alone, without tapes (the recompute
    plan: one CUDA graph of per-substep state checkpoints and plain substeps)."""
    import torch
    mode = sim.tape_memory
    sim.tape_memory = "recompute"
    out = []
    with torch.no_grad():
        for k in range(reps + 1):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            simulate(sim, x0, v0, log_E.detach(), nu.detach(), frames)
            b.record()
            b.synchronize()
            if k:
                out.append(a.elapsed_time(b))
    sim.tape_memory = mode
    return float(np.mean(out))


def tape_note(sim, frames):
    from xpbd_gpu.differentiable import _plan
    p = _plan(sim, frames)
    if p.stored:
        return ("stored: the forward records every substep's tape (%.1f GB), the backward reverses them"
                % (sum(t.numel() * t.element_size() for t in vars(p.tapes).values()
                       if hasattr(t, "numel")) / 1e9))
    return "recomputed: the backward restores each substep's checkpoint and re-runs it on a tape"


def c4_block(args):
    """Differentiable single body: forward (checkpointed) vs adjoint cost, gradient checks."""
    import torch
    from oracle.xpbd_adjoint import DiffOracle, lame_inverse, lame_inverse_grad
    from oracle.xpbd_oracle import OracleSdf
    from xpbd_gpu.differentiable import DiffSim, xpbd_simulate
    torch.cuda.set_device(0)
    dev = torch.device("cuda")
    mesh, specs, kw, log_E_target, desc = workload_c4()
    T = mesh.n_tets
    frames = args.c4_frames
    nu = np.full(T, 0.45)
    sim = DiffSim(mesh, product_sdfs(specs), log_E_target, nu, **kw)
    x0 = torch.tensor(mesh.points, dtype=torch.float32, device=dev)
    v0 = torch.zeros_like(x0)
    with torch.no_grad():
        x_target = xpbd_simulate(sim, x0, v0, torch.tensor(log_E_target, device=dev),
                                 torch.tensor(nu, device=dev), frames).clone()
    le = torch.full((T,), float(np.log(1e5)), dtype=torch.float64, device=dev, requires_grad=True)
    nu_t = torch.tensor([0.45], dtype=torch.float64, device=dev, requires_grad=True)
    v0r = v0.clone().requires_grad_(True)
    fwd, bwd = [], []
    for k in range(args.c4_reps + 1):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        xf = xpbd_simulate(sim, x0, v0r, le, nu_t, frames)
        loss = ((xf - x_target) ** 2).sum() / xf.shape[0]
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        le.grad = None
        nu_t.grad = None
        v0r.grad = None
        loss.backward()
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        if k > 0:
            fwd.append(t1 - t0)
            bwd.append(t2 - t1)
    fwd_ms, bwd_ms = 1e3 * float(np.mean(fwd)), 1e3 * float(np.mean(bwd))
    units = T * frames * kw["substeps_num"] * kw["constraints_iter"]
    plain_fwd_ms = plain_forward_ms(sim, xpbd_simulate, x0, v0, le, nu_t, frames, args.c4_reps)

    # gradient check on a short horizon that starts in contact (after c4_check_start
    # frames of the forward), against the FD-checked float64 adjoint
    hf = args.c4_check_frames
    rng = np.random.default_rng(123)
    le0 = np.log(1e5) + 0.2 * rng.normal(size=T)
    sim2 = DiffSim(mesh, product_sdfs(specs), le0, nu, **kw)
    with torch.no_grad():
        sim2.set_state(x0, v0)
        x_s = xpbd_simulate(sim2, x0, v0, torch.tensor(le0, device=dev), torch.tensor(nu, device=dev),
                            args.c4_check_start).clone()
        v_s = sim2.solver.mesh.verts.v.to_torch().clone()
    rho0 = sim2.solver.rho_hat
    sim2.initial_rho_hat = rho0
    xt = x_s.clone().requires_grad_(True)
    vt = v_s.clone().requires_grad_(True)
    let = torch.tensor(le0, dtype=torch.float64, device=dev, requires_grad=True)
    nut = torch.tensor([0.45], dtype=torch.float64, device=dev, requires_grad=True)
    c = rng.normal(size=mesh.points.shape)
    xf = xpbd_simulate(sim2, xt, vt, let, nut, hf)
    (xf.double() * torch.tensor(c, device=dev)).sum().backward()
    okw = {k: v for k, v in kw.items() if k != "block_neohookean_enable"}
    o = DiffOracle(mesh.points, mesh.tets, [OracleSdf(k, **p) for k, p in specs], *lame_inverse(le0, 0.45),
                   omega_grad=sim2.omega_grad, **okw)
    o.rho_hat = rho0
    _, xb, vb, gm, gl, _ = o.gradient(x_s.cpu().numpy().astype(np.float64), v_s.cpu().numpy().astype(np.float64),
                                      hf, c)
    g_le64, g_nu64 = lame_inverse_grad(le0, np.full(T, 0.45), gm, gl)
    g_le, g_v = let.grad.cpu().numpy(), vt.grad.cpu().numpy()
    rel = lambda a, b: float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))
    errs = {"log_E": [], "v0": []}
    for _ in range(32):
        d = rng.normal(size=T)
        errs["log_E"].append(abs(float((g_le - g_le64) @ d)) / (np.linalg.norm(g_le64) * np.linalg.norm(d) / np.sqrt(T)))
        dv = rng.normal(size=mesh.points.shape)
        errs["v0"].append(abs(float(((g_v - vb) * dv).sum())) / (np.linalg.norm(vb) * np.linalg.norm(dv) / np.sqrt(dv.size)))
    nu_err = abs(float(nut.grad.cpu().numpy().sum()) - float(g_nu64.sum())) / max(abs(float(g_nu64.sum())), 1e-30)
    line = {"metric": METRIC, "value": units / (fwd_ms * 1e-3), "unit": UNIT, "n_gpus": 1, "steps": args.c4_reps,
            "warmup": 1, "ms_per_step": fwd_ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic",
            "config": {"workload": desc, "step": "forward of %d frames with per-substep checkpoints" % frames},
            "adjoint": {"backward_ms": bwd_ms, "backward_over_forward": bwd_ms / fwd_ms,
                        "plain_forward_ms": plain_fwd_ms, "backward_over_plain_forward": bwd_ms / plain_fwd_ms,
                        "omega": "through omega (omega -> rho_hat -> r_hat adjoint)" if sim.omega_grad
                        else "stop-gradient",
                        "tapes": tape_note(sim, frames)},
            "gradient_check": {"start_frame": args.c4_check_start, "horizon_frames": hf, "directions": 32,
                               "reference": "float64 adjoint (oracle/xpbd_adjoint.py, itself checked against "
                                            "central finite differences), started from the GPU state",
                               "rel_l2_err": {"log_E": rel(g_le, g_le64), "v0": rel(g_v, vb), "nu": nu_err},
                               "max_directional_err_over_rms": {k: float(np.max(v)) for k, v in errs.items()}}}
    return line


def workload_c5(seed=0, n_bodies=64, h=1.0 / 16, sigma=2.0):
    """64 Kuhn bodies with per-axis cell counts U{8..24} (cell edge 1/16 m, jitter 0.1 cell), each with a
    hidden per-tet log E field (mean log-U[1e4, 1e6] + 0.5 g, g a unit-variance Gaussian field of sigma
    cells) and nu U[0.35, 0.48]; density 1000; dropped from 0.3 m onto the plane y = 0 (bodies on an 8 x 8
    grid of 2.5 m pitch, independent of each other); 30 frames x 5 substeps x 20 it."""
    from xpbd_gpu.mesh import kuhn_grid
    rng = np.random.default_rng(seed)
    dims = rng.integers(8, 25, size=(n_bodies, 3))
    mean = rng.uniform(np.log(1e4), np.log(1e6), n_bodies)
    nus = rng.uniform(0.35, 0.48, n_bodies)
    meshes, log_E = [], []
    for k in range(n_bodies):
        nx, ny, nz = (int(v) for v in dims[k])
        origin = (2.5 * (k % 8), 0.3, 2.5 * (k // 8))
        meshes.append(kuhn_grid(nx, ny, nz, h, origin=origin, jitter=0.1, seed=seed * 1000 + k))
        g = smooth_field((nx, ny, nz), sigma, rng)
        log_E.append(mean[k] + 0.5 * np.repeat(g.ravel(order="F"), 6))
    specs = [("plane", dict(point=[0.0, 0.0, 0.0], dir=[0.0, 1.0, 0.0], fixed=True))]
    kw = dict(frame_dt=1.0 / 60, dt=1.0 / 60, substeps_num=5, constraints_iter=20, cheb_enable=True,
              cheb_warmup=5, cheb_gamma=0.6666, block_neohookean_enable=True)
    desc = ("64 Kuhn bodies (cells U{8..24}^3, %d tets, %d verts), hidden per-tet log E (mean log-U[1e4,1e6], "
            "sigma 0.5), nu U[0.35,0.48], plane, 30 frames x 5 substeps x 20 it, MSE of final positions" % (
                sum(m.n_tets for m in meshes), sum(m.n_verts for m in meshes)))
    return meshes, log_E, nus, specs, kw, desc


def run_c5(args):
    print(json.dumps(c5_block(args, args.c5_adam_steps, plain_accuracy_bodies=args.c5_plain_bodies)), flush=True)


def c5_block(args, steps, plain_accuracy_bodies=4, plain_timing_steps=2, fp64_bodies=4):
    """Batched differentiable: Adam on every body's per-tet log E through the
    batched adjoint (forward + adjoint per substep, graph-captured), against the
    plain per-body form (one single-body adjoint per body, also captured):
    * timing: `steps` Adam steps of the batch; the plain form runs
      `plain_timing_steps` Adam steps of every one of the 64 bodies;
    * accuracy: the first `plain_accuracy_bodies` bodies run all `steps` Adam
      steps in the plain form too, and their recovered fields are compared;
    * error of the forward against FP64: `fp64_bodies` bodies (spread over the
      sizes), one frame from the initial state, against the float64 oracle run
      of each body with its own per-tet materials."""
    import torch
    from xpbd_gpu.batched import Body
    from xpbd_gpu.differentiable import BatchedDiffSim, DiffSim, xpbd_simulate, xpbd_simulate_batch
    torch.cuda.set_device(0)
    dev = torch.device("cuda")
    meshes, log_E_true, nus, specs, kw, desc = workload_c5()
    frames, lr = args.c5_frames, args.c5_lr
    nb = len(meshes)
    T_all = sum(m.n_tets for m in meshes)
    nu_tet = np.concatenate([np.full(m.n_tets, nus[k]) for k, m in enumerate(meshes)])
    le_true = np.concatenate(log_E_true)
    le0 = np.full(T_all, np.log(1e5))
    bodies = [Body(m, tet_young_modulus=np.exp(log_E_true[k]), tet_poisson_ratio=nus[k], density=1000.0,
                   poisson_ratio=float(nus[k])) for k, m in enumerate(meshes)]
    sim = BatchedDiffSim(bodies, product_sdfs(specs), **kw)
    x0 = torch.tensor(np.concatenate([m.points for m in meshes]), dtype=torch.float32, device=dev)
    v0 = torch.zeros_like(x0)
    nu_t = torch.tensor(nu_tet, dtype=torch.float64, device=dev)
    with torch.no_grad():
        x_target = xpbd_simulate_batch(sim, x0, v0, torch.tensor(le_true, device=dev), nu_t, frames).clone()
    vcount = torch.tensor(np.concatenate([np.full(m.n_verts, 1.0 / m.n_verts) for m in meshes]), device=dev)
    offs = np.concatenate([[0], np.cumsum([m.n_tets for m in meshes])])
    voffs = np.concatenate([[0], np.cumsum([m.n_verts for m in meshes])])

    def per_body_rel_err(theta, truth, start):
        return float(np.linalg.norm(theta - truth) / max(np.linalg.norm(start - truth), 1e-30))

    theta = torch.tensor(le0, dtype=torch.float64, device=dev, requires_grad=True)
    opt = torch.optim.Adam([theta], lr=lr)
    fwd_ms, bwd_ms, losses = [], [], []
    for it in range(steps):
        e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        opt.zero_grad()
        e0.record()
        xf = xpbd_simulate_batch(sim, x0, v0, theta, nu_t, frames)
        loss = (((xf - x_target) ** 2).sum(1).double() * vcount).sum()  # sum of per-body MSEs
        e1.record()
        loss.backward()
        e2.record()
        opt.step()
        e2.synchronize()
        fwd_ms.append(e0.elapsed_time(e1))
        bwd_ms.append(e1.elapsed_time(e2))
        losses.append(float(loss))
    sim.batch.check_status()
    plain_fwd_ms = plain_forward_ms(sim, xpbd_simulate_batch, x0, v0, theta, nu_t, frames, 3)
    th = theta.detach().cpu().numpy()
    errs = [per_body_rel_err(th[offs[k]:offs[k + 1]], le_true[offs[k]:offs[k + 1]], le0[offs[k]:offs[k + 1]])
            for k in range(nb)]
    rel_l2 = float(np.linalg.norm(th - le_true) / np.linalg.norm(le_true))
    # the body-mean log E and the fluctuation about it, recovered separately:
    # the loss (final positions after the drop) constrains the first far more
    mean_errs, fluct_errs = [], []
    for k in range(nb):
        a, b, c = th[offs[k]:offs[k + 1]], le_true[offs[k]:offs[k + 1]], le0[offs[k]:offs[k + 1]]
        mean_errs.append(abs(a.mean() - b.mean()) / max(abs(c.mean() - b.mean()), 1e-30))
        fluct_errs.append(per_body_rel_err(a - a.mean(), b - b.mean(), c - c.mean()))

    def plain_body(k, n_steps):
        m = meshes[k]
        ps = DiffSim(m, product_sdfs(specs), np.full(m.n_tets, np.log(1e5)), np.full(m.n_tets, nus[k]),
                     density=1000.0, poisson_ratio=float(nus[k]), **kw)
        xk0 = torch.tensor(m.points, dtype=torch.float32, device=dev)
        vk0 = torch.zeros_like(xk0)
        nuk = torch.full((m.n_tets,), float(nus[k]), dtype=torch.float64, device=dev)
        with torch.no_grad():
            xt = xpbd_simulate(ps, xk0, vk0, torch.tensor(log_E_true[k], device=dev), nuk, frames).clone()
        thk = torch.tensor(le0[offs[k]:offs[k + 1]], dtype=torch.float64, device=dev, requires_grad=True)
        optk = torch.optim.Adam([thk], lr=lr)
        ms = []
        for it in range(n_steps):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            optk.zero_grad()
            a.record()
            xf = xpbd_simulate(ps, xk0, vk0, thk, nuk, frames)
            lk = ((xf - xt) ** 2).sum(1).double().mean()
            lk.backward()
            b.record()
            optk.step()
            b.synchronize()
            ms.append(a.elapsed_time(b))
        ps.solver.check_status()
        return thk.detach().cpu().numpy(), ms

    # plain form, timing: every body, `plain_timing_steps` Adam steps each (the first
    # step of a body captures its graphs and is not counted when there are more)
    plain_ms = []
    for k in range(nb):
        _, ms = plain_body(k, plain_timing_steps)
        plain_ms.append(float(np.mean(ms[1:] if len(ms) > 1 else ms)))
    # plain form, accuracy: the first bodies through all the Adam steps
    plain = []
    for k in range(min(plain_accuracy_bodies, nb)):
        tk, _ = plain_body(k, steps)
        plain.append(dict(rel_err=per_body_rel_err(tk, log_E_true[k], le0[offs[k]:offs[k + 1]]),
                          batched_rel_err=errs[k],
                          theta_rel_diff_vs_batched=float(np.linalg.norm(tk - th[offs[k]:offs[k + 1]]) /
                                                          np.linalg.norm(th[offs[k]:offs[k + 1]]))))
    fp64 = c5_fp64_error(meshes, log_E_true, nus, specs, kw, sim, x0, v0, nu_t, le_true, voffs, fp64_bodies)
    sl = slice(1, None) if steps > 1 else slice(None)
    step_ms = float(np.mean(np.add(fwd_ms, bwd_ms)[sl]))
    units = T_all * frames * kw["substeps_num"] * kw["constraints_iter"]
    plain_total_ms = float(np.sum(plain_ms))
    return {"metric": METRIC, "value": units / (step_ms * 1e-3), "unit": UNIT, "n_gpus": 1, "steps": steps,
            "warmup": 1, "ms_per_step": step_ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic",
            "config": {"workload": desc,
                       "step": "one Adam step on all 64 bodies: checkpointed batched forward of %d frames + "
                               "batched adjoint (tet-iterations counted once, forward)" % frames,
                       "form": "batched (one launch per phase over all bodies, forward and adjoint each one "
                               "CUDA graph)"},
            "forward_ms": float(np.mean(np.asarray(fwd_ms)[sl])), "backward_ms": float(np.mean(np.asarray(bwd_ms)[sl])),
            "backward_over_forward": float(np.mean(np.asarray(bwd_ms)[sl]) / np.mean(np.asarray(fwd_ms)[sl])),
            "plain_forward_ms": plain_fwd_ms,
            "backward_over_plain_forward": float(np.mean(np.asarray(bwd_ms)[sl]) / plain_fwd_ms),
            "tapes": tape_note(sim, frames),
            "adam": {"steps": steps, "lr": lr, "init": "log E = log 1e5 everywhere",
                     "loss_first_last": [losses[0], losses[-1]],
                     "recovered_rel_err_median": float(np.median(errs)),
                     "recovered_rel_err_mean": float(np.mean(errs)),
                     "recovered_rel_l2_of_log_E": rel_l2,
                     "recovered_body_mean_rel_err_median": float(np.median(mean_errs)),
                     "recovered_fluctuation_rel_err_median": float(np.median(fluct_errs)),
                     "rel_err_definition": "|theta - theta*| / |theta_0 - theta*| per body"},
            "plain": {"form": "one single-body DiffSim per body (ATOMIC scatter, per-tet materials), same Adam, "
                              "forward and adjoint graph-captured",
                      "bodies_timed": nb, "ms_per_adam_step_all_bodies": plain_total_ms,
                      "value": units / (plain_total_ms * 1e-3),
                      "accuracy_bodies": len(plain), "per_body": plain},
            "batched_over_plain": plain_total_ms / step_ms,
            "fp64_error": fp64}


def c5_fp64_error(meshes, log_E, nus, specs, kw, sim, x0, v0, nu_t, le_true, voffs, n_bodies):
    """The batched forward of one frame (true materials, from the initial state)
    against the float64 oracle of each sampled body: max vertex deviation over
    the body's bounding-box diagonal."""
    import torch
    from oracle.xpbd_adjoint import DiffOracle, lame_inverse
    from oracle.xpbd_oracle import OracleSdf
    from xpbd_gpu.differentiable import xpbd_simulate_batch
    with torch.no_grad():
        xg = xpbd_simulate_batch(sim, x0, v0, torch.tensor(le_true, device=x0.device), nu_t, 1).cpu().numpy()
    sizes = np.array([m.n_tets for m in meshes])
    pick = [int(k) for k in np.argsort(sizes)[np.linspace(0, len(meshes) - 1, n_bodies).astype(int)]]
    okw = {k: v for k, v in kw.items() if k != "block_neohookean_enable"}
    out = []
    for k in pick:
        m = meshes[k]
        im, il = lame_inverse(log_E[k], nus[k])
        total = 1000.0 * float(np.abs(_volume(m)).sum())
        o = DiffOracle(m.points, m.tets, [OracleSdf(kk, **p) for kk, p in specs], im, il, total_mass=total, **okw)
        xe, _, _, _ = o.run(m.points.astype(np.float64), np.zeros((m.n_verts, 3)), 1)
        diag = float(np.linalg.norm(m.points.max(0) - m.points.min(0)))
        out.append(dict(body=k, tets=int(m.n_tets),
                        max_dev_over_bbox_diag=float(np.abs(xg[voffs[k]:voffs[k + 1]] - xe).max()) / diag))
    return {"reference": "float64 oracle (oracle/xpbd_adjoint.py forward) with each body's per-tet materials",
            "frames": 1, "bodies": out,
            "max_over_bodies": max(b["max_dev_over_bbox_diag"] for b in out)}


def c3_solvers(args, bodies, specs, kw, cap, target, floor):
    """The batched form and the plain form (one single-body solver per body) of
    the 256-body workload, both in stop mode with iteration cap `cap`."""
    from xpbd_gpu.batched import XPBDBatchedSolver
    from xpbd_gpu.mesh import TetMesh
    from xpbd_gpu.neohookean_solver import XPBDNeoHookeanSolver
    kwc = dict(kw, constraints_iter=cap)
    btpt = "auto" if args.batch_tpt == "auto" else int(args.batch_tpt)
    batch = XPBDBatchedSolver(bodies, product_sdfs(specs), tets_per_thread=btpt, pair_tets=bool(args.pair_tets),
                              target_rel_residual=target, residual_floor=floor, **kwc)
    plain = []
    for b in bodies:
        mesh = TetMesh(b.rest_pose.points @ b.rotation.T, b.rest_pose.tets)
        plain.append(XPBDNeoHookeanSolver(mesh, product_sdfs(specs), young_modulus=b.young_modulus,
                                          poisson_ratio=b.poisson_ratio, offset=b.offset, density=b.density,
                                          scatter="patch", tets_per_thread=args.tets_per_thread,
                                          pair_tets=bool(args.pair_tets), target_rel_residual=target,
                                          residual_floor=floor, **kwc))
    return batch, plain


def set_plain_mode(plain, target, floor, iters):
    for s in plain:
        s.target_rel_residual, s.residual_floor, s.constraints_iter = float(target), float(floor), int(iters)


def load_plain_state(plain, batch, state):
    """Positions, velocities and rho_hat of every body (the state a frame
    starts from; multipliers and predicted positions restart each substep)."""
    for k, s in enumerate(plain):
        sl = batch.body_vert_slices[k]
        s.mesh.verts.x.from_numpy(state["x"][sl])
        s.mesh.verts.v.from_numpy(state["v"][sl])
        s.rho_hat = float(state["rho"][k])


def loop_launches(n, per_iteration=4):
    """Kernel launches of one stop-mode substep whose longest body ran n
    iterations: begin + end + `per_iteration` per iteration (the batch:
    projection, residual, update and the next iteration's patch list); past
    the first two iterations the frame graph's WHILE node runs pairs of
    iterations."""
    it = n if n <= 2 else 2 + 2 * ((n - 1) // 2)
    return 2 + per_iteration * it


def run_frames(step, n, flush, stream, after=None):
    """n frames, each bracketed by CUDA events on `stream`, L2 flushed before
    each; `after()` (outside the events) collects per-frame data."""
    import torch
    ms, data = [], []
    for _ in range(n):
        flush.fill_(1.0)
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        step()
        b.record(stream)
        b.synchronize()
        ms.append(a.elapsed_time(b))
        if after is not None:
            data.append(after())
    return ms, data


def c3_headline(args, world=1, barrier=lambda: None):
    """The metric's configuration: the 256-body batch, batched form against the
    plain one-body-per-launch form at equal final relative residual.

    Both forms start from the same settled state (the batch stepped
    `c3_settle` frames at the reference's fixed 30 iterations, so every body
    has landed) and run in stop mode: each body's substep iterates until
    r_hat_k / r_hat_0 <= c3_target, or r_hat_k <= c3_floor (the FP32 round-off
    level of a resting or free-falling body), with c3_cap iterations at the
    most.  Both forms run the same per-body algorithm, so every body stops at
    the same iteration with the same residual in both; the line reports the
    counts' agreement.  `value` = executed tet-iterations per second of the
    batched form; the plain form is timed on the first frames of the same
    window.  The fixed 30-iteration comparison (the reference's own loop) is
    reported beside it."""
    import torch
    rank, local_rank, _ = dist_info()
    bodies, specs, kw, desc = workload_c3()
    cap, target, floor = args.c3_cap, args.c3_target, args.c3_floor
    K0 = kw["constraints_iter"]
    S = kw["substeps_num"]
    t_build = time.perf_counter()
    batch, plain = c3_solvers(args, bodies, specs, kw, cap, target, floor)
    t_build = time.perf_counter() - t_build
    Tb = np.array([b.rest_pose.n_tets for b in bodies], dtype=np.float64)
    Vb = np.array([b.rest_pose.n_verts for b in bodies], dtype=np.float64)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()

    # settle at the fixed iteration count, then the shared starting state
    batch.set_stop(0.0, 0.0, K0)
    for _ in range(args.c3_settle):
        batch.solve()
    batch.check_status()
    state = dict(x=batch.positions(), v=batch.velocities(), rho=batch.rho_hat, snap=batch.snapshot())

    def batch_counts():
        return batch.iterations_per_substep(S)

    def plain_counts():
        return np.stack([s.iterations_per_substep(S) for s in plain])

    # batched, stop mode: warm-up from the shared state, then K timed frames from it
    batch.set_stop(target, floor, cap)
    for _ in range(max(args.warmup, 3)):
        batch.solve()
    batch.restore(state["snap"])
    torch.cuda.synchronize()
    barrier()
    with ClockSampler(torch.cuda.current_device()) as clk_b:
        ms_b, cnt_b = run_frames(batch.solve, args.steps, flush, stream, batch_counts)
    barrier()
    batch.check_status()
    cnt_b = np.stack(cnt_b)  # frames, bodies, substeps
    units_b = (cnt_b * Tb[None, :, None]).sum(axis=(1, 2))  # executed tet-iterations per frame
    bytes_b = (cnt_b * (136.0 * Tb + 128.0 * Vb)[None, :, None]).sum(axis=(1, 2))
    total_ms = max_over_ranks(float(sum(ms_b)), device="cuda")
    value = float(units_b.sum()) * world / (total_ms * 1e-3)
    launches = int(sum(loop_launches(int(n)) for n in cnt_b.max(axis=1).ravel()))
    if rank != 0:
        return None

    # plain, stop mode, the first P frames of the same window
    P = max(1, min(args.c3_plain_frames, args.steps))
    load_plain_state(plain, batch, state)
    for s in plain:
        s.solve()  # warm-up: captures every body's frame graph
    load_plain_state(plain, batch, state)
    torch.cuda.synchronize()
    with ClockSampler(torch.cuda.current_device()) as clk_p:
        ms_p, cnt_p = run_frames(lambda: [s.solve() for s in plain], P, flush, stream, plain_counts)
    for s in plain:
        s.check_status()
    cnt_p = np.stack(cnt_p)
    units_p = (cnt_p * Tb[None, :, None]).sum(axis=(1, 2))
    hist_p = np.stack([s.read_history() for s in plain])

    def rel_final(hist, counts):
        """r_hat of each body-substep's last iteration over its first (last frame)."""
        r = hist[:, :S * cap, 0].reshape(hist.shape[0], S, cap)
        last = np.take_along_axis(r, (counts - 1)[:, :, None], axis=2)[:, :, 0]
        with np.errstate(divide="ignore", invalid="ignore"):
            return last / r[:, :, 0], last

    # the batch's residuals of frame P (the plain form's last), untimed
    batch.restore(state["snap"])
    for _ in range(P):
        batch.solve()
    cnt_bP = batch_counts()
    rel_b, last_b = rel_final(batch.read_history(), cnt_bP)
    rel_p, last_p = rel_final(hist_p, cnt_p[-1])
    met_b = (rel_b <= target) & (cnt_bP < cap)
    floor_b = (last_b <= floor) & ~met_b

    # the reference's fixed iteration count, both forms, the same P frames
    batch.set_stop(0.0, 0.0, K0)
    batch.restore(state["snap"])
    batch.solve()
    batch.restore(state["snap"])
    torch.cuda.synchronize()
    ms_bf, _ = run_frames(batch.solve, P, flush, stream)
    set_plain_mode(plain, 0.0, 0.0, K0)
    load_plain_state(plain, batch, state)
    for s in plain:
        s.solve()
    load_plain_state(plain, batch, state)
    torch.cuda.synchronize()
    ms_pf, _ = run_frames(lambda: [s.solve() for s in plain], P, flush, stream)
    units_f = float(Tb.sum()) * S * K0

    # error against FP64: one fixed-count frame of the batch from the settled state
    # against the float64 and the FP32 C restatement of a sample of bodies
    batch.restore(state["snap"])
    batch.solve()
    fp64 = c3_fp64_error(batch.positions(), state, batch, bodies, specs, kw, args.c3_fp64_bodies)

    # projection kernel of the batched form (fixed count: every patch works),
    # CUDA events around each launch of one frame
    batch.restore(state["snap"])
    batch.set_profiling(True)
    batch.read_profile(reset=True)
    flush.fill_(1.0)
    batch.solve()
    prof = batch.read_profile(reset=True)
    batch.set_profiling(False)
    T, V = float(Tb.sum()), float(Vb.sum())
    proj_ms = prof["project"]["ms"] / max(1, prof["project"]["launches"])
    peak, peak_src = measured_peak()
    proj_bytes = 72.0 * T + 32.0 * V

    # end to end through the public API: host state in, one frame, positions out
    batch.set_stop(target, floor, cap)
    x_host = torch.from_numpy(state["x"]).pin_memory()
    v_host = torch.from_numpy(state["v"]).pin_memory()
    e2e_ms, e2e_units = [], []
    for k in range(args.e2e_steps + 1):
        batch.restore(state["snap"])
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        batch.set_positions(x_host)
        batch.set_velocities(v_host)
        batch.solve()
        out = batch.positions()
        t1 = time.perf_counter()
        if k > 0:
            e2e_ms.append((t1 - t0) * 1e3)
            e2e_units.append(float((batch_counts() * Tb[:, None]).sum()))
    assert out.shape == state["x"].shape
    batch.check_status()

    ms_step = total_ms / args.steps
    n_sub = cnt_b.size
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": max(args.warmup, 3), "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": desc,
                   "step": ("one frame of all 256 bodies; every body's substep iterates until r_hat_k/r_hat_0 <= "
                            "%g or r_hat_k <= %g, at most %d iterations (value counts the tet-iterations run)"
                            % (target, floor, cap)),
                   "form": "batched (one launch per phase over all bodies; frame = one CUDA graph whose "
                           "iterations loop in a WHILE conditional node while any body iterates)",
                   "start": "the batch settled for %d frames at 30 iterations (all bodies landed); every timed "
                            "frame of both forms starts from that state" % args.c3_settle,
                   "l2": "flushed between steps (%d MiB write)" % (L2_FLUSH_BYTES >> 20),
                   "parallelism": "replicas" if world > 1 else "single GPU",
                   "construction_s": t_build},
        "frames_per_s": 1e3 / ms_step * world,
        "tet_iterations_per_frame": float(units_b.mean()),
        "gpu_launches": launches,
        "plain": {"form": "one body per launch sequence: 256 single-body solvers in stop mode, one CUDA graph "
                          "each (WHILE node per substep)",
                  "frames": P, "value": float(units_p.sum()) / (sum(ms_p) * 1e-3), "ms_per_step": float(np.mean(ms_p)),
                  "clocks": clk_p.summary()},
        "batched_over_plain": float(sum(ms_p) / sum(ms_b[:P])),
        "equal_residual": {
            "target_rel_residual": target, "residual_floor": floor, "iteration_cap": cap,
            "iteration_counts_equal_fraction": float(np.mean(cnt_b[:P] == cnt_p)),
            "iteration_counts_max_abs_diff": int(np.abs(cnt_b[:P] - cnt_p).max()),
            "executed_tet_iterations_ratio_plain_over_batched": float(units_p.sum() / units_b[:P].sum()),
            "rel_residual_final_median_frame_P": [float(np.nanmedian(rel_b)), float(np.nanmedian(rel_p))],
            "rel_residual_final_max_abs_diff_frame_P": float(np.nanmax(np.abs(rel_b - rel_p))),
            "body_substeps": int(n_sub),
            "fraction_met_target": float(np.mean(met_b)),
            "fraction_at_floor": float(np.mean(floor_b)),
            "fraction_at_cap": float(np.mean(cnt_b == cap)),
            "iterations_percentiles_10_50_90_max": [float(v) for v in np.percentile(cnt_b, [10, 50, 90, 100])],
            "note": "met/floor fractions and the final r_hat_K/r_hat_0 over frame P's body-substeps (batched, then "
                    "plain); cap fraction and percentiles over all timed frames of the batched form"},
        "fixed_iterations": {"iterations": K0, "frames": P,
                             "batched_ms_per_step": float(np.mean(ms_bf)), "plain_ms_per_step": float(np.mean(ms_pf)),
                             "batched_value": units_f / (np.mean(ms_bf) * 1e-3),
                             "plain_value": units_f / (np.mean(ms_pf) * 1e-3),
                             "batched_over_plain": float(np.mean(ms_pf) / np.mean(ms_bf)),
                             "note": "the reference's loop (neohookean_solver.py:474): every body runs 30 "
                                     "iterations per substep"},
        "roofline": {"bound": "hbm", "kernel": "kb_project (batched tile projection, all bodies active)",
                     "achieved": proj_bytes / (proj_ms * 1e-3) / 1e9, "peak": peak, "unit": "GB/s",
                     "frac": proj_bytes / (proj_ms * 1e-3) / 1e9 / peak, "peak_source": peak_src,
                     "traffic": None, "bytes_per_launch": proj_bytes, "ms_per_launch": proj_ms,
                     "timing": "CUDA events around each launch of one fixed-count frame (direct launches)"},
        "iteration_roofline": {"bytes_per_frame": float(bytes_b.mean()),
                               "achieved_GBps": float(bytes_b.sum()) / (sum(ms_b) * 1e-3) / 1e9,
                               "frac": float(bytes_b.sum()) / (sum(ms_b) * 1e-3) / 1e9 / peak,
                               "note": "136 B per tet + 128 B per vertex for every iteration a body ran"},
        "kernel_profile": {k: {"ms_per_launch": v["ms"] / max(1, v["launches"]), "launches": v["launches"]}
                           for k, v in prof.items() if v["launches"]},
        "fp64_error": fp64,
        "e2e": {"value": float(np.sum(e2e_units)) / (np.sum(e2e_ms) * 1e-3), "unit": UNIT,
                "h2d_bytes_per_step": 2 * int(state["x"].nbytes), "d2h_bytes_per_step": int(state["x"].nbytes),
                "ms_per_step": float(np.mean(e2e_ms)),
                "path": "XPBDBatchedSolver.set_positions / set_velocities from pinned host memory, solve(), "
                        "positions() to host"},
        "clocks": clk_b.summary(),
    }
    if batch.autotune_result is not None:
        line["config"]["autotune"] = {"tets_per_thread": batch.tets_per_thread,
                                      "cached": batch.autotune_result["cached"],
                                      "ms_per_substep": {"tpt%d" % r["tets_per_thread"]: r["ms"]
                                                         for r in batch.autotune_result["table"]}}
    return line


def c3_fp64_error(x_gpu, state, batch, bodies, specs, kw, n_sample):
    """Max vertex deviation over the bounding-box diagonal of `n_sample` bodies
    (spread over the sizes) after one fixed-count frame from the settled state:
    the GPU batch against the C restatement in FP64, and the same restatement in
    FP32 against FP64 (what an FP32 run of the reference algorithm departs)."""
    from xpbd_gpu.mesh import TetMesh
    sizes = np.array([b.rest_pose.n_tets for b in bodies])
    pick = [int(k) for k in np.argsort(sizes)[np.linspace(0, len(bodies) - 1, n_sample).astype(int)]]
    threads = os.cpu_count() or 1
    S = kw["substeps_num"]
    out = []
    for k in pick:
        b = bodies[k]
        sl = batch.body_vert_slices[k]
        pts = b.rest_pose.points @ b.rotation.T + np.asarray(b.offset, dtype=np.float64)
        mesh = TetMesh(pts, b.rest_pose.tets)
        kwb = dict(kw, young_modulus=b.young_modulus, poisson_ratio=b.poisson_ratio, density=b.density)
        devs = {}
        for name, dt_ in (("fp64", np.float64), ("fp32", np.float32)):
            o = cpu_oracle(mesh, specs, kwb, S, threads, dtype=dt_)
            o.x[:] = state["x"][sl]
            o.v[:] = state["v"][sl]
            o.rho_hat.value = float(state["rho"][k])
            o.solve()
            devs[name] = o.x.astype(np.float64)
        diag = float(np.linalg.norm(pts.max(0) - pts.min(0)))
        out.append(dict(body=k, tets=int(sizes[k]),
                        max_dev_over_bbox_diag=float(np.abs(x_gpu[sl] - devs["fp64"]).max()) / diag,
                        fp32_reference_max_dev_over_bbox_diag=float(np.abs(devs["fp32"] - devs["fp64"]).max()) / diag))
    return {"reference": "C restatement in FP64 (and FP32), %d threads" % threads, "frames": 1,
            "start": "the settled state of the timed window", "iterations": kw["constraints_iter"],
            "bodies": out, "max_over_bodies": max(b["max_dev_over_bbox_diag"] for b in out),
            "fp32_reference_max_over_bodies": max(b["fp32_reference_max_dev_over_bbox_diag"] for b in out)}


def measured_peak():
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(peaks_path):
        return float(json.load(open(peaks_path))["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


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

def cpu_oracle(mesh, specs, kw, substeps, threads=None, dtype=np.float32):
    """The threaded C restatement of the reference substep on the workload's mesh (FP32, or FP64
    for the float64 reference run), stepping `substeps` substeps of the workload's substep length
    per call."""
    from oracle.xpbd_oracle import OracleSdf
    from oracle.xpbd_oracle_c import COracle
    sub_dt = kw["dt"] / kw["substeps_num"]
    okw = {k: v for k, v in kw.items() if k != "density"}
    okw.update(substeps_num=substeps, frame_dt=sub_dt * substeps, dt=sub_dt * substeps)
    total = kw.get("density", 1.0) * float(np.abs(_volume(mesh)).sum()) if "density" in kw else 1.0
    return COracle(mesh.points, mesh.tets, [OracleSdf(k, **p) for k, p in specs], threads=threads,
                   total_mass=total, dtype=dtype, **okw)


def fp64_error(solver_factory, mesh, specs, kw, frames, warm_start=11, warm_frames=1):
    """Error of the GPU path against the float64 run of the reference algorithm (the C
    restatement in FP64 on every host core): max and RMS vertex deviation as fractions of the
    bounding-box diagonal (a) over `frames` frames from the initial state and (b) over
    `warm_frames` frames in contact, all runs started from the GPU state after `warm_start`
    frames; in (b) also the deviation of the FP32 C restatement from the same state (what an
    FP32 run of the reference algorithm itself departs from FP64), the GPU's deviation from
    that FP32 run, the FP32 run's deviation from itself with its tets renumbered (the same
    arithmetic summed in another order: what float-atomic order alone does to the
    reference), and the relative difference of the per-iteration residual curves (only
    where the float64 r_hat is above 1e-4, well above the FP32 floor of about 1e-5 of a
    body at rest on this mesh)."""
    from xpbd_gpu.mesh import TetMesh
    threads = os.cpu_count() or 1
    S, K = kw["substeps_num"], kw["constraints_iter"]
    diag = float(np.linalg.norm(mesh.points.max(0) - mesh.points.min(0)))
    out = {"tolerance": 1e-4, "reference": "C restatement in FP64, %d threads" % threads}

    def run(solver, ref, n, hist=None):
        worst, t = 0.0, 0.0
        for _ in range(n):
            solver.solve()
            t0 = time.perf_counter()
            ref.solve(1, hist)
            t += time.perf_counter() - t0
            d = np.abs(solver.mesh.verts.x.to_numpy().astype(np.float64) - ref.x)
            worst = max(worst, float(d.max()))
        return worst / diag, float(np.sqrt((d ** 2).sum(1).mean())) / diag, t / max(1, n)

    solver = solver_factory()
    ref = cpu_oracle(mesh, specs, kw, S, threads, dtype=np.float64)
    mx, rms, t = run(solver, ref, frames)
    out["from_rest"] = {"frames": frames, "max_dev_over_bbox_diag": mx, "rms_dev_over_bbox_diag": rms,
                        "fp64_s_per_frame": t}
    if warm_frames > 0:
        for _ in range(max(0, warm_start - frames)):
            solver.solve()
        ref.x[:] = solver.mesh.verts.x.to_numpy()
        ref.v[:] = solver.mesh.verts.v.to_numpy()
        ref.rho_hat.value = solver.rho_hat
        f32 = cpu_oracle(mesh, specs, kw, S, threads, dtype=np.float32)
        perm = np.random.default_rng(7).permutation(mesh.n_tets)
        f32p = cpu_oracle(TetMesh(mesh.points, mesh.tets[perm]), specs, kw, S, threads, dtype=np.float32)
        for o in (f32, f32p):
            o.x[:] = ref.x
            o.v[:] = ref.v
            o.rho_hat.value = ref.rho_hat.value
        hist = np.zeros(S * K)
        mx, rms, t = run(solver, ref, warm_frames, hist)
        h32, h32p = np.zeros(S * K), np.zeros(S * K)
        for _ in range(warm_frames):
            f32.solve(1, h32)
            f32p.solve(1, h32p)
        x_gpu = solver.mesh.verts.x.to_numpy().astype(np.float64)
        x32, x32p = f32.x.astype(np.float64), f32p.x.astype(np.float64)
        r_gpu = solver.read_history()[:S * K, 0]
        live = hist > 1e-4

        def curve(a, b):
            return float((np.abs(a - b)[live] / b[live]).max()) if live.any() else None

        out["in_contact"] = {"start_frame": max(warm_start, frames), "frames": warm_frames,
                             "max_dev_over_bbox_diag": mx, "rms_dev_over_bbox_diag": rms,
                             "fp32_reference_max_dev_over_bbox_diag": float(np.abs(x32 - ref.x).max()) / diag,
                             "gpu_vs_fp32_reference_max_dev_over_bbox_diag": float(np.abs(x_gpu - x32).max()) / diag,
                             "fp32_reference_reordered_vs_itself_max_dev_over_bbox_diag":
                                 float(np.abs(x32p - x32).max()) / diag,
                             "residual_curve_max_rel_diff": curve(r_gpu, hist),
                             "residual_curve_max_rel_diff_fp32_reference_vs_fp64": curve(h32, hist),
                             "residual_curve_max_rel_diff_gpu_vs_fp32_reference": curve(r_gpu, h32),
                             "residual_curve_max_rel_diff_fp32_reordered_vs_fp32": curve(h32p, h32),
                             "residual_iterations_compared": int(live.sum()), "fp64_s_per_frame": t,
                             "note": "every run starts from the GPU state (positions, velocities, rho_hat); the "
                                     "reordered FP32 run numbers the tets in a random order (seed 7)"}
    return out


def _volume(mesh):
    P = mesh.points[mesh.tets]
    return np.einsum("ij,ij->i", np.cross(P[:, 1] - P[:, 0], P[:, 2] - P[:, 0]), P[:, 3] - P[:, 0]) / 6.0


def cpu_baseline(mesh, specs, kw, substeps=5):
    """Time `substeps` substeps (x constraints_iter Jacobi iterations) of the workload with
    the C restatement on every host core; returns tet-iterations/s and the sample text."""
    threads = os.cpu_count() or 1
    c = cpu_oracle(mesh, specs, kw, substeps, threads)
    t0 = time.perf_counter()
    c.solve()
    el = time.perf_counter() - t0
    units = mesh.n_tets * substeps * kw["constraints_iter"]
    return dict(value=units / el, unit=UNIT, cores=threads, kind="port",
                sample="C restatement (FP32, %d threads), %d substeps x %d iterations of the same mesh and "
                       "substep length (%d tet-iterations, %.1f s)" % (threads, substeps, kw["constraints_iter"],
                                                                        units, el))


# ---------------------------------------------------------------------------
# clocks
# ---------------------------------------------------------------------------

class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap,clocks.mem,"
              "temperature.gpu")

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
        sm, smax, mem, temp, reasons = [], [], [], [], set()
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
            for lst, k in ((mem, 9), (temp, 10)):
                try:
                    lst.append(float(f[k]))
                except (ValueError, IndexError):
                    pass
        if not sm:
            return None
        out = {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(smax)), "reasons": sorted(reasons),
               "samples": len(sm)}
        if mem:
            out["mem_mhz"] = float(np.median(mem))
        if temp:
            out["temp_c"] = float(max(temp))
        return out


# ---------------------------------------------------------------------------
# arms
# ---------------------------------------------------------------------------

def dist_info():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("LOCAL_RANK", 0)), int(os.environ.get("WORLD_SIZE", 1))


def max_over_ranks(value, device=None):
    """MAX of a float over all ranks of the process group (the replicas' timing
    reduction); the value itself without a group or with one rank."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(units_per_step, steps, world, max_total_ms):
    """Whole-job throughput of `world` independent replicas that each processed
    `units_per_step` x `steps` units, timed by the slowest rank."""
    return units_per_step * steps * world / (max_total_ms * 1e-3)


def c3_oracles(bodies, specs, kw, dtype=np.float32):
    """The C restatement of every body of the 256-body workload, each stepping
    one substep (the workload's constraints_iter iterations) per call; a body
    uses one host thread per 8192 of its tets (all threads for the largest)."""
    from xpbd_gpu.mesh import TetMesh
    threads = os.cpu_count() or 1
    out = []
    for b in bodies:
        pts = b.rest_pose.points @ b.rotation.T + np.asarray(b.offset, dtype=np.float64)
        mesh = TetMesh(pts, b.rest_pose.tets)
        kwb = dict(kw, young_modulus=b.young_modulus, poisson_ratio=b.poisson_ratio, density=b.density)
        out.append(cpu_oracle(mesh, specs, kwb, 1, max(1, min(threads, mesh.n_tets // 8192)), dtype))
    return out, threads


def cpu_baseline_c3(bodies, specs, kw):
    """One substep of all 256 bodies (30 iterations each, the reference's loop)
    with the C restatement on the host cores: tet-iterations/s."""
    oracles, threads = c3_oracles(bodies, specs, kw)
    t0 = time.perf_counter()
    for c in oracles:
        c.solve()
    el = time.perf_counter() - t0
    units = sum(len(c.tets) for c in oracles) * kw["constraints_iter"]
    return dict(value=units / el, unit=UNIT, cores=threads, kind="port",
                sample="C restatement (FP32, up to %d threads per body): one substep of all 256 bodies x %d "
                       "iterations from the initial state (%d tet-iterations, %.1f s)"
                       % (threads, kw["constraints_iter"], units, el))


def run_reference(args):
    """The reference arm: the reference's algorithm on the host cores.  The reference's
    own Taichi CPU backend cannot be installed on this machine (no Taichi wheel for
    Python 3.12, no network), so this times the C restatement on all host threads;
    one step = one substep of the workload (constraints_iter Jacobi iterations; for
    c3 one substep of all 256 bodies, each at the reference's 30 iterations)."""
    rank, _, world = dist_info()
    if rank != 0:
        return
    if args.workload == "c3":
        bodies, specs, kw, desc = workload_c3()
        oracles, threads = c3_oracles(bodies, specs, kw)
        step = lambda: [c.solve() for c in oracles]
        for _ in range(args.warmup):
            step()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            step()
        el = time.perf_counter() - t0
        units = sum(len(c.tets) for c in oracles) * kw["constraints_iter"] * args.steps
        v = units / el
        sample = ("C restatement of the reference substep (FP32, up to %d threads per body): %d substeps of all 256 "
                  "bodies x %d iterations, %.1f s" % (threads, args.steps, kw["constraints_iter"], el))
        line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": el / args.steps * 1e3,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic",
                "config": {"workload": desc, "step": "one substep of all 256 bodies at the reference's fixed "
                                                     "30 iterations (%d tet-iterations)" % (units // args.steps)},
                "frames_per_s": v / (units / args.steps * kw["substeps_num"]),
                "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
                "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return
    mesh, specs, kw, desc = workload(args.workload)
    threads = os.cpu_count() or 1
    c = cpu_oracle(mesh, specs, kw, 1, threads)
    for _ in range(args.warmup):
        c.solve()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        c.solve()
    el = time.perf_counter() - t0
    units = mesh.n_tets * kw["constraints_iter"] * args.steps
    v = units / el
    frame_units = tet_iterations_per_frame(mesh, kw)
    sample = ("C restatement of the reference substep (FP32, %d threads): %d substeps x %d iterations, %.1f s"
              % (threads, args.steps, kw["constraints_iter"], el))
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": el / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": {"workload": desc, "step": "one substep (%d tet-iterations)"
                                            % (mesh.n_tets * kw["constraints_iter"])},
            "frames_per_s": v / frame_units,
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def c2_line(args, workload_name, world=1, barrier=lambda: None, cpu_substeps=None):
    """The single-body plain GPU form on `workload_name` (c2: the 64^3 cube):
    frames replayed from the frame graph, per-kernel times, e2e, CPU
    baseline, error against the FP64 run.  Returns the JSON dict (None on
    ranks other than 0)."""
    import torch
    from xpbd_gpu.neohookean_solver import XPBDNeoHookeanSolver, frame_chunks
    rank = dist_info()[0]
    mesh, specs, kw, desc = workload(workload_name)
    t_build = time.perf_counter()
    solver = XPBDNeoHookeanSolver(mesh, product_sdfs(specs), scatter=args.scatter, sweep_order=args.sweep_order,
                                  patch_pipeline=args.patch_pipeline, patch_reduce=args.patch_reduce,
                                  tets_per_thread=args.tets_per_thread, pair_tets=bool(args.pair_tets), **kw)
    t_build = time.perf_counter() - t_build
    # the configuration that runs (the autotuner's pick with --scatter auto)
    scatter, tpt, pipe = solver.scatter, solver.tets_per_thread, solver.patch_pipeline
    patch_tets = solver._patch_tets if scatter == "patch" else 0
    frame_units = tet_iterations_per_frame(mesh, kw)
    n_chunks = len(frame_chunks(kw["frame_dt"], kw["dt"]))
    per_substep = 2 + kw["constraints_iter"] * (3 + (1 if scatter == "gather" else 0))
    launches_per_frame = n_chunks * kw["substeps_num"] * per_substep
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()

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
    total_ms = max_over_ranks(float(sum(ms)), device="cuda")
    ms_per_step = total_ms / args.steps
    value = replica_throughput(frame_units, args.steps, world, total_ms)
    solver.check_status()

    # per-kernel durations: the same frames, each launch bracketed by events (event record
    # nodes in the frame graph)
    solver.set_profiling(True)
    solver.read_profile(reset=True)
    for _ in range(args.profile_steps):
        flush.fill_(1.0)
        solver.solve()
    prof = solver.read_profile(reset=True)
    solver.set_profiling(False)
    assert sum(v["launches"] for v in prof.values()) == launches_per_frame * args.profile_steps, prof

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
        return None
    peak, peak_src = measured_peak()
    K = kw["constraints_iter"]
    n_proj = prof["project"]["launches"]
    # algorithmic bytes of one projection launch (per-unit figures of the
    # reference-semantics accounting): per tet 16 ids + 36 inv_Dm + 4 V0 +
    # 8 lambda read + 8 lambda write = 72 B; per vertex 16 gather + 16 scatter
    proj_bytes = 72.0 * T + 32.0 * V
    proj_ms = prof["project"]["ms"] / max(1, n_proj)
    achieved = proj_bytes / (proj_ms * 1e-3) / 1e9
    if scatter == "patch" and pipe == 1 and patch_tets == 256:
        kernel_name = "k_project_tile (persistent CTAs, cp.async.bulk tet records, 256-tet patches)"
    elif scatter == "patch" and tpt > 1 and not args.patch_reduce:
        kernel_name = ("k_project_patchN (tile, %d-tet patches, %d consecutive tets per thread, shared corners "
                       "merged before red.global.add.v4)" % (patch_tets, tpt))
    elif scatter == "patch":
        kernel_name = "k_project_patch1 (tile, %d-tet patches, red.global.add.v4 per corner)" % patch_tets
    else:
        kernel_name = {"atomic": "k_project (one thread per tet, red.global.add.v4 per corner)",
                       "gather": "k_project (per-corner buffer + deterministic vertex gather)"}[scatter]
    iter_bytes = 136.0 * T + 128.0 * V
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": desc, "step": "one frame (%d tet-iterations)" % frame_units,
                   "scatter": scatter, "patch_tets": patch_tets, "sweep_order": args.sweep_order,
                   "patch_pipeline": pipe, "tets_per_thread": tpt, "tet_pairs": solver.n_tet_pairs,
                   "records_evict_last": bool(solver.set_l2_hint()),
                   "l2": "flushed between steps (%d MiB write)" % (L2_FLUSH_BYTES >> 20),
                   "parallelism": "replicas" if world > 1 else "single GPU", "graph": "one CUDA graph per frame"},
        "frames_per_s": 1e3 / ms_per_step * world,
        "gpu_launches": launches_per_frame * args.steps,
        "roofline": {"bound": "hbm", "kernel": kernel_name,
                     "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_source": peak_src, "traffic": None,
                     "bytes_per_launch": proj_bytes, "ms_per_launch": proj_ms,
                     "timing": "CUDA events recorded by event nodes inside the frame graph (the timed "
                               "region's graph plus those nodes), %d frames after the timed region"
                               % args.profile_steps},
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
    if solver.autotune_result is not None:
        r = solver.autotune_result
        line["config"]["autotune"] = {
            "cached": r["cached"], "construction_s": t_build,
            "ms_per_substep": {"%s/P%s/tpt%s/pipe%s" % (c["scatter"], c["patch_tets"], c["tets_per_thread"],
                                                         c["patch_pipeline"]): c["ms"] for c in r["table"]}}
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(mesh, specs, kw, substeps=cpu_substeps or args.cpu_substeps)
    if args.fp64_frames > 0:
        del solver
        line["fp64_error"] = fp64_error(
            lambda: XPBDNeoHookeanSolver(mesh, product_sdfs(specs), scatter=scatter, sweep_order=args.sweep_order,
                                         patch_pipeline=pipe, patch_reduce=args.patch_reduce, tets_per_thread=tpt,
                                         patch_tets=patch_tets or 256, pair_tets=bool(args.pair_tets), **kw),
            mesh, specs, kw, args.fp64_frames, warm_start=args.fp64_warm_start, warm_frames=args.fp64_warm_frames)
    return line


def run_gb300(args):
    """The GB300 arm.  Default (c3): the metric's 256-body batch at equal
    residual, with the 64^3 single body (c2), the differentiable cube's
    adjoint cost (c4) and the batched differentiable form against the plain
    per-body form (c5, a few Adam steps) as extra keys of the same line."""
    import torch
    rank, local_rank, world = dist_info()
    torch.cuda.set_device(local_rank)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    if args.workload == "c3":
        line = c3_headline(args, world, barrier)
        if line is None:
            return
        bodies, specs, kw, _ = workload_c3()
        line["cpu_baseline"] = cpu_baseline_c3(bodies, specs, kw)
        if not args.no_extra:
            line["c2"] = c2_line(args, "c2", cpu_substeps=5)
            line["c4"] = c4_block(args)
            line["c5"] = c5_block(args, args.c5_bench_steps, plain_accuracy_bodies=0, fp64_bodies=3)
    else:
        line = c2_line(args, args.workload, world, barrier)
        if line is None:
            return
    print(json.dumps(line), flush=True)


def run_profile(args):
    """Frames with direct launches and no timing, for an external profiler."""
    import torch
    from xpbd_gpu.neohookean_solver import XPBDNeoHookeanSolver
    if args.workload == "c3":  # the batched form alone
        # `profile_settle` frames at the fixed 30 iterations (frame graphs), then
        # `profile_frames` frames in stop mode (with --profile-stop) or at the fixed
        # count, as direct launches
        from xpbd_gpu.batched import XPBDBatchedSolver
        bodies, specs, kw, desc = workload_c3()
        cap = args.c3_cap if args.profile_stop else kw["constraints_iter"]
        batch = XPBDBatchedSolver(bodies, product_sdfs(specs), tets_per_thread=min(args.tets_per_thread, 2),
                                  use_graph=True, pair_tets=bool(args.pair_tets), **dict(kw, constraints_iter=cap))
        batch.set_stop(0.0, 0.0, kw["constraints_iter"])
        for _ in range(args.profile_settle):
            batch.solve()
        batch.use_graph = False
        if args.profile_stop:
            batch.set_stop(args.c3_target, args.c3_floor, cap)
        else:
            batch.set_stop(0.0, 0.0, kw["constraints_iter"])
        torch.cuda.synchronize()
        # the profiled frames sit in the NVTX range "frames" (ncu --nvtx --nvtx-include frames/)
        torch.cuda.nvtx.range_push("frames")
        for _ in range(args.profile_frames):
            batch.solve()
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_pop()
        batch.check_status()
        print("profile mode: %d settle frame(s) + %d %s frame(s) of %s (batched)" % (
            args.profile_settle, args.profile_frames, "stop-mode" if args.profile_stop else "fixed-count", desc))
        return
    if args.workload == "c5":  # batched forward + adjoint of `profile_frames` frames
        from xpbd_gpu.batched import Body
        from xpbd_gpu.differentiable import BatchedDiffSim, xpbd_simulate_batch
        meshes, log_E, nus, specs, kw, desc = workload_c5()
        bodies = [Body(m, tet_young_modulus=np.exp(log_E[k]), tet_poisson_ratio=nus[k], density=1000.0,
                       poisson_ratio=float(nus[k])) for k, m in enumerate(meshes)]
        sim = BatchedDiffSim(bodies, product_sdfs(specs), use_graphs=False, tape_memory=args.profile_tape_memory,
                             **kw)
        dev = torch.device("cuda")
        x0 = torch.tensor(np.concatenate([m.points for m in meshes]), dtype=torch.float32, device=dev)
        le = torch.tensor(np.concatenate(log_E), dtype=torch.float64, device=dev, requires_grad=True)
        nu = torch.tensor(np.concatenate([np.full(m.n_tets, nus[k]) for k, m in enumerate(meshes)]), device=dev)
        xf = xpbd_simulate_batch(sim, x0, torch.zeros_like(x0), le, nu, args.profile_frames)
        (xf ** 2).sum().backward()
        torch.cuda.synchronize()
        sim.batch.check_status()
        print("profile mode: forward + adjoint of %d frame(s) of %s" % (args.profile_frames, desc))
        return
    mesh, specs, kw, desc = workload(args.workload)
    scatter = "patch" if args.scatter == "auto" else args.scatter
    solver = XPBDNeoHookeanSolver(mesh, product_sdfs(specs), scatter=scatter, sweep_order=args.sweep_order,
                                  patch_pipeline=args.patch_pipeline, patch_reduce=args.patch_reduce,
                                  tets_per_thread=args.tets_per_thread, use_graph=False,
                                  pair_tets=bool(args.pair_tets), **kw)
    for _ in range(args.profile_frames):
        solver.solve()
    torch.cuda.synchronize()
    solver.check_status()
    print("profile mode: %d frame(s) of %s" % (args.profile_frames, desc))


def make_parser():
    """The command line of bench.py (also used to check the commands quoted in
    the profile summaries)."""
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="c3", choices=["c2", "c1", "c3", "c4", "c5", "matrix"])
    ap.add_argument("--mesh", default=None, help="matrix workload: a TetGen .node path (e.g. the reference's "
                                                 "assets/tetmesh/armadillo.node)")
    ap.add_argument("--matrix-frame", type=int, default=300, help="matrix workload: the recorded frame")
    ap.add_argument("--matrix-scale", type=float, default=0.01, help="matrix workload: the mesh scale")
    ap.add_argument("--c3-cap", type=int, default=200, help="iteration cap of the equal-residual runs")
    ap.add_argument("--c3-target", type=float, default=1e-3, help="r_hat_k / r_hat_0 target")
    ap.add_argument("--c3-floor", type=float, default=1e-5, help="r_hat below which a substep has converged")
    ap.add_argument("--c3-settle", type=int, default=90, help="frames stepped before the timed window")
    ap.add_argument("--c3-plain-frames", type=int, default=4, help="timed frames of the plain form")
    ap.add_argument("--c3-fp64-bodies", type=int, default=8, help="bodies checked against FP64")
    ap.add_argument("--no-extra", action="store_true", help="c3 line without the c2 / c4 / c5 keys")
    ap.add_argument("--c5-frames", type=int, default=30)
    ap.add_argument("--c5-adam-steps", type=int, default=200)
    ap.add_argument("--c5-lr", type=float, default=0.05)
    ap.add_argument("--c5-plain-bodies", type=int, default=4, help="bodies of the plain-form accuracy run")
    ap.add_argument("--c5-bench-steps", type=int, default=4, help="Adam steps of the c5 key of the default line")
    ap.add_argument("--c4-frames", type=int, default=60)
    ap.add_argument("--c4-reps", type=int, default=2)
    ap.add_argument("--c4-check-frames", type=int, default=1)
    ap.add_argument("--c4-check-start", type=int, default=20)
    ap.add_argument("--scatter", default="auto", choices=["auto", "atomic", "gather", "patch"])
    ap.add_argument("--sweep-order", type=int, default=1, choices=[0, 1])
    ap.add_argument("--patch-pipeline", type=int, default=0, choices=[0, 1])
    ap.add_argument("--patch-reduce", type=int, default=0, choices=[0, 1])
    ap.add_argument("--tets-per-thread", type=int, default=2, choices=[1, 2, 4])
    ap.add_argument("--batch-tpt", default="auto", choices=["auto", "1", "2"])
    ap.add_argument("--pair-tets", type=int, default=1, choices=[0, 1],
                    help="order face-adjacent tets in corner-aligned pairs (xpbd_pair_tets)")
    ap.add_argument("--profile-steps", type=int, default=2)
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--cpu-substeps", type=int, default=20)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--fp64-frames", type=int, default=1)
    ap.add_argument("--fp64-warm-start", type=int, default=11)
    ap.add_argument("--fp64-warm-frames", type=int, default=1)
    ap.add_argument("--mode", default="bench", choices=["bench", "profile"])
    ap.add_argument("--profile-frames", type=int, default=1)
    ap.add_argument("--profile-settle", type=int, default=0, help="c3 profile mode: frames stepped first (graphs)")
    ap.add_argument("--profile-stop", type=int, default=0, choices=[0, 1], help="c3 profile mode: stop-mode frames")
    ap.add_argument("--profile-tape-memory", default="auto", choices=["auto", "store", "recompute"],
                    help="c5 profile mode: tapes stored by the forward or recomputed by the backward")
    return ap


def main():
    ap = make_parser()
    args = ap.parse_args()
    if args.mode == "profile":
        run_profile(args)
    elif args.workload == "c4" and args.impl != "reference":
        run_c4(args)
    elif args.workload == "c5" and args.impl != "reference":
        run_c5(args)
    elif args.workload == "matrix":
        if not args.mesh:
            ap.error("--workload matrix needs --mesh")
        run_matrix(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
