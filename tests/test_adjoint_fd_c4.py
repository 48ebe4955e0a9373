"""The float64 adjoint at the differentiable workload's size, against FP64
central finite differences along 32 seeded directions.

Scene: the 16^3 Kuhn cube (24,576 tets, 4,913 vertices) with the per-tet
log E field of the differentiable workload (mean log 1e5, sigma 0.5), nu =
0.45, the plane y = 0, thrown at the plane so that the horizon -- two
substeps of 1/300 s with 20 Jacobi iterations each, the workload's substep --
runs in contact.  Loss: c . x_final for a seeded c.

Two finite-difference functions (step 1e-4, central):
* omega replayed: the Chebyshev factors of the unperturbed run are replayed,
  the stop-gradient convention of the adjoint (oracle/xpbd_adjoint.py).  This
  is the function the adjoint differentiates: the directional derivatives of
  log E, nu and the initial velocity must match within 1e-3 of the RMS of the
  finite differences (32 directions each for log E and v0, nu is a scalar).
* omega recomputed from the residuals, as the forward runs: the difference to
  the adjoint is the gradient error of treating omega as a stop-gradient,
  reported on 8 directions each.  It stays below 1e-2 of the RMS for log E
  and the initial velocity; for nu, which moves every tet's compliance and
  with it the residual curve that omega follows, it is large (measured
  0.41), so no bound is asserted for nu.

The finite-difference runs are spread over a spawn process pool.
"""
import multiprocessing as mp
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
H = 1e-4
N_DIR = 32
N_DIR_OMEGA = 8

_SCENE = {}


def _scene():
    for p in (ROOT, os.path.join(ROOT, "rdc-xpbd-taichi_gb300")):
        if p not in sys.path:
            sys.path.insert(0, p)
    import bench
    from oracle.xpbd_oracle import OracleSdf
    mesh, specs, kw, log_E, _ = bench.workload_c4()
    x0 = mesh.points.copy()
    x0[:, 1] -= x0[:, 1].min() - 0.002          # 2 mm above the plane
    v0 = np.zeros_like(x0)
    v0[:] = (0.3, -1.5, 0.2)                     # thrown at it
    sub_dt = kw["dt"] / kw["substeps_num"]
    okw = dict(frame_dt=2 * sub_dt, dt=2 * sub_dt, substeps_num=2, constraints_iter=kw["constraints_iter"],
               cheb_enable=True, cheb_warmup=kw["cheb_warmup"], cheb_gamma=kw["cheb_gamma"],
               total_mass=kw["total_mass"])
    sdfs = [OracleSdf(k, **p) for k, p in specs]
    c = np.random.default_rng(11).normal(size=x0.shape)
    return dict(points=mesh.points, tets=mesh.tets, sdfs=sdfs, okw=okw, log_E=log_E, nu=0.45, x0=x0, v0=v0, c=c)


def _direction(kind, k, shape):
    return np.random.default_rng(1000 * {"log_E": 1, "v0": 2, "nu": 3}[kind] + k).normal(size=shape)


def _loss(s, log_E, nu, v0, omegas):
    from oracle.xpbd_adjoint import DiffOracle, lame_inverse
    im, il = lame_inverse(log_E, nu)
    o = DiffOracle(s["points"], s["tets"], s["sdfs"], im, il, **s["okw"])
    xe, _, _, _ = o.run(s["x0"], v0, 1, omegas=omegas)
    return float((s["c"] * xe).sum())


def _init(omegas):
    _SCENE.update(_scene())
    _SCENE["omegas"] = omegas


def _fd_task(task):
    kind, k, replay = task
    s = _SCENE
    d = _direction(kind, k, np.shape(s[kind]) if kind != "nu" else ())
    vals = []
    for sign in (1.0, -1.0):
        args = dict(log_E=s["log_E"], nu=s["nu"], v0=s["v0"])
        args[kind] = args[kind] + sign * H * d
        vals.append(_loss(s, args["log_E"], args["nu"], args["v0"], s["omegas"] if replay else None))
    return kind, k, replay, (vals[0] - vals[1]) / (2 * H)


def _adjoint(s, omega_grad):
    from oracle.xpbd_adjoint import DiffOracle, lame_inverse, lame_inverse_grad
    im, il = lame_inverse(s["log_E"], s["nu"])
    o = DiffOracle(s["points"], s["tets"], s["sdfs"], im, il, omega_grad=omega_grad, **s["okw"])
    oms, xb, vb, gm, gl, _ = o.gradient(s["x0"], s["v0"], 1, s["c"])
    g_logE, g_nu = lame_inverse_grad(s["log_E"], np.full(len(s["log_E"]), s["nu"]), gm, gl)
    return oms, {"log_E": g_logE, "nu": float(g_nu.sum()), "v0": vb}


def test_c4_size_adjoint_against_central_differences():
    s = _scene()
    oms, grads = _adjoint(s, False)
    _, grads_om = _adjoint(s, True)
    tasks = [("log_E", k, True) for k in range(N_DIR)] + [("v0", k, True) for k in range(N_DIR)]
    tasks += [("nu", 0, True), ("nu", 0, False)]
    tasks += [("log_E", k, False) for k in range(N_DIR_OMEGA)] + [("v0", k, False) for k in range(N_DIR_OMEGA)]
    ctx = mp.get_context("spawn")
    with ctx.Pool(min(len(tasks), os.cpu_count() or 1), initializer=_init, initargs=(oms,)) as pool:
        results = pool.map(_fd_task, tasks)
    report = {}
    for replay in (True, False):
        for kind in ("log_E", "v0", "nu"):
            rows = [(k, fd) for kd, k, rp, fd in results if kd == kind and rp == replay]
            fd = np.array([r[1] for r in rows])
            rms = float(np.sqrt(np.mean(fd ** 2)))
            for label, g in (("stop", grads), ("through_omega", grads_om)):
                an = np.array([float(np.sum(g[kind] * _direction(kind, k, np.shape(g[kind]))))
                               if kind != "nu" else g[kind] * float(_direction(kind, k, ())) for k, _ in rows])
                report[(kind, replay, label)] = float(np.max(np.abs(fd - an))) / rms
    print("max |FD - adjoint| / RMS(FD):", {"%s/%s/%s" % (k, "replayed" if r else "recomputed", lb): "%.2e" % v
                                            for (k, r, lb), v in report.items()})
    for kind in ("log_E", "v0", "nu"):
        # the stop-gradient adjoint is the derivative of the omega-replayed function
        assert report[(kind, True, "stop")] <= 1e-3, (kind, report[(kind, True, "stop")])
        # through omega, the adjoint is the derivative of the forward as it runs
        assert report[(kind, False, "through_omega")] <= 1e-3, (kind, report[(kind, False, "through_omega")])
