"""The float64 adjoint (oracle/xpbd_adjoint.py) against central finite differences.

Two conventions for the Chebyshev omega.  With omega as a stop-gradient the
finite differences replay the recorded omega schedule; with omega_grad the
adjoint runs back through omega -> rho_hat -> the residual sweep, and the
finite differences recompute omega from the residuals as the forward does.
Gradients w.r.t. per-tet log E and nu, initial positions and initial
velocities are checked along random directions; relative error of the
directional derivatives <= 1e-5.
"""
import numpy as np
import pytest

from oracle.xpbd_adjoint import DiffOracle, lame_inverse, lame_inverse_grad, project_adjoint, project_forward
from oracle.xpbd_oracle import OracleSdf


def test_projection_adjoint_matches_finite_differences():
    rng = np.random.default_rng(0)
    T = 5
    P = rng.normal(size=(T, 4, 3)) * 0.3 + np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1.0]])
    Dm = np.linalg.inv(np.stack([[[1, 0, 0], [0, 1, 0], [0, 0, 1.0]]] * T) + rng.normal(size=(T, 3, 3)) * 0.1)
    w = rng.uniform(0.5, 2.0, size=(T, 4))
    w[0, 2] = 0.0
    lam = rng.normal(size=(T, 2)) * 0.1
    aD, aH = rng.uniform(0.1, 1.0, T), rng.uniform(0.01, 0.1, T)
    cdp = rng.normal(size=(T, 4, 3))
    cl = rng.normal(size=(T, 2))

    def f(P_, lam_, aD_, aH_):
        dp, dl, _ = project_forward(P_, Dm, w, lam_, aD_, aH_)
        return (cdp * dp).sum() + (cl * dl).sum()

    _, _, cache = project_forward(P, Dm, w, lam, aD, aH)
    Pb, lb, aDb, aHb = project_adjoint(P, Dm, w, lam, aD, aH, cdp, cl, cache)
    lb = lb + cl  # lambda_{k+1} = lambda_k + dlam
    h = 1e-6
    for arr, grad, name in ((P, Pb, "P"), (lam, lb - cl, "lam"), (aD, aDb, "aD"), (aH, aHb, "aH")):
        d = rng.normal(size=arr.shape)
        args = dict(P_=P, lam_=lam, aD_=aD, aH_=aH)
        key = {"P": "P_", "lam": "lam_", "aD": "aD_", "aH": "aH_"}[name]
        ap = dict(args)
        am = dict(args)
        ap[key] = arr + h * d
        am[key] = arr - h * d
        fd = (f(**ap) - f(**am)) / (2 * h)
        an = (grad * d).sum()
        assert abs(fd - an) <= 1e-6 * max(1.0, abs(fd)), (name, fd, an)


def _scene(seed=0):
    from xpbd_gpu.mesh import kuhn_grid
    m = kuhn_grid(2, 2, 2, 0.1, origin=(0.35, 0.012, 0.35), jitter=0.1, seed=seed)
    sdfs = [OracleSdf("plane", point=[0, 0, 0], dir=[0, 1, 0], fixed=True),
            OracleSdf("sphere", center=[0.45, -0.2, 0.45], radius=0.22, fixed=True),
            OracleSdf("cube", center=[0.55, 0.0, 0.55], size=[0.1, 0.03, 0.2], fixed=False)]
    return m, sdfs


@pytest.mark.parametrize("cheb,omega_grad", [(True, False), (False, False), (True, True)])
def test_trajectory_gradients_match_finite_differences(cheb, omega_grad):
    m, sdfs = _scene()
    T = m.n_tets
    rng = np.random.default_rng(1)
    logE = np.log(1e5) + 0.3 * rng.normal(size=T)
    nu = np.full(T, 0.4) + 0.02 * rng.normal(size=T)
    kw = dict(frame_dt=1 / 60, dt=1 / 60, substeps_num=2, constraints_iter=6, cheb_enable=cheb, cheb_warmup=2,
              cheb_gamma=0.6666, total_mass=1.0)
    x0 = m.points.copy()
    if omega_grad:
        # r_hat sums sqrt(rD^2 + rH^2) over tets, a cone with its apex at the rest
        # shape: a strained start keeps the tets off the apex, where the omega
        # chain is smooth enough for central differences
        x0 += 0.005 * np.random.default_rng(5).normal(size=x0.shape)
    v0 = rng.normal(size=x0.shape) * 0.05
    c = rng.normal(size=x0.shape)
    frames = 2

    def loss(logE_, nu_, x_, v_, oms):
        im, il = lame_inverse(logE_, nu_)
        o = DiffOracle(m.points, m.tets, sdfs, im, il, **kw)
        xe, _, _, _ = o.run(x_, v_, frames, omegas=None if omega_grad else oms)
        return float((c * xe).sum())

    im, il = lame_inverse(logE, nu)
    o = DiffOracle(m.points, m.tets, sdfs, im, il, omega_grad=omega_grad, **kw)
    oms, xb, vb, gm, gl, _ = o.gradient(x0, v0, frames, c)
    g_logE, g_nu = lame_inverse_grad(logE, nu, gm, gl)
    assert np.isfinite(g_logE).all()
    # FD steps: 1e-4 for the materials (the loss is O(10) while d/dlogE is O(1e-5),
    # smaller steps drown in round-off), 1e-5 for the states (1e-6 through omega)
    hs = 1e-6 if omega_grad else 1e-5
    for name, base, grad, h in (("logE", logE, g_logE, 1e-4), ("nu", nu, g_nu, 1e-4), ("x0", x0, xb, hs),
                                ("v0", v0, vb, hs)):
        d = rng.normal(size=base.shape)
        args = {"logE": logE, "nu": nu, "x0": x0, "v0": v0}
        ap = dict(args)
        am = dict(args)
        ap[name] = base + h * d
        am[name] = base - h * d
        fd = (loss(ap["logE"], ap["nu"], ap["x0"], ap["v0"], oms)
              - loss(am["logE"], am["nu"], am["x0"], am["v0"], oms)) / (2 * h)
        an = float((grad * d).sum())
        assert abs(fd - an) <= 1e-5 * max(abs(fd), 1e-8), (name, fd, an)
