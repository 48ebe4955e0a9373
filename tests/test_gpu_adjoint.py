"""GPU adjoint kernels against the float64 adjoint of the oracle.

The oracle adjoint (oracle/xpbd_adjoint.py) is checked against central finite
differences in tests/test_adjoint_oracle.py; here the GPU gradients of a
linear loss on the final positions w.r.t. per-tet log E, nu, the initial
positions and velocities must match it within 1e-3 relative (L2 norm of the
difference over the norm of the gradient), on a body with plane, sphere and
moving-box contact: with the adjoint run back through the Chebyshev omega
(omega_grad, the derivative of the forward as it runs) and with omega as a
stop-gradient, with the tapes stored by the forward and recomputed by the
backward.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


@pytest.mark.parametrize("cheb,omega_grad,tape_memory,iters", [
    (True, True, "store", 8), (True, True, "recompute", 8), (True, False, "store", 8), (False, False, "recompute", 8),
    # more than 32 iterations: the omega chain's table spans two warp scans
    (True, True, "store", 40)])
def test_gpu_gradients_match_float64_adjoint(cheb, omega_grad, tape_memory, iters):
    import torch
    from oracle.xpbd_adjoint import DiffOracle, lame_inverse, lame_inverse_grad
    from oracle.xpbd_oracle import OracleSdf
    from xpbd_gpu.differentiable import DiffSim, xpbd_simulate
    from xpbd_gpu.mesh import kuhn_grid
    from xpbd_gpu.sdf import CubeSdf, PlaneSdf, SphereSdf
    m = kuhn_grid(3, 3, 3, 0.08, origin=(0.3, 0.015, 0.3), jitter=0.1, seed=4)
    T = m.n_tets
    rng = np.random.default_rng(7)
    logE = np.log(1e5) + 0.3 * rng.normal(size=T)
    nu = np.clip(0.4 + 0.03 * rng.normal(size=T), 0.3, 0.48)
    v0 = rng.normal(size=m.points.shape) * 0.05
    c = rng.normal(size=m.points.shape)
    kw = dict(frame_dt=1 / 60, dt=1 / 60, substeps_num=2, constraints_iter=iters, cheb_enable=cheb, cheb_warmup=3,
              cheb_gamma=0.6666, total_mass=1.0)
    frames = 2
    o = DiffOracle(m.points, m.tets,
                   [OracleSdf("plane", point=[0, 0, 0], dir=[0, 1, 0], fixed=True),
                    OracleSdf("sphere", center=[0.42, -0.18, 0.42], radius=0.2, fixed=True),
                    OracleSdf("cube", center=[0.5, 0.0, 0.5], size=[0.1, 0.03, 0.2], fixed=False)],
                   *lame_inverse(logE, nu), omega_grad=omega_grad, **kw)
    _, xb, vb, gm, gl, xe64 = o.gradient(m.points.copy(), v0, frames, c)
    g_logE64, g_nu64 = lame_inverse_grad(logE, nu, gm, gl)

    sim = DiffSim(m, [PlaneSdf([0, 0, 0], [0, 1, 0], True), SphereSdf([0.42, -0.18, 0.42], 0.2, True),
                      CubeSdf([0.5, 0.0, 0.5], [0.1, 0.03, 0.2], False)], logE, nu, omega_grad=omega_grad,
                  tape_memory=tape_memory, **kw)
    dev = torch.device("cuda")
    x0_t = torch.tensor(m.points, dtype=torch.float32, device=dev, requires_grad=True)
    v0_t = torch.tensor(v0, dtype=torch.float32, device=dev, requires_grad=True)
    le_t = torch.tensor(logE, dtype=torch.float64, device=dev, requires_grad=True)
    nu_t = torch.tensor(nu, dtype=torch.float64, device=dev, requires_grad=True)
    xf = xpbd_simulate(sim, x0_t, v0_t, le_t, nu_t, frames)
    diag = float(np.linalg.norm(m.points.max(0) - m.points.min(0)))
    assert np.abs(xf.detach().cpu().numpy() - xe64).max() <= 1e-4 * diag
    loss = (xf.double() * torch.tensor(c, device=dev)).sum()
    loss.backward()
    assert _rel(le_t.grad.cpu().numpy(), g_logE64) < 1e-3
    assert _rel(nu_t.grad.cpu().numpy(), g_nu64) < 1e-3
    assert _rel(x0_t.grad.cpu().numpy(), xb) < 1e-3
    assert _rel(v0_t.grad.cpu().numpy(), vb) < 1e-3
