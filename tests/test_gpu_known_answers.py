"""GPU known-answer tests: analytic cases that need no oracle, up to the
largest single-body size of the benchmarks (64^3 cells, 1,572,864 tets).

* rest state: without gravity or contact a body at rest keeps its positions
  and its residual is zero (every constraint is satisfied at the rest pose);
* free fall: with gravity and no contact every vertex follows the discrete
  recurrence of apply_external_forces + advance (xpbd_base.py:139-160):
  v <- (v + g dt) e^(-5 dt), x <- x + (v + g dt) dt, since a rigidly moving
  body leaves every constraint satisfied;
* ragged batch: bodies of 1 tet, of less than one 256-tet patch and of one
  patch plus two tets step like their single-body solvers.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _far_plane():
    from xpbd_gpu.sdf import PlaneSdf
    return PlaneSdf([0.0, -100.0, 0.0], [0.0, 1.0, 0.0], True)


@pytest.mark.parametrize("n", [6, 64])
def test_rest_state_stays_at_rest_with_zero_residual(n):
    from xpbd_gpu.mesh import kuhn_grid
    from xpbd_gpu.neohookean_solver import XPBDNeoHookeanSolver
    m = kuhn_grid(n, n, n, 1.0 / n, origin=(0.0, 1.0, 0.0), jitter=0.05, seed=1)
    s = XPBDNeoHookeanSolver(m, _far_plane(), young_modulus=1e6, poisson_ratio=0.49, frame_dt=1 / 60, dt=1 / 60,
                             substeps_num=2, constraints_iter=10, block_neohookean_enable=True, cheb_enable=True,
                             cheb_warmup=3, gravity=(0.0, 0.0, 0.0), density=1000.0)
    x0 = s.mesh.verts.x.to_numpy().copy()
    s.solve()
    s.check_status()
    assert np.abs(s.mesh.verts.x.to_numpy() - x0).max() <= 1e-6
    assert np.abs(s.mesh.verts.v.to_numpy()).max() <= 1e-4
    r = s.read_history()[:, 0]
    assert np.abs(r).max() <= 1e-5


@pytest.mark.parametrize("n", [5, 64])
def test_free_fall_follows_the_discrete_recurrence(n):
    from xpbd_gpu.mesh import kuhn_grid
    from xpbd_gpu.neohookean_solver import XPBDNeoHookeanSolver
    m = kuhn_grid(n, n, n, 1.0 / n, origin=(0.0, 1.0, 0.0), jitter=0.05, seed=2)
    S, frames = 4, 3
    s = XPBDNeoHookeanSolver(m, _far_plane(), young_modulus=1e5, poisson_ratio=0.45, frame_dt=1 / 60, dt=1 / 60,
                             substeps_num=S, constraints_iter=8, block_neohookean_enable=True, cheb_enable=True,
                             cheb_warmup=3, density=1000.0)
    x0 = s.mesh.verts.x.to_numpy().astype(np.float64)
    for _ in range(frames):
        s.solve()
    s.check_status()
    dt = (1 / 60) / S
    g = -9.8
    y_shift, v = 0.0, 0.0
    for _ in range(S * frames):
        v1 = v + g * dt
        y_shift += v1 * dt
        v = v1 * np.exp(-5.0 * dt)
    x = s.mesh.verts.x.to_numpy().astype(np.float64)
    assert np.abs(x[:, 1] - (x0[:, 1] + y_shift)).max() <= 2e-5
    assert np.abs(x[:, [0, 2]] - x0[:, [0, 2]]).max() <= 2e-5
    vv = s.mesh.verts.v.to_numpy().astype(np.float64)
    assert np.abs(vv[:, 1] - v).max() <= 2e-3 * abs(v)


def test_ragged_batch_matches_single_bodies():
    from xpbd_gpu.batched import Body, XPBDBatchedSolver
    from xpbd_gpu.mesh import TetMesh, kuhn_grid
    from xpbd_gpu.neohookean_solver import XPBDNeoHookeanSolver
    from xpbd_gpu.sdf import PlaneSdf
    one = TetMesh(np.array([[0.0, 0.3, 0.0], [0.2, 0.3, 0.0], [0.0, 0.5, 0.0], [0.0, 0.3, 0.2]]),
                  np.array([[0, 1, 2, 3]], dtype=np.int32))
    g192 = kuhn_grid(8, 4, 1, 0.05, origin=(1.0, 0.1, 0.0), jitter=0.1, seed=3)      # 192 tets: under one patch
    g258 = kuhn_grid(43, 1, 1, 0.02, origin=(0.0, 0.2, 1.0), jitter=0.1, seed=4)     # 258 tets: one patch + 2
    meshes = [one, g192, g258]
    kw = dict(frame_dt=1 / 60, dt=1 / 60, substeps_num=3, constraints_iter=10, cheb_enable=True, cheb_warmup=4,
              cheb_gamma=0.6666, block_neohookean_enable=True)
    sdfs = lambda: [PlaneSdf([0, 0, 0], [0, 1, 0], True)]
    batch = XPBDBatchedSolver([Body(m, young_modulus=2e5, poisson_ratio=0.4, density=900.0) for m in meshes],
                              sdfs(), **kw)
    singles = [XPBDNeoHookeanSolver(m, sdfs(), young_modulus=2e5, poisson_ratio=0.4, density=900.0, **kw)
               for m in meshes]
    for _ in range(10):
        batch.solve()
        X = batch.positions()
        for k, s in enumerate(singles):
            s.solve()
            x = s.mesh.verts.x.to_numpy()
            diag = float(np.linalg.norm(meshes[k].points.max(0) - meshes[k].points.min(0)))
            assert np.abs(X[batch.body_vert_slices[k]] - x).max() <= 1e-4 * diag
    batch.check_status()
