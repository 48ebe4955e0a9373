"""GPU: the launch autotuner picks a measured configuration, caches it, and
the tuned solvers compute the same physics as the fixed configurations
(max vertex deviation <= 1e-4 of the bounding-box diagonal)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_single_body_autotune_picks_and_caches(tmp_path):
    from oracle.xpbd_oracle import OracleSdf, OracleSolver
    from xpbd_gpu.mesh import kuhn_grid
    from xpbd_gpu.neohookean_solver import XPBDNeoHookeanSolver
    from xpbd_gpu.sdf import PlaneSdf, SphereSdf
    m = kuhn_grid(6, 5, 7, 0.1, origin=(0.0, 0.65, 0.0), jitter=0.1, seed=2)
    kw = dict(young_modulus=1e5, poisson_ratio=0.45, frame_dt=1 / 60, dt=1 / 60, substeps_num=3,
              constraints_iter=10, cheb_enable=True, cheb_warmup=4, cheb_gamma=0.6666,
              block_neohookean_enable=True, total_mass=10.0)
    sdfs = lambda: [PlaneSdf([0, 0, 0], [0, 1, 0], True), SphereSdf([0.3, 0.3, 0.3], 0.3, True)]
    cache = str(tmp_path / "tune.json")
    s = XPBDNeoHookeanSolver(m, sdfs(), scatter="auto", autotune_cache=cache, **kw)
    r = s.autotune_result
    assert not r["cached"]
    timed = [row for row in r["table"] if row["ms"] is not None]
    assert len(timed) >= 4 and {row["scatter"] for row in timed} >= {"patch", "atomic", "gather"}
    assert r["ms_per_substep"] == min(row["ms"] for row in timed)
    assert (s.scatter, s.tets_per_thread, s.patch_pipeline) == (r["scatter"], r["tets_per_thread"],
                                                                r["patch_pipeline"])
    s2 = XPBDNeoHookeanSolver(m, sdfs(), scatter="auto", autotune_cache=cache, **kw)
    assert s2.autotune_result["cached"] and s2.scatter == s.scatter
    ref = OracleSolver(m.points, m.tets, [OracleSdf("plane", point=[0, 0, 0], dir=[0, 1, 0], fixed=True),
                                          OracleSdf("sphere", center=[0.3, 0.3, 0.3], radius=0.3, fixed=True)],
                       dtype=np.float64, **kw)
    diag = float(np.linalg.norm(m.points.max(0) - m.points.min(0)))
    for _ in range(3):
        s.solve()
        ref.solve()
        assert np.abs(s.mesh.verts.x.to_numpy() - ref.x).max() <= 1e-4 * diag
    s.check_status()


def test_batch_autotune_restores_state(tmp_path):
    from xpbd_gpu.batched import Body, XPBDBatchedSolver
    from xpbd_gpu.mesh import kuhn_grid
    from xpbd_gpu.sdf import PlaneSdf
    bodies = [Body(kuhn_grid(4, 3, 5, 0.1, origin=(0.0, 0.2, 0.0), jitter=0.1, seed=1), young_modulus=1e5,
                   poisson_ratio=0.45, density=1000.0),
              Body(kuhn_grid(7, 6, 6, 0.05, origin=(1.0, 0.3, 0.0), jitter=0.1, seed=2), young_modulus=3e5,
                   poisson_ratio=0.3, total_mass=2.0)]
    kw = dict(frame_dt=1 / 60, dt=1 / 60, substeps_num=3, constraints_iter=12, cheb_enable=True, cheb_warmup=4,
              cheb_gamma=0.6666, block_neohookean_enable=True)
    tuned = XPBDBatchedSolver(bodies, [PlaneSdf([0, 0, 0], [0, 1, 0], True)], tets_per_thread="auto",
                              autotune_cache=str(tmp_path / "b.json"), **kw)
    r = tuned.autotune_result
    assert r["tets_per_thread"] in (1, 2) and len(r["table"]) == 2
    assert tuned.tets_per_thread == r["tets_per_thread"]
    fixed = XPBDBatchedSolver(bodies, [PlaneSdf([0, 0, 0], [0, 1, 0], True)], tets_per_thread=1, **kw)
    np.testing.assert_array_equal(tuned.positions(), fixed.positions())
    np.testing.assert_array_equal(tuned.rho_hat, fixed.rho_hat)
    for _ in range(4):
        tuned.solve()
        fixed.solve()
    X, Y = tuned.positions(), fixed.positions()
    for sl in tuned.body_vert_slices:
        diag = float(np.linalg.norm(Y[sl].max(0) - Y[sl].min(0)))
        assert np.abs(X[sl] - Y[sl]).max() <= 1e-4 * diag
