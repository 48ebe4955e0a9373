"""GPU: stop mode, the residual-targeted iteration count (xpbd_params
target_rel_residual / residual_floor).

The reference always runs constraints_iter Jacobi iterations per substep
(neohookean_solver.py:474) and computes r_hat after each (:492-504).  In stop
mode a substep ends after the first iteration k with
r_hat_k <= target * r_hat_0 or r_hat_k <= floor, constraints_iter being the
cap.  So a stop-mode substep of n iterations must equal a fixed-count substep
of n iterations:

* single body, deterministic GATHER variant: bitwise, through the frame
  graph (a WHILE conditional node over pairs of iterations) and through
  direct launches;
* single body, PATCH variant (float atomics): within the parity tolerance,
  1e-4 of the bounding-box diagonal;
* batch: every body against a single-body solver run with that body's
  iteration counts, within the same tolerance.

Every substep's count must be the first iteration that meets the target
(or the cap), read from the residual history the same run recorded.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

POS_TOL = 1e-4
CAP = 60


def _sdfs():
    from xpbd_gpu.sdf import PlaneSdf, SphereSdf
    return [PlaneSdf([0, 0, 0], [0, 1, 0], True), SphereSdf([0.2, -0.05, 0.15], 0.12, True)]


def _kw(**extra):
    kw = dict(frame_dt=1 / 60, dt=1 / 60, substeps_num=3, constraints_iter=CAP, cheb_enable=True, cheb_warmup=5,
              cheb_gamma=0.6666, block_neohookean_enable=True, total_mass=5.0)
    kw.update(extra)
    return kw


def _mesh(seed=4, n=(6, 5, 6)):
    from xpbd_gpu.mesh import kuhn_grid
    return kuhn_grid(*n, 0.05, origin=(0.0, 0.002, 0.0), jitter=0.1, seed=seed)


def _solver(scatter, mesh=None, young=2e5, nu=0.35, **extra):
    from xpbd_gpu.neohookean_solver import XPBDNeoHookeanSolver
    s = XPBDNeoHookeanSolver(mesh if mesh is not None else _mesh(), _sdfs(), young_modulus=young, poisson_ratio=nu,
                             scatter=scatter, **_kw(**extra))
    # thrown at the ground: the substeps start in contact, with residuals well
    # above the FP32 floor
    v = np.zeros((s.n_verts, 3), dtype=np.float32)
    v[:, 1] = -3.0
    v[:, 0] = 0.5
    s.mesh.verts.v.from_numpy(v)
    return s


def _check_counts(hist, counts, K, target, floor=0.0):
    """counts[s] is the first iteration index + 1 whose r_hat meets the target, or K."""
    for s, n in enumerate(counts):
        r = hist[s * K:(s + 1) * K, 0]
        assert 1 <= n <= K
        met = (r[:n] <= target * r[0]) | (r[:n] <= floor)
        assert not met[:n - 1].any(), "substep %d stopped late: %s" % (s, r[:n])
        assert met[n - 1] or n == K, "substep %d stopped early at %d" % (s, n)


def _fixed_substeps(solver, counts, sub_dt):
    """Fixed-count substeps of the given lengths through direct launches."""
    from xpbd_gpu import _native
    for n in counts:
        solver.constraints_iter = int(n)
        solver._sync()
        _native.check(solver._lib.xpbd_substep(solver._handle, float(sub_dt), 0, solver._stream()))


@pytest.mark.parametrize("use_graph", [True, False])
def test_stop_mode_equals_truncated_fixed_run_gather_bitwise(use_graph):
    target = 3e-2
    stop = _solver("gather", target_rel_residual=target, use_graph=use_graph)
    fixed = _solver("gather")
    sub_dt = (1 / 60) / 3
    early = 0
    for frame in range(4):
        stop.solve()
        counts = stop.iterations_per_substep()
        hist = stop.read_history()
        _check_counts(hist, counts, CAP, target)
        early += int((counts < CAP).sum())
        _fixed_substeps(fixed, counts, sub_dt)
        np.testing.assert_array_equal(stop.mesh.verts.x.to_numpy(), fixed.mesh.verts.x.to_numpy())
        np.testing.assert_array_equal(stop.mesh.verts.v.to_numpy(), fixed.mesh.verts.v.to_numpy())
        assert stop.rho_hat == fixed.rho_hat
    stop.check_status()
    assert early > 0, "no substep met the target before the cap"


def test_stop_mode_graph_and_direct_launches_agree():
    target = 3e-2
    g = _solver("gather", target_rel_residual=target, use_graph=True)
    d = _solver("gather", target_rel_residual=target, use_graph=False)
    for _ in range(3):
        g.solve()
        d.solve()
        np.testing.assert_array_equal(g.iterations_per_substep(), d.iterations_per_substep())
        np.testing.assert_array_equal(g.mesh.verts.x.to_numpy(), d.mesh.verts.x.to_numpy())


def test_stop_mode_patch_variant_matches_truncated_run():
    target = 3e-2
    stop = _solver("patch", target_rel_residual=target)
    fixed = _solver("patch")
    assert stop.scatter == "patch"
    sub_dt = (1 / 60) / 3
    for frame in range(4):
        stop.solve()
        counts = stop.iterations_per_substep()
        _check_counts(stop.read_history(), counts, CAP, target)
        _fixed_substeps(fixed, counts, sub_dt)
        x, y = stop.mesh.verts.x.to_numpy(), fixed.mesh.verts.x.to_numpy()
        diag = float(np.linalg.norm(y.max(0) - y.min(0)))
        assert np.abs(x - y).max() <= POS_TOL * diag
    stop.check_status()


def test_stop_mode_floor_and_cap():
    """A residual floor above every r_hat stops each substep after one
    iteration; an unreachable target runs the cap, i.e. the fixed count."""
    floor = _solver("gather", residual_floor=1e3)
    floor.solve()
    np.testing.assert_array_equal(floor.iterations_per_substep(), np.ones(3, dtype=np.int32))
    cap = _solver("gather", target_rel_residual=1e-30)
    fixed = _solver("gather")
    for _ in range(2):
        cap.solve()
        fixed.solve()
        np.testing.assert_array_equal(cap.iterations_per_substep(), np.full(3, CAP, dtype=np.int32))
        np.testing.assert_array_equal(cap.mesh.verts.x.to_numpy(), fixed.mesh.verts.x.to_numpy())
    assert fixed.solve_compute_iterations == 2 * 3 * CAP
    assert cap.solve_compute_iterations == 2 * 3 * CAP
    assert floor.solve_compute_iterations == 3


def test_stop_mode_monitoring_records_stop_with_the_substep():
    target = 3e-2
    s = _solver("gather", target_rel_residual=target, monitor_convergence=True)
    got = []
    s.convergence_callback = lambda f, sub, recs: got.append(len(recs))
    s.solve()
    counts = [n for n in got]
    assert len(counts) == 3
    assert len(s.convergence_history) == sum(counts)
    assert s.solve_compute_iterations == sum(counts)
    assert min(counts) >= 1 and max(counts) <= CAP


def _batch_scene():
    from xpbd_gpu.batched import Body
    from xpbd_gpu.mesh import kuhn_grid
    bodies = [
        Body(kuhn_grid(6, 5, 6, 0.05, origin=(0.0, 0.002, 0.0), jitter=0.1, seed=4), young_modulus=2e5,
             poisson_ratio=0.35, total_mass=5.0),
        Body(kuhn_grid(9, 4, 7, 0.04, origin=(1.0, 0.002, 0.0), jitter=0.1, seed=5), young_modulus=2e6,
             poisson_ratio=0.45, total_mass=3.0),
        # high above the ground: free fall, r_hat at the FP32 floor
        Body(kuhn_grid(3, 3, 3, 0.05, origin=(0.0, 2.0, 1.0), jitter=0.1, seed=6), young_modulus=1e5,
             poisson_ratio=0.3, total_mass=1.0),
    ]
    return bodies


def _single_for(body, **extra):
    from xpbd_gpu.mesh import TetMesh
    from xpbd_gpu.neohookean_solver import XPBDNeoHookeanSolver
    kw = _kw(**extra)
    kw.pop("total_mass")
    return XPBDNeoHookeanSolver(TetMesh(body.rest_pose.points, body.rest_pose.tets), _sdfs(),
                                young_modulus=body.young_modulus, poisson_ratio=body.poisson_ratio,
                                total_mass=body.total_mass, scatter="patch", **kw)


def test_batched_stop_mode_matches_truncated_single_bodies():
    from xpbd_gpu.batched import XPBDBatchedSolver
    target, floor = 3e-2, 1e-4
    bodies = _batch_scene()
    kw = _kw()
    kw.pop("total_mass")
    batch = XPBDBatchedSolver(bodies, _sdfs(), target_rel_residual=target, residual_floor=floor, **kw)
    v = np.zeros((sum(b.rest_pose.n_verts for b in bodies), 3), dtype=np.float32)
    v[:, 1] = -3.0
    batch.set_velocities(v)
    singles = [_single_for(b) for b in bodies]
    for s in singles:
        s.mesh.verts.v.from_numpy(np.tile([0.0, -3.0, 0.0], (s.n_verts, 1)).astype(np.float32))
    sub_dt = (1 / 60) / 3
    early = 0
    for frame in range(4):
        batch.solve()
        counts = batch.iterations_per_substep()
        hist = batch.read_history()
        X = batch.positions()
        for k, s in enumerate(singles):
            _check_counts(hist[k], counts[k], CAP, target, floor)
            _fixed_substeps(s, counts[k], sub_dt)
            x = s.mesh.verts.x.to_numpy()
            diag = float(np.linalg.norm(x.max(0) - x.min(0)))
            err = np.abs(X[batch.body_vert_slices[k]] - x).max()
            assert err <= POS_TOL * diag, "frame %d body %d: %.3e" % (frame, k, err)
        early += int((counts < CAP).sum())
    batch.check_status()
    assert early > 0
    # the free-falling body: r_hat at FP32 round-off, below the floor, so each
    # of its substeps stops after one iteration
    r0 = hist[2, ::CAP, 0][:3]
    assert (r0 <= floor).all() and (counts[2] == 1).all(), (r0, counts[2])
