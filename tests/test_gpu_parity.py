"""GPU parity: the sm_103a solver against golden vectors of the reference.

The goldens come from the reference's own solver code run in FP64 (see
tests/golden/make_golden.py).  The GPU computes in FP32 with float atomics
(order nondeterministic) or with the deterministic gather, so positions are
compared within the stated tolerance: max vertex deviation <= 1e-4 of the
bounding-box diagonal after every frame; per-iteration residuals r_hat within
2e-3 relative (1e-2 on the stiff reference cow, where FP32 itself departs
4e-3) plus an absolute 2e-4 of the curve's maximum, the FP32
round-off floor of a body in free fall (there FP64 gives r_hat ~ 1e-16 and
FP32 ~ 1e-7, and rho_hat is driven by that noise, so it is compared only for
bodies that are in contact from the first frame).
"""
import numpy as np
import pytest

import golden_cases as gc

pytestmark = pytest.mark.gpu

POS_TOL = 1e-4   # of the bounding-box diagonal, after each frame
RES_RTOL = 2e-3
# The reference's cow at E 5e8: rD = C_D + aD lambda_D nearly cancels, and the
# reference algorithm's r_hat in FP32 (the C restatement) departs up to 4.1e-3
# from FP64 there, 2.5e-3 at the first iteration
RES_RTOL_CASE = {"cow_block_cheb": 1e-2}


def make_solver(d, **over):
    from xpbd_gpu.neohookean_solver import XPBDNeoHookeanSolver
    kw = gc.solver_kwargs(d)
    kw.update(over)
    return XPBDNeoHookeanSolver(rest_pose=(d["points"], d["tets"]), sdf=gc.product_sdfs(d), **kw)


@pytest.mark.parametrize("name", gc.golden_names())
@pytest.mark.parametrize("scatter", ["atomic", "gather", "patch", "patch-tma", "patch-tma-1tpt", "patch-reduce",
                                     "patch-1tpt", "patch-4tpt", "patch-128", "patch-64", "patch-64-1tpt"])
def test_frames_match_reference(name, scatter):
    d = gc.load(name)
    if scatter.startswith(("patch-128", "patch-64")):
        # the smaller patches the autotuner may pick (kernels compiled per patch size)
        P = 128 if scatter.startswith("patch-128") else 64
        s = make_solver(d, scatter="patch", patch_tets=P, tets_per_thread=1 if scatter.endswith("1tpt") else 2,
                        monitor_convergence=False)
        assert s.scatter == "patch" and s._patch_tets == P
    elif scatter == "patch-tma":
        s = make_solver(d, scatter="patch", patch_pipeline=1, monitor_convergence=False)
    elif scatter == "patch-tma-1tpt":
        s = make_solver(d, scatter="patch", patch_pipeline=1, tets_per_thread=1, monitor_convergence=False)
    elif scatter == "patch-reduce":
        s = make_solver(d, scatter="patch", patch_reduce=1, monitor_convergence=False)
    elif scatter == "patch-1tpt":
        s = make_solver(d, scatter="patch", tets_per_thread=1, monitor_convergence=False)
    elif scatter == "patch-4tpt":
        s = make_solver(d, scatter="patch", tets_per_thread=4, monitor_convergence=False)
    else:
        s = make_solver(d, scatter=scatter, monitor_convergence=False)
    diag = gc.bbox_diag(d["x_init"])
    np.testing.assert_allclose(s.mesh.verts.x.to_numpy(), d["x_init"], rtol=0, atol=1e-6 * diag)
    np.testing.assert_array_equal(s.mesh.verts.inv_m.to_numpy() == 0, d["inv_m"] == 0)
    r_hat = []
    for f in range(int(d["frames"])):
        s.solve()
        x = s.mesh.verts.x.to_numpy()
        err = np.abs(x - d["x"][f]).max()
        assert err <= POS_TOL * diag, "frame %d: max deviation %.3e > %.3e" % (f, err, POS_TOL * diag)
        if s.cheb_enable:
            r_hat.append(s.read_history()[:, 0])
    s.check_status()
    if r_hat:
        r = np.concatenate(r_hat)
        g = d["r_hat"]
        np.testing.assert_allclose(r, g, rtol=RES_RTOL_CASE.get(name, RES_RTOL), atol=2e-4 * np.abs(g).max())
        if not name.startswith("tet1"):
            assert abs(s.rho_hat - float(d["rho_hat_frame"][-1])) < 2e-3


@pytest.mark.parametrize("name", ["kuhn2_block_cheb", "kuhn2_split_nocheb", "kuhn3_block_cheb_nu049"])
@pytest.mark.parametrize("scatter", ["atomic", "patch", "patch-1tpt"])
def test_monitoring_records_match_reference(name, scatter):
    d = gc.load(name)
    if scatter == "patch-1tpt":
        s = make_solver(d, monitor_convergence=True, scatter="patch", tets_per_thread=1)
    else:
        s = make_solver(d, monitor_convergence=True, scatter=scatter)
    seen = []
    s.convergence_callback = lambda frame, substep, recs: seen.append((frame, substep, len(recs)))
    for _ in range(int(d["frames"])):
        s.solve()
    h = np.array([r["hydro_error"] for r in s.convergence_history])
    dv = np.array([r["dev_error"] for r in s.convergence_history])
    np.testing.assert_allclose(h, d["hydro_error"], rtol=5e-3, atol=1e-6 * np.abs(d["hydro_error"]).max())
    np.testing.assert_allclose(dv, d["dev_error"], rtol=5e-3, atol=1e-6 * np.abs(d["dev_error"]).max())
    K = s.constraints_iter
    assert all(n == K for _, _, n in seen)
    assert len(seen) == len(s.convergence_history) // K
    rec = s.convergence_history[0]
    assert set(rec) == {"frame", "substep", "iter", "iter_compute_time_sec", "hydro_error", "dev_error"}
    assert s.solve_compute_iterations == len(s.convergence_history)
    assert s.solve_compute_time_total > 0.0


def test_gather_variant_is_deterministic():
    d = gc.load("kuhn3_block_cheb_nu049")
    outs = []
    for _ in range(2):
        s = make_solver(d, scatter="gather", monitor_convergence=False)
        for _ in range(2):
            s.solve()
        outs.append((s.mesh.verts.x.to_numpy(), s.read_history()))
    np.testing.assert_array_equal(outs[0][0], outs[1][0])
    np.testing.assert_array_equal(outs[0][1], outs[1][1])


def test_graph_and_direct_launch_agree():
    d = gc.load("kuhn2_block_cheb")
    res = []
    for g in (True, False):
        s = make_solver(d, scatter="gather", monitor_convergence=False, use_graph=g)
        for _ in range(3):
            s.solve()
        res.append(s.mesh.verts.x.to_numpy())
    np.testing.assert_array_equal(res[0], res[1])


def test_granular_methods_equal_fused_substep():
    """apply_external_forces + solve_step + advance (the reference's three calls,
    neohookean_solver.py:577-579) equals the fused substep."""
    d = gc.load("kuhn2_block_cheb")
    a = make_solver(d, scatter="gather", monitor_convergence=False, substeps_num=1, frame_dt=0.01, dt=0.01)
    b = make_solver(d, scatter="gather", monitor_convergence=False, substeps_num=1, frame_dt=0.01, dt=0.01)
    for _ in range(3):
        a.solve()
        b.apply_external_forces(0.01)
        b.solve_step(0.01)
        b.advance(0.01, b.damping)
    np.testing.assert_array_equal(a.mesh.verts.x.to_numpy(), b.mesh.verts.x.to_numpy())
    np.testing.assert_array_equal(a.mesh.verts.v.to_numpy(), b.mesh.verts.v.to_numpy())
    assert a.rho_hat == b.rho_hat


@pytest.mark.parametrize("scatter", ["atomic", "patch"])
def test_one_frame_against_f32_oracle_larger_grid(scatter):
    """A 6x6x6 Kuhn body (1,296 tets) dropped on the plane + sphere scene, one
    frame of 5 substeps x 20 iterations, against the float64 oracle."""
    from oracle.xpbd_oracle import OracleSdf, OracleSolver
    from xpbd_gpu.mesh import kuhn_grid
    from xpbd_gpu.neohookean_solver import XPBDNeoHookeanSolver
    from xpbd_gpu.sdf import PlaneSdf, SphereSdf
    m = kuhn_grid(6, 6, 6, 1.0 / 6, origin=(0.0, 0.61, 0.0), jitter=0.1, seed=0)
    kw = dict(young_modulus=1e5, poisson_ratio=0.45, frame_dt=1 / 60, dt=1 / 60, substeps_num=5,
              constraints_iter=20, cheb_enable=True, cheb_warmup=5, cheb_gamma=0.6666,
              block_neohookean_enable=True, total_mass=1000.0)
    o = OracleSolver(m.points, m.tets, [OracleSdf("plane", point=[0, 0, 0], dir=[0, 1, 0], fixed=True),
                                        OracleSdf("sphere", center=[0.5, 0.3, 0.5], radius=0.3, fixed=True)],
                     dtype=np.float64, **kw)
    s = XPBDNeoHookeanSolver(m, [PlaneSdf([0, 0, 0], [0, 1, 0], True), SphereSdf([0.5, 0.3, 0.5], 0.3, True)],
                             scatter=scatter, **kw)
    diag = gc.bbox_diag(m.points)
    for f in range(8):
        o.solve()
        s.solve()
        err = np.abs(s.mesh.verts.x.to_numpy() - o.x).max()
        assert err <= POS_TOL * diag, "frame %d: %.3e" % (f, err)

