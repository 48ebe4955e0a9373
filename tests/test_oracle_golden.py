"""The CPU oracle against golden vectors from the reference's own code.

The fixtures were produced by tests/golden/make_golden.py, which runs the
reference's xpbd_gpu package unmodified under a Taichi-semantics shim in
FP64.  The oracle in float64 must reproduce them to round-off; in float32 it
must stay within the parity tolerance used for the GPU (1e-4 of the bounding
box diagonal per frame).
"""
import numpy as np
import pytest

import golden_cases as gc
from oracle.xpbd_oracle import OracleSolver, frame_chunks


@pytest.mark.parametrize("name", gc.golden_names())
def test_oracle_f64_matches_reference(name):
    d = gc.load(name)
    s = OracleSolver(d["points"], d["tets"], gc.oracle_sdfs(d), dtype=np.float64, **gc.solver_kwargs(d))
    np.testing.assert_allclose(s.x, d["x_init"], rtol=0, atol=1e-15)
    np.testing.assert_allclose(s.inv_m, d["inv_m"], rtol=1e-12)
    if "V0" in d.files:  # the fixtures of reference assets keep only the mesh, states and curves
        np.testing.assert_allclose(s.V0, d["V0"], rtol=1e-12)
        np.testing.assert_allclose(s.inv_Dm, d["inv_Dm"], rtol=1e-10, atol=1e-10)
        np.testing.assert_array_equal(s.indices, d["indices"])
    # tet1 free-falls first: r_hat is round-off noise there, so omega differs at 1e-8;
    # the cow (E 5e8, 17,360 tets) amplifies the FP64 round-off of the sums to ~3e-11
    tol = 1e-8 if name.startswith("tet1") else (1e-10 if name.startswith("cow") else 1e-11)
    for f in range(int(d["frames"])):
        s.solve()
        np.testing.assert_allclose(s.x, d["x"][f], rtol=0, atol=tol)
        np.testing.assert_allclose(s.v, d["v"][f], rtol=0, atol=tol * 100)
    rmax = float(np.abs(d["r_hat"]).max()) if len(d["r_hat"]) else 0.0
    np.testing.assert_allclose(s.r_hat_history, d["r_hat"], rtol=1e-9, atol=1e-9 * rmax)
    np.testing.assert_allclose(s.omega_history, d["omega"], rtol=1e-6)
    he = [h["hydro_error"] for h in s.convergence_history]
    de = [h["dev_error"] for h in s.convergence_history]
    np.testing.assert_allclose(he, d["hydro_error"], rtol=1e-6, atol=1e-14)
    np.testing.assert_allclose(de, d["dev_error"], rtol=1e-6, atol=1e-14)
    assert abs(s.rho_hat - float(d["rho_hat_frame"][-1])) < (1e-5 if name.startswith("tet1") else 1e-8)


@pytest.mark.parametrize("name", ["kuhn2_block_cheb", "kuhn2_split_cheb", "kuhn3_block_cheb_nu049"])
def test_oracle_f32_within_parity_tolerance(name):
    d = gc.load(name)
    s = OracleSolver(d["points"], d["tets"], gc.oracle_sdfs(d), dtype=np.float32, **gc.solver_kwargs(d))
    diag = gc.bbox_diag(d["x_init"])
    s.solve()
    assert np.abs(s.x - d["x"][0]).max() <= 1e-4 * diag


def test_frame_chunks_match_reference_loop():
    # neohookean_solver.py:563-568 with the driver defaults (fps 60, dt 0.01)
    ch = frame_chunks(1.0 / 60, 0.01)
    assert len(ch) == 2 and ch[0] == 0.01 and abs(ch[1] - (1.0 / 60 - 0.01)) < 1e-18
    assert frame_chunks(1.0 / 60, 1.0 / 60) == [1.0 / 60]


def test_oracle_single_tet_known_answer():
    """Hand-checkable block projection of one stretched tet (neohookean_solver.py:365-451)."""
    from oracle.xpbd_oracle import OracleSdf, calc_first_lame, calc_second_lame
    pts = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], dtype=np.float64)
    s = OracleSolver(pts, [[0, 1, 2, 3]], [OracleSdf("plane", point=[0, -10, 0], dir=[0, 1, 0], fixed=True)],
                     young_modulus=1000.0, poisson_ratio=0.3, block_neohookean_enable=True, dtype=np.float64)
    s.pred_x = pts.copy()
    s.pred_x[1, 0] = 1.1  # F = diag(1.1, 1, 1)
    s.lambda_D[:] = 0
    s.lambda_H[:] = 0
    s.delta_x = np.zeros((4, 3))
    s.cons_num = np.zeros(4, dtype=np.uint32)
    dt = 0.01
    s.solve_neohookean_block(dt)
    C_D = 1.1 ** 2 - 1.0  # |F|^2 - 3
    C_H = 0.1             # det F - 1
    # corner gradients: dC_D/dx1 = 2 F Dm^-T e1 = (2.2, 0, 0); dC_H/dx1 = cof(F) e1 = (1, 0, 0)
    w = s.inv_m
    gD = np.array([[-2.2, -2, -2], [2.2, 0, 0], [0, 2, 0], [0, 0, 2]])
    gH = np.array([[-1, -1.1, -1.1], [1, 0, 0], [0, 1.1, 0], [0, 0, 1.1]])
    V0 = 1.0 / 6.0
    aD = 1.0 / (calc_second_lame(1000.0, 0.3) * V0) / dt ** 2
    aH = 1.0 / (calc_first_lame(1000.0, 0.3) * V0) / dt ** 2
    A = np.array([[(w[:, None] * gD * gD).sum() + aD, (w[:, None] * gD * gH).sum()],
                  [(w[:, None] * gD * gH).sum(), (w[:, None] * gH * gH).sum() + aH]])
    dl = np.linalg.solve(A, [-C_D, -C_H])
    np.testing.assert_allclose([s.lambda_D[0], s.lambda_H[0]], dl, rtol=1e-12)
    np.testing.assert_allclose(s.delta_x, w[:, None] * (gD * dl[0] + gH * dl[1]), rtol=1e-12, atol=1e-15)
    np.testing.assert_array_equal(s.cons_num, [1, 1, 1, 1])
