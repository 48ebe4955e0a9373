"""GPU test of xpbd_residual_noalloc, the residual sweep that allocates nothing.

Some callers may not allocate device memory: an engine or plugin host that
owns every device allocation and hands this library only its buffers, or a
frame loop that cannot afford cudaMalloc's implicit device synchronisation.
For them the C ABI has one entry point whose scratch is a static device array
instead of an allocation.  This test calls it through ctypes and checks its
three outputs (r_hat, mean |det F - 1|, mean |tr F^T F - 3|) against the
values the allocating path (xpbd_solve_step's residual sweep, read back as
history row 0) computed for the same state, twice in a row, within the
residual tolerance of the parity tests (2e-3 relative above a 1e-6 floor).

The state: one substep of one Jacobi iteration with Chebyshev gamma = 1 and
omega = 1 (warm-up), so the positions left in the predicted buffer are the
post-Jacobi positions the sweep measured (up to one rounding) and the Jacobi
accumulator is back at zero.  This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL, ATOL = 2e-3, 1e-6


def _state(scatter="atomic", tet_materials=False):
    import torch
    from xpbd_gpu.mesh import kuhn_grid
    from xpbd_gpu.neohookean_solver import XPBDNeoHookeanSolver
    from xpbd_gpu.sdf import PlaneSdf, SphereSdf
    m = kuhn_grid(8, 6, 7, 0.05, origin=(0.1, 0.02, 0.1), jitter=0.1, seed=11)
    extra = {}
    if tet_materials:  # per-tet Young's moduli spread over two decades
        extra["tet_young_modulus"] = np.exp(np.random.default_rng(5).uniform(np.log(2e4), np.log(2e6), m.n_tets))
    s = XPBDNeoHookeanSolver(m, [PlaneSdf([0, 0, 0], [0, 1, 0], True), SphereSdf([0.3, 0.0, 0.3], 0.1, True)],
                             young_modulus=2e5, poisson_ratio=0.45, frame_dt=0.01, dt=0.01, substeps_num=1,
                             constraints_iter=1, cheb_enable=True, cheb_warmup=5, cheb_gamma=1.0,
                             block_neohookean_enable=True, monitor_convergence=True, scatter=scatter,
                             total_mass=10.0, **extra)
    assert s.scatter == scatter
    assert (s._tinv_mu is not None) == tet_materials
    # deform the body so the residual is well above round-off
    x = s.mesh.verts.x.to_numpy()
    s.mesh.verts.x.from_numpy(x * np.array([1.0, 0.9, 1.05], dtype=np.float32))
    dt = 0.01
    s.apply_external_forces(dt)
    s.solve_step(dt)
    torch.cuda.synchronize()
    row = s.read_history(1)[0]  # r_hat, omega, hydro, dev of the allocating path
    pred = s._p4[1]             # one Chebyshev iteration: the prediction moved to p1
    assert float(s._dx4.abs().max()) == 0.0
    return s, row, pred


@pytest.mark.parametrize("scatter,tet_materials", [("atomic", False), ("patch", False), ("atomic", True)])
def test_noalloc_residual_matches_allocating_path(scatter, tet_materials):
    """The entry point reads the per-tet records every scatter variant shares, and
    with per-tet materials the compliance of each tet from its own 1 / mu, 1 / lambda."""
    import torch
    from xpbd_gpu import _native
    s, row, pred = _state(scatter, tet_materials)
    lib = _native.load()
    body = s._body()
    out = torch.full((3,), -1.0, dtype=torch.float64, device=pred.device)
    stream = torch.cuda.current_stream().cuda_stream
    expect = np.array([row[0], row[2], row[3]])
    assert expect[0] > 1e-4
    for _ in range(2):  # the static scratch is reused; the second call must agree too
        out.fill_(-1.0)
        st = lib.xpbd_residual_noalloc(ctypes.byref(body), pred.data_ptr(), ctypes.c_float(0.01),
                                       ctypes.c_float(s.lame2), ctypes.c_float(s.lame1),
                                       1 if s.precise_hydro else 0, out.data_ptr(), stream)
        _native.check(st)
        got = out.cpu().numpy()
        np.testing.assert_allclose(got, expect, rtol=RTOL, atol=ATOL)


def test_noalloc_rejects_meshes_beyond_its_scratch():
    from xpbd_gpu import _native
    lib = _native.load()
    body = _native.XpbdBody()
    body.n_verts = 10
    body.n_tets = 8192 * 256 + 1
    out = ctypes.c_double()
    st = lib.xpbd_residual_noalloc(ctypes.byref(body), ctypes.c_void_p(1), ctypes.c_float(0.01),
                                   ctypes.c_float(1.0), ctypes.c_float(1.0), 0, ctypes.addressof(out), None)
    assert st == 1
    assert b"2097152" in lib.xpbd_last_error()
