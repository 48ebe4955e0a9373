"""GPU checks of the reference-facing interface (xpbd_gpu package)."""
import numpy as np
import pytest

import golden_cases as gc

pytestmark = pytest.mark.gpu


def _solver(**over):
    from xpbd_gpu.neohookean_solver import XPBDNeoHookeanSolver
    d = gc.load("kuhn2_block_cheb")
    kw = gc.solver_kwargs(d)
    kw.update(over)
    return d, XPBDNeoHookeanSolver(rest_pose=(d["points"], d["tets"]), sdf=gc.product_sdfs(d), **kw)


def test_fields_and_indices_match_reference_setup():
    d, s = _solver()
    np.testing.assert_array_equal(s.indices.to_numpy(), d["indices"])
    assert s.indices.shape[0] == 12 * len(d["tets"])
    np.testing.assert_allclose(s.mesh.cells.V0.to_numpy(), d["V0"], rtol=1e-6)
    np.testing.assert_allclose(s.mesh.cells.inv_Dm.to_numpy(), d["inv_Dm"], rtol=1e-5, atol=1e-5)
    np.testing.assert_allclose(s.mesh.verts.m.to_numpy(), d["mass"], rtol=1e-6)
    np.testing.assert_allclose(s.mesh.verts.inv_m.to_numpy(), d["inv_m"], rtol=1e-6)
    assert len(s.mesh.verts) == len(d["points"]) and len(s.mesh.cells) == len(d["tets"])
    assert s.mesh.verts.x.to_numpy().dtype == np.float32


def test_from_numpy_roundtrip_in_caller_order():
    _, s = _solver()
    rng = np.random.default_rng(0)
    a = rng.normal(size=(s.n_verts, 3)).astype(np.float32)
    s.mesh.verts.v.from_numpy(a)
    np.testing.assert_array_equal(s.mesh.verts.v.to_numpy(), a)
    x = s.mesh.verts.x.to_numpy()
    s.mesh.verts.x.from_numpy(x + 1.0)
    np.testing.assert_array_equal(s.mesh.verts.x.to_numpy(), x + 1.0)
    # inv_m survives a position import
    np.testing.assert_array_equal(s.mesh.verts.inv_m.to_numpy() == 0, s._host_inv_m == 0)


def test_no_sdf_raises_value_error():
    from xpbd_gpu.neohookean_solver import XPBDNeoHookeanSolver
    d = gc.load("kuhn2_block_cheb")
    with pytest.raises(ValueError, match="SDF"):
        XPBDNeoHookeanSolver(rest_pose=(d["points"], d["tets"]), sdf=[])
    with pytest.raises(ValueError):
        XPBDNeoHookeanSolver(rest_pose=(d["points"], d["tets"]), sdf=None)


def test_bad_tets_per_thread_is_rejected():
    with pytest.raises(RuntimeError, match="tets_per_thread"):
        _solver(tets_per_thread=3)


def test_rho_hat_persists_across_frames_and_is_settable():
    _, s = _solver(monitor_convergence=False)
    assert abs(s.rho_hat - 0.999) < 1e-15
    s.solve()
    r1 = s.rho_hat
    assert r1 != 0.999
    s.rho_hat = 0.5
    assert s.rho_hat == 0.5


def test_sdf_parameter_change_reaches_device():
    """Moving the plane from y=0 to y=0.5 lifts the body (y in [0.05, 0.25]) at
    the next substep's SDF projection; the iterations then re-expand the
    flattened body, so only its mean height is checked."""
    from xpbd_gpu.neohookean_solver import XPBDNeoHookeanSolver
    from xpbd_gpu.sdf import PlaneSdf
    from xpbd_gpu.mesh import kuhn_grid
    m = kuhn_grid(2, 2, 2, 0.1, origin=(0, 0.05, 0))
    plane = PlaneSdf(point=[0, 0, 0], dir=[0, 1, 0], fixed=False)
    s = XPBDNeoHookeanSolver(m, plane, frame_dt=1 / 60, dt=1 / 60, substeps_num=1, constraints_iter=2,
                             block_neohookean_enable=True)
    plane.point[None] = [0.0, 0.5, 0.0]
    s.solve()
    assert s.mesh.verts.x.to_numpy()[:, 1].mean() > 0.45


def test_nonfinite_residual_sets_status():
    from xpbd_gpu._native import XpbdError
    _, s = _solver(monitor_convergence=False)
    x = s.mesh.verts.x.to_numpy()
    x[0, 0] = np.nan
    s.mesh.verts.x.from_numpy(x)
    s.solve()
    with pytest.raises(XpbdError):
        s.check_status()


def test_usd_export_accessors():
    """What usd_export.py:58-92 reads from the solver and the SDFs."""
    from xpbd_gpu.sdf import CubeSdf, PlaneSdf, SphereSdf
    d, s = _solver()
    verts = s.mesh.verts.x
    assert verts.to_numpy().shape == (len(d["points"]), 3)
    face = s.indices
    assert face.shape[0] // 3 * [3] == [3] * (face.shape[0] // 3)
    for sdf in s.sdfs:
        if isinstance(sdf, SphereSdf):
            assert sdf.center[None].to_numpy().shape == (3,)
            float(sdf.radius[None])
        elif isinstance(sdf, CubeSdf):
            assert (sdf.half_size[None].to_numpy() * 2.0).astype(np.float32).shape == (3,)
        elif isinstance(sdf, PlaneSdf):
            assert sdf.point[None].to_numpy().shape == (3,)
            np.testing.assert_allclose(np.linalg.norm(sdf.dir[None].to_numpy()), 1.0, rtol=1e-6)


@pytest.mark.parametrize("use_graph", [True, False])
def test_profiling_counts_launches_and_keeps_results(use_graph):
    """Event brackets per kernel class (event record nodes inside the frame
    graph, or direct launches) count every launch of the profiled frames and
    leave the results bitwise unchanged (deterministic gather variant)."""
    from xpbd_gpu.neohookean_solver import frame_chunks
    _, ref = _solver(scatter="gather", monitor_convergence=False, use_graph=use_graph)
    _, s = _solver(scatter="gather", monitor_convergence=False, use_graph=use_graph)
    K = s.constraints_iter
    per_frame = len(frame_chunks(s.frame_dt, s.dt)) * s.substeps_num
    s.set_profiling(True)
    s.read_profile(reset=True)
    for f in range(3):  # frames 0 and 2 profiled, frame 1 not
        ref.solve()
        s.solve()
        s.set_profiling(f == 1)
    prof = s.read_profile(reset=True)
    n_sub = 2 * per_frame
    assert prof["begin"]["launches"] == n_sub and prof["end"]["launches"] == n_sub
    for k in ("project", "gather", "update"):
        assert prof[k]["launches"] == n_sub * K, (k, prof)
    for k, v in prof.items():
        assert (v["ms"] > 0.0) == (v["launches"] > 0), (k, v)
    np.testing.assert_array_equal(s.mesh.verts.x.to_numpy(), ref.mesh.verts.x.to_numpy())
    assert s.read_profile()["project"]["launches"] == 0


def test_residual_history_is_the_last_frames_curve():
    _, s = _solver(monitor_convergence=False)
    s.solve()
    from xpbd_gpu.neohookean_solver import frame_chunks
    r = s.residual_history
    assert len(r) == len(frame_chunks(s.frame_dt, s.dt)) * s.substeps_num * s.constraints_iter
    np.testing.assert_array_equal(np.asarray(r), s.read_history()[:, 0])
    assert all(np.isfinite(r)) and max(r) > 0.0


def test_usda_export_from_device(tmp_path):
    """The solver's positions leave the GPU through pinned buffers and land in
    the layer as one time sample per rendered frame (usd_export.py:58-92)."""
    from xpbd_gpu.usda import USDMeshRenderer, add_sdfs, read_usda_points
    _, s = _solver(monitor_convergence=False)
    r = USDMeshRenderer(str(tmp_path / "run.usda"), 4, 60)
    r.add_dynamic_mesh(s.mesh.verts.x, s.indices, "deformable_mesh")
    add_sdfs(r, s.sdfs)
    frames = []
    for _ in range(4):
        s.solve()
        r.render()
        frames.append(s.mesh.verts.x.to_numpy())
    r.save()
    r.close()
    samples = read_usda_points(r.filepath)
    assert sorted(samples) == [1, 2, 3, 4]
    for t, x in enumerate(frames, start=1):
        np.testing.assert_allclose(samples[t], x, rtol=1e-7, atol=1e-7)
    text = open(r.filepath).read()
    assert text.count("def Sphere") + text.count("def Cube") + text.count("def Mesh") == 1 + len(s.sdfs)


def test_l2_hint_modes_keep_results():
    """The tile sweeps' L2 policy (evict_last records or plain loads) changes
    no result beyond the float-atomic ordering noise of the patch scatter;
    the automatic policy keeps records of a small mesh, and the forced
    modes are reported back."""
    import os
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    from xpbd_gpu.neohookean_solver import XPBDNeoHookeanSolver
    mesh, specs, kw, _ = bench.workload("c1")
    kw = dict(kw, scatter="patch")
    xs = []
    for mode in (0, 1):
        s = XPBDNeoHookeanSolver(mesh, bench.product_sdfs(specs), **kw)
        assert s.set_l2_hint() == 1
        assert s.set_l2_hint(mode) == mode
        for _ in range(3):
            s.solve()
        s.check_status()
        xs.append(s.mesh.verts.x.to_numpy())
    with pytest.raises(RuntimeError):
        s.set_l2_hint(2)
    diag = float(np.linalg.norm(mesh.points.max(0) - mesh.points.min(0)))
    assert np.abs(xs[0] - xs[1]).max() <= 1e-5 * diag
