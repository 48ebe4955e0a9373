"""GPU: an irregular TetGen-like mesh (a Delaunay tetrahedralisation, 19,229
tets) through the tile layout (Morton patches of 256 tets, face pairs) and
the ATOMIC variant, dropped onto a sphere and the plane, against the float64
run of the reference algorithm (the C restatement in FP64).  After every
frame the GPU must stay within 1e-4 of the bounding-box diagonal of it, or
within twice the deviation of the same algorithm run in FP32 (the C
restatement in FP32), whichever is larger: in contact with nu = 0.45, FP32
itself drifts from FP64."""
import os
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("scatter", ["patch", "atomic"])
def test_delaunay_mesh_against_float64(scatter):
    sys.path.insert(0, ROOT)
    import bench
    from test_mesh_layouts_irregular import delaunay_blob
    from xpbd_gpu.mesh import TetMesh
    from xpbd_gpu.neohookean_solver import XPBDNeoHookeanSolver
    pts, tets = delaunay_blob()
    pts = pts + np.array([0.5, 0.32, 0.5])
    mesh = TetMesh(pts, tets)
    specs = [("plane", dict(point=[0.0, 0.0, 0.0], dir=[0.0, 1.0, 0.0], fixed=True)),
             ("sphere", dict(center=[0.55, -0.1, 0.45], radius=0.2, fixed=True))]
    kw = dict(young_modulus=1e5, poisson_ratio=0.45, frame_dt=1 / 60, dt=1 / 60, substeps_num=5,
              constraints_iter=20, cheb_enable=True, cheb_warmup=5, cheb_gamma=0.6666,
              block_neohookean_enable=True, density=1000.0)
    gpu = XPBDNeoHookeanSolver(mesh, bench.product_sdfs(specs), scatter=scatter, **kw)
    assert gpu.scatter == scatter
    if scatter == "patch":
        assert gpu._patch_tets == 256 and gpu.n_tet_pairs > 0.4 * mesh.n_tets
    threads = os.cpu_count() or 1
    S = kw["substeps_num"]
    ref = bench.cpu_oracle(mesh, specs, kw, S, threads, dtype=np.float64)
    f32 = bench.cpu_oracle(mesh, specs, kw, S, threads, dtype=np.float32)
    diag = float(np.linalg.norm(pts.max(0) - pts.min(0)))
    contact = False
    for frame in range(12):
        gpu.solve()
        ref.solve()
        f32.solve()
        x = gpu.mesh.verts.x.to_numpy().astype(np.float64)
        dev = np.abs(x - ref.x).max() / diag
        dev32 = np.abs(f32.x.astype(np.float64) - ref.x).max() / diag
        assert dev <= max(1e-4, 2.0 * dev32), (frame, dev, dev32)
        contact |= bool(ref.x[:, 1].min() < 0.105)  # down to the sphere top (y = 0.1)
    gpu.check_status()
    assert contact, "the body never reached the sphere"
