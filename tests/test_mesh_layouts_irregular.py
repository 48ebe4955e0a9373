"""Host-side layouts (Morton order, face pairs, 256-tet patches) on irregular
TetGen meshes: a Delaunay tetrahedralisation made here, and -- where the
reference checkout is available (XPBD_REFERENCE_DIR) -- the reference's own
assets (assets/tetmesh/*.node, loaded by xpbd_base.py:42).  The tile kernels
need every 256-tet patch to touch at most 256 vertices, and the
two-tets-per-thread kernels gain from face pairs."""
import glob
import os

import numpy as np
import pytest

from xpbd_gpu import _native
from xpbd_gpu.mesh import read_tetgen


def delaunay_blob(n_points=3000, seed=0):
    """An irregular tet mesh: the Delaunay tetrahedralisation of random points
    in an ellipsoid, without near-degenerate tets, positively oriented."""
    from scipy.spatial import Delaunay
    rng = np.random.default_rng(seed)
    p = rng.normal(size=(4 * n_points, 3))
    p /= np.linalg.norm(p, axis=1, keepdims=True)
    p *= rng.uniform(0, 1, size=(len(p), 1)) ** (1 / 3)
    p = p[:n_points] * np.array([0.3, 0.2, 0.25])
    tets = Delaunay(p).simplices.astype(np.int64)
    P = p[tets]
    vol = np.einsum("ij,ij->i", np.cross(P[:, 1] - P[:, 0], P[:, 2] - P[:, 0]), P[:, 3] - P[:, 0]) / 6.0
    keep = np.abs(vol) > 1e-3 * np.abs(vol).mean()
    tets, vol = tets[keep], vol[keep]
    tets[vol < 0, 1], tets[vol < 0, 2] = tets[vol < 0, 2].copy(), tets[vol < 0, 1].copy()
    used = np.unique(tets)
    remap = np.full(len(p), -1)
    remap[used] = np.arange(len(used))
    return p[used], remap[tets]


def layout_stats(points, tets, patch_tets=256):
    lib = _native.load()
    V, T = len(points), len(tets)
    pts = np.ascontiguousarray(points, dtype=np.float64)
    tt = np.ascontiguousarray(tets, dtype=np.int32)
    vperm, tperm = np.empty(V, dtype=np.int32), np.empty(T, dtype=np.int32)
    _native.check(lib.xpbd_morton_order(pts.ctypes.data, V, tt.ctypes.data, T, vperm.ctypes.data, tperm.ctypes.data))
    inv = np.empty(V, dtype=np.int64)
    inv[vperm] = np.arange(V)
    tets_new = inv[tets[tperm]].astype(np.int32)
    order, cperm, n_pairs = _native.pair_tets(lib, tets_new, V)
    paired = np.ascontiguousarray(np.take_along_axis(tets_new[order], cperm, axis=1), dtype=np.int32)
    assert sorted(map(tuple, np.sort(paired, axis=1))) == sorted(map(tuple, np.sort(tets_new, axis=1)))
    npat = -(-T // patch_tets)
    voff = np.empty(npat + 1, dtype=np.int32)
    pverts = np.empty(4 * T, dtype=np.int32)
    lid = np.zeros(-(-T // 256) * 256, dtype=np.uint32)
    mx = _native.ctypes.c_int32()
    _native.check(lib.xpbd_build_patches(paired.ctypes.data, T, V, patch_tets, voff.ctypes.data, pverts.ctypes.data,
                                         lid.ctypes.data, _native.ctypes.byref(mx)))
    return dict(pair_fraction=2.0 * n_pairs / T, max_patch_verts=mx.value,
                mean_patch_verts=float(np.diff(voff).mean()))


def test_delaunay_mesh_layout():
    pts, tets = delaunay_blob()
    st = layout_stats(pts, tets)
    assert st["max_patch_verts"] <= 256, st
    assert st["pair_fraction"] > 0.8, st


REF = os.environ.get("XPBD_REFERENCE_DIR", "")


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "assets", "tetmesh")),
                    reason="needs the reference checkout (XPBD_REFERENCE_DIR)")
@pytest.mark.parametrize("name", ["cow", "horse", "beast", "armadillo", "lucy", "dragon"])
def test_reference_asset_layout(name):
    path = os.path.join(REF, "assets", "tetmesh", name + ".node")
    m = read_tetgen(path)
    st = layout_stats(m.points, m.tets)
    assert st["max_patch_verts"] <= 256, (name, st)
    assert st["pair_fraction"] > 0.8, (name, st)
