import os
import sys

import numpy as np

from conftest import ROOT
from xpbd_gpu.mesh import TetMesh, kuhn_grid, read_tetgen
from xpbd_gpu.xpbd_base import calc_tet_volume

sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))


def test_kuhn_grid_counts_and_orientation():
    m = kuhn_grid(4, 3, 2, 0.25, origin=(1, 2, 3), jitter=0.1, seed=5)
    assert m.n_verts == 5 * 4 * 3 and m.n_tets == 6 * 24
    P = m.points[m.tets]
    vol = calc_tet_volume(P[:, 0], P[:, 1], P[:, 2], P[:, 3])
    assert (vol > 0).all()
    np.testing.assert_allclose(vol.sum(), 1.0 * 0.75 * 0.5, rtol=1e-12)


def test_kuhn_grid_matches_golden_generator():
    import make_golden
    a = kuhn_grid(3, 2, 2, 0.1, (0.3, 0.1, 0.2), 0.1, 7)
    pts, tets = make_golden.kuhn_grid(3, 2, 2, 0.1, (0.3, 0.1, 0.2), 0.1, 7)
    np.testing.assert_array_equal(a.points, pts)
    np.testing.assert_array_equal(a.tets, tets)


def test_read_tetgen_roundtrip(tmp_path):
    m = kuhn_grid(2, 2, 1, 1.0)
    base = tmp_path / "box"
    with open(str(base) + ".node", "w") as f:
        f.write("%d 3 0 0\n" % m.n_verts)
        for i, p in enumerate(m.points):
            f.write("%d %.17g %.17g %.17g\n" % (i + 1, *p))
    with open(str(base) + ".ele", "w") as f:
        f.write("# comment line\n%d 4 0\n" % m.n_tets)
        for i, t in enumerate(m.tets):
            f.write("%d %d %d %d %d\n" % (i + 1, *(t + 1)))
    r = read_tetgen(str(base) + ".node")
    assert isinstance(r, TetMesh)
    np.testing.assert_array_equal(r.points, m.points)
    np.testing.assert_array_equal(r.tets, m.tets)
