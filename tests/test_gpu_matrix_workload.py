"""GPU: bench.py --workload matrix (the reference's NH / NH-DC / BNH / BNH-DC
comparison) on a small TetGen mesh written here, for a few frames: the four
configurations run, record the convergence rows of the recorded frame, and
that frame matches the C restatement in FP64 from the same state within the
single-body parity tolerance."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _write_tetgen(path, pts, tets):
    with open(path + ".node", "w") as f:
        f.write("%d 3 0 0\n" % len(pts))
        for i, p in enumerate(pts):
            f.write("%d %.17g %.17g %.17g\n" % (i, p[0], p[1], p[2]))
    with open(path + ".ele", "w") as f:
        f.write("%d 4 0\n" % len(tets))
        for i, t in enumerate(tets):
            f.write("%d %d %d %d %d\n" % (i, t[0], t[1], t[2], t[3]))


def test_matrix_workload_runs_the_four_configurations(tmp_path):
    sys.path.insert(0, os.path.join(ROOT, "rdc-xpbd-taichi_gb300"))
    from xpbd_gpu.mesh import kuhn_grid
    # 1.2 m across at scale 1, dropped from y = 0.8 onto the fixed sphere within a few frames
    m = kuhn_grid(4, 3, 4, 0.3, origin=(-0.6, -0.2, -0.6), jitter=0.1, seed=5)
    base = str(tmp_path / "kuhn")
    _write_tetgen(base, m.points, m.tets)
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--workload", "matrix", "--mesh",
                        base + ".node", "--matrix-frame", "20", "--matrix-scale", "1.0"],
                       capture_output=True, text=True, cwd=ROOT, timeout=900)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads([ln for ln in r.stdout.splitlines() if ln.startswith("{")][-1])
    assert line["tets"] == m.n_tets and line["frames"] == 21
    assert list(line["configs"]) == ["NH", "NH-DC", "BNH", "BNH-DC"]
    for label, c in line["configs"].items():
        assert len(c["chunks"]) == 2  # dt 0.01 at 60 fps: two chunks per frame
        for ch in c["chunks"]:
            assert len(ch["hydro_error"]) == 200 and len(ch["dev_error"]) == 200
            assert (ch["r_hat"] is not None) == label.endswith("DC")
        assert np.isfinite(c["ms_per_frame"])
        assert c["fp64_max_dev_over_bbox_diag"] <= 1e-4 + 2 * c["fp32_vs_fp64_max_dev_over_bbox_diag"]
