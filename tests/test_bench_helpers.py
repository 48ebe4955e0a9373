"""Host-side helpers of bench.py that need no GPU: the launch count of a
stop-mode frame and the 256-body workload's shape."""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def test_stop_mode_launch_count():
    import bench
    # begin + end, three kernels per iteration (single body); after iterations
    # 0 and 1 the frame graph's WHILE node launches iterations two at a time
    assert bench.loop_launches(1, 3) == 2 + 3
    assert bench.loop_launches(2, 3) == 2 + 6
    assert bench.loop_launches(3, 3) == 2 + 12
    assert bench.loop_launches(4, 3) == 2 + 12
    assert bench.loop_launches(5, 3) == 2 + 18
    assert bench.loop_launches(200, 3) == 2 + 600
    # the batch adds the next iteration's patch list to every iteration
    assert bench.loop_launches(5) == 2 + 24


def test_c3_workload_shape():
    import bench
    bodies, specs, kw, desc = bench.workload_c3()
    assert len(bodies) == 256
    assert kw["substeps_num"] == 5 and kw["constraints_iter"] == 30
    # per-axis cells U{4..32}: between 384 and 196,608 tets per body
    nt = np.array([b.rest_pose.n_tets for b in bodies])
    assert nt.min() >= 6 * 4 ** 3 and nt.max() <= 6 * 32 ** 3
    E = np.array([b.young_modulus for b in bodies])
    nu = np.array([b.poisson_ratio for b in bodies])
    assert E.min() >= 1e4 and E.max() <= 1e7
    assert nu.min() >= 0.30 and nu.max() <= 0.495
    assert sum(1 for k, _ in specs if k == "sphere") == 32


def test_matrix_scene_is_the_reference_comparison():
    """bench.py --workload matrix uses the scene of the reference's convergence
    comparison (scripts/compare_convergence_armadillo.bat:14-17 with the
    driver's scene, run_neohookean_usd.py:82-106)."""
    import bench

    class A:
        matrix_scale = 0.01
    kw, sdfs = bench.matrix_scene(A)
    assert kw["scale"] == 0.01 and kw["offset"] == (0.0, 1.0, 0.0)
    assert kw["young_modulus"] == 5e8 and kw["poisson_ratio"] == 0.4999
    assert kw["dt"] == 0.01 and abs(kw["frame_dt"] - 1.0 / 60) < 1e-15
    assert kw["substeps_num"] == 1 and kw["constraints_iter"] == 200
    assert kw["cheb_warmup"] == 5 and kw["cheb_gamma"] == 0.666
    assert kw["hydrostatic_relaxation"] == 1.2 and kw["deviatoric_relaxation"] == 1.2
    assert kw["monitor_convergence"]
    assert [k for k, _ in sdfs] == ["plane", "sphere"]
    assert sdfs[0][1]["point"] == [0.0, -2.0, 0.0] and sdfs[1][1]["radius"] == 0.3
    assert [(lab, b, c) for lab, b, c in bench.MATRIX] == [("NH", False, False), ("NH-DC", False, True),
                                                           ("BNH", True, False), ("BNH-DC", True, True)]
