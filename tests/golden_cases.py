"""Helpers to rebuild solvers from the golden fixtures in tests/golden/."""
import ast
import glob
import os

import numpy as np

GOLDEN_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def golden_names():
    """The solver fixtures of make_golden.py (not the driver trace of make_driver_trace.py)."""
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN_DIR, "*.npz"))
                  if not p.endswith("_f32.npz") and not os.path.basename(p).startswith("driver_trace"))


def load(name):
    return np.load(os.path.join(GOLDEN_DIR, name + ".npz"))


def solver_kwargs(d):
    return ast.literal_eval(str(d["solver_kw"]))


def sdf_specs(d):
    return [(str(k), ast.literal_eval(str(p))) for k, p in zip(d["sdf_kinds"], d["sdf_params"])]


def oracle_sdfs(d):
    from oracle.xpbd_oracle import OracleSdf
    return [OracleSdf(k, **p) for k, p in sdf_specs(d)]


def product_sdfs(d):
    from xpbd_gpu.sdf import CubeSdf, PlaneSdf, SphereSdf
    out = []
    for k, p in sdf_specs(d):
        if k == "plane":
            out.append(PlaneSdf(point=p["point"], dir=p["dir"], fixed=p["fixed"]))
        elif k == "sphere":
            out.append(SphereSdf(center=p["center"], radius=p["radius"], fixed=p["fixed"]))
        else:
            out.append(CubeSdf(center=p["center"], size=p["size"], fixed=p["fixed"]))
    return out


def bbox_diag(points):
    p = np.asarray(points)
    return float(np.linalg.norm(p.max(0) - p.min(0)))
