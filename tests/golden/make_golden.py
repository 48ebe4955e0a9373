"""Generate golden vectors by running the reference solver under the Taichi shim.

Usage (only where the reference checkout is present):

    python tests/golden/make_golden.py --ref PATH [--out DIR] [--only NAME ...]

It imports the reference's ``xpbd_gpu.neohookean_solver`` and ``xpbd_gpu.sdf``
unmodified (``neohookean_solver.py:16-587``, ``xpbd_base.py:11-204``,
``sdf.py:7-124``), with ``taichi`` and ``meshtaichi_patcher`` replaced by
``taichi_shim`` (FP64 storage and arithmetic: an FP64 run of the reference's
kernels with sequential atomics).  For every case it records, per frame, the
vertex positions and velocities and, per Jacobi iteration, the residual
r_hat (``neohookean_solver.py:494-496``), the Chebyshev omega passed to
``_chebyshev_update`` (``:548``) and, when monitoring is on, the
hydrostatic/deviatoric errors (``:509-532``).  Results are written as
``<name>.npz`` next to this script.  The mesh inputs are stored in the
fixture, so the tests need neither the reference nor this script.
"""
import argparse
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)


def kuhn_grid(nx, ny, nz, h, origin, jitter, seed):
    """Kuhn grid: every cell split into 6 tets around its main diagonal.

    Interior vertices are jittered by U(-jitter, jitter)*h per coordinate.
    Tets are oriented so that (p1-p0)x(p2-p0).(p3-p0) > 0.
    """
    rng = np.random.default_rng(seed)
    I, J, K = np.meshgrid(np.arange(nx + 1), np.arange(ny + 1), np.arange(nz + 1), indexing="ij")
    ijk = np.stack([I.ravel(order="F"), J.ravel(order="F"), K.ravel(order="F")], 1)
    pts = np.asarray(origin, dtype=np.float64) + h * ijk.astype(np.float64)
    interior = ((ijk > 0) & (ijk < np.array([nx, ny, nz]))).all(1)
    pts[interior] += rng.uniform(-jitter, jitter, size=(int(interior.sum()), 3)) * h

    def vid(i, j, k):
        return i + (nx + 1) * (j + (ny + 1) * k)

    perms = [(0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0)]
    tets = []
    for k in range(nz):
        for j in range(ny):
            for i in range(nx):
                for p in perms:
                    c = [i, j, k]
                    a = list(c)
                    a[p[0]] += 1
                    b = list(a)
                    b[p[1]] += 1
                    t = [vid(*c), vid(*a), vid(*b), vid(i + 1, j + 1, k + 1)]
                    tets.append(t)
    tets = np.array(tets, dtype=np.int64)
    p0, p1, p2, p3 = (pts[tets[:, q]] for q in range(4))
    vol = np.einsum("ij,ij->i", np.cross(p1 - p0, p2 - p0), p3 - p0)
    neg = vol < 0
    tets[neg, 1], tets[neg, 2] = tets[neg, 2].copy(), tets[neg, 1].copy()
    return pts, tets


def single_tet():
    pts = np.array([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [0.0, 1.0, 0.0], [0.0, 0.0, 1.0]]) * 0.1
    pts += np.array([0.0, 0.12, 0.0])
    pts[3] += np.array([0.013, -0.004, 0.021])
    tets = np.array([[0, 1, 2, 3]])
    return pts, tets


def read_tetgen(node_path):
    """TetGen .node / .ele pair (the reference's assets/tetmesh format) ->
    (points, tets); the first index of each file is the base (0 or 1)."""
    def rows(path):
        lines = [ln.split("#")[0].split() for ln in open(path)]
        lines = [ln for ln in lines if ln]
        n = int(lines[0][0])
        return lines[1:n + 1]
    nodes = rows(node_path)
    base = int(nodes[0][0])
    pts = np.array([[float(v) for v in ln[1:4]] for ln in nodes], dtype=np.float64)
    tets = np.array([[int(v) - base for v in ln[1:5]] for ln in rows(node_path[:-5] + ".ele")], dtype=np.int64)
    return pts, tets


# name -> dict(mesh, sdfs, solver kwargs, frames)
def cases(ref=None):
    c = {}
    k2 = kuhn_grid(2, 2, 2, 0.1, (0.35, 0.02, 0.35), 0.1, 1)
    k3 = kuhn_grid(3, 3, 3, 0.08, (0.3, 0.015, 0.3), 0.1, 2)
    sdf_a = [("plane", dict(point=[0.0, 0.0, 0.0], dir=[0.0, 1.0, 0.0], fixed=True)),
             ("sphere", dict(center=[0.5, -0.17, 0.5], radius=0.2, fixed=True)),
             ("cube", dict(center=[0.6, 0.0, 0.58], size=[0.2, 0.06, 0.3], fixed=True))]
    base = dict(young_modulus=1e5, poisson_ratio=0.45, frame_dt=1.0 / 60, dt=1.0 / 60,
                substeps_num=2, constraints_iter=10, cheb_enable=True, cheb_warmup=3,
                cheb_gamma=0.6666, block_neohookean_enable=True, monitor_convergence=True)
    c["tet1_block_cheb"] = dict(mesh=single_tet(), sdfs=[sdf_a[0]],
                                kw=dict(base, substeps_num=2, constraints_iter=8), frames=24)
    c["kuhn2_block_cheb"] = dict(mesh=k2, sdfs=sdf_a, kw=dict(base), frames=8)
    c["kuhn2_block_nocheb"] = dict(mesh=k2, sdfs=sdf_a, kw=dict(base, cheb_enable=False), frames=8)
    c["kuhn2_split_cheb"] = dict(mesh=k2, sdfs=sdf_a, kw=dict(base, block_neohookean_enable=False), frames=8)
    c["kuhn2_split_nocheb"] = dict(mesh=k2, sdfs=sdf_a,
                                   kw=dict(base, block_neohookean_enable=False, cheb_enable=False), frames=8)
    # near-incompressible, multi-chunk frame (dt < frame_dt) with scale/offset
    c["kuhn3_block_cheb_nu049"] = dict(
        mesh=k3, sdfs=sdf_a,
        kw=dict(base, young_modulus=1e6, poisson_ratio=0.49, frame_dt=1.0 / 60, dt=0.01,
                substeps_num=2, constraints_iter=12, cheb_warmup=5, scale=1.1,
                offset=(-0.03, 0.0, -0.03)),
        frames=4)
    # vertices starting inside a fixed sphere are pinned (xpbd_base.py:125-131);
    # a non-fixed plane exercises the dot(n, v_sdf - v) > 0 branch (sdf.py:24-25)
    sdf_pin = [("plane", dict(point=[0.0, 0.0, 0.0], dir=[0.05, 1.0, 0.0], fixed=False)),
               ("sphere", dict(center=[0.45, 0.3, 0.45], radius=0.14, fixed=True))]
    c["kuhn2_pinned_nonfixed"] = dict(mesh=kuhn_grid(2, 2, 2, 0.1, (0.35, 0.2, 0.35), 0.1, 3),
                                      sdfs=sdf_pin, kw=dict(base), frames=6)
    if ref is not None:
        # the reference's own cow (assets/tetmesh/cow.node: 4,784 vertices, 17,360
        # tets) with the driver's material (run_neohookean_usd.py:27-30: E 5e8,
        # nu 0.4999), its hooves 3 mm into the plane; one frame, since this stiff
        # contact scene amplifies round-off from frame to frame (FP32 departs
        # 3e-5 of the diagonal from FP64 after one frame, 1.5e-4 after two)
        cow = read_tetgen(os.path.join(ref, "assets", "tetmesh", "cow.node"))
        floor = float(cow[0][:, 1].min()) + 0.003
        c["cow_block_cheb"] = dict(
            mesh=cow, sdfs=[("plane", dict(point=[0.0, floor, 0.0], dir=[0.0, 1.0, 0.0], fixed=True))],
            kw=dict(base, young_modulus=5e8, poisson_ratio=0.4999, substeps_num=1, constraints_iter=20,
                    cheb_warmup=5, cheb_gamma=0.666),
            frames=1)
    return c


def run_case(ref, name, spec, precision):
    import taichi_shim
    patcher = taichi_shim.install(precision, meshes={"mesh:" + name: spec["mesh"]})
    if ref not in sys.path:
        sys.path.insert(0, ref)
    from xpbd_gpu import neohookean_solver as nh  # the reference's module
    from xpbd_gpu import sdf as sdfmod

    sdfs = []
    for kind, kw in spec["sdfs"]:
        if kind == "plane":
            sdfs.append(sdfmod.PlaneSdf(point=kw["point"], dir=kw["dir"], fixed=kw["fixed"]))
        elif kind == "sphere":
            sdfs.append(sdfmod.SphereSdf(center=kw["center"], radius=kw["radius"], fixed=kw["fixed"]))
        elif kind == "cube":
            sdfs.append(sdfmod.CubeSdf(center=kw["center"], size=kw["size"], fixed=kw["fixed"]))
    solver = nh.XPBDNeoHookeanSolver(rest_pose="mesh:" + name, sdf=sdfs, **spec["kw"])

    r_hat, omega = [], []
    orig_res = solver.compute_xpbd_residual
    orig_cheb = solver._chebyshev_update

    def res_hook(dt):
        orig_res(dt)
        cnt = solver.residual_count[None]
        r_hat.append(solver.residual_sum[None] / cnt if cnt > 0 else 0.0)

    def cheb_hook(w):
        omega.append(float(w))
        orig_cheb(w)

    solver.compute_xpbd_residual = res_hook
    solver._chebyshev_update = cheb_hook

    x0 = solver.mesh.verts.x.to_numpy()
    inv_m = solver.mesh.verts.inv_m.to_numpy()
    xs, vs, rho = [], [], []
    for _ in range(spec["frames"]):
        solver.solve()
        xs.append(solver.mesh.verts.x.to_numpy())
        vs.append(solver.mesh.verts.v.to_numpy())
        rho.append(solver.rho_hat)
    hist = solver.convergence_history
    out = dict(
        points=np.asarray(spec["mesh"][0], dtype=np.float64),
        tets=np.asarray(spec["mesh"][1], dtype=np.int64),
        x_init=x0, inv_m=inv_m,
        x=np.array(xs), v=np.array(vs), rho_hat_frame=np.array(rho),
        r_hat=np.array(r_hat, dtype=np.float64), omega=np.array(omega, dtype=np.float64),
        hydro_error=np.array([h["hydro_error"] for h in hist], dtype=np.float64),
        dev_error=np.array([h["dev_error"] for h in hist], dtype=np.float64),
        indices=solver.indices.to_numpy(),
        V0=solver.mesh.cells.V0.to_numpy(), inv_Dm=solver.mesh.cells.inv_Dm.to_numpy(),
        mass=solver.mesh.verts.m.to_numpy(),
        frames=spec["frames"],
        sdf_kinds=np.array([k for k, _ in spec["sdfs"]]),
        sdf_params=np.array([repr(kw) for _, kw in spec["sdfs"]]),
        solver_kw=repr(spec["kw"]),
        precision=precision,
    )
    if len(out["tets"]) > 5000:
        # a reference asset: the setup arrays follow from the mesh (and are checked
        # on the small cases), so the fixture keeps the mesh, the states and the curves
        for k in ("V0", "inv_Dm", "indices", "mass"):
            del out[k]
        out["tets"] = out["tets"].astype(np.int32)
    for m in [m for m in list(sys.modules) if m == "xpbd_gpu" or m.startswith("xpbd_gpu.")]:
        del sys.modules[m]
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("XPBD_REFERENCE_DIR"),
                    help="the reference checkout (or set XPBD_REFERENCE_DIR)")
    ap.add_argument("--out", default=HERE)
    ap.add_argument("--only", nargs="*", default=None)
    ap.add_argument("--precision", default="f64", choices=["f64", "f32"])
    args = ap.parse_args()
    if not args.ref:
        ap.error("give --ref or set XPBD_REFERENCE_DIR")
    for name, spec in cases(os.path.abspath(args.ref)).items():
        if args.only and name not in args.only:
            continue
        t0 = time.time()
        out = run_case(args.ref, name, spec, args.precision)
        suffix = "" if args.precision == "f64" else "_f32"
        path = os.path.join(args.out, name + suffix + ".npz")
        np.savez_compressed(path, **out)
        print("%-28s T=%-5d V=%-5d frames=%d  %.1fs -> %s" % (
            name, len(out["tets"]), len(out["points"]), out["frames"], time.time() - t0,
            os.path.relpath(path)))


if __name__ == "__main__":
    main()
