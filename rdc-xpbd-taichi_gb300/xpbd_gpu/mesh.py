"""Tetrahedral mesh input: TetGen ``.node/.ele`` files and Kuhn-split grids.

The reference loads meshes through meshtaichi_patcher
(``Patcher.load_mesh(path, relations=["VV", "CV"])``, xpbd_base.py:42), which
reads a TetGen pair named by its ``.node`` path.  ``read_tetgen`` reads the
same pair in file order (ids may start at 0 or 1).  ``kuhn_grid`` builds the
synthetic benchmark bodies: every cube cell split into 6 tets around its main
diagonal, interior vertices jittered from a seeded generator, every tet
positively oriented under ``calc_tet_volume`` (xpbd_base.py:7-8).
"""
from dataclasses import dataclass

import numpy as np


@dataclass
class TetMesh:
    points: np.ndarray  # (V, 3) float64
    tets: np.ndarray    # (T, 4) int32

    @property
    def n_verts(self):
        return len(self.points)

    @property
    def n_tets(self):
        return len(self.tets)


def _rows(path):
    with open(path) as f:
        for ln in f:
            s = ln.split("#", 1)[0].split()
            if s:
                yield s


def read_tetgen(node_path):
    """Read ``<name>.node`` and ``<name>.ele``; returns a TetMesh with 0-based ids."""
    base_path = node_path[:-5] if node_path.endswith(".node") else node_path
    it = _rows(base_path + ".node")
    head = next(it)
    nv = int(head[0])
    ids = np.empty(nv, dtype=np.int64)
    pts = np.empty((nv, 3), dtype=np.float64)
    for k in range(nv):
        r = next(it)
        ids[k] = int(r[0])
        pts[k] = (float(r[1]), float(r[2]), float(r[3]))
    first = int(ids[0]) if nv else 0
    it = _rows(base_path + ".ele")
    head = next(it)
    nt = int(head[0])
    tets = np.empty((nt, 4), dtype=np.int64)
    for k in range(nt):
        r = next(it)
        tets[k] = (int(r[1]), int(r[2]), int(r[3]), int(r[4]))
    tets -= first
    if nt and (tets.min() < 0 or tets.max() >= nv):
        raise ValueError("tet indices out of range in %s.ele" % base_path)
    return TetMesh(pts, tets.astype(np.int32))


# the 6 axis orders of the Kuhn split
_PERMS = np.array([(0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0)])


def kuhn_grid(nx, ny, nz, h=1.0, origin=(0.0, 0.0, 0.0), jitter=0.0, seed=0, rng=None):
    """(nx, ny, nz) cells of edge ``h``: (nx+1)(ny+1)(nz+1) vertices, 6 nx ny nz tets.

    Vertex (i, j, k) has id i + (nx+1)(j + (ny+1)k).  Interior vertices move
    by U(-jitter, jitter) * h per coordinate (numpy PCG64 with ``seed`` unless
    ``rng`` is given).  Tets whose signed volume is negative get corners 1 and
    2 swapped.
    """
    rng = np.random.default_rng(seed) if rng is None else rng
    gi, gj, gk = np.meshgrid(np.arange(nx + 1), np.arange(ny + 1), np.arange(nz + 1), indexing="ij")
    ijk = np.stack([gi.ravel(order="F"), gj.ravel(order="F"), gk.ravel(order="F")], 1)
    pts = np.asarray(origin, dtype=np.float64) + h * ijk.astype(np.float64)
    if jitter > 0.0:
        interior = ((ijk > 0) & (ijk < np.array([nx, ny, nz]))).all(1)
        pts[interior] += rng.uniform(-jitter, jitter, size=(int(interior.sum()), 3)) * h

    ci, cj, ck = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    cell = np.stack([ci.ravel(order="F"), cj.ravel(order="F"), ck.ravel(order="F")], 1)  # (C,3)

    def vid(c):
        return c[..., 0] + (nx + 1) * (c[..., 1] + (ny + 1) * c[..., 2])

    eye = np.eye(3, dtype=np.int64)
    c0 = cell[:, None, :]                              # (C,1,3)
    c1 = c0 + eye[_PERMS[:, 0]][None]                  # (C,6,3)
    c2 = c1 + eye[_PERMS[:, 1]][None]
    c3 = c0 + 1
    tets = np.stack([np.broadcast_to(vid(c0), (len(cell), 6)), vid(c1), vid(c2),
                     np.broadcast_to(vid(c3), (len(cell), 6))], axis=-1).reshape(-1, 4)
    tets = tets.astype(np.int64)
    p0, p1, p2, p3 = (pts[tets[:, q]] for q in range(4))
    vol = np.einsum("ij,ij->i", np.cross(p1 - p0, p2 - p0), p3 - p0)
    neg = vol < 0
    tets[neg, 1], tets[neg, 2] = tets[neg, 2].copy(), tets[neg, 1].copy()
    return TetMesh(pts, tets.astype(np.int32))


def random_rotation(rng):
    """Uniform random rotation matrix (QR of a Gaussian matrix, sign-fixed)."""
    q, r = np.linalg.qr(rng.normal(size=(3, 3)))
    q = q * np.sign(np.diag(r))
    if np.linalg.det(q) < 0:
        q[:, 0] = -q[:, 0]
    return q
