"""XPBDSolverBase: mesh, device buffers and the vertex-level steps (xpbd_gpu/xpbd_base.py).

Interface kept from the reference (``xpbd_base.py:11-204``): constructor
arguments, ``mesh.verts.{x,pred_x,v,m,inv_m}``, ``indices``, ``sdfs``/``sdf``,
``gravity``/``damping``/``total_mass``, ``apply_external_forces``,
``advance``, ``solve_sdf_collision``, ``compute_lumped_mass`` and ``solve``.

Layout on the device (torch CUDA tensors, handed to ``libxpbd_gb300.so`` as
raw pointers): per vertex float4 ``x``, ``v``, two predicted-position buffers
``p0``/``p1`` and the Jacobi accumulator ``dx``; per tet ``int4`` corner ids,
``inv_Dm`` as float4/float4/float, ``V0`` and ``(lambda_D, lambda_H)`` as
float2 (tet records padded to a multiple of 256 tets), plus, for the tile
variant, 4 u8 patch-local corner ids per tet and the patch vertex lists.  Vertices and tets are stored in Morton order; the field accessors
return and accept arrays in the caller's (file) order.
"""
import os

import numpy as np

from xpbd_gpu import _native
from xpbd_gpu.constants import EPSILON
from xpbd_gpu.mesh import TetMesh, read_tetgen

FACE_TABLE = np.array([[0, 2, 1], [0, 3, 2], [0, 1, 3], [1, 2, 3]])  # xpbd_base.py:83


def calc_tet_volume(p0, p1, p2, p3):
    """xpbd_base.py:6-8 (vectorised over leading axes)."""
    return np.einsum("...i,...i->...", np.cross(p1 - p0, p2 - p0), p3 - p0) / 6.0


def inv_dm_of(x, tets):
    """inverse([x1 - x0, x2 - x0, x3 - x0]) of every tet (neohookean_solver.py:97-107), float64."""
    P = np.asarray(x, dtype=np.float64)[tets]
    Ds = np.stack([P[:, 1] - P[:, 0], P[:, 2] - P[:, 0], P[:, 3] - P[:, 0]], axis=-1)
    with np.errstate(divide="ignore", invalid="ignore"):
        return np.linalg.inv(Ds)


def _torch():
    import torch
    return torch


def _require_cuda():
    torch = _torch()
    if not torch.cuda.is_available():
        raise RuntimeError("xpbd_gpu runs only on a CUDA GPU (sm_103a); no CUDA device is visible "
                           "and there is no CPU fallback")
    return torch


class VertexVec3Field:
    """``mesh.verts.<name>`` for a vec3 stored in a float4 device buffer."""

    def __init__(self, solver, field_id):
        self._s = solver
        self._id = field_id

    @property
    def shape(self):
        return (self._s.n_verts,)

    def to_numpy(self):
        return self._s._export_vec3(self._id)

    def from_numpy(self, arr):
        self._s._import_vec3(self._id, arr)

    def to_torch(self, device=None):
        t = self._s._export_vec3_device(self._id)
        return t if device is None else t.to(device)


class VertexScalarField:
    """``mesh.verts.m`` / ``mesh.verts.inv_m``."""

    def __init__(self, solver, name):
        self._s = solver
        self._name = name

    @property
    def shape(self):
        return (self._s.n_verts,)

    def to_numpy(self):
        return getattr(self._s, "_host_" + self._name).astype(np.float32).copy()

    def from_numpy(self, arr):
        if self._name != "inv_m":
            raise AttributeError("only inv_m can be written")
        self._s._set_inv_m(np.asarray(arr, dtype=np.float64))


class CellField:
    """``mesh.cells.<name>`` read back in the caller's tet order."""

    def __init__(self, solver, getter):
        self._s = solver
        self._get = getter

    @property
    def shape(self):
        return (self._s.n_tets,)

    def to_numpy(self):
        return self._get()

    def fill(self, value):
        if value != 0.0:
            raise ValueError("only fill(0.0) is supported")
        self._s._lam.zero_()


class HostField:
    """A host array with the Taichi field accessors (``indices``)."""

    def __init__(self, arr):
        self._a = arr

    @property
    def shape(self):
        return self._a.shape

    def to_numpy(self):
        return self._a.copy()

    def __len__(self):
        return len(self._a)


class ElementSet:
    def __init__(self, n, fields):
        self._n = n
        self.__dict__.update(fields)

    def __len__(self):
        return self._n


class DeviceMesh:
    """``solver.mesh``: ``verts``/``cells`` element sets and the rest positions."""

    def __init__(self, points, verts, cells):
        self._points = points
        self.verts = verts
        self.cells = cells

    def get_position_as_numpy(self):
        return self._points.copy()


def load_rest_pose(rest_pose):
    """``rest_pose`` as in the reference (a ``.node`` path) or, as extensions, a
    TetMesh or a ``(points, tets)`` pair."""
    if isinstance(rest_pose, TetMesh):
        return rest_pose
    if isinstance(rest_pose, (tuple, list)) and len(rest_pose) == 2:
        return TetMesh(np.asarray(rest_pose[0], dtype=np.float64), np.asarray(rest_pose[1], dtype=np.int32))
    if isinstance(rest_pose, (str, os.PathLike)):
        return read_tetgen(os.fspath(rest_pose))
    raise TypeError("rest_pose must be a .node path, a TetMesh or (points, tets)")


class XPBDSolverBase:
    """Base class for deformable object solvers (xpbd_base.py:11-204)."""

    def __init__(self, rest_pose, sdf, scale=1.0, offset=(0.0, 0.0, 0.0), frame_dt=1e-2, dt=1e-2,
                 substeps_num=20, reorder_all=False, block_size=128, total_mass=1.0, density=None,
                 gravity=(0.0, -9.8, 0.0), reorder=True, pair_tets=True):
        # Collision list first: the reference raises ValueError for an empty list (:60-67)
        if isinstance(sdf, (list, tuple)):
            self.sdfs = [s for s in sdf if s is not None]
        else:
            self.sdfs = [sdf] if sdf is not None else []
        if len(self.sdfs) == 0:
            raise ValueError("At least one SDF object must be provided.")
        self.sdf = self.sdfs[0]

        torch = _require_cuda()
        self._lib = _native.load()
        self._device = torch.device("cuda", torch.cuda.current_device())

        self.time = 0.0
        self.frame_dt = frame_dt
        self.dt = dt
        self.substeps_num = substeps_num
        self.gravity = np.asarray(gravity, dtype=np.float64)  # xpbd_base.py:33-34
        self.damping = 5.0                                    # :35
        self.total_mass = 1.0 if total_mass is None else float(total_mass)  # :36
        self._density = density
        self.block_size = block_size
        self.reorder_all = reorder_all
        self._handle = None

        mesh = load_rest_pose(rest_pose)
        self._rest = mesh
        self.n_verts = mesh.n_verts
        self.n_tets = mesh.n_tets
        if self.n_verts == 0 or self.n_tets == 0:
            raise ValueError("mesh has no vertices or no tets")
        tets = np.asarray(mesh.tets, dtype=np.int64)
        if tets.min() < 0 or tets.max() >= self.n_verts:
            raise ValueError("tet indices out of range")
        self._tets_host = tets

        # xpbd_base.py:56-58, :78-87: per-tet face triangles in caller vertex ids
        self.indices = HostField(tets[:, FACE_TABLE].reshape(-1).astype(np.uint32))

        self._reorder = bool(reorder)
        self.pair_tets = bool(pair_tets)
        self.initialize_specific(scale, offset)

    # -- setup ----------------------------------------------------------------
    def _orderings(self, x):
        V, T = self.n_verts, self.n_tets
        if not self._reorder:
            return np.arange(V, dtype=np.int32), np.arange(T, dtype=np.int32)
        vperm = np.empty(V, dtype=np.int32)
        tperm = np.empty(T, dtype=np.int32)
        pts = np.ascontiguousarray(x, dtype=np.float64)
        tt = np.ascontiguousarray(self._tets_host, dtype=np.int32)
        _native.check(self._lib.xpbd_morton_order(pts.ctypes.data, V, tt.ctypes.data, T,
                                                  vperm.ctypes.data, tperm.ctypes.data))
        return vperm, tperm

    def initialize(self, scale, offset):
        """neohookean_solver.py:97-107 in float64 on the host: x = x*scale + offset,
        V0 = calc_tet_volume, inv_Dm = inverse([x1-x0, x2-x0, x3-x0])."""
        x = self._rest.points * float(scale) + np.asarray(offset, dtype=np.float64)
        P = x[self._tets_host]
        Ds = np.stack([P[:, 1] - P[:, 0], P[:, 2] - P[:, 0], P[:, 3] - P[:, 0]], axis=-1)
        V0 = calc_tet_volume(P[:, 0], P[:, 1], P[:, 2], P[:, 3])
        with np.errstate(divide="ignore", invalid="ignore"):
            inv_Dm = np.linalg.inv(Ds)
        return x, V0, inv_Dm

    def compute_lumped_mass(self, x, V0):
        """xpbd_base.py:89-137: lumped masses scaled to ``total_mass``, then vertices
        initially inside a fixed SDF are pinned (inv_m = 0)."""
        bad = int((V0 <= EPSILON).sum())
        if bad:
            print("Warning: %d cells have negative or zero volume" % bad)
        m = np.zeros(self.n_verts, dtype=np.float64)
        np.add.at(m, self._tets_host.reshape(-1), np.repeat(V0 * 0.25, 4))
        total_volume = float(V0.sum())
        total_mass = self.total_mass
        if self._density is not None:  # extension: total mass from a density
            total_mass = float(self._density) * total_volume
            self.total_mass = total_mass
        m *= total_mass / total_volume
        inv_m = np.where(m > 0.0, 1.0 / np.where(m > 0.0, m, 1.0), 0.0)
        v0 = np.zeros((self.n_verts, 3))
        for s in self.sdfs:
            live = inv_m > 0.0
            fixed, inside, _ = s.check(x, v0)
            if fixed:
                inv_m[live & inside] = 0.0
        return m, inv_m

    def _upload(self, x, V0, inv_Dm, m, inv_m):
        self._inv_dm_file = inv_Dm
        torch = _torch()
        dev = self._device
        V, T = self.n_verts, self.n_tets
        vperm, tperm = self._orderings(x)
        inv_vperm = np.empty(V, dtype=np.int64)
        inv_vperm[vperm] = np.arange(V)
        self._vperm, self._tperm = vperm, tperm
        tets_new = inv_vperm[self._tets_host[tperm]].astype(np.int32)
        self.n_tet_pairs = 0
        dm_solver = inv_Dm[tperm]
        if self.pair_tets:
            order, cperm, self.n_tet_pairs = _native.pair_tets(self._lib, tets_new, V)
            tperm = tperm[order]
            self._tperm = tperm
            tets_new = np.ascontiguousarray(np.take_along_axis(tets_new[order], cperm, axis=1), dtype=np.int32)
            dm_solver = inv_dm_of(x, np.take_along_axis(self._tets_host[tperm], cperm, axis=1))
        self._tets_solver = tets_new
        x4 = np.zeros((V, 4), dtype=np.float32)
        x4[:, :3] = x[vperm]
        x4[:, 3] = inv_m[vperm]
        # tet records are padded to a multiple of the largest patch (256 tets)
        # so that every patch's slice can be bulk-copied whole
        Tp = -(-T // 256) * 256
        D = np.zeros((Tp, 9), dtype=np.float32)
        D[:T] = dm_solver.reshape(T, 9)
        dm_a = np.ascontiguousarray(D[:, 0:4])
        dm_b = np.ascontiguousarray(D[:, 4:8])
        dm_c = np.ascontiguousarray(D[:, 8])
        v0 = V0[tperm].astype(np.float32)

        def dt_(a, dtype=torch.float32):
            return torch.from_numpy(np.ascontiguousarray(a)).to(device=dev, dtype=dtype)

        self._x4 = dt_(x4)
        self._v4 = torch.zeros((V, 4), dtype=torch.float32, device=dev)
        self._p4 = [self._x4.clone(), self._x4.clone()]
        self._dx4 = torch.zeros((V, 4), dtype=torch.float32, device=dev)
        self._tets = dt_(tets_new, torch.int32)
        self._dm_a, self._dm_b, self._dm_c = dt_(dm_a), dt_(dm_b), dt_(dm_c)
        self._v0 = dt_(v0)
        self._lam = torch.zeros((Tp, 2), dtype=torch.float32, device=dev)
        self._perm = dt_(vperm, torch.int32)
        self._stage = torch.empty((V, 3), dtype=torch.float32, device=dev)
        self._v2t_off = self._v2t_slots = self._corner = None
        self._tet_lid = self._patch_voff = self._patch_verts = None
        self._patch_tets = 0
        self._host_m = m
        self._host_inv_m = inv_m.copy()

    def _ensure_gather_buffers(self):
        if self._corner is not None:
            return
        torch = _torch()
        V, T = self.n_verts, self.n_tets
        off = np.empty(V + 1, dtype=np.int32)
        slots = np.empty(4 * T, dtype=np.int32)
        tt = np.ascontiguousarray(self._tets_solver)
        _native.check(self._lib.xpbd_build_vertex_csr(tt.ctypes.data, T, V, off.ctypes.data, slots.ctypes.data))
        self._v2t_off = torch.from_numpy(off).to(self._device)
        self._v2t_slots = torch.from_numpy(slots).to(self._device)
        self._corner = torch.zeros((4 * T, 4), dtype=torch.float32, device=self._device)

    def _ensure_patch_buffers(self):
        """Patches of P consecutive tets (solver order) with <= 256 vertices each (P =
        the largest of 256, 128, 64 not above ``patch_tets`` whose patches all
        fit); returns False if none fits."""
        if self._tet_lid is not None:
            return True
        torch = _torch()
        V, T = self.n_verts, self.n_tets
        tt = np.ascontiguousarray(self._tets_solver)
        for P in (p for p in (256, 128, 64) if p <= getattr(self, "patch_tets", 256)):
            npat = (T + P - 1) // P
            voff = np.empty(npat + 1, dtype=np.int32)
            pverts = np.empty(4 * T, dtype=np.int32)
            lid = np.zeros(-(-T // 256) * 256, dtype=np.uint32)
            mx = _native.ctypes.c_int32()
            _native.check(self._lib.xpbd_build_patches(tt.ctypes.data, T, V, P, voff.ctypes.data, pverts.ctypes.data,
                                                       lid.ctypes.data, _native.ctypes.byref(mx)))
            if mx.value <= 256:
                self._patch_tets = P
                self._n_patches = npat
                self._tet_lid = torch.from_numpy(lid.view(np.int32)).to(self._device)
                self._patch_voff = torch.from_numpy(voff).to(self._device)
                self._patch_verts = torch.from_numpy(pverts[:voff[-1]].copy()).to(self._device)
                self.patch_max_verts = mx.value
                pv_start = np.empty(int(voff[-1]), dtype=np.uint16)
                pv_slots = np.empty(4 * npat * P, dtype=np.uint16)
                _native.check(self._lib.xpbd_build_patch_csr(voff.ctypes.data, lid.ctypes.data, T, P,
                                                             pv_start.ctypes.data, pv_slots.ctypes.data))
                self._pv_start = torch.from_numpy(pv_start.view(np.int16)).to(self._device)
                self._pv_slots = torch.from_numpy(pv_slots.view(np.int16)).to(self._device)
                return True
        return False

    def _body(self):
        b = _native.XpbdBody()
        b.n_verts, b.n_tets = self.n_verts, self.n_tets
        b.x, b.v = self._x4.data_ptr(), self._v4.data_ptr()
        b.p0, b.p1 = self._p4[0].data_ptr(), self._p4[1].data_ptr()
        b.dx = self._dx4.data_ptr()
        b.tets = self._tets.data_ptr()
        b.dm_a, b.dm_b, b.dm_c = self._dm_a.data_ptr(), self._dm_b.data_ptr(), self._dm_c.data_ptr()
        b.v0 = self._v0.data_ptr()
        b.lam = self._lam.data_ptr()
        if getattr(self, "_tinv_mu", None) is not None:
            b.tet_inv_mu = self._tinv_mu.data_ptr()
            b.tet_inv_lambda = self._tinv_la.data_ptr()
        if self._tet_lid is not None:
            b.n_patches, b.patch_tets = self._n_patches, self._patch_tets
            b.tet_lid = self._tet_lid.data_ptr()
            b.patch_voff = self._patch_voff.data_ptr()
            b.patch_verts = self._patch_verts.data_ptr()
            b.pv_start = self._pv_start.data_ptr()
            b.pv_slots = self._pv_slots.data_ptr()
        if self._corner is not None:
            b.v2t_offsets = self._v2t_off.data_ptr()
            b.v2t_slots = self._v2t_slots.data_ptr()
            b.corner_dx = self._corner.data_ptr()
        b.vert_perm = self._perm.data_ptr()
        b.tet_pairs = 1 if self.pair_tets else 0
        return b

    def _sdf_table(self):
        arr = (_native.XpbdSdf * len(self.sdfs))()
        for k, s in enumerate(self.sdfs):
            arr[k] = s.to_struct()
        self._sdf_versions = [s._version for s in self.sdfs]
        return arr

    def _build_mesh_view(self):
        verts = ElementSet(self.n_verts, dict(
            x=VertexVec3Field(self, _native.FIELD_X),
            v=VertexVec3Field(self, _native.FIELD_V),
            pred_x=VertexVec3Field(self, _native.FIELD_PRED_X),
            m=VertexScalarField(self, "m"),
            inv_m=VertexScalarField(self, "inv_m")))
        cells = ElementSet(self.n_tets, dict(
            V0=CellField(self, lambda: self._cell_array(self._v0)),
            inv_Dm=CellField(self, self._inv_dm_array),
            lambda_D=CellField(self, lambda: self._cell_array(self._lam[:self.n_tets, 0])),
            lambda_H=CellField(self, lambda: self._cell_array(self._lam[:self.n_tets, 1]))))
        self.mesh = DeviceMesh(self._rest.points, verts, cells)

    # -- device access helpers -------------------------------------------------
    def _stream(self):
        return _torch().cuda.current_stream(self._device).cuda_stream

    def _cell_array(self, t):
        a = t.detach().cpu().numpy()
        out = np.empty_like(a)
        out[self._tperm] = a
        return out

    def _inv_dm_array(self):
        """inv_Dm in the caller's tet and corner order (the device copy of a
        face-paired tet is that of its reordered corners)."""
        return self._inv_dm_file.astype(np.float32)

    def _export_vec3_device(self, field_id):
        out = _torch().empty((self.n_verts, 3), dtype=_torch().float32, device=self._device)
        _native.check(self._lib.xpbd_export_vec3(self._handle, field_id, out.data_ptr(), self._stream()))
        return out

    def _export_vec3(self, field_id):
        return self._export_vec3_device(field_id).cpu().numpy()

    def _import_vec3(self, field_id, arr):
        torch = _torch()
        a = arr if isinstance(arr, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(arr, dtype=np.float32))
        if tuple(a.shape) != (self.n_verts, 3):
            raise ValueError("expected shape (%d, 3), got %s" % (self.n_verts, tuple(a.shape)))
        self._stage.copy_(a, non_blocking=True)
        _native.check(self._lib.xpbd_import_vec3(self._handle, field_id, self._stage.data_ptr(), self._stream()))

    def _set_inv_m(self, inv_m):
        torch = _torch()
        self._host_inv_m = inv_m.copy()
        w = torch.from_numpy(inv_m[self._vperm].astype(np.float32)).to(self._device)
        self._x4[:, 3] = w
        self._p4[0][:, 3] = w
        self._p4[1][:, 3] = w

    # -- reference methods -----------------------------------------------------
    def apply_external_forces(self, dt):
        """xpbd_base.py:139-146."""
        self._sync()
        _native.check(self._lib.xpbd_apply_external_forces(self._handle, float(dt), self._stream()))

    def advance(self, dt, damping):
        """xpbd_base.py:148-160."""
        _native.check(self._lib.xpbd_advance(self._handle, float(dt), float(damping), self._stream()))

    def solve_sdf_collision(self, dt):
        """xpbd_base.py:176-178: every SDF in list order, one vertex pass."""
        self._sync()
        _native.check(self._lib.xpbd_solve_sdf_collision(self._handle, float(dt), self._stream()))

    def _sync(self):
        """Push host-side changes (SDF parameters, constants) to the device."""
        if [s._version for s in self.sdfs] != getattr(self, "_sdf_versions", None):
            table = self._sdf_table()
            _native.check(self._lib.xpbd_set_sdfs(self._handle, table, len(self.sdfs), self._stream()))

    def initialize_specific(self, scale, offset):
        raise NotImplementedError("Derived classes must implement initialize_specific")

    def solve_step(self, dt):
        raise NotImplementedError("Derived classes must implement solve_step")

    def __del__(self):
        h = getattr(self, "_handle", None)
        if h is not None:
            try:
                self._lib.xpbd_destroy(h)
            except Exception:
                pass
            self._handle = None
