"""SDF obstacles with the reference's constructors and accessors (xpbd_gpu/sdf.py).

The reference keeps SDF parameters in 0-d Taichi fields, read as
``sdf.center[None].to_numpy()`` / ``float(sdf.radius[None])`` by
``usd_export.py:75-92``.  Here each parameter is a small host-side ``Param``
that supports the same ``[None]`` get/set; the solver packs the SDF list into
an ``xpbd_sdf`` table on the device (``include/xpbd_gb300.h``) and re-uploads
it whenever a parameter changes.  Distance and normal are evaluated by the
CUDA kernels; ``dist``/``normal`` here are float64 host versions used for the
one-time pinning test at construction (``xpbd_base.py:124-137``).
"""
import numpy as np

from xpbd_gpu import _native
from xpbd_gpu.constants import EPSILON


class Value(np.ndarray):
    """A parameter value: a float32 numpy vector with Taichi's ``.to_numpy()``."""

    def to_numpy(self):
        return np.array(self)


class Param:
    """0-d field stand-in: ``p[None]`` reads, ``p[None] = v`` writes."""

    def __init__(self, owner, value, scalar=False):
        self._owner = owner
        self._scalar = scalar
        self._set(value)

    def _set(self, value):
        if self._scalar:
            self._v = float(np.float32(value))
        else:
            self._v = np.asarray(value, dtype=np.float32).reshape(3).copy()
        self._owner._version += 1

    def __getitem__(self, key):
        if key is not None:
            raise IndexError("SDF parameters are 0-d; index with [None]")
        if self._scalar:
            return self._v
        return self._v.copy().view(Value)

    def __setitem__(self, key, value):
        if key is not None:
            raise IndexError("SDF parameters are 0-d; index with [None]")
        self._set(value)

    def to_numpy(self):
        return np.array(self._v)


class SdfModel:
    """sdf.py:7-27.  ``fixed`` obstacles project every penetrating vertex;
    moving ones only vertices approaching them (dot(n, v_sdf - v) > 0)."""

    kind = None

    def __init__(self, fixed):
        self._version = 0
        self.vel = Param(self, (0.0, 0.0, 0.0))
        self.fixed = Param(self, 1.0 if fixed else 0.0, scalar=True)

    # host float64 versions (pinning at construction only)
    def dist(self, pos):
        raise NotImplementedError

    def normal(self, pos):
        raise NotImplementedError

    def check(self, pos, vel):
        """sdf.py:14-27 over arrays: returns (fixed, inside mask, normals)."""
        pos = np.asarray(pos, dtype=np.float64)
        phi = self.dist(pos)
        neg = phi < 0.0
        n = np.zeros_like(pos)
        if neg.any():
            n[neg] = self.normal(pos[neg])
        diff_vel = self.vel[None].astype(np.float64) - vel
        dotnv = (n * diff_vel).sum(-1)
        fixed = bool(self.fixed[None])
        inside = neg & ((dotnv > 0.0) | fixed)
        return fixed, inside, n

    def _pack(self, s):
        raise NotImplementedError

    def to_struct(self):
        s = _native.XpbdSdf()
        s.kind = self.kind
        s.fixed = 1 if self.fixed[None] else 0
        s.vel[:] = [float(c) for c in self.vel[None]]
        self._pack(s)
        return s


class PlaneSdf(SdfModel):
    """sdf.py:59-74: dist = (p - point) . dir with dir normalised at construction."""

    kind = _native.SDF_PLANE

    def __init__(self, point, dir, fixed=False):  # noqa: A002 - reference keyword
        super().__init__(fixed=fixed)
        d = np.asarray(dir, dtype=np.float64)
        self.point = Param(self, point)
        self.dir = Param(self, d / np.sqrt((d * d).sum()))

    def dist(self, pos):
        return ((pos - self.point[None]) * self.dir[None]).sum(-1)

    def normal(self, pos):
        return np.broadcast_to(self.dir[None].astype(np.float64), pos.shape).copy()

    def _pack(self, s):
        s.a[:] = [float(c) for c in self.point[None]]
        s.b[:] = [float(c) for c in self.dir[None]]


class SphereSdf(SdfModel):
    """sdf.py:77-95: dist = |p - c| - r, normal = (p - c) / (|p - c| + EPS)."""

    kind = _native.SDF_SPHERE

    def __init__(self, center, radius, fixed=False):
        super().__init__(fixed=fixed)
        self.center = Param(self, center)
        self.radius = Param(self, radius, scalar=True)

    def dist(self, pos):
        d = pos - self.center[None]
        return np.sqrt((d * d).sum(-1)) - self.radius[None]

    def normal(self, pos):
        d = pos - self.center[None]
        return d / (np.sqrt((d * d).sum(-1)) + EPSILON)[:, None]

    def _pack(self, s):
        s.a[:] = [float(c) for c in self.center[None]]
        s.b[:] = [float(self.radius[None]), 0.0, 0.0]


class CubeSdf(SdfModel):
    """sdf.py:98-124: box SDF; the normal is the sign of the dominant axis of (p - c)."""

    kind = _native.SDF_CUBE

    def __init__(self, center, size, fixed=False):
        super().__init__(fixed=fixed)
        self.center = Param(self, center)
        self.half_size = Param(self, np.asarray(size, dtype=np.float64) * 0.5)

    def dist(self, pos):
        d = np.abs(pos - self.center[None]) - self.half_size[None]
        m = np.maximum(d, 0.0)
        return np.sqrt((m * m).sum(-1)) + np.minimum(d.max(-1), 0.0)

    def normal(self, pos):
        d = pos - self.center[None]
        a = np.abs(d)
        axis = np.zeros(len(pos), dtype=np.int64)
        axis = np.where(a[:, 1] > a[:, 0], 1, axis)
        axis = np.where(a[:, 2] > a[np.arange(len(pos)), axis], 2, axis)
        n = np.zeros_like(pos)
        sel = d[np.arange(len(pos)), axis]
        n[np.arange(len(pos)), axis] = np.where(sel > 0, 1.0, -1.0)
        return n

    def _pack(self, s):
        s.a[:] = [float(c) for c in self.center[None]]
        s.b[:] = [float(c) for c in self.half_size[None]]
