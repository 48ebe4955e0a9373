"""Test-only emulation of the Taichi 1.6 subset that the reference solver uses.

This module exists so that the reference's own solver code
(``xpbd_gpu/neohookean_solver.py``, ``xpbd_gpu/xpbd_base.py``, ``xpbd_gpu/sdf.py``)
can be executed unmodified in a container where Taichi is not installed, to
produce golden vectors.  It is test infrastructure only: nothing in the
product imports it.

Semantics emulated (call sites in the reference):

* ``@ti.kernel``: the body runs as plain Python, each top-level ``for`` over
  mesh elements executes sequentially in element order.  Float atomics
  therefore add in a fixed order (Taichi's GPU order is nondeterministic).
* ``ti.field`` / ``ti.Vector.field`` / ``mesh.verts.place``: numpy storage.
  Inside a kernel, ``field[None]`` and ``elem.attr`` return *views* so that
  ``ti.atomic_add``, ``+=`` and ``.fill`` write through, as Taichi lvalues do.
  At Python scope, reads return copies / Python scalars as Taichi does.
* Matrix helpers: ``norm_sqr``, ``norm(eps)`` = sqrt(|v|^2 + eps),
  ``normalized(eps)`` = v / (sqrt(|v|^2) + eps), 3x3 ``determinant`` by
  cofactor expansion along the first column, ``inverse`` = adjugate / det.
* Precision: ``set_precision('f64')`` stores every float field (including
  fields declared ``ti.f32``) in float64 and casts ``ti.f32`` kernel
  arguments to float64, i.e. an FP64 run of the reference's kernels.
  ``set_precision('f32')`` keeps float32 storage and arguments.
"""
import inspect
import sys
import types

import numpy as np

_PREC = {"float": np.float64}
_IN_KERNEL = [0]


def set_precision(name):
    _PREC["float"] = np.float64 if name == "f64" else np.float32


def _fdt():
    return _PREC["float"]


class _DType:
    def __init__(self, name, kind):
        self.name = name
        self.kind = kind

    def np(self):
        if self.kind == "f":
            return _fdt()
        if self.name == "u32":
            return np.uint32
        if self.name == "i64":
            return np.int64
        return np.int32

    def __repr__(self):
        return "ti." + self.name


f32 = _DType("f32", "f")
f64 = _DType("f64", "f")
i32 = _DType("i32", "i")
u32 = _DType("u32", "i")
i64 = _DType("i64", "i")


def _np_dtype(dt):
    if isinstance(dt, _DType):
        return dt.np()
    if dt is float:
        return _fdt()
    if dt is int:
        return np.int32
    raise TypeError("unsupported dtype %r" % (dt,))


class TiArr(np.ndarray):
    """ndarray with the Taichi matrix/vector methods the reference calls."""

    def norm_sqr(self):
        return (np.asarray(self) ** 2).sum()

    def norm(self, eps=0):
        return np.sqrt(self.norm_sqr() + eps)

    def normalized(self, eps=0):
        invlen = 1.0 / (self.norm() + eps)
        return self * invlen

    def cross(self, o):
        a = np.asarray(self)
        b = np.asarray(o)
        return np.array([a[1] * b[2] - a[2] * b[1],
                         a[2] * b[0] - a[0] * b[2],
                         a[0] * b[1] - a[1] * b[0]]).view(TiArr)

    def determinant(self):
        x = np.asarray(self)
        return (x[0, 0] * (x[1, 1] * x[2, 2] - x[2, 1] * x[1, 2])
                - x[1, 0] * (x[0, 1] * x[2, 2] - x[2, 1] * x[0, 2])
                + x[2, 0] * (x[0, 1] * x[1, 2] - x[1, 1] * x[0, 2]))

    def inverse(self):
        x = np.asarray(self)
        inv_det = 1.0 / self.determinant()
        adj = np.empty_like(x)
        adj[0, 0] = x[1, 1] * x[2, 2] - x[2, 1] * x[1, 2]
        adj[1, 0] = x[1, 2] * x[2, 0] - x[1, 0] * x[2, 2]
        adj[2, 0] = x[1, 0] * x[2, 1] - x[2, 0] * x[1, 1]
        adj[0, 1] = x[0, 2] * x[2, 1] - x[0, 1] * x[2, 2]
        adj[1, 1] = x[0, 0] * x[2, 2] - x[0, 2] * x[2, 0]
        adj[2, 1] = x[2, 0] * x[0, 1] - x[0, 0] * x[2, 1]
        adj[0, 2] = x[0, 1] * x[1, 2] - x[0, 2] * x[1, 1]
        adj[1, 2] = x[1, 0] * x[0, 2] - x[0, 0] * x[1, 2]
        adj[2, 2] = x[0, 0] * x[1, 1] - x[1, 0] * x[0, 1]
        return (adj * inv_det).view(TiArr)

    def to_numpy(self):
        return np.array(self)

    @property
    def x(self):
        return self[0]

    @property
    def y(self):
        return self[1]

    @property
    def z(self):
        return self[2]


def _arr(obj):
    return np.asarray(obj, dtype=_fdt()).view(TiArr)


class Vector:
    def __new__(cls, data, dt=None):
        return _arr([np.asarray(d).item() if np.ndim(d) == 0 else d for d in data])

    @staticmethod
    def zero(dt, n):
        return np.zeros(n, dtype=_np_dtype(dt)).view(TiArr)

    @staticmethod
    def field(n, dtype, shape=()):
        return Field(dtype, shape, (n,))


class Matrix:
    @staticmethod
    def cols(cols):
        return np.stack([np.asarray(c) for c in cols], axis=1).astype(_fdt()).view(TiArr)

    @staticmethod
    def field(n, m, dtype, shape=()):
        return Field(dtype, shape, (n, m))


class Field:
    def __init__(self, dtype, shape, elem=()):
        if isinstance(shape, int):
            shape = (shape,)
        self.dtype = dtype
        self.shape = tuple(shape)
        self.elem = tuple(elem)
        self.data = np.zeros(self.shape + self.elem, dtype=_np_dtype(dtype)).view(TiArr)

    def _key(self, key):
        if key is None:
            return Ellipsis
        return key

    def __getitem__(self, key):
        v = self.data[self._key(key)] if key is not None else self.data[...]
        if _IN_KERNEL[0]:
            return v
        if v.ndim == 0:
            return v.item()
        return np.array(v).view(TiArr)

    def __setitem__(self, key, val):
        self.data[self._key(key)] = np.asarray(val)

    def fill(self, val):
        self.data.fill(val)

    def to_numpy(self):
        return np.array(self.data)

    def from_numpy(self, arr):
        self.data[...] = arr


def field(dtype, shape=()):
    return Field(dtype, shape)


# ---- element storage for meshes --------------------------------------------

class _Elem:
    __slots__ = ("_set", "_i")

    def __init__(self, eset, i):
        object.__setattr__(self, "_set", eset)
        object.__setattr__(self, "_i", i)

    @property
    def id(self):
        return self._i

    @property
    def verts(self):
        rel = self._set.relations["verts"]
        vset = self._set.mesh.verts
        row = rel[self._i]
        return [_Elem(vset, int(j)) for j in row]

    def __getattr__(self, name):
        f = self._set.fields[name]
        return f.data[self._i, ...]

    def __setattr__(self, name, val):
        f = self._set.fields[name]
        f.data[self._i] = np.asarray(val)


class _ElemSet:
    def __init__(self, mesh, n):
        self.mesh = mesh
        self.n = n
        self.fields = {}
        self.relations = {}

    def place(self, spec, reorder=False):
        for name, t in spec.items():
            if isinstance(t, tuple) and t[0] == "vec":
                fld = Field(f32 if t[2] == "f" else i32, (self.n,), (t[1],))
            elif isinstance(t, tuple) and t[0] == "mat":
                fld = Field(f32, (self.n,), (t[1], t[2]))
            else:
                fld = Field(t, (self.n,))
            self.fields[name] = fld

    def __getattr__(self, name):
        if name in ("mesh", "n", "fields", "relations"):
            raise AttributeError(name)
        try:
            return self.fields[name]
        except KeyError:
            raise AttributeError(name)

    def __len__(self):
        return self.n

    def __iter__(self):
        for i in range(self.n):
            yield _Elem(self, i)


class TetMeshShim:
    def __init__(self, points, tets):
        self._points = np.asarray(points, dtype=np.float64)
        self.verts = _ElemSet(self, len(points))
        self.cells = _ElemSet(self, len(tets))
        self.cells.relations["verts"] = np.asarray(tets, dtype=np.int64)

    def get_position_as_numpy(self):
        return self._points.copy()


# ---- decorators and intrinsics ---------------------------------------------

def kernel(fn):
    ann = dict(getattr(fn, "__annotations__", {}))
    sig = inspect.signature(fn)

    def wrapper(*args, **kwargs):
        bound = sig.bind(*args, **kwargs)
        for name, val in list(bound.arguments.items()):
            t = ann.get(name)
            if isinstance(t, _DType):
                bound.arguments[name] = (_fdt()(val) if t.kind == "f" else t.np()(val))
        _IN_KERNEL[0] += 1
        try:
            return fn(*bound.args, **bound.kwargs)
        finally:
            _IN_KERNEL[0] -= 1

    wrapper.__name__ = fn.__name__
    return wrapper


def func(fn):
    return fn


def data_oriented(cls):
    return cls


def template():
    return None


def static(x):
    return x


def loop_config(**kw):
    return None


def mesh_local(*args):
    return None


def atomic_add(ref, val):
    old = np.array(ref)
    ref += val
    return old


def abs(x):  # noqa: A001 - mirrors ti.abs
    return np.abs(x)


def sqrt(x):
    return np.sqrt(x)


def exp(x):
    return np.exp(x)


def max(a, b):  # noqa: A001
    return np.maximum(a, b)


def min(a, b):  # noqa: A001
    return np.minimum(a, b)


def init(arch=None, **kw):
    return None


cpu = "cpu"
gpu = "gpu"
cuda = "cuda"

math_mod = types.ModuleType("taichi.math")
math_mod.vec3 = ("vec", 3, "f")
math_mod.mat3 = ("mat", 3, 3)
math = math_mod


def read_tetgen(node_path):
    """Read a TetGen .node/.ele pair (0- or 1-based ids)."""
    with open(node_path) as f:
        toks = [ln.split() for ln in f if ln.strip() and not ln.lstrip().startswith("#")]
    nv = int(toks[0][0])
    rows = toks[1:1 + nv]
    base = int(rows[0][0])
    pts = np.array([[float(r[1]), float(r[2]), float(r[3])] for r in rows])
    ele_path = node_path[:-5] + ".ele" if node_path.endswith(".node") else node_path + ".ele"
    with open(ele_path) as f:
        toks = [ln.split() for ln in f if ln.strip() and not ln.lstrip().startswith("#")]
    nt = int(toks[0][0])
    tets = np.array([[int(r[1]), int(r[2]), int(r[3]), int(r[4])] for r in toks[1:1 + nt]]) - base
    return pts, tets


def install(precision="f64", meshes=None):
    """Register the shim as ``taichi`` and a fake ``meshtaichi_patcher``.

    ``meshes`` maps a path string to (points, tets); other paths are read as
    TetGen files.  Vertex and cell order is kept as given (no reorder).
    """
    set_precision(precision)
    me = sys.modules[__name__]
    sys.modules["taichi"] = me
    sys.modules["taichi.math"] = math_mod
    patcher = types.ModuleType("meshtaichi_patcher")
    registry = dict(meshes or {})

    def load_mesh(path, relations=None):
        if path in registry:
            pts, tets = registry[path]
        else:
            pts, tets = read_tetgen(path)
        return TetMeshShim(pts, tets)

    patcher.load_mesh = load_mesh
    patcher._registry = registry
    sys.modules["meshtaichi_patcher"] = patcher
    return patcher
