"""Build and run oracle/xpbd_oracle_c.c -- TEST INFRASTRUCTURE ONLY.

The threaded C restatement of the reference substep: FP32 (the reference's
arithmetic type) as the timed CPU baseline and a second checker, and FP64 as
the float64 reference run of meshes too large for the NumPy oracle.  Built
with gcc into oracle/_build/liboracle_xpbd.so and liboracle_xpbd64.so (no
-march=native, no fast-math).
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "xpbd_oracle_c.c")
LIB = os.path.join(HERE, "_build", "liboracle_xpbd.so")
LIB64 = os.path.join(HERE, "_build", "liboracle_xpbd64.so")


class OcSdf(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("fixed", ctypes.c_int), ("a", ctypes.c_float * 3),
                ("b", ctypes.c_float * 3), ("vel", ctypes.c_float * 3)]


class OcParams(ctypes.Structure):
    _fields_ = [("mu", ctypes.c_float), ("lam", ctypes.c_float), ("gravity", ctypes.c_float * 3),
                ("damping", ctypes.c_float), ("relax_h", ctypes.c_float), ("relax_d", ctypes.c_float),
                ("gamma", ctypes.c_float), ("cheb", ctypes.c_int), ("warmup", ctypes.c_int),
                ("block", ctypes.c_int), ("iters", ctypes.c_int), ("precise", ctypes.c_int),
                ("rho_min", ctypes.c_double), ("rho_max", ctypes.c_double), ("rho_beta", ctypes.c_double)]


def _build_one(lib, defines, force):
    if not force and os.path.exists(lib) and os.path.getmtime(lib) >= os.path.getmtime(SRC):
        return lib
    os.makedirs(os.path.dirname(lib), exist_ok=True)
    tmp = lib + ".tmp"
    cmd = ["gcc", "-O3", "-std=c11", "-fPIC", "-shared", "-pthread"] + defines + ["-o", tmp, SRC, "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("gcc failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
    os.replace(tmp, lib)
    return lib


def build(force=False):
    """Build the FP32 and the FP64 library; returns the FP32 path."""
    _build_one(LIB64, ["-DOC_DOUBLE"], force)
    return _build_one(LIB, [], force)


_libs = {}


def load(double=False):
    key = bool(double)
    if key not in _libs:
        build()
        lib = ctypes.CDLL(LIB64 if key else LIB)
        lib.oc_run.restype = ctypes.c_int
        lib.oc_run.argtypes = [ctypes.c_int, ctypes.c_int] + [ctypes.c_void_p] * 6 + [
            ctypes.POINTER(OcSdf), ctypes.c_int, ctypes.POINTER(OcParams), ctypes.c_double, ctypes.c_double,
            ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_double), ctypes.c_int, ctypes.c_void_p]
        _libs[key] = lib
    return _libs[key]


class COracle:
    """Same constructor as oracle.xpbd_oracle.OracleSolver (setup computed by it in
    float64), stepping frames with the C restatement in `dtype` (np.float32, the
    reference's arithmetic, or np.float64)."""

    def __init__(self, points, tets, sdf, threads=None, dtype=np.float32, **kw):
        from oracle.xpbd_oracle import OracleSolver
        o = OracleSolver(points, tets, sdf, dtype=np.float64, **kw)
        self._o = o
        self.dtype = np.dtype(dtype)
        if self.dtype not in (np.float32, np.float64):
            raise ValueError("dtype must be float32 or float64")
        dt_ = self.dtype
        self.x = o.x.astype(dt_).copy()
        self.v = o.v.astype(dt_).copy()
        self.tets = np.ascontiguousarray(o.tets, dtype=np.int32)
        self.inv_Dm = np.ascontiguousarray(o.inv_Dm.reshape(-1, 9), dtype=dt_)
        self.V0 = np.ascontiguousarray(o.V0, dtype=dt_)
        self.inv_m = np.ascontiguousarray(o.inv_m, dtype=dt_)
        self.rho_hat = ctypes.c_double(0.999)
        self.threads = threads or os.cpu_count() or 1
        self.sdfs = (OcSdf * len(o.sdfs))()
        for k, s in enumerate(o.sdfs):
            e = self.sdfs[k]
            e.kind = {"plane": 0, "sphere": 1, "cube": 2}[s.kind]
            e.fixed = 1 if s.fixed else 0
            if s.kind == "plane":
                e.a[:], e.b[:] = list(s.point), list(s.dir)
            elif s.kind == "sphere":
                e.a[:], e.b[:] = list(s.center), [s.radius, 0.0, 0.0]
            else:
                e.a[:], e.b[:] = list(s.center), list(s.half_size)
        p = OcParams()
        p.mu, p.lam = o.lame2, o.lame1
        p.gravity[:] = list(o.gravity)
        p.damping = o.damping
        p.relax_h, p.relax_d = o.hydrostatic_relaxation, o.deviatoric_relaxation
        p.gamma = o.cheb_gamma
        p.cheb, p.warmup = int(o.cheb_enable), int(o.cheb_warmup)
        p.block, p.iters = int(o.block_neohookean_enable), int(o.constraints_iter)
        p.precise = int(kw.get("poisson_ratio", 0.495) >= 0.49)
        p.rho_min, p.rho_max, p.rho_beta = o.rho_min, o.rho_max, o.rho_beta
        self.p = p
        self.frame_dt, self.dt, self.substeps = o.frame_dt, o.dt, o.substeps_num

    def solve(self, frames=1, r_hat_hist=None):
        buf = None
        if r_hat_hist is not None:
            buf = r_hat_hist.ctypes.data
        rc = load(self.dtype == np.float64).oc_run(len(self.x), len(self.tets), self.x.ctypes.data, self.v.ctypes.data,
                           self.tets.ctypes.data, self.inv_Dm.ctypes.data, self.V0.ctypes.data,
                           self.inv_m.ctypes.data, self.sdfs, len(self.sdfs), ctypes.byref(self.p),
                           self.frame_dt, self.dt, self.substeps, frames, ctypes.byref(self.rho_hat),
                           self.threads, buf)
        if rc != 0:
            raise RuntimeError("oc_run failed")
