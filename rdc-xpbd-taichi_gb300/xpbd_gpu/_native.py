"""Build and load ``libxpbd_gb300.so`` (hand-written sm_103a CUDA + C ABI).

The library is compiled in-tree with nvcc (``build()``) and bound with
ctypes.  The structures below mirror ``include/xpbd_gb300.h`` field for
field.  There is no CPU fallback: ``load()`` raises if the library is missing
and the solver classes raise if no CUDA device is visible.
"""
import ctypes
import os
import subprocess
import threading
from concurrent.futures import ThreadPoolExecutor

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
SRC_DIR = os.path.join(os.path.dirname(PKG_DIR), "csrc")
REPO_DIR = os.path.dirname(os.path.dirname(PKG_DIR))
INCLUDE_DIR = os.path.join(REPO_DIR, "include")
LIB_NAME = "libxpbd_gb300.so"
LIB_PATH = os.path.join(PKG_DIR, LIB_NAME)
BUILD_DIR = os.path.join(os.path.dirname(PKG_DIR), "_build")

ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O3"]
SOURCES = ["xpbd_solver.cu", "xpbd_batch.cu", "xpbd_mesh.cpp"]

ABI_VERSION = 3  # XPBD_ABI_VERSION of include/xpbd_gb300.h
XPBD_OK = 0
STATUS_NAMES = {
    0: "XPBD_OK", 1: "XPBD_ERR_INVALID_ARGUMENT", 2: "XPBD_ERR_CUDA",
    3: "XPBD_ERR_NONFINITE", 4: "XPBD_ERR_NO_SDF", 5: "XPBD_ERR_BAD_MESH",
    6: "XPBD_ERR_HISTORY_FULL", 7: "XPBD_ERR_TIMEOUT",
}
SDF_PLANE, SDF_SPHERE, SDF_CUBE = 0, 1, 2
SCATTER_ATOMIC, SCATTER_GATHER, SCATTER_PATCH = 0, 1, 2
SCATTERS = {"atomic": SCATTER_ATOMIC, "gather": SCATTER_GATHER, "patch": SCATTER_PATCH}
FIELD_X, FIELD_V, FIELD_PRED_X = 0, 1, 2
KERNEL_CLASSES = ("begin", "project", "gather", "residual", "update", "end")


class XpbdSdf(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("fixed", ctypes.c_int32),
                ("a", ctypes.c_float * 3), ("b", ctypes.c_float * 3),
                ("vel", ctypes.c_float * 3), ("pad", ctypes.c_float)]


class XpbdParams(ctypes.Structure):
    _fields_ = [("lame_mu", ctypes.c_float), ("lame_lambda", ctypes.c_float),
                ("gravity", ctypes.c_float * 3), ("damping", ctypes.c_float),
                ("hydrostatic_relaxation", ctypes.c_float),
                ("deviatoric_relaxation", ctypes.c_float),
                ("cheb_gamma", ctypes.c_float),
                ("cheb_enable", ctypes.c_int32), ("cheb_warmup", ctypes.c_int32),
                ("block_mode", ctypes.c_int32), ("constraints_iter", ctypes.c_int32),
                ("monitor", ctypes.c_int32), ("precise_hydro", ctypes.c_int32),
                ("scatter", ctypes.c_int32), ("use_graph", ctypes.c_int32),
                ("sweep_order", ctypes.c_int32), ("patch_pipeline", ctypes.c_int32),
                ("patch_reduce", ctypes.c_int32), ("tets_per_thread", ctypes.c_int32),
                ("rho_min", ctypes.c_double), ("rho_max", ctypes.c_double),
                ("rho_beta", ctypes.c_double),
                ("target_rel_residual", ctypes.c_double), ("residual_floor", ctypes.c_double)]


_P = ctypes.c_void_p


class XpbdBody(ctypes.Structure):
    _fields_ = [("n_verts", ctypes.c_int32), ("n_tets", ctypes.c_int32),
                ("x", _P), ("v", _P), ("p0", _P), ("p1", _P), ("dx", _P),
                ("tets", _P), ("dm_a", _P), ("dm_b", _P), ("dm_c", _P), ("v0", _P), ("lam", _P),
                ("tet_inv_mu", _P), ("tet_inv_lambda", _P),
                ("v2t_offsets", _P), ("v2t_slots", _P), ("corner_dx", _P),
                ("vert_perm", _P),
                ("n_patches", ctypes.c_int32), ("patch_tets", ctypes.c_int32),
                ("tet_lid", _P), ("patch_voff", _P), ("patch_verts", _P),
                ("pv_start", _P), ("pv_slots", _P), ("tet_pairs", ctypes.c_int32)]


class XpbdBatch(ctypes.Structure):
    _fields_ = [("n_bodies", ctypes.c_int32), ("n_verts", ctypes.c_int32), ("n_tets", ctypes.c_int32),
                ("n_patches", ctypes.c_int32), ("n_patch_verts", ctypes.c_int32), ("n_out_verts", ctypes.c_int32),
                ("x", _P), ("v", _P), ("p0", _P), ("p1", _P), ("dx", _P),
                ("dm_a", _P), ("dm_b", _P), ("dm_c", _P), ("lam", _P), ("tet_lid", _P),
                ("patch_voff", _P), ("patch_verts", _P), ("patch_body", _P), ("patch_ntets", _P),
                ("vblock_body", _P), ("body_inv_mu", _P), ("body_inv_lambda", _P),
                ("body_n_patches", _P), ("body_n_tets", _P), ("vert_perm", _P),
                ("tet_inv_mu", _P), ("tet_inv_lambda", _P), ("tet_pairs", ctypes.c_int32)]


class XpbdTape(ctypes.Structure):
    _fields_ = [("xs", _P), ("lams", _P), ("xpre", _P), ("v1", _P), ("posts", _P), ("rho_in", _P), ("hist", _P)]


class XpbdAdjoint(ctypes.Structure):
    _fields_ = [("gx", _P), ("gv", _P), ("g_inv_mu", _P), ("g_inv_lambda", _P), ("work0", _P), ("work1", _P),
                ("ybar", _P), ("dxbar", _P), ("lambar", _P), ("cnt", _P), ("omega_state", _P),
                ("work_res_tet", _P)]


# name -> (restype, argtypes); every symbol declared in include/xpbd_gb300.h
_SIGNATURES = {
    "xpbd_abi_version": (ctypes.c_int, []),
    "xpbd_status_string": (ctypes.c_char_p, [ctypes.c_int]),
    "xpbd_last_error": (ctypes.c_char_p, []),
    "xpbd_device_count": (ctypes.c_int, []),
    "xpbd_create": (ctypes.c_int, [ctypes.POINTER(XpbdParams), ctypes.POINTER(XpbdBody),
                                   ctypes.POINTER(XpbdSdf), ctypes.c_int32, ctypes.c_int32,
                                   ctypes.POINTER(ctypes.c_void_p)]),
    "xpbd_destroy": (ctypes.c_int, [_P]),
    "xpbd_set_params": (ctypes.c_int, [_P, ctypes.POINTER(XpbdParams)]),
    "xpbd_set_sdfs": (ctypes.c_int, [_P, ctypes.POINTER(XpbdSdf), ctypes.c_int32, _P]),
    "xpbd_apply_external_forces": (ctypes.c_int, [_P, ctypes.c_float, _P]),
    "xpbd_solve_sdf_collision": (ctypes.c_int, [_P, ctypes.c_float, _P]),
    "xpbd_solve_step": (ctypes.c_int, [_P, ctypes.c_float, ctypes.c_int32, _P]),
    "xpbd_advance": (ctypes.c_int, [_P, ctypes.c_float, ctypes.c_float, _P]),
    "xpbd_substep": (ctypes.c_int, [_P, ctypes.c_float, ctypes.c_int32, _P]),
    "xpbd_solve": (ctypes.c_int, [_P, ctypes.c_double, ctypes.c_double, ctypes.c_int32, _P]),
    "xpbd_read_history": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_double), ctypes.c_int32, _P]),
    "xpbd_read_iterations": (ctypes.c_int, [_P, _P, ctypes.c_int32, ctypes.POINTER(ctypes.c_int64), _P]),
    "xpbd_get_rho_hat": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_double), _P]),
    "xpbd_set_rho_hat": (ctypes.c_int, [_P, ctypes.c_double, _P]),
    "xpbd_import_vec3": (ctypes.c_int, [_P, ctypes.c_int32, _P, _P]),
    "xpbd_export_vec3": (ctypes.c_int, [_P, ctypes.c_int32, _P, _P]),
    "xpbd_check_status": (ctypes.c_int, [_P, _P]),
    "xpbd_save_rho_hat": (ctypes.c_int, [_P, _P, _P]),
    "xpbd_load_rho_hat": (ctypes.c_int, [_P, _P, _P]),
    "xpbd_substep_tape": (ctypes.c_int, [_P, ctypes.c_float, ctypes.POINTER(XpbdTape), _P]),
    "xpbd_substep_adjoint": (ctypes.c_int, [_P, ctypes.c_float, ctypes.POINTER(XpbdTape),
                                            ctypes.POINTER(XpbdAdjoint), _P]),
    "xpbd_residual_noalloc": (ctypes.c_int, [ctypes.POINTER(XpbdBody), _P, ctypes.c_float, ctypes.c_float,
                                             ctypes.c_float, ctypes.c_int32, _P, _P]),
    "xpbd_set_profiling": (ctypes.c_int, [_P, ctypes.c_int32]),
    "xpbd_set_l2_hint": (ctypes.c_int, [_P, ctypes.c_int32, ctypes.POINTER(ctypes.c_int32)]),
    "xpbd_read_profile": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int64),
                                         ctypes.c_int32, ctypes.c_int32, _P]),
    "xpbd_morton_order": (ctypes.c_int, [_P, ctypes.c_int32, _P, ctypes.c_int32, _P, _P]),
    "xpbd_build_vertex_csr": (ctypes.c_int, [_P, ctypes.c_int32, ctypes.c_int32, _P, _P]),
    "xpbd_pair_tets": (ctypes.c_int, [_P, ctypes.c_int32, ctypes.c_int32, _P, _P, ctypes.POINTER(ctypes.c_int32)]),
    "xpbd_batch_last_error": (ctypes.c_char_p, []),
    "xpbd_batch_create": (ctypes.c_int, [ctypes.POINTER(XpbdParams), ctypes.POINTER(XpbdBatch),
                                         ctypes.POINTER(XpbdSdf), ctypes.c_int32, ctypes.c_int32,
                                         ctypes.POINTER(ctypes.c_void_p)]),
    "xpbd_batch_destroy": (ctypes.c_int, [_P]),
    "xpbd_batch_substep": (ctypes.c_int, [_P, ctypes.c_float, ctypes.c_int32, _P]),
    "xpbd_batch_solve": (ctypes.c_int, [_P, ctypes.c_double, ctypes.c_double, ctypes.c_int32, _P]),
    "xpbd_batch_read_history": (ctypes.c_int, [_P, _P, ctypes.c_int32, _P]),
    "xpbd_batch_read_iterations": (ctypes.c_int, [_P, _P, ctypes.c_int32, _P]),
    "xpbd_batch_get_rho_hat": (ctypes.c_int, [_P, _P, _P]),
    "xpbd_batch_check_status": (ctypes.c_int, [_P, _P]),
    "xpbd_batch_import_vec3": (ctypes.c_int, [_P, ctypes.c_int32, _P, _P]),
    "xpbd_batch_export_vec3": (ctypes.c_int, [_P, ctypes.c_int32, _P, _P]),
    "xpbd_batch_set_profiling": (ctypes.c_int, [_P, ctypes.c_int32]),
    "xpbd_batch_read_profile": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int64),
                                               ctypes.c_int32, ctypes.c_int32, _P]),
    "xpbd_batch_set_params": (ctypes.c_int, [_P, ctypes.POINTER(XpbdParams)]),
    "xpbd_batch_save_rho_hat": (ctypes.c_int, [_P, _P, _P]),
    "xpbd_batch_load_rho_hat": (ctypes.c_int, [_P, _P, _P]),
    "xpbd_batch_substep_tape": (ctypes.c_int, [_P, ctypes.c_float, ctypes.POINTER(XpbdTape), _P]),
    "xpbd_batch_substep_adjoint": (ctypes.c_int, [_P, ctypes.c_float, ctypes.POINTER(XpbdTape),
                                                  ctypes.POINTER(XpbdAdjoint), _P]),
    "xpbd_build_patch_csr": (ctypes.c_int, [_P, _P, ctypes.c_int32, ctypes.c_int32, _P, _P]),
    "xpbd_build_patches": (ctypes.c_int, [_P, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, _P, _P, _P,
                                          ctypes.POINTER(ctypes.c_int32)]),
}

_lock = threading.Lock()
_lib = None


def _nvcc():
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def _stale():
    if not os.path.exists(LIB_PATH):
        return True
    t = os.path.getmtime(LIB_PATH)
    deps = [os.path.join(SRC_DIR, f) for f in os.listdir(SRC_DIR)]
    deps.append(os.path.join(INCLUDE_DIR, "xpbd_gb300.h"))
    return any(os.path.getmtime(p) > t for p in deps)


def build(force=False, verbose=False):
    """Compile the CUDA/C++ sources for sm_103a into ``libxpbd_gb300.so``.

    Translation units compile in parallel; the link is a shared library with
    the CUDA runtime linked statically.  Returns the library path.
    """
    if not force and not _stale():
        return LIB_PATH
    os.makedirs(BUILD_DIR, exist_ok=True)
    nvcc = _nvcc()
    objs = []

    def compile_one(src):
        obj = os.path.join(BUILD_DIR, src + ".o")
        cmd = [nvcc] + ARCH_FLAGS + NVCC_FLAGS + ["-I", INCLUDE_DIR, "-c",
                                                  os.path.join(SRC_DIR, src), "-o", obj]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr))
        if verbose and r.stderr:
            print(r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB_PATH + ".tmp"
    cmd = [nvcc] + ARCH_FLAGS + ["-shared", "-o", tmp] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc link failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


def load():
    """Load the library (building it first if it is missing or stale)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if _stale():
            build()
        lib = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in _SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        if lib.xpbd_abi_version() != ABI_VERSION:
            raise RuntimeError("libxpbd_gb300.so ABI mismatch")
        _lib = lib
        return lib


class XpbdError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s (%d): %s" % (STATUS_NAMES.get(status, "?"), status, msg))
        self.status = status


def check(status, batch=False):
    """Raise for a non-zero status with the library's last error message."""
    if status == XPBD_OK:
        return
    lib = load()
    last = lib.xpbd_batch_last_error() if batch else lib.xpbd_last_error()
    msg = last.decode() or lib.xpbd_status_string(status).decode()
    if status == 4:  # XPBD_ERR_NO_SDF mirrors xpbd_base.py:66-67
        raise ValueError(msg)
    raise XpbdError(status, msg)


def pair_tets(lib, tets, n_verts):
    """Face pairs of `tets` ([T, 4] int, solver order) for the two-tets-per-thread
    kernels: returns (order [T], corner permutation [T, 4], number of pairs);
    new tet i is old tet order[i] with corners old[perm[i]]."""
    import numpy as np
    tt = np.ascontiguousarray(tets, dtype=np.int32)
    T = len(tt)
    order = np.empty(T, dtype=np.int32)
    packed = np.empty(T, dtype=np.uint8)
    n = ctypes.c_int32()
    check(lib.xpbd_pair_tets(tt.ctypes.data, T, int(n_verts), order.ctypes.data, packed.ctypes.data,
                             ctypes.byref(n)))
    perm = np.stack([(packed >> (2 * c)) & 3 for c in range(4)], axis=1).astype(np.int64)
    return order, perm, n.value
