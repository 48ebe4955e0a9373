"""C ABI checks that need no GPU: the library loads, exports every function
declared in include/xpbd_gb300.h, and the host-only entry points and error
paths behave."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT
from xpbd_gpu import _native
from xpbd_gpu.mesh import kuhn_grid

HEADER = os.path.join(ROOT, "include", "xpbd_gb300.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(xpbd_[a-z0-9_]+)\s*\(", src)))


def test_header_declares_bound_functions():
    assert set(declared_functions()) == set(_native._SIGNATURES)


def test_library_exports_every_declared_symbol(native_lib):
    for name in declared_functions():
        assert hasattr(native_lib, name), name
    assert native_lib.xpbd_abi_version() == _native.ABI_VERSION
    m = re.search(r"#define XPBD_ABI_VERSION (\d+)", open(HEADER).read())
    assert int(m.group(1)) == _native.ABI_VERSION


def test_stop_mode_parameters_are_checked(native_lib):
    prm = _native.XpbdParams()
    prm.lame_mu = prm.lame_lambda = 1.0
    body = _native.XpbdBody()
    sdf = (_native.XpbdSdf * 1)()
    h = ctypes.c_void_p()
    prm.target_rel_residual = -1e-3
    assert native_lib.xpbd_create(prm, body, sdf, 1, 1, ctypes.byref(h)) == 1
    assert b"target_rel_residual" in native_lib.xpbd_last_error()
    prm.target_rel_residual = 1e-3
    prm.residual_floor = float("nan")
    assert native_lib.xpbd_create(prm, body, sdf, 1, 1, ctypes.byref(h)) == 1
    prm.residual_floor = 0.0
    assert native_lib.xpbd_create(prm, body, sdf, 1, 1, ctypes.byref(h)) == 5  # valid stop mode, empty mesh


def test_status_strings(native_lib):
    assert native_lib.xpbd_status_string(0) == b"ok"
    assert b"SDF" in native_lib.xpbd_status_string(4)


def test_create_without_sdf_is_value_error(native_lib):
    prm = _native.XpbdParams()
    prm.lame_mu = prm.lame_lambda = 1.0
    body = _native.XpbdBody()
    h = ctypes.c_void_p()
    st = native_lib.xpbd_create(prm, body, None, 0, 1, ctypes.byref(h))
    assert st == 4
    with pytest.raises(ValueError):
        _native.check(st)


def test_create_rejects_bad_arguments(native_lib):
    prm = _native.XpbdParams()
    prm.lame_mu = prm.lame_lambda = 1.0
    prm.scatter = 7
    body = _native.XpbdBody()
    sdf = (_native.XpbdSdf * 1)()
    h = ctypes.c_void_p()
    assert native_lib.xpbd_create(prm, body, sdf, 1, 1, ctypes.byref(h)) == 1
    prm.scatter = 0
    assert native_lib.xpbd_create(prm, body, sdf, 1, 1, ctypes.byref(h)) == 5  # empty mesh
    assert native_lib.xpbd_create(None, body, sdf, 1, 1, ctypes.byref(h)) == 1
    assert native_lib.xpbd_destroy(None) == 0
    assert native_lib.xpbd_substep(None, ctypes.c_float(0.01), 0, None) == 1
    on = ctypes.c_int32(-1)
    assert native_lib.xpbd_set_l2_hint(None, -1, ctypes.byref(on)) == 1 and on.value == -1


def test_morton_order_is_a_permutation_with_locality(native_lib):
    m = kuhn_grid(8, 8, 8, 0.1, jitter=0.1, seed=0)
    V, T = m.n_verts, m.n_tets
    vp = np.empty(V, dtype=np.int32)
    tp = np.empty(T, dtype=np.int32)
    pts = np.ascontiguousarray(m.points)
    tt = np.ascontiguousarray(m.tets, dtype=np.int32)
    assert native_lib.xpbd_morton_order(pts.ctypes.data, V, tt.ctypes.data, T, vp.ctypes.data, tp.ctypes.data) == 0
    assert sorted(vp.tolist()) == list(range(V))
    assert sorted(tp.tolist()) == list(range(T))
    # consecutive tets are spatially compact: windows of 64 tets span a smaller box
    cen = m.points[m.tets].mean(1)

    def window_extent(order):
        c = cen[order][: (T // 64) * 64].reshape(-1, 64, 3)
        return np.linalg.norm(c.max(1) - c.min(1), axis=1).mean()

    assert window_extent(tp) < 0.75 * window_extent(np.arange(T))
    # vertices are numbered by first use: the first tet's corners come first
    assert set(vp[:4].tolist()) == set(m.tets[tp[0]].tolist())


def test_morton_rejects_bad_index(native_lib):
    pts = np.zeros((4, 3))
    tt = np.array([[0, 1, 2, 9]], dtype=np.int32)
    vp = np.empty(4, dtype=np.int32)
    tp = np.empty(1, dtype=np.int32)
    assert native_lib.xpbd_morton_order(pts.ctypes.data, 4, tt.ctypes.data, 1, vp.ctypes.data, tp.ctypes.data) == 5


def test_vertex_csr(native_lib):
    m = kuhn_grid(3, 2, 2, 1.0)
    V, T = m.n_verts, m.n_tets
    off = np.empty(V + 1, dtype=np.int32)
    slots = np.empty(4 * T, dtype=np.int32)
    tt = np.ascontiguousarray(m.tets, dtype=np.int32)
    assert native_lib.xpbd_build_vertex_csr(tt.ctypes.data, T, V, off.ctypes.data, slots.ctypes.data) == 0
    assert off[0] == 0 and off[-1] == 4 * T
    flat = m.tets.reshape(-1)
    for v in range(V):
        s = slots[off[v]:off[v + 1]]
        assert np.all(np.diff(s) > 0)
        assert np.all(flat[s] == v)
        assert len(s) == (flat == v).sum()


def test_device_count_without_gpu_is_zero_or_more(native_lib):
    assert native_lib.xpbd_device_count() >= 0


def test_build_patches_layout(native_lib):
    m = kuhn_grid(6, 5, 4, 1.0, jitter=0.1, seed=1)
    V, T = m.n_verts, m.n_tets
    tt = np.ascontiguousarray(m.tets, dtype=np.int32)
    for P in (256, 128, 64):
        npat = (T + P - 1) // P
        voff = np.empty(npat + 1, dtype=np.int32)
        pv = np.empty(4 * T, dtype=np.int32)
        lid = np.empty(T, dtype=np.uint32)
        mx = ctypes.c_int32()
        assert native_lib.xpbd_build_patches(tt.ctypes.data, T, V, P, voff.ctypes.data, pv.ctypes.data,
                                             lid.ctypes.data, ctypes.byref(mx)) == 0
        assert voff[0] == 0 and np.all(np.diff(voff) > 0) and mx.value == np.diff(voff).max() <= 256
        for p in range(npat):
            verts = pv[voff[p]:voff[p + 1]]
            assert np.all(np.diff(verts) > 0)
            for t in range(p * P, min(T, (p + 1) * P)):
                loc = [(int(lid[t]) >> (8 * q)) & 0xFF for q in range(4)]
                assert list(verts[loc]) == list(m.tets[t])
        start = np.empty(voff[-1], dtype=np.uint16)
        slots = np.empty(4 * npat * P, dtype=np.uint16)
        assert native_lib.xpbd_build_patch_csr(voff.ctypes.data, lid.ctypes.data, T, P, start.ctypes.data,
                                               slots.ctypes.data) == 0
        for p in range(npat):
            nv = voff[p + 1] - voff[p]
            ntet = min(T, (p + 1) * P) - p * P
            blk = slots[4 * P * p: 4 * P * (p + 1)]
            st = list(start[voff[p]:voff[p + 1]]) + [4 * ntet]
            assert np.all(blk[4 * ntet:] == 0xFFFF)
            for k in range(nv):
                seg = blk[st[k]:st[k + 1]]
                assert np.all(np.diff(seg.astype(int)) > 0)
                for sl in seg:
                    t, q = p * P + int(sl) // 4, int(sl) % 4
                    assert (int(lid[t]) >> (8 * q)) & 0xFF == k


def _signed_volumes(pts, tets):
    P = pts[tets]
    return np.einsum("ij,ij->i", np.cross(P[:, 1] - P[:, 0], P[:, 2] - P[:, 0]), P[:, 3] - P[:, 0]) / 6.0


def test_pair_tets_on_a_kuhn_grid(native_lib):
    """Every tet of a Kuhn grid (6 tets around each cell diagonal) finds a face
    partner; pairs are laid out as (u, v, w, a*), (v, u, w, b*) with even corner
    permutations, so every signed volume is unchanged."""
    from xpbd_gpu import _native
    from xpbd_gpu.mesh import kuhn_grid
    m = kuhn_grid(5, 4, 3, 0.1, jitter=0.1, seed=3)
    tets = np.asarray(m.tets, dtype=np.int64)
    order, perm, n_pairs = _native.pair_tets(native_lib, tets, m.n_verts)
    T = len(tets)
    assert n_pairs == T // 2
    assert sorted(order.tolist()) == list(range(T))
    assert all(sorted(p.tolist()) == [0, 1, 2, 3] for p in perm)
    new = np.take_along_axis(tets[order], perm, axis=1)
    np.testing.assert_allclose(_signed_volumes(m.points, new), _signed_volumes(m.points, tets)[order], rtol=1e-12)
    a, b = new[0::2], new[1::2]
    np.testing.assert_array_equal(b[:, 0], a[:, 1])
    np.testing.assert_array_equal(b[:, 1], a[:, 0])
    np.testing.assert_array_equal(b[:, 2], a[:, 2])
    assert not np.any(b[:, 3] == a[:, 3])


def test_pair_tets_leaves_unpairable_tets_last(native_lib):
    """Two tets sharing only an edge cannot pair, nor can a tet inverted
    against its face neighbour (odd orientation).  Unpaired tets keep their
    corners and are grouped two by two; every tet keeps its signed volume."""
    from xpbd_gpu import _native
    tets = np.array([[0, 1, 2, 3], [0, 1, 4, 5], [1, 2, 3, 6], [7, 8, 9, 10], [2, 3, 1, 12]], dtype=np.int64)
    pts = np.random.default_rng(0).normal(size=(13, 3))
    order, perm, n_pairs = _native.pair_tets(native_lib, tets, 13)
    assert sorted(order.tolist()) == [0, 1, 2, 3, 4]
    paired = set(order[:0].tolist())
    for i in range(5):
        if perm[i].tolist() != [0, 1, 2, 3]:
            paired.add(int(order[i]))
    assert len(paired) <= 2 * n_pairs
    new = np.take_along_axis(tets[order], perm, axis=1)
    np.testing.assert_allclose(_signed_volumes(pts, new), _signed_volumes(pts, tets)[order], rtol=1e-12)
    with pytest.raises(Exception):
        _native.pair_tets(native_lib, np.array([[0, 1, 2, 13]]), 13)


def test_batch_create_rejects_bad_arguments(native_lib):
    """xpbd_batch_create checks its arguments before any device work, in this
    order: NULL arguments, the SDF list, an empty batch, the padded sizes
    (n_verts a multiple of 256, n_tets = 256 n_patches), NULL buffers,
    half-given per-tet materials, max_records and the stop-mode parameters.
    The pointers here are never dereferenced: each case fails a check first."""
    prm = _native.XpbdParams()
    prm.lame_mu = prm.lame_lambda = 1.0
    b = _native.XpbdBatch()
    sdf = (_native.XpbdSdf * 1)()
    h = ctypes.c_void_p()

    def create(n_sdf=1, sdfs=sdf, max_records=1):
        st = native_lib.xpbd_batch_create(prm, b, sdfs, n_sdf, max_records, ctypes.byref(h))
        assert h.value is None
        return st, native_lib.xpbd_batch_last_error().decode()

    assert native_lib.xpbd_batch_create(None, b, sdf, 1, 1, ctypes.byref(h)) == 1
    assert create(n_sdf=0, sdfs=None)[0] == 4
    sdf[0].kind = 3
    assert create() == (1, "unknown SDF kind")
    sdf[0].kind = 0
    assert create() == (5, "empty batch")
    b.n_bodies, b.n_verts, b.n_tets, b.n_patches = 1, 256, 300, 1
    assert create()[0] == 5
    b.n_verts, b.n_tets = 257, 256
    assert create()[0] == 5
    b.n_verts = 256
    assert create() == (1, "NULL batch buffer")
    for name, _ in _native.XpbdBatch._fields_[6:-3]:
        setattr(b, name, 256)  # non-NULL, never read
    b.tet_inv_mu = 256
    assert create()[0] == 1 and "tet_inv_mu" in create()[1]
    b.tet_inv_mu = None
    assert create(max_records=-1) == (1, "max_records < 0")
    prm.target_rel_residual = -1.0
    assert create()[0] == 1
    prm.target_rel_residual, prm.residual_floor = 0.0, float("nan")
    assert create()[0] == 1
    assert native_lib.xpbd_batch_destroy(None) == 0


def test_tape_and_adjoint_entries_reject_missing_buffers(native_lib):
    """The forward-with-tape and adjoint entries of both forms refuse a NULL
    handle or a tape / adjoint without its required buffers
    (XPBD_ERR_INVALID_ARGUMENT) before touching the device."""
    tape, adj = _native.XpbdTape(), _native.XpbdAdjoint()
    dt = ctypes.c_float(0.01)
    for tape_fn, adj_fn, err in ((native_lib.xpbd_substep_tape, native_lib.xpbd_substep_adjoint,
                                  native_lib.xpbd_last_error),
                                 (native_lib.xpbd_batch_substep_tape, native_lib.xpbd_batch_substep_adjoint,
                                  native_lib.xpbd_batch_last_error)):
        assert tape_fn(None, dt, tape, None) == 1 and b"NULL" in err()
        assert tape_fn(None, dt, None, None) == 1
        assert adj_fn(None, dt, tape, adj, None) == 1 and b"NULL" in err()
        assert adj_fn(None, dt, tape, None, None) == 1
