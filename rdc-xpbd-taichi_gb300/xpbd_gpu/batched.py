"""XPBDBatchedSolver: many independent soft bodies of uneven size in one set of launches.

The reference steps one body per ``XPBDNeoHookeanSolver``
(``neohookean_solver.py:16-587``).  A batch holds a list of bodies that share
the SDF list, time stepping and iteration settings; each body keeps its own
mesh, Lame parameters, mass, pinning and Chebyshev state (``rho_hat``
persists per body across substeps and frames, as in the reference).  One
frame of every body is one CUDA-graph replay of
``xpbd_batch_solve`` (``include/xpbd_gb300.h``): each phase of the substep is
a single launch over the flattened tets or vertices of all bodies.

Per-body setup (x = points * scale + offset, V0, inv_Dm, lumped mass scaled
to the body's total mass, pinning inside fixed SDFs) is the single-body
setup of ``xpbd_base.py:89-137`` / ``neohookean_solver.py:97-107``.
"""
from dataclasses import dataclass

import numpy as np

from xpbd_gpu import _native
from xpbd_gpu.neohookean_solver import calc_first_lame, calc_second_lame, frame_chunks
from xpbd_gpu.xpbd_base import _require_cuda, _torch, calc_tet_volume, inv_dm_of, load_rest_pose

PATCH = 256


@dataclass
class Body:
    """One body of a batch.  ``rotation`` (3x3) is applied before ``scale`` and ``offset``.
    ``tet_young_modulus`` / ``tet_poisson_ratio`` (file tet order) give per-tet
    materials; a batch uses them for every body once any body has them."""

    rest_pose: object
    young_modulus: float = 200000.0
    poisson_ratio: float = 0.495
    scale: float = 1.0
    offset: tuple = (0.0, 0.0, 0.0)
    rotation: np.ndarray = None
    total_mass: float = 1.0
    density: float = None
    tet_young_modulus: np.ndarray = None
    tet_poisson_ratio: np.ndarray = None


def _pad(n, m=PATCH):
    return -(-n // m) * m


class XPBDBatchedSolver:
    def __init__(self, bodies, sdf, frame_dt=1e-2, dt=1e-2, substeps_num=20, constraints_iter=5,
                 hydrostatic_relaxation=1.2, deviatoric_relaxation=1.2, cheb_enable=True, cheb_warmup=5,
                 cheb_gamma=0.6666, block_neohookean_enable=True, monitor_convergence=False,
                 gravity=(0.0, -9.8, 0.0), precise_hydro=None, use_graph=True, tets_per_thread=2,
                 autotune_cache=True, pair_tets=True, target_rel_residual=0.0, residual_floor=0.0):
        if isinstance(sdf, (list, tuple)):
            self.sdfs = [s for s in sdf if s is not None]
        else:
            self.sdfs = [sdf] if sdf is not None else []
        if not self.sdfs:
            raise ValueError("At least one SDF object must be provided.")
        if not bodies:
            raise ValueError("a batch needs at least one body")
        torch = _require_cuda()
        self._lib = _native.load()
        self._device = torch.device("cuda", torch.cuda.current_device())
        self.bodies = list(bodies)
        self.frame_dt, self.dt, self.substeps_num = frame_dt, dt, substeps_num
        self.constraints_iter = constraints_iter
        # stop mode: each body ends its substep at r_hat <= target * r_hat_0 or
        # r_hat <= floor (constraints_iter is then the cap)
        self.target_rel_residual = float(target_rel_residual)
        self.residual_floor = float(residual_floor)
        self.hydrostatic_relaxation = hydrostatic_relaxation
        self.deviatoric_relaxation = deviatoric_relaxation
        self.cheb_enable, self.cheb_warmup, self.cheb_gamma = cheb_enable, cheb_warmup, cheb_gamma
        self.block_neohookean_enable = block_neohookean_enable
        self.monitor_convergence = monitor_convergence
        self.gravity = np.asarray(gravity, dtype=np.float64)
        self.damping = 5.0
        self.rho_min, self.rho_max, self.rho_beta = 0.00001, 0.99999, 0.2
        nus = [b.poisson_ratio for b in self.bodies]
        self.precise_hydro = (max(nus) >= 0.49) if precise_hydro is None else bool(precise_hydro)
        self.use_graph = bool(use_graph)
        if tets_per_thread not in (1, 2, "auto"):
            raise ValueError("tets_per_thread must be 1, 2 or 'auto'")
        self.tets_per_thread = 2 if tets_per_thread == "auto" else int(tets_per_thread)
        self.per_tet_materials = any(b.tet_young_modulus is not None for b in self.bodies)
        self.pair_tets = bool(pair_tets)
        self.time = 0.0
        self.current_frame = 0
        self._handle = None
        self._build()
        self.autotune_result = None
        if tets_per_thread == "auto":
            from xpbd_gpu import autotune
            self.autotune_result = autotune.tune_batch(self, cache=autotune_cache)
            self.set_tets_per_thread(self.autotune_result["tets_per_thread"])

    # -- setup ------------------------------------------------------------------
    def _prepare_body(self, b):
        mesh = load_rest_pose(b.rest_pose)
        pts = np.asarray(mesh.points, dtype=np.float64)
        if b.rotation is not None:
            pts = pts @ np.asarray(b.rotation, dtype=np.float64).T
        x = pts * float(b.scale) + np.asarray(b.offset, dtype=np.float64)
        tets = np.asarray(mesh.tets, dtype=np.int64)
        V, T = len(x), len(tets)
        if V == 0 or T == 0 or tets.min() < 0 or tets.max() >= V:
            raise ValueError("bad body mesh")
        P = x[tets]
        V0 = calc_tet_volume(P[:, 0], P[:, 1], P[:, 2], P[:, 3])
        Ds = np.stack([P[:, 1] - P[:, 0], P[:, 2] - P[:, 0], P[:, 3] - P[:, 0]], axis=-1)
        inv_Dm = np.linalg.inv(Ds)
        m = np.zeros(V)
        np.add.at(m, tets.reshape(-1), np.repeat(V0 * 0.25, 4))
        total_volume = float(V0.sum())
        total_mass = float(b.density) * total_volume if b.density is not None else float(b.total_mass)
        m *= total_mass / total_volume
        inv_m = np.where(m > 0.0, 1.0 / np.where(m > 0.0, m, 1.0), 0.0)
        for s in self.sdfs:
            live = inv_m > 0.0
            fixed, inside, _ = s.check(x, np.zeros_like(x))
            if fixed:
                inv_m[live & inside] = 0.0
        # Morton tets, first-touch vertices, 256-tet patches
        vperm = np.empty(V, dtype=np.int32)
        tperm = np.empty(T, dtype=np.int32)
        tt = np.ascontiguousarray(tets, dtype=np.int32)
        _native.check(self._lib.xpbd_morton_order(np.ascontiguousarray(x).ctypes.data, V, tt.ctypes.data, T,
                                                  vperm.ctypes.data, tperm.ctypes.data))
        inv_vperm = np.empty(V, dtype=np.int64)
        inv_vperm[vperm] = np.arange(V)
        tets_s = np.ascontiguousarray(inv_vperm[tets[tperm]], dtype=np.int32)
        dm_solver = inv_Dm[tperm]
        if self.pair_tets:  # face pairs with aligned corners (xpbd_pair_tets)
            order, cperm, _ = _native.pair_tets(self._lib, tets_s, V)
            tperm = tperm[order]
            tets_s = np.ascontiguousarray(np.take_along_axis(tets_s[order], cperm, axis=1), dtype=np.int32)
            dm_solver = inv_dm_of(x, np.take_along_axis(tets[tperm], cperm, axis=1))
        npat = -(-T // PATCH)
        voff = np.empty(npat + 1, dtype=np.int32)
        pverts = np.empty(4 * T, dtype=np.int32)
        lid = np.zeros(npat * PATCH, dtype=np.uint32)
        mx = _native.ctypes.c_int32()
        _native.check(self._lib.xpbd_build_patches(tets_s.ctypes.data, T, V, PATCH, voff.ctypes.data,
                                                   pverts.ctypes.data, lid.ctypes.data, _native.ctypes.byref(mx)))
        if mx.value > 256:
            raise ValueError("a 256-tet patch of this body touches more than 256 vertices")
        lame_mu = calc_second_lame(b.young_modulus, b.poisson_ratio)
        lame_la = calc_first_lame(b.young_modulus, b.poisson_ratio)
        if b.tet_young_modulus is not None:
            tE = np.asarray(b.tet_young_modulus, dtype=np.float64).reshape(-1)
            if tE.shape != (T,):
                raise ValueError("tet_young_modulus must have one entry per tet")
            tnu = b.poisson_ratio if b.tet_poisson_ratio is None else b.tet_poisson_ratio
            tnu = np.broadcast_to(np.asarray(tnu, dtype=np.float64), tE.shape)
        else:
            tE = np.full(T, float(b.young_modulus))
            tnu = np.full(T, float(b.poisson_ratio))
        # valence (constraints per vertex in block mode), solver vertex order
        cnt = np.bincount(tets_s.reshape(-1), minlength=V).astype(np.float32)
        return dict(x=x, V0=V0, inv_Dm=inv_Dm, dm_solver=dm_solver, m=m, inv_m=inv_m, vperm=vperm, tperm=tperm,
                    T=T, V=V, npat=npat,
                    voff=voff, pverts=pverts[:voff[-1]], lid=lid, mu=lame_mu, la=lame_la, tet_E=tE, tet_nu=tnu,
                    cnt=cnt, indices=tets[:, np.array([[0, 2, 1], [0, 3, 2], [0, 1, 3], [1, 2, 3]])].reshape(-1))

    def _build(self):
        torch = _torch()
        preps = [self._prepare_body(b) for b in self.bodies]
        nb = len(preps)
        Vp = [_pad(p["V"]) for p in preps]
        Tp = [p["npat"] * PATCH for p in preps]
        voffs = np.concatenate([[0], np.cumsum(Vp)]).astype(np.int64)
        toffs = np.concatenate([[0], np.cumsum(Tp)]).astype(np.int64)
        outoffs = np.concatenate([[0], np.cumsum([p["V"] for p in preps])]).astype(np.int64)
        Vt, Tt = int(voffs[-1]), int(toffs[-1])
        NP = Tt // PATCH
        x4 = np.zeros((Vt, 4), dtype=np.float32)
        perm = np.full(Vt, -1, dtype=np.int32)
        vblock_body = np.empty(Vt // PATCH, dtype=np.int32)
        D = np.zeros((Tt, 9), dtype=np.float32)
        lid = np.zeros(Tt, dtype=np.uint32)
        patch_body = np.empty(NP, dtype=np.int32)
        patch_ntets = np.empty(NP, dtype=np.int32)
        pv_list, pvoff = [], [0]
        for k, p in enumerate(preps):
            vo, to, oo = int(voffs[k]), int(toffs[k]), int(outoffs[k])
            x4[vo:vo + p["V"], :3] = p["x"][p["vperm"]]
            x4[vo:vo + p["V"], 3] = p["inv_m"][p["vperm"]]
            perm[vo:vo + p["V"]] = oo + p["vperm"]
            vblock_body[vo // PATCH:(vo + Vp[k]) // PATCH] = k
            D[to:to + p["T"]] = p["dm_solver"].reshape(-1, 9)
            lid[to:to + Tp[k]] = p["lid"]
            p0 = to // PATCH
            patch_body[p0:p0 + p["npat"]] = k
            nt = np.full(p["npat"], PATCH, dtype=np.int32)
            nt[-1] = p["T"] - (p["npat"] - 1) * PATCH
            patch_ntets[p0:p0 + p["npat"]] = nt
            pv_list.append(p["pverts"] + vo)
            base = pvoff[-1]
            pvoff.extend((base + p["voff"][1:]).tolist())
        pverts = np.concatenate(pv_list).astype(np.int32)
        pvoff = np.asarray(pvoff, dtype=np.int32)
        dev = self._device

        def T_(a, dtype=torch.float32):
            return torch.from_numpy(np.ascontiguousarray(a)).to(device=dev, dtype=dtype)

        self._x4 = T_(x4)
        self._v4 = torch.zeros((Vt, 4), dtype=torch.float32, device=dev)
        self._p4 = [self._x4.clone(), self._x4.clone()]
        self._dx4 = torch.zeros((Vt, 4), dtype=torch.float32, device=dev)
        self._dm_a = T_(D[:, 0:4])
        self._dm_b = T_(D[:, 4:8])
        self._dm_c = T_(D[:, 8])
        self._lam = torch.zeros((Tt, 2), dtype=torch.float32, device=dev)
        self._lid = T_(lid.view(np.int32), torch.int32)
        self._voff = T_(pvoff, torch.int32)
        self._pverts = T_(pverts, torch.int32)
        self._patch_body = T_(patch_body, torch.int32)
        self._patch_ntets = T_(patch_ntets, torch.int32)
        self._vblock_body = T_(vblock_body, torch.int32)
        self._inv_mu = T_(np.array([1.0 / p["mu"] for p in preps]))
        self._inv_la = T_(np.array([1.0 / p["la"] for p in preps]))
        self._body_patches = T_(np.array([p["npat"] for p in preps]), torch.int32)
        self._body_tets = T_(np.array([p["T"] for p in preps]), torch.int32)
        self._perm = T_(perm, torch.int32)
        # tet slot of every caller tet (body order, then file order) and vertex valence
        slot = np.concatenate([toffs[k] + np.argsort(p["tperm"]) for k, p in enumerate(preps)]).astype(np.int64)
        self._tet_slot = torch.from_numpy(slot).to(dev)
        cnt = np.zeros(Vt, dtype=np.float32)
        for k, p in enumerate(preps):
            cnt[voffs[k]:voffs[k] + p["V"]] = p["cnt"]
        self._cnt = T_(cnt)
        self._vert_slot = torch.from_numpy(
            np.concatenate([voffs[k] + np.argsort(p["vperm"]) for k, p in enumerate(preps)]).astype(np.int64)).to(dev)
        self._tinv_mu = self._tinv_la = None
        if self.per_tet_materials:
            self._tinv_mu = torch.ones(Tt, dtype=torch.float32, device=dev)
            self._tinv_la = torch.ones(Tt, dtype=torch.float32, device=dev)
            self.set_tet_materials(np.log(np.concatenate([p["tet_E"] for p in preps])),
                                   np.concatenate([p["tet_nu"] for p in preps]))
        self.n_bodies, self.n_verts_padded, self.n_tets_padded, self.n_patches = nb, Vt, Tt, NP
        self.n_verts = int(outoffs[-1])
        self.n_tets = int(sum(p["T"] for p in preps))
        self.body_vert_slices = [slice(int(outoffs[k]), int(outoffs[k + 1])) for k in range(nb)]
        self.body_n_tets = [p["T"] for p in preps]
        self.body_indices = [p["indices"].astype(np.uint32) for p in preps]
        self._host_inv_m = [p["inv_m"] for p in preps]
        self._stage = torch.empty((self.n_verts, 3), dtype=torch.float32, device=dev)

        b = _native.XpbdBatch()
        b.n_bodies, b.n_verts, b.n_tets, b.n_patches = nb, Vt, Tt, NP
        b.n_patch_verts, b.n_out_verts = int(pvoff[-1]), self.n_verts
        b.x, b.v = self._x4.data_ptr(), self._v4.data_ptr()
        b.p0, b.p1, b.dx = self._p4[0].data_ptr(), self._p4[1].data_ptr(), self._dx4.data_ptr()
        b.dm_a, b.dm_b, b.dm_c = self._dm_a.data_ptr(), self._dm_b.data_ptr(), self._dm_c.data_ptr()
        b.lam, b.tet_lid = self._lam.data_ptr(), self._lid.data_ptr()
        b.patch_voff, b.patch_verts = self._voff.data_ptr(), self._pverts.data_ptr()
        b.patch_body, b.patch_ntets = self._patch_body.data_ptr(), self._patch_ntets.data_ptr()
        b.vblock_body = self._vblock_body.data_ptr()
        b.body_inv_mu, b.body_inv_lambda = self._inv_mu.data_ptr(), self._inv_la.data_ptr()
        b.body_n_patches, b.body_n_tets = self._body_patches.data_ptr(), self._body_tets.data_ptr()
        b.vert_perm = self._perm.data_ptr()
        if self._tinv_mu is not None:
            b.tet_inv_mu, b.tet_inv_lambda = self._tinv_mu.data_ptr(), self._tinv_la.data_ptr()
        b.tet_pairs = 1 if self.pair_tets else 0
        self._max_records = max(1, len(frame_chunks(self.frame_dt, self.dt)) * self.substeps_num
                                * self.constraints_iter)
        table = (_native.XpbdSdf * len(self.sdfs))()
        for k, s in enumerate(self.sdfs):
            table[k] = s.to_struct()
        h = _native.ctypes.c_void_p()
        _native.check(self._lib.xpbd_batch_create(self._params(), b, table, len(self.sdfs), self._max_records,
                                                  _native.ctypes.byref(h)), batch=True)
        self._handle = h.value

    def set_tet_materials(self, log_E, nu):
        """Per-tet log Young's modulus and Poisson ratio of every body (numpy or
        torch; all bodies' tets in body order, each body in file order; nu may be
        a scalar).  Uploads 1/mu and 1/lambda into the tet slots."""
        torch = _torch()
        if self._tinv_mu is None:
            raise RuntimeError("the batch was built without per-tet materials")
        le = torch.as_tensor(log_E, dtype=torch.float64, device=self._device).reshape(-1)
        nu_t = torch.as_tensor(nu, dtype=torch.float64, device=self._device).reshape(-1).expand(le.shape[0])
        E = torch.exp(le)
        self._tinv_mu[self._tet_slot] = (2.0 * (1.0 + nu_t) / E).to(torch.float32)
        self._tinv_la[self._tet_slot] = ((1.0 + nu_t) * (1.0 - 2.0 * nu_t) / (E * nu_t)).to(torch.float32)

    def _params(self):
        p = _native.XpbdParams()
        p.lame_mu = p.lame_lambda = 1.0
        p.gravity[:] = [float(g) for g in self.gravity]
        p.damping = self.damping
        p.hydrostatic_relaxation = self.hydrostatic_relaxation
        p.deviatoric_relaxation = self.deviatoric_relaxation
        p.cheb_gamma = self.cheb_gamma
        p.cheb_enable = 1 if self.cheb_enable else 0
        p.cheb_warmup = int(self.cheb_warmup)
        p.block_mode = 1 if self.block_neohookean_enable else 0
        p.constraints_iter = int(self.constraints_iter)
        p.monitor = 1 if self.monitor_convergence else 0
        p.precise_hydro = 1 if self.precise_hydro else 0
        p.scatter = _native.SCATTER_PATCH
        p.use_graph = 1 if self.use_graph else 0
        p.tets_per_thread = self.tets_per_thread
        p.rho_min, p.rho_max, p.rho_beta = self.rho_min, self.rho_max, self.rho_beta
        p.target_rel_residual = self.target_rel_residual
        p.residual_floor = self.residual_floor
        return p

    def set_stop(self, target_rel_residual, residual_floor=0.0, constraints_iter=None):
        """Switch stop mode (0, 0: the fixed iteration count) and optionally the
        iteration cap between frames; the frame graph is recaptured."""
        self.target_rel_residual = float(target_rel_residual)
        self.residual_floor = float(residual_floor)
        if constraints_iter is not None:
            if int(constraints_iter) * len(frame_chunks(self.frame_dt, self.dt)) * self.substeps_num > self._max_records:
                raise ValueError("constraints_iter above the history capacity given at construction")
            self.constraints_iter = int(constraints_iter)
        _native.check(self._lib.xpbd_batch_set_params(self._handle, self._params()), batch=True)

    def iterations_per_substep(self, n=None):
        """(n_bodies, n) Jacobi iterations every body ran in each substep of the last frame."""
        n = len(frame_chunks(self.frame_dt, self.dt)) * self.substeps_num if n is None else int(n)
        out = np.zeros((self.n_bodies, n), dtype=np.int32)
        _native.check(self._lib.xpbd_batch_read_iterations(self._handle, out.ctypes.data, n, self._stream()),
                      batch=True)
        return out

    def _stream(self):
        return _torch().cuda.current_stream(self._device).cuda_stream

    # -- stepping ------------------------------------------------------------------
    def solve(self):
        """One frame of every body (neohookean_solver.py:562-587)."""
        _native.check(self._lib.xpbd_batch_solve(self._handle, float(self.frame_dt), float(self.dt),
                                                 int(self.substeps_num), self._stream()), batch=True)
        self.time += sum(frame_chunks(self.frame_dt, self.dt))
        self.current_frame += 1

    def substep(self, dt):
        _native.check(self._lib.xpbd_batch_substep(self._handle, float(dt), 0, self._stream()), batch=True)

    # -- state access ----------------------------------------------------------------
    def _export(self, field_id):
        torch = _torch()
        out = torch.empty((self.n_verts, 3), dtype=torch.float32, device=self._device)
        _native.check(self._lib.xpbd_batch_export_vec3(self._handle, field_id, out.data_ptr(), self._stream()),
                      batch=True)
        return out

    def positions(self):
        """All bodies' positions, (sum V_b, 3) float32 in body order then file order."""
        return self._export(_native.FIELD_X).cpu().numpy()

    def velocities(self):
        return self._export(_native.FIELD_V).cpu().numpy()

    def positions_device(self):
        return self._export(_native.FIELD_X)

    def body_positions(self, k):
        return self.positions()[self.body_vert_slices[k]]

    def set_positions(self, arr, field_id=_native.FIELD_X):
        torch = _torch()
        a = arr if isinstance(arr, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(arr, dtype=np.float32))
        self._stage.copy_(a, non_blocking=True)
        _native.check(self._lib.xpbd_batch_import_vec3(self._handle, field_id, self._stage.data_ptr(),
                                                       self._stream()), batch=True)

    def set_velocities(self, arr):
        self.set_positions(arr, _native.FIELD_V)

    @property
    def rho_hat(self):
        out = np.zeros(self.n_bodies, dtype=np.float64)
        _native.check(self._lib.xpbd_batch_get_rho_hat(self._handle, out.ctypes.data, self._stream()), batch=True)
        return out

    def read_history(self, n=None):
        """(n_bodies, n, 4) rows {r_hat, omega, hydro_error, dev_error} of the last frame."""
        n = self._max_records if n is None else int(n)
        out = np.zeros((self.n_bodies, n, 4), dtype=np.float64)
        _native.check(self._lib.xpbd_batch_read_history(self._handle, out.ctypes.data, n, self._stream()),
                      batch=True)
        return out

    def check_status(self):
        _native.check(self._lib.xpbd_batch_check_status(self._handle, self._stream()), batch=True)

    # -- in-place tuning support ---------------------------------------------------
    def set_tets_per_thread(self, tpt):
        if tpt not in (1, 2):
            raise ValueError("tets_per_thread must be 1 or 2")
        self.tets_per_thread = int(tpt)
        _native.check(self._lib.xpbd_batch_set_params(self._handle, self._params()), batch=True)

    def snapshot(self):
        """Device copies of the whole mutable state (positions, velocities,
        predicted positions, Jacobi accumulator, multipliers, rho_hat)."""
        torch = _torch()
        rho = torch.empty(self.n_bodies, dtype=torch.float64, device=self._device)
        _native.check(self._lib.xpbd_batch_save_rho_hat(self._handle, rho.data_ptr(), self._stream()), batch=True)
        return dict(x=self._x4.clone(), v=self._v4.clone(), p0=self._p4[0].clone(), p1=self._p4[1].clone(),
                    dx=self._dx4.clone(), lam=self._lam.clone(), rho=rho)

    def restore(self, snap):
        self._x4.copy_(snap["x"])
        self._v4.copy_(snap["v"])
        self._p4[0].copy_(snap["p0"])
        self._p4[1].copy_(snap["p1"])
        self._dx4.copy_(snap["dx"])
        self._lam.copy_(snap["lam"])
        _native.check(self._lib.xpbd_batch_load_rho_hat(self._handle, snap["rho"].data_ptr(), self._stream()),
                      batch=True)

    def time_substeps(self, sub_dt, warmup, reps):
        """ms per substep over `reps` replays of a one-substep frame graph."""
        torch = _torch()
        lib, h, st = self._lib, self._handle, self._stream()
        for _ in range(max(1, warmup)):
            _native.check(lib.xpbd_batch_solve(h, float(sub_dt), float(sub_dt), 1, st), batch=True)
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(reps):
            _native.check(lib.xpbd_batch_solve(h, float(sub_dt), float(sub_dt), 1, st), batch=True)
        b.record()
        b.synchronize()
        self.check_status()
        return a.elapsed_time(b) / reps

    def set_profiling(self, enable):
        _native.check(self._lib.xpbd_batch_set_profiling(self._handle, 1 if enable else 0), batch=True)

    def read_profile(self, reset=False):
        n = len(_native.KERNEL_CLASSES)
        ms = (_native.ctypes.c_double * n)()
        cnt = (_native.ctypes.c_int64 * n)()
        _native.check(self._lib.xpbd_batch_read_profile(self._handle, ms, cnt, n, 1 if reset else 0,
                                                        self._stream()), batch=True)
        return {k: {"ms": ms[i], "launches": int(cnt[i])} for i, k in enumerate(_native.KERNEL_CLASSES)}

    def __del__(self):
        h = getattr(self, "_handle", None)
        if h is not None:
            try:
                self._lib.xpbd_batch_destroy(h)
            except Exception:
                pass
            self._handle = None
