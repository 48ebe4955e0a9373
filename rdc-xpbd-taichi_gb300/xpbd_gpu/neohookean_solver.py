"""XPBDNeoHookeanSolver: residual-driven Chebyshev Jacobi block Neo-Hookean XPBD.

Drop-in for the reference class (``xpbd_gpu/neohookean_solver.py:16-587``):
same constructor arguments, ``solve()`` / ``solve_step(dt)``, monitoring
attributes (``convergence_history``, ``convergence_callback``,
``monitor_convergence``, ``current_frame``/``current_substep``), timing
attributes (``solve_compute_time_total/calls/iterations``) and the
Chebyshev state (``rho_hat`` persists across substeps and frames).

Every substep runs on the GPU as hand-written sm_103a kernels
(``libxpbd_gb300.so``, ``include/xpbd_gb300.h``).  The residual r_hat, the
spectral-radius estimate rho_hat and the omega recurrence are evaluated on
the device in FP64, so a frame needs no host round trip; ``solve()`` replays
one cached CUDA graph per frame.  With ``monitor_convergence`` the frame is
driven substep by substep so that ``convergence_callback`` fires after each
substep, as in the reference (:574-583).

Extensions (keyword-only): ``total_mass`` / ``density`` (the reference fixes
1 kg, xpbd_base.py:36), ``gravity``, ``scatter`` ('atomic' = vector
red.global.add, 'gather' = deterministic vertex->tet CSR), ``precise_hydro``
(cancellation-free det F - 1; default on for poisson_ratio >= 0.49),
``use_graph``, ``reorder`` (Morton order on the device) and ``pair_tets``
(face-adjacent tets ordered in pairs with aligned corners, so the
two-tets-per-thread kernels merge their shared corners without comparing
vertex ids; on by default), and ``target_rel_residual`` / ``residual_floor``
(stop mode: each substep ends after the first iteration whose r_hat is at most
``target_rel_residual`` times the substep's first r_hat, or at most
``residual_floor``, with ``constraints_iter`` as the cap; the reference always
runs ``constraints_iter`` iterations, :474; ``iterations_per_substep()``
returns the counts of the last frame).  With
``scatter="auto"`` the scatter variant, patch size, tets per thread and
tile pipeline are measured on this mesh and GPU (``xpbd_gpu.autotune``) and
the choice is kept in ``autotune_result``.
"""
import numpy as np

from xpbd_gpu import _native
from xpbd_gpu.xpbd_base import XPBDSolverBase, _torch, calc_tet_volume  # noqa: F401


def calc_first_lame(E, nu):
    """neohookean_solver.py:7-8."""
    return 2.0 * nu / (1.0 - 2.0 * nu) * calc_second_lame(E, nu)


def calc_second_lame(E, nu):
    """neohookean_solver.py:11-12."""
    return E / (2.0 * (1.0 + nu))


def frame_chunks(frame_dt, dt):
    """dt0 of each chunk of one frame, in float64 (neohookean_solver.py:563-568)."""
    out = []
    left = frame_dt
    while left > 0.0:
        d = min(dt, left)
        left -= d
        out.append(d)
    return out


class XPBDNeoHookeanSolver(XPBDSolverBase):

    def __init__(self, rest_pose, sdf, young_modulus=200000.0, poisson_ratio=0.495, scale=1.0,
                 offset=(0.0, 0.0, 0.0), frame_dt=1e-2, dt=1e-2, substeps_num=20, constraints_iter=5,
                 reorder_all=False, block_size=256, hydrostatic_relaxation=1.2, deviatoric_relaxation=1.2,
                 cheb_enable=True, cheb_warmup=5, cheb_gamma=0.6666, block_neohookean_enable=False,
                 monitor_convergence=False, *, total_mass=1.0, density=None, gravity=(0.0, -9.8, 0.0),
                 scatter="patch", precise_hydro=None, use_graph=True, reorder=True, sweep_order=1,
                 patch_pipeline=0, patch_reduce=0, tets_per_thread=2, patch_tets=256, tet_young_modulus=None,
                 tet_poisson_ratio=None, autotune_cache=True, pair_tets=True, target_rel_residual=0.0,
                 residual_floor=0.0):
        self.autotune_result = None
        if scatter == "auto":
            from xpbd_gpu import autotune
            args = {k: v for k, v in locals().items() if k not in ("self", "autotune", "__class__")}
            args.pop("autotune_cache")
            self.autotune_result = autotune.tune_single(type(self), args, cache=autotune_cache)
            r = self.autotune_result
            scatter, patch_tets = r["scatter"], r["patch_tets"]
            tets_per_thread, patch_pipeline = r["tets_per_thread"], r["patch_pipeline"]
        self.constraints_iter = constraints_iter
        self.target_rel_residual = float(target_rel_residual)
        self.residual_floor = float(residual_floor)
        self.hydrostatic_relaxation = hydrostatic_relaxation
        self.deviatoric_relaxation = deviatoric_relaxation
        self.young_modulus = young_modulus
        self.poisson_ratio = poisson_ratio
        self.lame1 = calc_first_lame(young_modulus, poisson_ratio)
        self.lame2 = calc_second_lame(young_modulus, poisson_ratio)
        self.cheb_enable = cheb_enable
        self.cheb_gamma = cheb_gamma
        self.cheb_warmup = cheb_warmup
        self.block_neohookean_enable = block_neohookean_enable
        self.monitor_convergence = monitor_convergence
        self.convergence_history = []
        self.current_substep_convergence = []
        self.current_frame = 0
        self.current_substep = 0
        self.convergence_callback = None
        self.rho_min = 0.00001  # :66-68
        self.rho_max = 0.99999
        self.rho_beta = 0.2
        self.prev_r_hat = None
        self._timing_events = []
        self._time_done = 0.0
        self.solve_compute_calls = 0
        self._iterations_fixed = 0
        self._iterations_device_base = 0
        if scatter not in _native.SCATTERS:
            raise ValueError("scatter must be one of %s" % sorted(_native.SCATTERS))
        self.scatter = scatter
        self.sweep_order = int(sweep_order)
        self.patch_pipeline = int(patch_pipeline)
        self.patch_reduce = int(patch_reduce)
        self.tets_per_thread = int(tets_per_thread)
        self.patch_tets = int(patch_tets)
        # per-tet materials (file tet order); they need a per-tet scatter variant
        self._tet_E = None if tet_young_modulus is None else np.asarray(tet_young_modulus, dtype=np.float64)
        self._tet_nu = None
        if self._tet_E is not None:
            nu_t = poisson_ratio if tet_poisson_ratio is None else tet_poisson_ratio
            self._tet_nu = np.broadcast_to(np.asarray(nu_t, dtype=np.float64), self._tet_E.shape).copy()
            if scatter == "patch":
                scatter = "atomic"
                self.scatter = scatter
        self.precise_hydro = (poisson_ratio >= 0.49) if precise_hydro is None else bool(precise_hydro)
        self.use_graph = bool(use_graph)
        self.block_size = block_size
        super().__init__(rest_pose, sdf, scale, offset, frame_dt, dt, substeps_num, reorder_all, block_size,
                         total_mass=total_mass, density=density, gravity=gravity, reorder=reorder,
                         pair_tets=pair_tets)

    # -- construction (neohookean_solver.py:79-95) ------------------------------
    def initialize_specific(self, scale, offset):
        x, V0, inv_Dm = self.initialize(scale, offset)
        m, inv_m = self.compute_lumped_mass(x, V0)
        self._upload(x, V0, inv_Dm, m, inv_m)
        if self.scatter == "gather":
            self._ensure_gather_buffers()
        self._tinv_mu = self._tinv_la = None
        if self._tet_E is not None:
            torch = _torch()
            T = self.n_tets
            if self._tet_E.shape != (T,):
                raise ValueError("tet_young_modulus must have one entry per tet")
            self._tinv_mu = torch.empty(T, dtype=torch.float32, device=self._device)
            self._tinv_la = torch.empty(T, dtype=torch.float32, device=self._device)
            self.set_tet_materials(np.log(self._tet_E), self._tet_nu)
        if self.scatter == "patch" and not self._ensure_patch_buffers():
            # no patch size keeps every patch within 256 vertices: per-tet variant
            self.scatter = "atomic"
        self._build_mesh_view()
        self._max_records = max(1, self._records_per_frame())
        prm = self._params()
        self._prm_bytes = bytes(prm)
        h = _native.ctypes.c_void_p()
        table = self._sdf_table()
        body = self._body()
        _native.check(self._lib.xpbd_create(prm, body, table, len(self.sdfs), self._max_records,
                                            _native.ctypes.byref(h)))
        self._handle = h.value

    def set_tet_materials(self, log_E, nu):
        """Per-tet log Young's modulus and Poisson ratio (file tet order; numpy or
        torch).  Uploads 1/mu and 1/lambda in solver order."""
        torch = _torch()
        if self._tinv_mu is None:
            raise RuntimeError("the solver was built without per-tet materials")
        le = torch.as_tensor(log_E, dtype=torch.float64, device=self._device).reshape(-1)
        nu_t = torch.as_tensor(nu, dtype=torch.float64, device=self._device).reshape(-1).expand(le.shape[0])
        E = torch.exp(le)
        inv_mu = 2.0 * (1.0 + nu_t) / E
        inv_la = (1.0 + nu_t) * (1.0 - 2.0 * nu_t) / (E * nu_t)
        perm = torch.as_tensor(self._tperm, dtype=torch.int64, device=self._device)
        self._tinv_mu.copy_(inv_mu[perm].to(torch.float32))
        self._tinv_la.copy_(inv_la[perm].to(torch.float32))

    def _records_per_frame(self):
        return len(frame_chunks(self.frame_dt, self.dt)) * self.substeps_num * self.constraints_iter

    def _params(self):
        p = _native.XpbdParams()
        p.lame_mu = self.lame2
        p.lame_lambda = self.lame1
        p.gravity[:] = [float(g) for g in np.asarray(self.gravity, dtype=np.float64).reshape(3)]
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
        p.scatter = _native.SCATTERS[self.scatter]
        p.use_graph = 1 if self.use_graph else 0
        p.sweep_order = self.sweep_order
        p.patch_pipeline = self.patch_pipeline
        p.patch_reduce = self.patch_reduce
        p.tets_per_thread = self.tets_per_thread
        p.rho_min, p.rho_max, p.rho_beta = self.rho_min, self.rho_max, self.rho_beta
        p.target_rel_residual = self.target_rel_residual
        p.residual_floor = self.residual_floor
        return p

    @property
    def stop_mode(self):
        return self.target_rel_residual > 0.0 or self.residual_floor > 0.0

    # -- iteration counts (neohookean_solver.py:71-73) -----------------------------
    def _device_iterations(self):
        total = _native.ctypes.c_int64(0)
        _native.check(self._lib.xpbd_read_iterations(self._handle, None, 0, _native.ctypes.byref(total),
                                                     self._stream()))
        return int(total.value)

    @property
    def solve_compute_iterations(self):
        """Jacobi iterations run so far (reference attribute, :73); in stop mode
        the device's count of the iterations that actually ran (synchronises)."""
        if getattr(self, "_handle", None) is not None and self.stop_mode:
            return self._iterations_fixed + self._device_iterations() - self._iterations_device_base
        return self._iterations_fixed

    @solve_compute_iterations.setter
    def solve_compute_iterations(self, value):
        self._iterations_fixed = int(value)
        if getattr(self, "_handle", None) is not None:
            self._iterations_device_base = self._device_iterations()

    def _count_iterations(self, n):
        if not self.stop_mode:
            self._iterations_fixed += n

    def iterations_per_substep(self, n=None):
        """Jacobi iterations each substep of the last frame ran (constraints_iter
        in the reference's fixed mode; in stop mode up to it)."""
        n = len(frame_chunks(self.frame_dt, self.dt)) * self.substeps_num if n is None else int(n)
        out = np.zeros(n, dtype=np.int32)
        if n:
            _native.check(self._lib.xpbd_read_iterations(self._handle, out.ctypes.data, n, None, self._stream()))
        return out

    def _sync(self):
        super()._sync()
        if self.scatter == "gather" and self._corner is None:
            raise RuntimeError("scatter='gather' needs the CSR buffers built at construction")
        if self.scatter == "patch" and self._tet_lid is None:
            raise RuntimeError("scatter='patch' needs the patch layout built at construction")
        prm = self._params()
        b = bytes(prm)
        if b != self._prm_bytes:
            _native.check(self._lib.xpbd_set_params(self._handle, prm))
            self._prm_bytes = b

    # -- Chebyshev state ---------------------------------------------------------
    @property
    def rho_hat(self):
        out = _native.ctypes.c_double()
        _native.check(self._lib.xpbd_get_rho_hat(self._handle, _native.ctypes.byref(out), self._stream()))
        return out.value

    @rho_hat.setter
    def rho_hat(self, value):
        if getattr(self, "_handle", None) is None:
            return  # set by the reference's constructor order; device starts at 0.999
        _native.check(self._lib.xpbd_set_rho_hat(self._handle, float(value), self._stream()))

    # -- timing attributes (neohookean_solver.py:71-73, :558-560) --------------
    @property
    def solve_compute_time_total(self):
        if self._timing_events:
            for a, b in self._timing_events:
                b.synchronize()
                self._time_done += a.elapsed_time(b) * 1e-3
            self._timing_events = []
        return self._time_done

    def _events(self):
        torch = _torch()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        return a, b

    # -- history ------------------------------------------------------------------
    @property
    def residual_history(self):
        """r_hat of every Jacobi iteration of the last frame (or of the last
        monitored substep), in iteration order: the residual curve that drives
        the Chebyshev omega (neohookean_solver.py:492-504)."""
        rows = self.read_history(self.constraints_iter if self.monitor_convergence else None)
        return rows[:, 0].tolist()

    def read_history(self, n=None):
        """(n, 4) float64 rows {r_hat, omega, hydro_error, dev_error} of the last
        frame (or of the last solve_step), in iteration order."""
        n = self._max_records if n is None else int(n)
        out = np.zeros((n, 4), dtype=np.float64)
        if n:
            _native.check(self._lib.xpbd_read_history(
                self._handle, out.ctypes.data_as(_native.ctypes.POINTER(_native.ctypes.c_double)), n,
                self._stream()))
        return out

    def set_profiling(self, enable):
        """Bracket every kernel launch with CUDA events (with use_graph the
        frame graph carries them as event record nodes)."""
        _native.check(self._lib.xpbd_set_profiling(self._handle, 1 if enable else 0))

    def set_l2_hint(self, mode=-1):
        """L2 policy of the tile sweeps' read-only tet records: -1 automatic
        (evict_last when records + state fit in 80% of L2), 0 plain loads,
        1 evict_last.  Returns the policy in force (0 or 1)."""
        on = _native.ctypes.c_int32(0)
        _native.check(self._lib.xpbd_set_l2_hint(self._handle, int(mode), _native.ctypes.byref(on)))
        return int(on.value)

    def read_profile(self, reset=False):
        """{kernel class: {'ms': total device ms, 'launches': n}} since the last reset."""
        n = len(_native.KERNEL_CLASSES)
        ms = (_native.ctypes.c_double * n)()
        cnt = (_native.ctypes.c_int64 * n)()
        _native.check(self._lib.xpbd_read_profile(self._handle, ms, cnt, n, 1 if reset else 0, self._stream()))
        return {k: {"ms": ms[i], "launches": int(cnt[i])} for i, k in enumerate(_native.KERNEL_CLASSES)}

    def check_status(self):
        """Raise if a residual reduction produced NaN/Inf (sticky device flag)."""
        _native.check(self._lib.xpbd_check_status(self._handle, self._stream()))

    def _records_to_history(self, rows, K=None):
        K = self.constraints_iter if K is None else K
        for it in range(K):
            rec = dict(frame=self.current_frame, substep=self.current_substep, iter=it,
                       iter_compute_time_sec=0.0, hydro_error=float(rows[it, 2]),
                       dev_error=float(rows[it, 3]))
            self.convergence_history.append(rec)
            self.current_substep_convergence.append(rec)

    # -- stepping -------------------------------------------------------------------
    def solve_step(self, dt):
        """neohookean_solver.py:453-560 (predicted positions must be set, e.g. by
        apply_external_forces)."""
        self._sync()
        a, b = self._events()
        a.record()
        _native.check(self._lib.xpbd_solve_step(self._handle, float(dt), 0, self._stream()))
        b.record()
        self._timing_events.append((a, b))
        self.solve_compute_calls += 1
        self._count_iterations(self.constraints_iter)
        n_it = int(self.iterations_per_substep(1)[0]) if self.stop_mode else self.constraints_iter
        if self.monitor_convergence:
            rows = self.read_history(self.constraints_iter)
            t_it = a.elapsed_time(b) * 1e-3 / max(1, n_it)
            start = len(self.convergence_history)
            self._records_to_history(rows, n_it)
            for r in self.convergence_history[start:]:
                r["iter_compute_time_sec"] = t_it
        if self.cheb_enable and n_it > 0:
            self.prev_r_hat = float(self.read_history(self.constraints_iter)[n_it - 1, 0])

    def solve(self):
        """neohookean_solver.py:562-587: one frame."""
        self._sync()
        stream = self._stream()
        self.current_substep = 0
        if not self.monitor_convergence:
            a, b = self._events()
            a.record()
            _native.check(self._lib.xpbd_solve(self._handle, float(self.frame_dt), float(self.dt),
                                               int(self.substeps_num), stream))
            b.record()
            self._timing_events.append((a, b))
            chunks = frame_chunks(self.frame_dt, self.dt)
            self.solve_compute_calls += len(chunks) * self.substeps_num
            self._count_iterations(len(chunks) * self.substeps_num * self.constraints_iter)
            self.time += sum(chunks)
            if chunks:
                self.current_substep = self.substeps_num - 1
            self.current_frame += 1
            return
        for dt0 in frame_chunks(self.frame_dt, self.dt):
            sub_dt = dt0 / self.substeps_num
            for substep in range(self.substeps_num):
                self.current_substep = substep
                self.current_substep_convergence = []
                a, b = self._events()
                a.record()
                _native.check(self._lib.xpbd_substep(self._handle, float(sub_dt), 0, stream))
                b.record()
                self._timing_events.append((a, b))
                self.solve_compute_calls += 1
                self._count_iterations(self.constraints_iter)
                n_it = int(self.iterations_per_substep(1)[0]) if self.stop_mode else self.constraints_iter
                rows = self.read_history(self.constraints_iter)
                t_it = a.elapsed_time(b) * 1e-3 / max(1, n_it)
                self._records_to_history(rows, n_it)
                for r in self.current_substep_convergence:
                    r["iter_compute_time_sec"] = t_it
                if self.convergence_callback:
                    self.convergence_callback(self.current_frame, self.current_substep,
                                              self.current_substep_convergence)
            self.time += dt0
        self.current_frame += 1
