"""Differentiable XPBD simulation: gradients of a loss on the final positions
w.r.t. per-tet log Young's modulus and Poisson ratio, initial positions and
initial velocities.

The reference has no gradients.  The forward is the reference's substep
(``neohookean_solver.py:453-587``) run on the GPU with per-tet materials;
``xpbd_simulate`` wraps it in a ``torch.autograd.Function`` whose backward
runs hand-written adjoint kernels (``xpbd_substep_adjoint``) over a tape of
each substep: the predicted positions and multipliers entering every Jacobi
iteration, the states around predict and the SDF list, and the substep's
history rows (omega, r_hat).

Each simulation length gets a plan (``_Plan``) in one of two forms:
* tapes stored (``tape_memory="store"``): the forward records every
  substep's tape as it runs; the backward only reverses them.  A tape is
  about (K + 1) (32 V + 8 T) bytes per substep (K iterations, V vertices, T
  tets), e.g. 80 GB for 64 bodies of 1.75 M tets over 150 substeps of 20
  iterations -- HBM that a GB300 has;
* recomputed (``tape_memory="recompute"``): the forward checkpoints the
  state once per substep (positions, velocities, rho_hat); the backward
  restores each checkpoint and re-runs the substep on one shared tape before
  reversing it, which costs one more forward.
``tape_memory="auto"`` (default) stores when the plan's tapes take at most
half of the free device memory at plan creation.  Each pass is captured
once as a CUDA graph and replayed, so an optimisation loop launches two
graphs per step.  A simulation object holds one simulation in flight: its
backward must run before its next forward.

Differentiation conventions: active contact sets and the 2x2 pivot branch
are piecewise constant.  By default (``omega_grad=True``) the adjoint also
runs back through the Chebyshev factor: omega_k depends on the spectral
estimate rho_hat, which follows the residual ratio r_hat_k / r_hat_{k-1}
(neohookean_solver.py:495-546), and r_hat on the post-Jacobi positions, the
multipliers and the compliances (:298-329); the tape then also records the
post-Jacobi positions of every iteration.  ``omega_grad=False`` treats omega
as a stop-gradient, the derivative of the run with its omega schedule
replayed: cheaper, but for a uniform Poisson ratio, which moves the whole
residual curve, far from the derivative of the forward as it runs.
"""
import numpy as np

from xpbd_gpu import _native
from xpbd_gpu.neohookean_solver import XPBDNeoHookeanSolver, frame_chunks
from xpbd_gpu.xpbd_base import _torch


class _Plan:
    """Tapes or checkpoints and the two passes of one simulation length of `sim`
    (a DiffSim or a BatchedDiffSim): captured as two CUDA graphs with
    `use_graphs`, else run directly."""

    def __init__(self, sim, frames, use_graphs):
        torch = _torch()
        self.dts = sim.substep_dts(frames)
        n = len(self.dts)
        self.stored = sim._store_tapes(n)
        if self.stored:
            self.tapes = _Tapes(sim, n)
        else:
            x4, v4 = sim._state()
            self.ck_x = torch.empty((n,) + tuple(x4.shape), dtype=x4.dtype, device=x4.device)
            self.ck_v = torch.empty((n,) + tuple(v4.shape), dtype=v4.dtype, device=v4.device)
            self.ck_rho = torch.empty((n, sim.n_rho), dtype=torch.float64, device=x4.device)
        self.generation = 0
        self._graphs = None
        if use_graphs:
            gf, gb = torch.cuda.CUDAGraph(), torch.cuda.CUDAGraph()
            with torch.cuda.graph(gf):
                self._forward(sim)
            with torch.cuda.graph(gb):
                self._backward(sim)
            self._graphs = (gf, gb)

    def _forward(self, sim):
        if self.stored:
            for k, dt in enumerate(self.dts):
                sim._tape(dt, self.tapes.structs[k])
            return
        x4, v4 = sim._state()
        for k, dt in enumerate(self.dts):
            self.ck_x[k].copy_(x4)
            self.ck_v[k].copy_(v4)
            sim.rho_copy_to(self.ck_rho[k])
            sim._substep(dt)

    def _backward(self, sim):
        if self.stored:
            for k in reversed(range(len(self.dts))):
                sim._adjoint(self.dts[k], self.tapes.structs[k])
            return
        x4, v4 = sim._state()
        for k in reversed(range(len(self.dts))):
            x4.copy_(self.ck_x[k])
            v4.copy_(self.ck_v[k])
            sim.rho_load_from(self.ck_rho[k])
            sim._tape(self.dts[k])
            sim._adjoint(self.dts[k])

    def forward(self, sim):
        self.generation += 1
        if self._graphs:
            self._graphs[0].replay()
        else:
            self._forward(sim)
        return self.generation

    def backward(self, sim, generation):
        if generation != self.generation:
            raise RuntimeError("a later forward of this simulation object overwrote the checkpoints; run "
                               "each backward before the next forward")
        if self._graphs:
            self._graphs[1].replay()
        else:
            self._backward(sim)


class _Tapes:
    """The tapes of `n` substeps of `sim`, one slice of each buffer per substep."""

    def __init__(self, sim, n):
        torch = _torch()
        V, T, K, nb = sim.V, sim.T, sim.K, sim.n_rho
        dev = sim._gx.device
        f32 = dict(dtype=torch.float32, device=dev)
        f64 = dict(dtype=torch.float64, device=dev)
        self.xs = torch.empty((n, (K + 1) * V, 4), **f32)
        self.lams = torch.empty((n, _lam_rows(sim), 2), **f32)
        self.xpre = torch.empty((n, V, 4), **f32)
        self.v1 = torch.empty((n, V, 4), **f32)
        self.posts = torch.empty((n, K * V, 4), **f32) if sim.omega_grad else None
        self.rho_in = torch.empty((n, nb), **f64) if sim.omega_grad else None
        self.hist = torch.empty((n, nb * K * 4), **f64)
        p = lambda t, k: t[k].data_ptr() if t is not None else None
        self.structs = [_native.XpbdTape(p(self.xs, k), p(self.lams, k), p(self.xpre, k), p(self.v1, k),
                                         p(self.posts, k), p(self.rho_in, k), p(self.hist, k)) for k in range(n)]

    @staticmethod
    def nbytes(sim, n):
        V, T, K, nb = sim.V, sim.T, sim.K, sim.n_rho
        per = 16 * ((K + 1) * V + 2 * V) + 8 * _lam_rows(sim) + 32 * nb * K
        if sim.omega_grad:
            per += 16 * K * V + 8 * nb
        return n * per


def _lam_rows(sim):
    """Multiplier rows of one tape: those entering every iteration, and with
    omega_grad those after the last."""
    return (sim.K + 1 if sim.omega_grad else max(sim.K, 1)) * sim.T


def _plan(sim, frames):
    """The plan of `frames` frames under the simulation's current tape_memory
    (an "auto" plan keeps the choice it made when it was created)."""
    plans = sim.__dict__.setdefault("_plans", {})
    key = (frames, sim.tape_memory)
    if key not in plans:
        plans[key] = _Plan(sim, frames, sim.use_graphs)
    return plans[key]


class DiffSim:
    """A single body with per-tet materials and the buffers of its adjoint."""

    n_rho = 1

    def __init__(self, rest_pose, sdf, log_E, nu, scatter="atomic", use_graphs=True, omega_grad=True,
                 tape_memory="auto", **kw):
        _check_solver_kwargs(kw)
        log_E = np.asarray(log_E, dtype=np.float64)
        self.solver = XPBDNeoHookeanSolver(rest_pose, sdf, tet_young_modulus=np.exp(log_E),
                                           tet_poisson_ratio=np.asarray(nu, dtype=np.float64), scatter=scatter,
                                           use_graph=False, **kw)
        s = self.solver
        torch = _torch()
        dev = s._device
        V, T, K = s.n_verts, s.n_tets, s.constraints_iter
        self.V, self.T, self.K = V, T, K
        self._alloc_adjoint_buffers(V, T, K, 1, dev, omega_grad)
        cnt = np.bincount(s._tets_solver.reshape(-1), minlength=V).astype(np.float32)
        self._cnt = torch.from_numpy(cnt).to(dev)
        self._vperm = torch.as_tensor(s._vperm, dtype=torch.int64, device=dev)
        self._tperm = torch.as_tensor(s._tperm, dtype=torch.int64, device=dev)
        self._bind()
        self.initial_rho_hat = s.rho_hat
        self.use_graphs = bool(use_graphs)
        self.tape_memory = _check_tape_memory(tape_memory)

    def _store_tapes(self, n_substeps):
        """Whether a plan of `n_substeps` substeps stores its tapes (tape_memory)."""
        if self.tape_memory != "auto":
            return self.tape_memory == "store"
        free, _ = _torch().cuda.mem_get_info(self._gx.device)
        return _Tapes.nbytes(self, n_substeps) <= free // 2

    def _alloc_adjoint_buffers(self, V, T, K, n_bodies, dev, omega_grad):
        """Tape and adjoint buffers; with omega_grad the tape also keeps the
        post-Jacobi positions, the multipliers after the last iteration and the
        rho_hat entering the substep, and the adjoint a chain state per body."""
        torch = _torch()
        f4 = lambda n: torch.zeros((n, 4), dtype=torch.float32, device=dev)
        self.omega_grad = bool(omega_grad)
        self._xs = torch.zeros(((K + 1) * V, 4), dtype=torch.float32, device=dev)
        self._lams = torch.zeros((_lam_rows(self), 2), dtype=torch.float32, device=dev)
        self._xpre, self._v1 = f4(V), f4(V)
        self._gx, self._gv = f4(V), f4(V)
        self._w0, self._w1, self._yb, self._dxb = f4(V), f4(V), f4(V), f4(V)
        self._lamb = torch.zeros((T, 2), dtype=torch.float32, device=dev)
        self._gmu = torch.zeros(T, dtype=torch.float64, device=dev)
        self._gla = torch.zeros(T, dtype=torch.float64, device=dev)
        self._posts = f4(K * V) if omega_grad else None
        self._rho_in = torch.zeros(n_bodies, dtype=torch.float64, device=dev) if omega_grad else None
        self._om = (torch.zeros((n_bodies, 8 + 6 * K), dtype=torch.float64, device=dev) if omega_grad
                    else None)
        # the batch hands the residual adjoint's tet parts to the tet adjoint through this
        self._rtet = f4(T) if omega_grad else None

    def _bind(self):
        ptr = lambda t: t.data_ptr() if t is not None else None
        self.tape = _native.XpbdTape(self._xs.data_ptr(), self._lams.data_ptr(), self._xpre.data_ptr(),
                                     self._v1.data_ptr(), ptr(self._posts), ptr(self._rho_in))
        self.adj = _native.XpbdAdjoint(self._gx.data_ptr(), self._gv.data_ptr(), self._gmu.data_ptr(),
                                       self._gla.data_ptr(), self._w0.data_ptr(), self._w1.data_ptr(),
                                       self._yb.data_ptr(), self._dxb.data_ptr(), self._lamb.data_ptr(),
                                       self._cnt.data_ptr(), ptr(self._om), ptr(self._rtet))

    def reset_adjoint(self):
        """Zero what a backward pass accumulates (the omega chain included)."""
        self._gx.zero_()
        self._gv.zero_()
        self._gmu.zero_()
        self._gla.zero_()
        if self._om is not None:
            self._om.zero_()

    # -- the steps of a plan ---------------------------------------------------
    def _state(self):
        return self.solver._x4, self.solver._v4

    def _substep(self, dt):
        s = self.solver
        _native.check(s._lib.xpbd_substep(s._handle, float(dt), 0, s._stream()))

    def _tape(self, dt, tape=None):
        s = self.solver
        tape = self.tape if tape is None else tape
        _native.check(s._lib.xpbd_substep_tape(s._handle, float(dt), tape, s._stream()))

    def _adjoint(self, dt, tape=None):
        s = self.solver
        tape = self.tape if tape is None else tape
        _native.check(s._lib.xpbd_substep_adjoint(s._handle, float(dt), tape, self.adj, s._stream()))

    def rho_copy_to(self, dst):
        """Stream-ordered copy of the device rho_hat into a 1-element float64 tensor."""
        s = self.solver
        _native.check(s._lib.xpbd_save_rho_hat(s._handle, dst.data_ptr(), s._stream()))

    def rho_load_from(self, src):
        s = self.solver
        _native.check(s._lib.xpbd_load_rho_hat(s._handle, src.data_ptr(), s._stream()))

    def substep_dts(self, frames):
        s = self.solver
        out = []
        for _ in range(frames):
            for d in frame_chunks(s.frame_dt, s.dt):
                out.extend([d / s.substeps_num] * s.substeps_num)
        return out

    # caller order (V, 3) <-> solver order (V, 4) with w = inv_m
    def set_state(self, x, v):
        s = self.solver
        s._x4[:, :3] = x.to(s._x4)[self._vperm]
        s._v4[:, :3] = v.to(s._v4)[self._vperm]

    def positions(self):
        s = self.solver
        out = s._x4.new_empty((self.V, 3))
        out[self._vperm] = s._x4[:, :3]
        return out


class _Simulate(_torch().autograd.Function):
    @staticmethod
    def forward(ctx, x0, v0, log_E, nu, sim, frames):
        s = sim.solver
        s.set_tet_materials(log_E.detach(), nu.detach())
        sim.set_state(x0.detach(), v0.detach())
        s.rho_hat = sim.initial_rho_hat
        plan = _plan(sim, frames)
        ctx.sim, ctx.plan, ctx.generation = sim, plan, plan.forward(sim)
        ctx.save_for_backward(log_E, nu)
        return sim.positions()

    @staticmethod
    def backward(ctx, g_out):
        torch = _torch()
        sim = ctx.sim
        log_E, nu = ctx.saved_tensors
        sim.reset_adjoint()
        sim._gx[:, :3] = g_out.to(torch.float32)[sim._vperm]
        ctx.plan.backward(sim, ctx.generation)
        gx = torch.empty((sim.V, 3), dtype=torch.float32, device=g_out.device)
        gv = torch.empty_like(gx)
        gx[sim._vperm] = sim._gx[:, :3]
        gv[sim._vperm] = sim._gv[:, :3]
        # d/d(1/mu), d/d(1/lambda) (solver tet order) -> d/dlog E, d/dnu (file order)
        gmu = torch.empty_like(sim._gmu)
        gla = torch.empty_like(sim._gla)
        gmu[sim._tperm] = sim._gmu
        gla[sim._tperm] = sim._gla
        E = torch.exp(log_E.detach().to(torch.float64))
        n = nu.detach().to(torch.float64).expand_as(E)
        inv_mu = 2.0 * (1.0 + n) / E
        inv_la = (1.0 + n) * (1.0 - 2.0 * n) / (E * n)
        g_logE = -(gmu * inv_mu + gla * inv_la)
        g_nu = gmu * 2.0 / E + gla * (-1.0 - 2.0 * n * n) / (n * n * E)
        if nu.numel() == 1:
            g_nu = g_nu.sum().reshape(nu.shape)
        return (gx.to(g_out.dtype), gv.to(g_out.dtype), g_logE.to(log_E.dtype), g_nu.to(nu.dtype), None, None)


def xpbd_simulate(sim, x0, v0, log_E, nu, frames):
    """Final positions (V, 3) after `frames` frames from (x0, v0) with per-tet
    log E and nu; differentiable w.r.t. all four tensors."""
    return _Simulate.apply(x0, v0, log_E, nu, sim, frames)


def _lame_inverse_grads(gmu, gla, log_E, nu):
    """d/d(1/mu), d/d(1/lambda) -> d/dlog E, d/dnu (float64 tensors, per tet)."""
    torch = _torch()
    E = torch.exp(log_E.detach().to(torch.float64))
    n = nu.detach().to(torch.float64).expand_as(E)
    inv_mu = 2.0 * (1.0 + n) / E
    inv_la = (1.0 + n) * (1.0 - 2.0 * n) / (E * n)
    g_logE = -(gmu * inv_mu + gla * inv_la)
    g_nu = gmu * 2.0 / E + gla * (-1.0 - 2.0 * n * n) / (n * n * E)
    return g_logE, g_nu


class BatchedDiffSim:
    """A batch of bodies (``XPBDBatchedSolver``) with per-tet materials and the
    buffers of its adjoint.  Forward and adjoint of a substep are each one
    launch per phase over the tets or vertices of all bodies; every body keeps
    its own Chebyshev state, so the gradients of each body equal those of the
    same body simulated alone."""

    def __init__(self, bodies, sdf, use_graphs=True, omega_grad=True, tape_memory="auto", **kw):
        from xpbd_gpu.batched import Body, XPBDBatchedSolver
        _check_solver_kwargs(kw)
        bodies = [b if b.tet_young_modulus is not None else
                  Body(**dict(b.__dict__, tet_young_modulus=np.full(_n_tets(b.rest_pose), b.young_modulus)))
                  for b in bodies]
        self.batch = XPBDBatchedSolver(bodies, sdf, **kw)
        s = self.batch
        torch = _torch()
        dev = s._device
        V, T, K = s.n_verts_padded, s.n_tets_padded, s.constraints_iter
        self.V, self.T, self.K = V, T, K
        self.n_verts, self.n_tets = s.n_verts, s.n_tets
        DiffSim._alloc_adjoint_buffers(self, V, T, K, s.n_bodies, dev, omega_grad)
        self._cnt = s._cnt
        DiffSim._bind(self)
        self.initial_rho_hat = torch.empty(s.n_bodies, dtype=torch.float64, device=dev)
        self.rho_copy_to(self.initial_rho_hat)
        self.n_rho = s.n_bodies
        self.use_graphs = bool(use_graphs)
        self.tape_memory = _check_tape_memory(tape_memory)

    _store_tapes = DiffSim._store_tapes

    # -- the steps of a plan ---------------------------------------------------
    def _state(self):
        return self.batch._x4, self.batch._v4

    def _substep(self, dt):
        s = self.batch
        _native.check(s._lib.xpbd_batch_substep(s._handle, float(dt), 0, s._stream()), batch=True)

    def _tape(self, dt, tape=None):
        s = self.batch
        tape = self.tape if tape is None else tape
        _native.check(s._lib.xpbd_batch_substep_tape(s._handle, float(dt), tape, s._stream()), batch=True)

    def _adjoint(self, dt, tape=None):
        s = self.batch
        tape = self.tape if tape is None else tape
        _native.check(s._lib.xpbd_batch_substep_adjoint(s._handle, float(dt), tape, self.adj, s._stream()),
                      batch=True)

    def rho_copy_to(self, dst):
        s = self.batch
        _native.check(s._lib.xpbd_batch_save_rho_hat(s._handle, dst.data_ptr(), s._stream()), batch=True)

    def rho_load_from(self, src):
        s = self.batch
        _native.check(s._lib.xpbd_batch_load_rho_hat(s._handle, src.data_ptr(), s._stream()), batch=True)

    def substep_dts(self, frames):
        s = self.batch
        out = []
        for _ in range(frames):
            for d in frame_chunks(s.frame_dt, s.dt):
                out.extend([d / s.substeps_num] * s.substeps_num)
        return out

    def set_state(self, x, v):
        """x, v: (n_verts, 3) of all bodies in body order, each in file order."""
        s = self.batch
        s._x4[s._vert_slot, :3] = x.to(s._x4)
        s._v4[s._vert_slot, :3] = v.to(s._v4)

    def positions(self):
        s = self.batch
        return s._x4[s._vert_slot, :3].clone()


def _check_solver_kwargs(kw):
    """The adjoint reverses the block projection over a fixed number of
    iterations (the library checks the same at every taped substep)."""
    kw.setdefault("block_neohookean_enable", True)
    if not kw["block_neohookean_enable"]:
        raise ValueError("the adjoint supports the block projection only")
    if kw.get("target_rel_residual", 0.0) > 0.0 or kw.get("residual_floor", 0.0) > 0.0:
        raise ValueError("the adjoint needs a fixed iteration count: no target_rel_residual or residual_floor")


def _check_tape_memory(mode):
    if mode not in ("auto", "store", "recompute"):
        raise ValueError("tape_memory must be 'auto', 'store' or 'recompute', not %r" % (mode,))
    return mode


def _n_tets(rest_pose):
    from xpbd_gpu.xpbd_base import load_rest_pose
    return load_rest_pose(rest_pose).n_tets


class _SimulateBatch(_torch().autograd.Function):
    @staticmethod
    def forward(ctx, x0, v0, log_E, nu, sim, frames):
        s = sim.batch
        s.set_tet_materials(log_E.detach(), nu.detach())
        sim.set_state(x0.detach(), v0.detach())
        sim.rho_load_from(sim.initial_rho_hat)
        plan = _plan(sim, frames)
        ctx.sim, ctx.plan, ctx.generation = sim, plan, plan.forward(sim)
        ctx.save_for_backward(log_E, nu)
        return sim.positions()

    @staticmethod
    def backward(ctx, g_out):
        torch = _torch()
        sim = ctx.sim
        log_E, nu = ctx.saved_tensors
        s = sim.batch
        DiffSim.reset_adjoint(sim)
        sim._gx[s._vert_slot, :3] = g_out.to(torch.float32)
        ctx.plan.backward(sim, ctx.generation)
        gx = sim._gx[s._vert_slot, :3].clone()
        gv = sim._gv[s._vert_slot, :3].clone()
        gmu = sim._gmu[s._tet_slot]
        gla = sim._gla[s._tet_slot]
        g_logE, g_nu = _lame_inverse_grads(gmu, gla, log_E, nu)
        if nu.numel() == 1:
            g_nu = g_nu.sum().reshape(nu.shape)
        return (gx.to(g_out.dtype), gv.to(g_out.dtype), g_logE.to(log_E.dtype), g_nu.to(nu.dtype), None, None)


def xpbd_simulate_batch(sim, x0, v0, log_E, nu, frames):
    """Final positions (n_verts, 3) of every body after `frames` frames from
    (x0, v0) with per-tet log E and nu (all bodies' vertices and tets in body
    order); differentiable w.r.t. all four tensors."""
    return _SimulateBatch.apply(x0, v0, log_E, nu, sim, frames)
