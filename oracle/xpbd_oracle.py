"""CPU oracle for the RDC-XPBD substep -- TEST INFRASTRUCTURE ONLY.

A NumPy restatement of the reference solver (RaymondMcGuire/rdc-xpbd-taichi),
vectorised over tets / vertices, in float64 or float32.  Only the tests,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg use it, and
only as the checker; the product (``xpbd_gpu`` + ``libxpbd_gb300.so``) never
imports it.

Parity pin: the fixtures in ``tests/golden/*.npz`` were produced by executing
the reference's own ``xpbd_gpu`` package unmodified under a Taichi-semantics
shim (``tests/golden/make_golden.py``, FP64, sequential atomics).  This oracle
in float64 mode reproduces those fixtures to ~1e-12 (``tests/test_oracle_golden.py``).

Ordering conventions that make float64 results match the shim run:
* scatters are applied with ``np.add.at`` over (tet, corner) pairs in
  tet-major order, which is the sequential order of the reference's
  ``ti.atomic_add`` calls (``neohookean_solver.py:443-451``);
* global reductions (residual, monitoring errors) are summed in float64.

Every function cites the reference file:line it restates.
"""
import numpy as np

EPSILON = 1e-12  # xpbd_gpu/constants.py:3

# xpbd_base.py:7-8 / :79-87 face table
FACE_TABLE = ((0, 2, 1), (0, 3, 2), (0, 1, 3), (1, 2, 3))


def calc_second_lame(E, nu):  # neohookean_solver.py:11-12
    return E / (2.0 * (1.0 + nu))


def calc_first_lame(E, nu):  # neohookean_solver.py:7-8
    return 2.0 * nu / (1.0 - 2.0 * nu) * calc_second_lame(E, nu)


def _dot(a, b):
    return a[..., 0] * b[..., 0] + a[..., 1] * b[..., 1] + a[..., 2] * b[..., 2]


def _cross(a, b):
    return np.stack([a[..., 1] * b[..., 2] - a[..., 2] * b[..., 1],
                     a[..., 2] * b[..., 0] - a[..., 0] * b[..., 2],
                     a[..., 0] * b[..., 1] - a[..., 1] * b[..., 0]], axis=-1)


def _matmul(A, B):
    """(N,3,3) @ (N,3,3) with k summed left to right, like an unrolled 3x3 product."""
    return (A[..., :, 0, None] * B[..., None, 0, :]
            + A[..., :, 1, None] * B[..., None, 1, :]
            + A[..., :, 2, None] * B[..., None, 2, :])


def _det3(x):
    """3x3 determinant by cofactor expansion along the first column."""
    return (x[..., 0, 0] * (x[..., 1, 1] * x[..., 2, 2] - x[..., 2, 1] * x[..., 1, 2])
            - x[..., 1, 0] * (x[..., 0, 1] * x[..., 2, 2] - x[..., 2, 1] * x[..., 0, 2])
            + x[..., 2, 0] * (x[..., 0, 1] * x[..., 1, 2] - x[..., 1, 1] * x[..., 0, 2]))


def _inv3(x):
    """3x3 inverse = adjugate / det (neohookean_solver.py:105-107 ``.inverse()``)."""
    inv_det = 1.0 / _det3(x)
    adj = np.empty_like(x)
    adj[..., 0, 0] = x[..., 1, 1] * x[..., 2, 2] - x[..., 2, 1] * x[..., 1, 2]
    adj[..., 1, 0] = x[..., 1, 2] * x[..., 2, 0] - x[..., 1, 0] * x[..., 2, 2]
    adj[..., 2, 0] = x[..., 1, 0] * x[..., 2, 1] - x[..., 2, 0] * x[..., 1, 1]
    adj[..., 0, 1] = x[..., 0, 2] * x[..., 2, 1] - x[..., 0, 1] * x[..., 2, 2]
    adj[..., 1, 1] = x[..., 0, 0] * x[..., 2, 2] - x[..., 0, 2] * x[..., 2, 0]
    adj[..., 2, 1] = x[..., 2, 0] * x[..., 0, 1] - x[..., 0, 0] * x[..., 2, 1]
    adj[..., 0, 2] = x[..., 0, 1] * x[..., 1, 2] - x[..., 0, 2] * x[..., 1, 1]
    adj[..., 1, 2] = x[..., 1, 0] * x[..., 0, 2] - x[..., 0, 0] * x[..., 1, 2]
    adj[..., 2, 2] = x[..., 0, 0] * x[..., 1, 1] - x[..., 1, 0] * x[..., 0, 1]
    return adj * inv_det[..., None, None]


# ---------------------------------------------------------------------------
# SDFs (xpbd_gpu/sdf.py)
# ---------------------------------------------------------------------------

class OracleSdf:
    """One SDF: kind in {'plane','sphere','cube'}; params as the ref ctor takes them."""

    def __init__(self, kind, fixed=False, **kw):
        self.kind = kind
        self.fixed = bool(fixed)
        self.vel = np.zeros(3)  # sdf.py:9 (zero-initialised field)
        if kind == "plane":  # sdf.py:60-66
            d = np.asarray(kw["dir"], dtype=np.float64)
            self.point = np.asarray(kw["point"], dtype=np.float64)
            self.dir = d / np.sqrt((d * d).sum())
        elif kind == "sphere":  # sdf.py:78-84
            self.center = np.asarray(kw["center"], dtype=np.float64)
            self.radius = float(kw["radius"])
        elif kind == "cube":  # sdf.py:99-105
            self.center = np.asarray(kw["center"], dtype=np.float64)
            self.half_size = np.asarray(kw["size"], dtype=np.float64) * 0.5
        else:
            raise ValueError("unknown SDF kind %r" % kind)

    def dist(self, p, dt):
        if self.kind == "plane":  # sdf.py:68-70
            return _dot(p - self.point.astype(dt), self.dir.astype(dt))
        if self.kind == "sphere":  # sdf.py:86-88
            d = p - self.center.astype(dt)
            return np.sqrt(_dot(d, d)) - dt.type(self.radius)
        d = np.abs(p - self.center.astype(dt)) - self.half_size.astype(dt)  # sdf.py:107-110
        m = np.maximum(d, dt.type(0.0))
        return np.sqrt(_dot(m, m)) + np.minimum(
            np.maximum(d[:, 0], np.maximum(d[:, 1], d[:, 2])), dt.type(0.0))

    def normal(self, p, dt):
        if self.kind == "plane":  # sdf.py:72-74
            return np.broadcast_to(self.dir.astype(dt), p.shape).copy()
        if self.kind == "sphere":  # sdf.py:90-92, Taichi normalized(eps): v / (|v| + eps)
            d = p - self.center.astype(dt)
            inv = dt.type(1.0) / (np.sqrt(_dot(d, d)) + dt.type(EPSILON))
            return d * inv[:, None]
        d = p - self.center.astype(dt)  # sdf.py:112-124: dominant axis of (p - c)
        a = np.abs(d)
        axis = np.zeros(len(p), dtype=np.int64)
        axis = np.where(a[:, 1] > a[:, 0], 1, axis)
        axis = np.where(a[:, 2] > a[np.arange(len(p)), axis], 2, axis)
        n = np.zeros_like(p)
        sel = d[np.arange(len(p)), axis]
        n[np.arange(len(p)), axis] = np.where(sel > 0, 1.0, -1.0)
        return n

    def check(self, pos, vel, dt):
        """sdf.py:14-27 -> (fixed, inside mask, normals)."""
        phi = self.dist(pos, dt)
        neg = phi < 0.0
        n = np.zeros_like(pos)
        n[neg] = self.normal(pos[neg], dt)
        diff_vel = self.vel.astype(dt) - vel
        dotnv = _dot(n, diff_vel)
        inside = neg & ((dotnv > 0.0) | self.fixed)
        return inside, n


# ---------------------------------------------------------------------------
# Solver
# ---------------------------------------------------------------------------

class OracleSolver:
    """Restates XPBDNeoHookeanSolver (neohookean_solver.py:16-587) + XPBDSolverBase
    (xpbd_base.py:11-204).  Constructor arguments mirror the reference's
    (``neohookean_solver.py:18-38``); ``points``/``tets`` replace the mesh path,
    ``total_mass`` mirrors ``xpbd_base.py:36`` and ``dtype`` picks the precision.
    """

    def __init__(self, points, tets, sdf, young_modulus=200000.0, poisson_ratio=0.495,
                 scale=1.0, offset=(0.0, 0.0, 0.0), frame_dt=1e-2, dt=1e-2, substeps_num=20,
                 constraints_iter=5, hydrostatic_relaxation=1.2, deviatoric_relaxation=1.2,
                 cheb_enable=True, cheb_warmup=5, cheb_gamma=0.6666,
                 block_neohookean_enable=False, monitor_convergence=False,
                 total_mass=1.0, gravity=(0.0, -9.8, 0.0), damping=5.0, dtype=np.float64,
                 **_ignored):
        self.dt_ = np.dtype(dtype)
        f = self.dt_.type
        self.constraints_iter = constraints_iter
        self.hydrostatic_relaxation = hydrostatic_relaxation
        self.deviatoric_relaxation = deviatoric_relaxation
        self.lame1 = calc_first_lame(young_modulus, poisson_ratio)   # :43
        self.lame2 = calc_second_lame(young_modulus, poisson_ratio)  # :44
        self.cheb_enable = cheb_enable
        self.cheb_gamma = cheb_gamma
        self.cheb_warmup = cheb_warmup
        self.block_neohookean_enable = block_neohookean_enable
        self.monitor_convergence = monitor_convergence
        self.convergence_history = []
        self.current_frame = 0
        self.current_substep = 0
        self.rho_hat = 0.999          # :65-68
        self.rho_min = 0.00001
        self.rho_max = 0.99999
        self.rho_beta = 0.2
        self.prev_r_hat = None
        self.r_hat_history = []
        self.omega_history = []
        self.time = 0.0
        self.frame_dt = frame_dt
        self.dt = dt
        self.substeps_num = substeps_num
        self.gravity = np.asarray(gravity, dtype=np.float64)
        self.damping = damping
        self.total_mass = total_mass
        sdfs = list(sdf) if isinstance(sdf, (list, tuple)) else [sdf]
        self.sdfs = [s for s in sdfs if s is not None]
        if not self.sdfs:  # xpbd_base.py:66-67
            raise ValueError("At least one SDF object must be provided.")

        self.tets = np.asarray(tets, dtype=np.int64)
        T = len(self.tets)
        # xpbd_base.py:79-87
        self.indices = self.tets[:, np.array(FACE_TABLE)].reshape(-1).astype(np.uint32)
        # initialize (neohookean_solver.py:97-107)
        x = np.asarray(points, dtype=np.float64).astype(self.dt_)
        self.x = x * f(scale) + np.asarray(offset, dtype=np.float64).astype(self.dt_)
        P = self.x[self.tets]
        e1, e2, e3 = P[:, 1] - P[:, 0], P[:, 2] - P[:, 0], P[:, 3] - P[:, 0]
        self.V0 = _dot(_cross(e1, e2), e3) / f(6.0)
        self.inv_Dm = _inv3(np.stack([e1, e2, e3], axis=-1))
        self.lambda_H = np.zeros(T, dtype=self.dt_)
        self.lambda_D = np.zeros(T, dtype=self.dt_)
        V = len(self.x)
        self.v = np.zeros((V, 3), dtype=self.dt_)
        self.pred_x = np.zeros((V, 3), dtype=self.dt_)
        self._compute_lumped_mass()

    # xpbd_base.py:89-137
    def _compute_lumped_mass(self):
        f = self.dt_.type
        vol = self.V0  # same expression as calc_tet_volume on the same x
        m = np.zeros(len(self.x), dtype=self.dt_)
        np.add.at(m, self.tets.reshape(-1), np.repeat(vol * f(0.25), 4))
        total_volume = vol.astype(np.float64).sum()
        mass_scale = f(self.total_mass / total_volume)
        m = m * mass_scale
        self.m = m
        self.inv_m = np.where(m > 0.0, f(1.0) / np.where(m > 0.0, m, f(1.0)), f(0.0)).astype(self.dt_)
        for s in self.sdfs:
            live = self.inv_m > 0.0
            inside, _ = s.check(self.x, self.v, self.dt_)
            self.inv_m[live & s.fixed & inside] = 0.0

    # xpbd_base.py:139-146
    def apply_external_forces(self, dt):
        dt = self.dt_.type(dt)
        live = self.inv_m > 0.0
        self.v[live] += self.gravity.astype(self.dt_) * dt
        self.pred_x = self.x + self.v * dt

    # xpbd_base.py:148-160
    def advance(self, dt, damping):
        f = self.dt_.type
        dt = f(dt)
        fixed = self.inv_m <= 0.0
        self.pred_x[fixed] = self.x[fixed]
        live = ~fixed
        raw_v = (self.pred_x[live] - self.x[live]) / dt
        self.v[live] = raw_v * np.exp(-dt * f(damping))
        self.x[live] = self.pred_x[live]

    # xpbd_base.py:162-178
    def solve_sdf_collision(self, dt):
        for s in self.sdfs:
            live = self.inv_m > 0.0
            inside, n = s.check(self.pred_x, self.v, self.dt_)
            pen = -s.dist(self.pred_x, self.dt_)
            hit = live & inside & (pen > 0.0)
            self.pred_x[hit] += n[hit] * pen[hit][:, None]

    # -- per-tet kinematics shared by the sweeps ---------------------------
    def _F(self, xp):
        P = xp[self.tets]
        Ds = np.stack([P[:, 1] - P[:, 0], P[:, 2] - P[:, 0], P[:, 3] - P[:, 0]], axis=-1)
        return _matmul(Ds, self.inv_Dm)

    def _corner_grads(self, gradF):
        g123 = _matmul(gradF, np.swapaxes(self.inv_Dm, -1, -2))
        g1, g2, g3 = g123[..., :, 0], g123[..., :, 1], g123[..., :, 2]
        g0 = -(g1 + g2 + g3)
        return [g0, g1, g2, g3]

    def _scatter(self, dps, mask=None):
        T = len(self.tets)
        dp = np.stack(dps, axis=1)  # (T,4,3) tet-major, corner order 0..3
        cnt = np.ones((T, 4), dtype=np.uint32)
        if mask is not None:
            dp = dp[mask]
            cnt = cnt[mask]
            idx = self.tets[mask].reshape(-1)
        else:
            idx = self.tets.reshape(-1)
        np.add.at(self.delta_x, idx, dp.reshape(-1, 3))
        np.add.at(self.cons_num, idx, cnt.reshape(-1))

    # neohookean_solver.py:331-356 (vectorised, same branches)
    @staticmethod
    def solve2x2_pivot_lu(A00, A01, A10, A11, b0, b1, eps):
        swap = np.abs(A00) < np.abs(A10)
        A00, A10 = np.where(swap, A10, A00), np.where(swap, A00, A10)
        A01, A11 = np.where(swap, A11, A01), np.where(swap, A01, A11)
        b0, b1 = np.where(swap, b1, b0), np.where(swap, b0, b1)
        ok = ~(np.abs(A00) < eps)
        safe00 = np.where(ok, A00, 1.0)
        m = A10 / safe00
        A11_ = A11 - m * A01
        b1_ = b1 - m * b0
        ok2 = ok & ~(np.abs(A11_) < eps)
        x1 = np.where(ok2, b1_ / np.where(ok2, A11_, 1.0), 0.0)
        x0 = np.where(ok2, (b0 - A01 * x1) / safe00, 0.0)
        return ok2, x0.astype(A00.dtype), x1.astype(A00.dtype)

    # neohookean_solver.py:358-451
    def solve_neohookean_block(self, dt):
        f = self.dt_.type
        dt = f(dt)
        eps = f(EPSILON)
        w = self.inv_m[self.tets]
        F = self._F(self.pred_x)
        C_D = _normsq9(F) - f(3.0)
        C_H = _det3(F) - f(1.0)
        gD = self._corner_grads(F * f(2.0))
        F0, F1, F2 = F[..., :, 0], F[..., :, 1], F[..., :, 2]
        gH = self._corner_grads(np.stack([_cross(F1, F2), _cross(F2, F0), _cross(F0, F1)], axis=-1))
        A11 = (w[:, 0] * _dot(gD[0], gD[0]) + w[:, 1] * _dot(gD[1], gD[1])
               + w[:, 2] * _dot(gD[2], gD[2]) + w[:, 3] * _dot(gD[3], gD[3]))
        A22 = (w[:, 0] * _dot(gH[0], gH[0]) + w[:, 1] * _dot(gH[1], gH[1])
               + w[:, 2] * _dot(gH[2], gH[2]) + w[:, 3] * _dot(gH[3], gH[3]))
        A12 = (w[:, 0] * _dot(gD[0], gH[0]) + w[:, 1] * _dot(gD[1], gH[1])
               + w[:, 2] * _dot(gD[2], gH[2]) + w[:, 3] * _dot(gD[3], gH[3]))
        alpha_D = f(1.0) / (f(self.lame2) * self.V0)
        alpha_H = f(1.0) / (f(self.lame1) * self.V0)
        aD = alpha_D / (dt * dt)
        aH = alpha_H / (dt * dt)
        A11 = A11 + aD
        A22 = A22 + aH
        b1 = -(C_D + aD * self.lambda_D)
        b2 = -(C_H + aH * self.lambda_H)
        ok, dlamD, dlamH = self.solve2x2_pivot_lu(A11, A12, A12, A22, b1, b2, eps)
        # :425-432 diagonal fallback
        fbD = np.where(np.abs(A11) > eps, b1 / np.where(np.abs(A11) > eps, A11, f(1.0)), f(0.0))
        fbH = np.where(np.abs(A22) > eps, b2 / np.where(np.abs(A22) > eps, A22, f(1.0)), f(0.0))
        dlamD = np.where(ok, dlamD, fbD).astype(self.dt_)
        dlamH = np.where(ok, dlamH, fbH).astype(self.dt_)
        self.lambda_D += dlamD
        self.lambda_H += dlamH
        dps = [w[:, i, None] * (gD[i] * dlamD[:, None] + gH[i] * dlamH[:, None]) for i in range(4)]
        self._scatter(dps)

    def _split_update(self, C, g, lam, alpha, relax, dt):
        f = self.dt_.type
        w = self.inv_m[self.tets]
        w_sum = w[:, 0] * _dot(g[0], g[0])
        w_sum = w_sum + w[:, 1] * _dot(g[1], g[1])
        w_sum = w_sum + w[:, 2] * _dot(g[2], g[2])
        w_sum = w_sum + w[:, 3] * _dot(g[3], g[3])
        act = w_sum > f(EPSILON)
        alpha_tilde = alpha / (dt ** 2)
        d_lambda = -(C + alpha_tilde * lam) / (w_sum + alpha_tilde)
        d_lambda = d_lambda * f(relax)
        d_lambda = np.where(act, d_lambda, f(0.0)).astype(self.dt_)
        lam += d_lambda
        dps = [d_lambda[:, None] * w[:, i, None] * g[i] for i in range(4)]
        self._scatter(dps, mask=act)

    # neohookean_solver.py:144-194
    def solve_deviatoric(self, dt):
        f = self.dt_.type
        dt = f(dt)
        F = self._F(self.pred_x)
        C = _normsq9(F) - f(3.0)
        g = self._corner_grads(f(2.0) * F)
        alpha_D = f(1.0) / (f(self.lame2) * self.V0)
        self._split_update(C, g, self.lambda_D, alpha_D, self.deviatoric_relaxation, dt)

    # neohookean_solver.py:196-254
    def solve_hydrostatic(self, dt):
        f = self.dt_.type
        dt = f(dt)
        F = self._F(self.pred_x)
        C = _det3(F) - f(1.0)
        F0, F1, F2 = F[..., :, 0], F[..., :, 1], F[..., :, 2]
        g = self._corner_grads(np.stack([_cross(F1, F2), _cross(F2, F0), _cross(F0, F1)], axis=-1))
        alpha_H = f(1.0) / (f(self.lame1) * self.V0)
        self._split_update(C, g, self.lambda_H, alpha_H, self.hydrostatic_relaxation, dt)

    # neohookean_solver.py:298-329 (sum carried in float64)
    def compute_xpbd_residual(self, dt):
        f = self.dt_.type
        dt = f(dt)
        F = self._F(self.pred_x)
        C_D = _normsq9(F) - f(3.0)
        C_H = _det3(F) - f(1.0)
        alpha_D = f(1.0) / (f(self.lame2) * self.V0)
        alpha_H = f(1.0) / (f(self.lame1) * self.V0)
        aD = alpha_D / (dt * dt)
        aH = alpha_H / (dt * dt)
        rD = C_D + aD * self.lambda_D
        rH = C_H + aH * self.lambda_H
        r = np.sqrt(rD * rD + rH * rH)
        return float(r.astype(np.float64).sum()), len(r)

    # neohookean_solver.py:256-296
    def compute_errors(self):
        F = self._F(self.pred_x)
        f = self.dt_.type
        h = np.abs(_det3(F) - f(1.0)).astype(np.float64).sum()
        d = np.abs(_normsq9(F) - f(3.0)).astype(np.float64).sum()
        n = len(self.tets)
        return (h / n, d / n) if n > 0 else (0.0, 0.0)

    # neohookean_solver.py:453-560
    def solve_step(self, dt):
        f = self.dt_.type
        self.lambda_H[:] = 0.0
        self.lambda_D[:] = 0.0
        self.prev_r_hat = None
        self.solve_sdf_collision(dt)
        use_cheb = self.cheb_enable
        omega = 1.0
        if use_cheb:
            pred_x_prev = self.pred_x.copy()
        for it in range(self.constraints_iter):
            if use_cheb:
                pred_x_curr = self.pred_x.copy()
            # pre_solve :109-113
            self.delta_x = np.zeros_like(self.pred_x)
            self.cons_num = np.zeros(len(self.pred_x), dtype=np.uint32)
            if self.block_neohookean_enable:
                self.solve_neohookean_block(dt)
            else:
                self.solve_hydrostatic(dt)
                self.solve_deviatoric(dt)
            # post_solve :115-119
            c = self.cons_num > 0
            self.pred_x[c] += self.delta_x[c] / self.cons_num[c, None].astype(self.dt_)
            if use_cheb:
                s, cnt = self.compute_xpbd_residual(dt)
                r_hat = s / cnt if cnt > 0 else 0.0
                self.r_hat_history.append(r_hat)
                if self.prev_r_hat is not None and self.prev_r_hat > EPSILON:
                    rho_inst = r_hat / (self.prev_r_hat + EPSILON)
                    rho_inst = max(self.rho_min, min(self.rho_max, float(rho_inst)))
                    self.rho_hat = (1.0 - self.rho_beta) * self.rho_hat + self.rho_beta * rho_inst
                self.prev_r_hat = r_hat
            if self.monitor_convergence:
                he, de = self.compute_errors()
                self.convergence_history.append(dict(
                    frame=self.current_frame, substep=self.current_substep, iter=it,
                    iter_compute_time_sec=0.0, hydro_error=he, dev_error=de))
            if use_cheb:
                rho = float(self.rho_hat)
                rho2 = rho * rho
                if it < self.cheb_warmup:
                    omega = 1.0
                elif it == self.cheb_warmup:
                    omega = 2.0 / (2.0 - rho2)
                else:
                    omega = 4.0 / (4.0 - rho2 * omega)
                self.omega_history.append(omega)
                # _chebyshev_update :131-137 (omega and gamma are f32 kernel constants)
                w_ = f(omega)
                g_ = f(self.cheb_gamma)
                x_new = g_ * (self.pred_x - pred_x_curr) + pred_x_curr
                self.pred_x = pred_x_prev + w_ * (x_new - pred_x_prev)
                pred_x_prev = pred_x_curr  # _rotate_prev_with_save :139-142

    # neohookean_solver.py:562-587
    def solve(self):
        frame_time_left = self.frame_dt
        self.current_substep = 0
        while frame_time_left > 0.0:
            dt0 = min(self.dt, frame_time_left)
            frame_time_left -= dt0
            sub_dt = dt0 / self.substeps_num
            for substep in range(self.substeps_num):
                self.current_substep = substep
                self.apply_external_forces(sub_dt)
                self.solve_step(sub_dt)
                self.advance(sub_dt, self.damping)
            self.time += dt0
        self.current_frame += 1


def _normsq9(F):
    """Frobenius norm squared, entries summed row-major left to right (``norm_sqr``)."""
    s = F[..., 0, 0] * F[..., 0, 0]
    for i in range(3):
        for j in range(3):
            if i == 0 and j == 0:
                continue
            s = s + F[..., i, j] * F[..., i, j]
    return s


def frame_chunks(frame_dt, dt):
    """The (dt0) sequence of one frame, computed in float64 like neohookean_solver.py:563-568."""
    out = []
    left = frame_dt
    while left > 0.0:
        d = min(dt, left)
        left -= d
        out.append(d)
    return out
