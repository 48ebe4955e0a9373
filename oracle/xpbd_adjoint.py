"""Float64 adjoint of the RDC-XPBD substep -- TEST INFRASTRUCTURE ONLY.

A NumPy restatement of the block Neo-Hookean substep (neohookean_solver.py:
453-587, xpbd_base.py:139-178, sdf.py) with per-tet materials, recorded on a
tape, and its hand-written reverse pass.  It is the checker of the GPU
adjoint kernels (``xpbd_substep_adjoint``) and is itself checked against
central finite differences in ``tests/test_adjoint_oracle.py``.

Differentiation conventions (the GPU adjoint follows the same):
* The Chebyshev factor omega: by default a stop-gradient, a control heuristic
  driven by the residual ratio (neohookean_solver.py:495-546); finite
  differences that check such gradients replay the recorded omega schedule.
  With ``omega_grad=True`` the adjoint also runs backwards through omega:
  omega_k depends on rho_hat_k (and omega_{k-1}), rho_hat_k on the clamped
  ratio r_hat_k / r_hat_{k-1} (and rho_hat_{k-1}, which persists across
  substeps), and r_hat_k on the post-Jacobi positions, the multipliers after
  the iteration and the compliances (compute_xpbd_residual, :298-329).  The
  clamp of the ratio and the warm-up are piecewise constant.
* The active-contact sets (inside a SDF) and the 2x2 pivot branch are
  piecewise constant; the derivative is the derivative of A^-1 b.
* Materials enter as per-tet inverse Lame parameters inv_mu = 1/mu,
  inv_la = 1/lambda (time-scaled compliance aD = inv_mu / (V0 dt^2)).
"""
import numpy as np

from oracle.xpbd_oracle import EPSILON, OracleSdf, _cross, _det3, _dot, _inv3, calc_first_lame, calc_second_lame


def lame_inverse(log_E, nu):
    """Per-tet (1/mu, 1/lambda) from log E and nu (neohookean_solver.py:7-12)."""
    E = np.exp(np.asarray(log_E, dtype=np.float64))
    nu = np.broadcast_to(np.asarray(nu, dtype=np.float64), E.shape)
    return 1.0 / calc_second_lame(E, nu), 1.0 / calc_first_lame(E, nu)


def lame_inverse_grad(log_E, nu, g_inv_mu, g_inv_la):
    """Chain rule from d/d(1/mu), d/d(1/lambda) to d/d(log E), d/d(nu)."""
    E = np.exp(np.asarray(log_E, dtype=np.float64))
    nu = np.broadcast_to(np.asarray(nu, dtype=np.float64), E.shape)
    inv_mu = 2.0 * (1.0 + nu) / E
    inv_la = (1.0 + nu) * (1.0 - 2.0 * nu) / (E * nu)
    g_logE = -(g_inv_mu * inv_mu + g_inv_la * inv_la)
    g_nu = g_inv_mu * 2.0 / E + g_inv_la * (-1.0 - 2.0 * nu * nu) / (nu * nu * E)
    return g_logE, g_nu


def _cof(F):
    F0, F1, F2 = F[..., :, 0], F[..., :, 1], F[..., :, 2]
    return np.stack([_cross(F1, F2), _cross(F2, F0), _cross(F0, F1)], axis=-1)


def _corner(G, Dm):
    g = G @ np.swapaxes(Dm, -1, -2)  # g[:, r, c] = sum_k G[r, k] Dm[c, k]
    g1, g2, g3 = g[..., :, 0], g[..., :, 1], g[..., :, 2]
    return np.stack([-(g1 + g2 + g3), g1, g2, g3], axis=1)  # (T, 4, 3)


def project_forward(P, Dm, w, lam, aD, aH):
    """Block projection of every tet (neohookean_solver.py:365-451): returns dp
    (T,4,3), dlam (T,2) and the intermediates of the reverse pass."""
    E = np.stack([P[:, 1] - P[:, 0], P[:, 2] - P[:, 0], P[:, 3] - P[:, 0]], axis=-1)
    F = E @ Dm
    CD = (F * F).sum((1, 2)) - 3.0
    CH = _det3(F) - 1.0
    H = _cof(F)
    gD = _corner(2.0 * F, Dm)
    gH = _corner(H, Dm)
    A11 = (w[:, :, None] * gD * gD).sum((1, 2)) + aD
    A22 = (w[:, :, None] * gH * gH).sum((1, 2)) + aH
    A12 = (w[:, :, None] * gD * gH).sum((1, 2))
    b1 = -(CD + aD * lam[:, 0])
    b2 = -(CH + aH * lam[:, 1])
    det = A11 * A22 - A12 * A12
    dD = (A22 * b1 - A12 * b2) / det
    dH = (A11 * b2 - A12 * b1) / det
    dp = w[:, :, None] * (gD * dD[:, None, None] + gH * dH[:, None, None])
    cache = dict(F=F, H=H, gD=gD, gH=gH, A11=A11, A22=A22, A12=A12, det=det, dD=dD, dH=dH)
    return dp, np.stack([dD, dH], axis=1), cache


def project_adjoint(P, Dm, w, lam, aD, aH, dp_bar, dlam_bar, cache):
    """Reverse of project_forward.  dlam_bar is the adjoint of the multiplier
    increment.  Returns (P_bar (T,4,3), lam_bar (T,2), aD_bar (T), aH_bar (T))."""
    F, H, gD, gH = cache["F"], cache["H"], cache["gD"], cache["gH"]
    A11, A22, A12, det, dD, dH = (cache[k] for k in ("A11", "A22", "A12", "det", "dD", "dH"))
    wb = w[:, :, None]
    dD_bar = dlam_bar[:, 0] + (wb * gD * dp_bar).sum((1, 2))
    dH_bar = dlam_bar[:, 1] + (wb * gH * dp_bar).sum((1, 2))
    gD_bar = wb * dp_bar * dD[:, None, None]
    gH_bar = wb * dp_bar * dH[:, None, None]
    # d = A^-1 b with A symmetric: b_bar = A^-1 d_bar, A_bar = -b_bar d^T
    bb1 = (A22 * dD_bar - A12 * dH_bar) / det
    bb2 = (A11 * dH_bar - A12 * dD_bar) / det
    A11_bar = -bb1 * dD
    A22_bar = -bb2 * dH
    A12_bar = -(bb1 * dH + bb2 * dD)
    CD_bar = -bb1
    CH_bar = -bb2
    lam_bar = np.stack([-aD * bb1, -aH * bb2], axis=1)
    aD_bar = -lam[:, 0] * bb1 + A11_bar
    aH_bar = -lam[:, 1] * bb2 + A22_bar
    gD_bar = gD_bar + wb * (2.0 * A11_bar[:, None, None] * gD + A12_bar[:, None, None] * gH)
    gH_bar = gH_bar + wb * (2.0 * A22_bar[:, None, None] * gH + A12_bar[:, None, None] * gD)
    # corners g_{c+1} = (G Dm^T)[:, :, c], g_0 = -sum: G_bar = Gt @ Dm
    GtD = np.stack([gD_bar[:, c + 1] - gD_bar[:, 0] for c in range(3)], axis=-1)
    GtH = np.stack([gH_bar[:, c + 1] - gH_bar[:, 0] for c in range(3)], axis=-1)
    GD_bar = GtD @ Dm
    H_bar = GtH @ Dm
    F_bar = 2.0 * GD_bar + 2.0 * CD_bar[:, None, None] * F + CH_bar[:, None, None] * H
    F0, F1, F2 = F[..., :, 0], F[..., :, 1], F[..., :, 2]
    H0b, H1b, H2b = H_bar[..., :, 0], H_bar[..., :, 1], H_bar[..., :, 2]
    Fb0 = _cross(H1b, F2) + _cross(F1, H2b)
    Fb1 = _cross(F2, H0b) + _cross(H2b, F0)
    Fb2 = _cross(H0b, F1) + _cross(F0, H1b)
    F_bar = F_bar + np.stack([Fb0, Fb1, Fb2], axis=-1)
    E_bar = F_bar @ np.swapaxes(Dm, -1, -2)
    P_bar = np.zeros_like(P)
    for c in range(3):
        P_bar[:, c + 1] += E_bar[:, :, c]
        P_bar[:, 0] -= E_bar[:, :, c]
    return P_bar, lam_bar, aD_bar, aH_bar


def _sdf_step(s, q, vel):
    """One SDF of the list (sdf.py:14-27 + xpbd_base.py:162-174) on live vertices;
    returns the projected positions and the active mask."""
    dt = np.dtype(np.float64)
    inside, n = s.check(q, vel, dt)
    pen = -s.dist(q, dt)
    act = inside & (pen > 0.0)
    out = q.copy()
    out[act] += n[act] * pen[act][:, None]
    return out, act


def _sdf_adjoint(s, q, act, qbar):
    """q_bar = J^T q_bar' for the vertices projected by SDF s at positions q."""
    out = qbar.copy()
    if not act.any():
        return out
    qa, gb = q[act], qbar[act]
    if s.kind == "plane":
        n = s.dir
        out[act] = gb - n[None, :] * (gb @ n)[:, None]
    elif s.kind == "sphere":
        d = qa - s.center
        sl = np.sqrt(_dot(d, d))
        u = d / sl[:, None]
        k = (s.radius + EPSILON) / (sl + EPSILON)
        c = sl / (sl + EPSILON)
        out[act] = k[:, None] * (gb - c[:, None] * u * _dot(u, gb)[:, None])
    else:  # cube: J = I - n grad(phi)^T, n: dominant axis of (q - c), grad: argmax of |q - c| - h
        d = qa - s.center
        a = np.abs(d)
        nax = np.zeros(len(d), dtype=np.int64)
        nax = np.where(a[:, 1] > a[:, 0], 1, nax)
        nax = np.where(a[:, 2] > a[np.arange(len(d)), nax], 2, nax)
        dd = a - s.half_size
        gax = np.argmax(dd, axis=1)  # first maximum, like max(d.x, max(d.y, d.z))
        r = np.arange(len(d))
        sn = np.where(d[r, nax] > 0, 1.0, -1.0)
        sg = np.where(d[r, gax] > 0, 1.0, -1.0)
        res = gb.copy()
        res[r, gax] -= sg * sn * gb[r, nax]
        out[act] = res
    return out


class DiffOracle:
    """Differentiable float64 restatement of one body (block mode, Chebyshev
    optional), with per-tet inverse Lame parameters."""

    def __init__(self, points, tets, sdfs, inv_mu, inv_la, frame_dt, dt, substeps_num, constraints_iter,
                 cheb_enable=True, cheb_warmup=5, cheb_gamma=0.6666, total_mass=1.0, damping=5.0,
                 gravity=(0.0, -9.8, 0.0), omega_grad=False):
        self.omega_grad = bool(omega_grad)
        self.tets = np.asarray(tets, dtype=np.int64)
        self.x0 = np.asarray(points, dtype=np.float64).copy()
        P = self.x0[self.tets]
        e1, e2, e3 = P[:, 1] - P[:, 0], P[:, 2] - P[:, 0], P[:, 3] - P[:, 0]
        self.V0 = _dot(_cross(e1, e2), e3) / 6.0
        self.Dm = _inv3(np.stack([e1, e2, e3], axis=-1))
        m = np.zeros(len(self.x0))
        np.add.at(m, self.tets.reshape(-1), np.repeat(self.V0 * 0.25, 4))
        m *= total_mass / self.V0.sum()
        self.inv_m = np.where(m > 0, 1.0 / np.where(m > 0, m, 1.0), 0.0)
        self.sdfs = list(sdfs)
        for s in self.sdfs:
            live = self.inv_m > 0.0
            inside, _ = s.check(self.x0, np.zeros_like(self.x0), np.dtype(np.float64))
            if s.fixed:
                self.inv_m[live & inside] = 0.0
        self.cnt = np.bincount(self.tets.reshape(-1), minlength=len(self.x0)).astype(np.float64)
        self.inv_mu = np.broadcast_to(np.asarray(inv_mu, dtype=np.float64), self.V0.shape).copy()
        self.inv_la = np.broadcast_to(np.asarray(inv_la, dtype=np.float64), self.V0.shape).copy()
        self.frame_dt, self.dt, self.substeps, self.K = frame_dt, dt, substeps_num, constraints_iter
        self.cheb, self.warmup, self.gamma = cheb_enable, cheb_warmup, cheb_gamma
        self.damping = damping
        self.gravity = np.asarray(gravity, dtype=np.float64)
        self.rho_hat = 0.999

    def _substep_dts(self, frames):
        out = []
        for _ in range(frames):
            left = self.frame_dt
            while left > 0.0:
                d = min(self.dt, left)
                left -= d
                out.extend([d / self.substeps] * self.substeps)
        return out

    def _residual(self, xp, lam, aD, aH):
        P = xp[self.tets]
        E = np.stack([P[:, 1] - P[:, 0], P[:, 2] - P[:, 0], P[:, 3] - P[:, 0]], axis=-1)
        F = E @ self.Dm
        rD = (F * F).sum((1, 2)) - 3.0 + aD * lam[:, 0]
        rH = _det3(F) - 1.0 + aH * lam[:, 1]
        return float(np.sqrt(rD * rD + rH * rH).sum() / len(F))

    def substep(self, x, v, sdt, omegas=None, tape=None):
        """One substep; `omegas` replays a recorded omega list (else computed and
        returned); `tape` (dict) receives what the reverse pass needs."""
        live = self.inv_m > 0.0
        w = self.inv_m[self.tets]
        aD = self.inv_mu / (self.V0 * sdt * sdt)
        aH = self.inv_la / (self.V0 * sdt * sdt)
        v1 = v.copy()
        v1[live] += self.gravity * sdt
        q = x + v1 * sdt
        sdf_q, sdf_act = [], []
        for s in self.sdfs:
            nq, act = _sdf_step(s, q, v1)
            act &= live
            nq[~live] = q[~live]
            sdf_q.append(q)
            sdf_act.append(act)
            q = nq
        xt = q
        yprev = xt.copy()
        lam = np.zeros((len(self.tets), 2))
        xs, lams, oms = [xt.copy()], [], []
        prev, omega = None, 1.0
        # the omega chain: r_hat_k, rho_hat_k, whether rho_hat was updated and the
        # ratio clamped at iteration k, and the post-Jacobi positions
        chain = dict(rho_in=self.rho_hat, r=[], rho=[], upd=[], clamped=[], post=[], lam_next=[])
        for it in range(self.K):
            lams.append(lam.copy())
            dp, dlam, _ = project_forward(xt[self.tets], self.Dm, w, lam, aD, aH)
            lam = lam + dlam
            dx = np.zeros_like(xt)
            np.add.at(dx, self.tets.reshape(-1), dp.reshape(-1, 3))
            post = xt + dx / self.cnt[:, None]
            if self.cheb:
                if omegas is None:
                    r = self._residual(post, lam, aD, aH)
                    upd = prev is not None and prev > EPSILON
                    clamped = False
                    if upd:
                        ratio = r / (prev + EPSILON)
                        ri = max(1e-5, min(0.99999, ratio))
                        clamped = ri != ratio
                        self.rho_hat = 0.8 * self.rho_hat + 0.2 * ri
                    prev = r
                    if tape is not None:
                        chain["r"].append(r)
                        chain["rho"].append(self.rho_hat)
                        chain["upd"].append(upd)
                        chain["clamped"].append(clamped)
                        chain["post"].append(post.copy())
                        chain["lam_next"].append(lam.copy())
                    r2 = self.rho_hat ** 2
                    omega = 1.0 if it < self.warmup else (2.0 / (2.0 - r2) if it == self.warmup
                                                          else 4.0 / (4.0 - r2 * omega))
                else:
                    omega = omegas[it]
                oms.append(omega)
                xn = self.gamma * (post - xt) + xt
                nxt = yprev + omega * (xn - yprev)
                yprev = xt
                xt = nxt
            else:
                xt = post
            xs.append(xt.copy())
        e = np.exp(-sdt * self.damping)
        xo, vo = x.copy(), v1.copy()
        vo[live] = (xt[live] - x[live]) / sdt * e
        xo[live] = xt[live]
        if tape is not None:
            tape.update(x=x.copy(), v=v.copy(), v1=v1, sdf_q=sdf_q, sdf_act=sdf_act, xs=xs, lams=lams, oms=oms,
                        aD=aD, aH=aH, sdt=sdt, chain=chain)
        return xo, vo, oms

    def run(self, x, v, frames, omegas=None, record=False):
        dts = self._substep_dts(frames)
        tapes, all_om = [], []
        for k, sdt in enumerate(dts):
            tape = {} if record else None
            x, v, om = self.substep(x, v, sdt, None if omegas is None else omegas[k], tape)
            all_om.append(om)
            if record:
                tapes.append(tape)
        return x, v, all_om, tapes

    def substep_adjoint(self, tape, xbar, vbar):
        """Reverse of one substep: (xbar, vbar) at its end -> at its start, plus the
        per-tet adjoints of inv_mu and inv_la."""
        live = self.inv_m > 0.0
        w = self.inv_m[self.tets]
        sdt = tape["sdt"]
        e = np.exp(-sdt * self.damping)
        # advance (xpbd_base.py:148-160)
        xt_bar = np.zeros_like(xbar)
        xt_bar[live] = xbar[live] + vbar[live] * (e / sdt)
        x_bar = np.where(live[:, None], -vbar * (e / sdt), xbar)
        v1_bar = np.where(live[:, None], 0.0, vbar)
        g_mu = np.zeros(len(self.tets))
        g_la = np.zeros(len(self.tets))
        yprev_bar_next = np.zeros_like(xbar)
        chain = tape.get("chain")
        through_omega = self.omega_grad and self.cheb and chain is not None and len(chain["r"]) == self.K
        om_carry = r_carry = 0.0  # adjoints of omega_{k} and r_hat_{k} from iteration k + 1
        for it in reversed(range(self.K)):
            xt = tape["xs"][it]
            lam = tape["lams"][it]
            lam_next_bar = tape.setdefault("_lam_bar", np.zeros_like(lam))
            if self.cheb:
                om = tape["oms"][it]
                post_bar = om * self.gamma * xt_bar
                if through_omega:
                    post_bar = post_bar + self._omega_chain(tape, it, xt_bar, om_carry, r_carry, lam_next_bar,
                                                            g_mu, g_la, sdt)
                    om_carry, r_carry = self._carry
                cur_bar = om * (1.0 - self.gamma) * xt_bar + post_bar + yprev_bar_next
                yprev_bar = (1.0 - om) * xt_bar
            else:
                post_bar = xt_bar
                cur_bar = post_bar.copy()
                yprev_bar = np.zeros_like(xt_bar)
            dx_bar = post_bar / self.cnt[:, None]
            dp_bar = dx_bar[self.tets]
            P = xt[self.tets]
            _, _, cache = project_forward(P, self.Dm, w, lam, tape["aD"], tape["aH"])
            # lambda_{k+1} = lambda_k + dlam: the adjoint of lambda_{k+1} flows to both
            P_bar, lam_bar, aD_bar, aH_bar = project_adjoint(P, self.Dm, w, lam, tape["aD"], tape["aH"], dp_bar,
                                                             lam_next_bar, cache)
            tape["_lam_bar"] = lam_next_bar + lam_bar
            np.add.at(cur_bar, self.tets.reshape(-1), P_bar.reshape(-1, 3))
            g_mu += aD_bar / (self.V0 * sdt * sdt)
            g_la += aH_bar / (self.V0 * sdt * sdt)
            xt_bar = cur_bar
            if it == 0:
                xt_bar = xt_bar + yprev_bar  # y_prev of iteration 0 is x~_0
            yprev_bar_next = yprev_bar
        tape.pop("_lam_bar", None)
        # SDF list in reverse (fixed vertices pass through)
        qbar = xt_bar
        for s, q, act in reversed(list(zip(self.sdfs, tape["sdf_q"], tape["sdf_act"]))):
            qbar = _sdf_adjoint(s, q, act, qbar)
        # predict (xpbd_base.py:139-146)
        x_bar = x_bar + qbar
        v1_bar = v1_bar + qbar * sdt
        return x_bar, v1_bar, g_mu, g_la

    def _omega_chain(self, tape, k, xt_bar, om_carry, r_carry, lam_next_bar, g_mu, g_la, sdt):
        """Iteration k of the reverse pass through omega (omega_grad): from the
        adjoint of x~_{k+1} to that of omega_k, rho_hat_k and r_hat_k, and from
        r_hat_k (the residual at the post-Jacobi positions with lambda_{k+1},
        neohookean_solver.py:298-329) to the post-Jacobi positions (returned),
        the multipliers after the iteration (added to lam_next_bar) and the
        compliances (added to g_mu, g_la).  self._rho_bar carries the adjoint of
        rho_hat backwards; self._carry receives the adjoints of omega_{k-1} and
        r_hat_{k-1} that iteration k contributes."""
        ch = tape["chain"]
        xs, oms = tape["xs"], tape["oms"]
        W = self.warmup
        om = oms[k]
        y = xs[k - 1] if k > 0 else xs[0]
        wb = float((xt_bar * (xs[k + 1] - y)).sum()) / om + om_carry  # x~_{k+1} - y = om (xn - y)
        rho = ch["rho"][k]
        om_prev = oms[k - 1] if k > 0 else 1.0
        next_om_carry = 0.0
        if k == W:
            self._rho_bar += wb * 4.0 * rho / (2.0 - rho * rho) ** 2
        elif k > W:
            den = 4.0 - rho * rho * om_prev
            self._rho_bar += wb * 8.0 * rho * om_prev / (den * den)
            next_om_carry = wb * 4.0 * rho * rho / (den * den)
        r_bar = r_carry
        next_r_carry = 0.0
        if ch["upd"][k]:
            ri_bar = 0.2 * self._rho_bar
            self._rho_bar *= 0.8
            if not ch["clamped"][k]:
                d = ch["r"][k - 1] + EPSILON
                r_bar += ri_bar / d
                next_r_carry = -ri_bar * ch["r"][k] / (d * d)
        self._carry = (next_om_carry, next_r_carry)
        if r_bar == 0.0:
            return np.zeros_like(xt_bar)
        # r_hat = (1/T) sum_t sqrt(rD^2 + rH^2), rD = C_D + aD lambda_D, rH = C_H + aH lambda_H
        post, lamn = ch["post"][k], ch["lam_next"][k]
        aD, aH = tape["aD"], tape["aH"]
        P = post[self.tets]
        E = np.stack([P[:, 1] - P[:, 0], P[:, 2] - P[:, 0], P[:, 3] - P[:, 0]], axis=-1)
        F = E @ self.Dm
        rD = (F * F).sum((1, 2)) - 3.0 + aD * lamn[:, 0]
        rH = _det3(F) - 1.0 + aH * lamn[:, 1]
        sq = np.sqrt(rD * rD + rH * rH)
        sb = r_bar / len(F)
        nz = sq > 0.0
        rDb = np.where(nz, sb * rD / np.where(nz, sq, 1.0), 0.0)
        rHb = np.where(nz, sb * rH / np.where(nz, sq, 1.0), 0.0)
        Fb = rDb[:, None, None] * 2.0 * F + rHb[:, None, None] * _cof(F)
        Pb = _corner(Fb, self.Dm)
        out = np.zeros_like(xt_bar)
        np.add.at(out, self.tets.reshape(-1), Pb.reshape(-1, 3))
        lam_next_bar[:, 0] += rDb * aD
        lam_next_bar[:, 1] += rHb * aH
        g_mu += rDb * lamn[:, 0] / (self.V0 * sdt * sdt)
        g_la += rHb * lamn[:, 1] / (self.V0 * sdt * sdt)
        return out

    def gradient(self, x, v, frames, xbar_final, vbar_final=None):
        """Adjoint of `frames` frames from (x, v): returns (omegas, x_bar, v_bar,
        g_inv_mu, g_inv_la) for the loss whose gradient w.r.t. the final
        positions is xbar_final."""
        xe, ve, oms, tapes = self.run(x, v, frames, record=True)
        xb = np.asarray(xbar_final, dtype=np.float64).copy()
        vb = np.zeros_like(xb) if vbar_final is None else np.asarray(vbar_final, dtype=np.float64).copy()
        gm = np.zeros(len(self.tets))
        gl = np.zeros(len(self.tets))
        self._rho_bar = 0.0  # the loss does not read rho_hat; it flows back through omega
        for tape in reversed(tapes):
            xb, vb, a, b = self.substep_adjoint(tape, xb, vb)
            gm += a
            gl += b
        return oms, xb, vb, gm, gl, xe
