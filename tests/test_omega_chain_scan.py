"""The omega chain's table (the adjoint's per-iteration coefficients of the
rho_hat recurrence, neohookean_solver.py:495-504, :537-546) is built on the GPU
by a warp scan of affine maps, 32 iterations at a time (ka_chain in
csrc/xpbd_adjoint.cuh).  This restates that scan in NumPy and checks it
against the sequential recurrence: rho_hat_j = a_j rho_hat_{j-1} + b_j, with
(a_j, b_j) = (1 - beta, beta ri_j) where rho_hat is updated and (1, 0) where it
is not, composed by an inclusive Hillis-Steele scan across the lanes and
carried from one group of 32 to the next."""
import numpy as np
import pytest


def _sequential(r, rho_in, beta, rmin, rmax):
    rho, prev, out = rho_in, 0.0, []
    for j, rj in enumerate(r):
        if j > 0 and prev > 1e-12:
            ratio = rj / (prev + 1e-12)
            rho = (1.0 - beta) * rho + beta * min(rmax, max(rmin, ratio))
        out.append(rho)
        prev = rj
    return np.array(out)


def _warp_scan(r, rho_in, beta, rmin, rmax, width=32):
    K = len(r)
    out = np.zeros(K)
    carry = rho_in
    for j0 in range(0, K, width):
        lanes = np.arange(width)
        j = j0 + lanes
        inn = j < K
        a = np.ones(width)
        b = np.zeros(width)
        for l in lanes:
            if inn[l] and j[l] > 0 and r[j[l] - 1] > 1e-12:
                ratio = r[j[l]] / (r[j[l] - 1] + 1e-12)
                a[l], b[l] = 1.0 - beta, beta * min(rmax, max(rmin, ratio))
        off = 1
        while off < width:  # every lane reads its neighbour's value from before the step
            pa, pb = np.roll(a, off), np.roll(b, off)
            upd = lanes >= off
            b = np.where(upd, a * pb + b, b)
            a = np.where(upd, a * pa, a)
            off <<= 1
        rho = a * carry + b
        out[j[inn]] = rho[inn]
        carry = rho[width - 1]
    return out


@pytest.mark.parametrize("K", [1, 8, 31, 32, 33, 40, 200])
def test_scan_equals_the_sequential_recurrence(K):
    rng = np.random.default_rng(K)
    # a decreasing residual curve with plateaus, a clamped ratio (a jump up) and
    # a zero stretch (no update while r_hat_{j-1} <= 1e-12)
    r = np.cumprod(rng.uniform(0.7, 1.05, size=K)) * 1e-2
    if K > 10:
        r[5] = 3.0 * r[4]
        r[7:9] = 0.0
    for rho_in in (0.999, 0.5):
        want = _sequential(r, rho_in, 0.2, 1e-5, 0.99999)
        got = _warp_scan(r, rho_in, 0.2, 1e-5, 0.99999)
        np.testing.assert_allclose(got, want, rtol=1e-13, atol=0)
