"""Host logic of the differentiable plans that needs no GPU: the tape-memory
policy and the size of a stored tape."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "rdc-xpbd-taichi_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)


class _Sim:
    """The attributes _Tapes.nbytes reads from a DiffSim / BatchedDiffSim."""

    def __init__(self, V, T, K, n_bodies, omega_grad):
        self.V, self.T, self.K, self.n_rho, self.omega_grad = V, T, K, n_bodies, omega_grad


def test_tape_memory_modes_are_checked():
    from xpbd_gpu.differentiable import _check_tape_memory
    for m in ("auto", "store", "recompute"):
        assert _check_tape_memory(m) == m
    with pytest.raises(ValueError):
        _check_tape_memory("keep")


@pytest.mark.parametrize("omega_grad", [True, False])
def test_stored_tape_size(omega_grad):
    from xpbd_gpu.differentiable import _Tapes
    V, T, K, nb, n = 1000, 5000, 20, 3, 7
    s = _Sim(V, T, K, nb, omega_grad)
    per = 16 * (K + 1) * V + 16 * 2 * V + 8 * (K + 1 if omega_grad else K) * T + 32 * nb * K
    if omega_grad:
        per += 16 * K * V + 8 * nb
    assert _Tapes.nbytes(s, n) == n * per
    # the C5 workload: 64 bodies, 1.75 M tets, 20 iterations, 150 substeps -- about 80 GB
    big = _Tapes.nbytes(_Sim(348087, 1753152, 20, 64, True), 150)
    assert 7.0e10 < big < 9.0e10


def test_solver_kwargs_are_checked():
    """The adjoint reverses the block projection at a fixed iteration count:
    the split projection and stop mode are refused before any device work."""
    from xpbd_gpu.differentiable import _check_solver_kwargs
    kw = {}
    _check_solver_kwargs(kw)
    assert kw["block_neohookean_enable"] is True
    _check_solver_kwargs(dict(target_rel_residual=0.0, residual_floor=0.0))
    for bad in (dict(block_neohookean_enable=False), dict(target_rel_residual=1e-3), dict(residual_floor=1e-6)):
        with pytest.raises(ValueError):
            _check_solver_kwargs(bad)
