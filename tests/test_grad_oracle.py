"""CPU checks of the FP64 differentiable-form oracle (oracle/adjoint.py): the
adjoint identity, finite differences of the loss (h = 1e-3, 64 voxels, real and
imaginary perturbations) and the TV gradient."""
import numpy as np
import pytest

import adjoint as AD


def _case(r=16, frac=0.3, seed=0):
    rng = np.random.default_rng(seed)
    mask = rng.random(r ** 3) < frac
    idx = np.flatnonzero(mask).astype(np.uint32)
    y = rng.standard_normal(idx.size) + 1j * rng.standard_normal(idx.size)
    V = 0.1 * (rng.standard_normal((r, r, r)) + 1j * rng.standard_normal((r, r, r)))
    return idx, y, V, rng


def test_adjoint_identity():
    idx, y, V, _ = _case()
    lhs = np.vdot(y, AD.forward(V, idx))
    rhs = np.vdot(AD.adjoint(y, idx, V.shape[0]), V)
    assert abs(lhs - rhs) <= 1e-12 * abs(lhs)


@pytest.mark.parametrize("lam", [0.0, 0.05])
def test_gradient_finite_differences(lam):
    idx, y, V, rng = _case(seed=1)
    eps, h = 1e-2, 1e-3
    _, g = AD.loss_grad(V, idx, y, lam, eps)
    picks = rng.choice(V.size, 64, replace=False)
    # central differences: truncation error O(h^2 |L'''|), well under 1e-5 |g|_max here
    atol = 1e-5 * np.abs(g).max()
    for p in picks:
        for unit, comp in ((1.0, g.ravel()[p].real), (1j, g.ravel()[p].imag)):
            Vp = V.copy().ravel(); Vp[p] += h * unit
            Vm = V.copy().ravel(); Vm[p] -= h * unit
            fd = (AD.loss(Vp.reshape(V.shape), idx, y, lam, eps) - AD.loss(Vm.reshape(V.shape), idx, y, lam, eps)) / (2 * h)
            assert abs(fd - comp) <= atol + 1e-4 * abs(comp)


def test_measured_indices_predicate():
    F2 = np.zeros(8, np.complex64)
    F2[[1, 4, 6]] = [1 + 1j, 2 + 0j, -1 - 2j]   # 4: imaginary part zero -> not measured
    assert list(AD.measured_indices(F2)) == [1, 6]
    counts = np.array([0, 1, 0, 0, 3, 0, 0, 0])
    assert list(AD.measured_indices(F2, counts)) == [1, 4]


def test_contrast_to_ri_principal_root():
    V = np.array([-2.0 + 0j, -2.0 - 0.0j, 0.5 + 0.2j, -1 + 0j]).reshape(1, 1, 4)
    V = np.broadcast_to(V, (4, 4, 4)).copy()
    n = AD.contrast_to_ri(V, 1.0)
    np.testing.assert_allclose(np.roll(n, (-2, -2, -2), axis=(0, 1, 2))[0, 0], np.sqrt(1 + V[0, 0]))
