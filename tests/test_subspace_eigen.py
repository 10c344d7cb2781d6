"""Rayleigh-Ritz eigen-solve of the Davidson subspace matrix (host code in the library; no GPU).

psoci_subspace_eigen stands in for the dsygv call of PsociGAsubspace::diagSubspaceGOP with the
unit metric of an orthonormal basis.  Checked against LAPACK (numpy.linalg.eigh): eigenvalues,
orthonormal eigenvectors, residuals, ascending order, on random, graded, clustered and
diagonal matrices of the orders the solver uses (1 to 96).
"""
import numpy as np
import pytest


def _check(api, A, tol=1e-13):
    w, Y = api.subspace_eigen(A)
    ref = np.linalg.eigvalsh(A)
    scale = max(1.0, np.abs(ref).max())
    n = A.shape[0]
    assert np.all(np.diff(w) >= 0)
    assert np.abs(w - ref).max() <= tol * scale * max(1, n ** 0.5)
    assert np.abs(Y.T @ Y - np.eye(n)).max() <= 1e-13 * max(1, n)
    assert np.abs(A @ Y - Y * w).max() <= tol * scale * max(1, n)


@pytest.mark.parametrize("n", [1, 2, 3, 5, 8, 16, 33, 40, 64, 96])
def test_random_symmetric(gpu_lib, n):
    from psoci_gb300 import api

    rng = np.random.default_rng(n)
    B = rng.standard_normal((n, n))
    _check(api, B + B.T)


def test_subspace_like_spectrum(gpu_lib):
    """Rayleigh matrix of a CI-like operator: a large negative shift, close low eigenvalues."""
    from psoci_gb300 import api

    rng = np.random.default_rng(7)
    n = 40
    Q, _ = np.linalg.qr(rng.standard_normal((n, n)))
    lam = np.concatenate([-18.7687 + 1e-6 * np.arange(4), -18.0 + rng.random(n - 4) * 10.0])
    _check(api, (Q * lam) @ Q.T)


def test_diagonal_degenerate_and_tiny_border(gpu_lib):
    from psoci_gb300 import api

    n = 24
    A = np.diag(np.repeat(np.arange(6, dtype=float), 4))
    w, Y = api.subspace_eigen(A)
    assert np.array_equal(w, np.sort(np.diag(A)))
    assert np.abs(np.abs(Y) - np.eye(n)[:, np.argsort(np.diag(A), kind="stable")]).max() == 0.0
    # a diagonal block with a small border, as after a collapse and one expansion
    rng = np.random.default_rng(3)
    A = np.diag(np.linspace(-20, -5, n))
    b = 1e-3 * rng.standard_normal(n - 1)
    A[-1, :-1] = b
    A[:-1, -1] = b
    _check(api, A)


def test_rejects_bad_input(gpu_lib):
    from psoci_gb300 import api

    with pytest.raises(ValueError):
        api.subspace_eigen(np.zeros((3, 4)))
    A = np.eye(3)
    A[1, 2] = np.nan
    with pytest.raises(api.PsociError):
        api.subspace_eigen(A)
