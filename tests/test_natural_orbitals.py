"""Natural-orbital consumer of the 1-particle density (host code in the library; no GPU).

psoci_natural_orbitals restates the MO-basis part of PsociNOpopulations::
constructNaturalOrbitals: per symmetry block, eigenpairs of the density with a unit metric,
largest occupation first.  Checked against LAPACK (numpy.linalg.eigh) and, on densities of
CI vectors from the oracle, against the N-representability bounds 0 <= n <= 2, sum = nelec.
"""
import numpy as np
import pytest

from helpers import small_problem


def _packed(M):
    n = M.shape[0]
    return np.array([M[p, q] for p in range(n) for q in range(p + 1)])


def _block_density(rng, sym):
    n = len(sym)
    M = np.zeros((n, n))
    for s in np.unique(sym):
        idx = np.nonzero(sym == s)[0]
        A = rng.standard_normal((len(idx), len(idx)))
        M[np.ix_(idx, idx)] = A + A.T
    return M


@pytest.mark.parametrize("nbf,nsym", [(1, 1), (7, 1), (20, 4), (72, 8), (128, 3)])
def test_blocks_match_lapack(gpu_lib, nbf, nsym):
    from psoci_gb300 import api

    rng = np.random.default_rng(nbf)
    sym = rng.integers(1, nsym + 1, nbf).astype(np.int32)
    M = _block_density(rng, sym)
    occ, blocks = api.natural_orbitals(_packed(M), sym)
    assert len(occ) == nbf
    assert [b["sym"] for b in blocks] == sorted(set(sym.tolist()))
    e = 0
    for b in blocks:
        idx = b["orbitals"]
        assert (np.diff(idx) > 0).all() and (sym[idx] == b["sym"]).all()
        A = M[np.ix_(idx, idx)]
        w = np.linalg.eigh(A)[0][::-1]
        n = b["occupations"]
        assert np.abs(n - w).max() <= 1e-12 * max(1.0, np.abs(w).max())
        assert np.array_equal(occ[e:e + len(idx)], n)
        V = b["vectors"]  # row i = natural orbital i
        assert np.abs(V @ V.T - np.eye(len(idx))).max() <= 1e-12
        assert np.abs(V @ A @ V.T - np.diag(n)).max() <= 1e-11 * max(1.0, np.abs(w).max())
        e += len(idx)


def test_degenerate_and_diagonal(gpu_lib):
    from psoci_gb300 import api

    M = np.diag([2.0, 0.0, 2.0, 1.0, 1.0, 0.5])
    occ, blocks = api.natural_orbitals(_packed(M), np.ones(6, np.int32))
    assert np.array_equal(occ, [2.0, 2.0, 1.0, 1.0, 0.5, 0.0])
    # equal occupations keep the solver's ascending order: orbitals 0, 2 then 3, 4
    V = blocks[0]["vectors"]
    assert np.array_equal(np.abs(V), np.eye(6)[[0, 2, 3, 4, 5, 1]])


def test_rejects_bad_sizes(gpu_lib):
    from psoci_gb300 import api

    with pytest.raises(ValueError):
        api.natural_orbitals(np.zeros(5), np.ones(3, np.int32))


@pytest.mark.parametrize("name,ksym", [("fci_6e8o", 1), ("fci_5e6o", 2)])
def test_ci_density_occupations(gpu_lib, oracle_mod, name, ksym):
    """Densities of normalised CI vectors: occupations in [0, 2], summing to nelec."""
    from psoci_gb300 import api

    p = small_problem(name, ksym, seed=8)
    O = oracle_mod.Oracle(p)
    v = np.random.default_rng(3).standard_normal((2, O.num_sefs()))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    for d in O.density1(v):
        occ, _ = api.natural_orbitals(d, p.irreps)
        assert occ.min() >= -1e-12 and occ.max() <= 2.0 + 1e-12
        assert abs(occ.sum() - p.nelec) <= 1e-11
