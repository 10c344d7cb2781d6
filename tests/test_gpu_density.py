"""1-particle density (CIDEN path) on the GPU vs the oracle, through the C ABI.

The oracle restates generateSOCIblocksForCIDEN + transformSEFSEFtoMOGET and is pinned bit
for bit to the reference (test_oracle_vs_reference.py, golden fixtures).  The GPU sums in
an order set by atomics, so the bar is DENS_TOL absolute on densities of unit vectors
(entries are O(1); the largest possible entry is nelec).
"""
import numpy as np
import pytest

from helpers import high_open_problem, small_problem

pytestmark = pytest.mark.gpu

DENS_TOL = 1e-12


def _unit(rng, k, n):
    v = rng.standard_normal((k, n))
    return v / np.linalg.norm(v, axis=1, keepdims=True)


def _ctx(p):
    from psoci_gb300 import api

    c = api.Context(0)
    c.load_problem(p)
    c.build_determinants()
    return c


def _cases():
    from psoci_gb300.inputs import make_problem

    return {
        "fci_6e8o_k1": lambda: small_problem("fci_6e8o", 1, seed=2),
        "fci_5e6o_k2": lambda: small_problem("fci_5e6o", 2, seed=2),
        "fci_4e6o_k3": lambda: small_problem("fci_4e6o", 3, seed=2),
        "mrcisd_4e6o_v8": lambda: make_problem("mrcisd", seed=11, ksym=1, nact=6, nelec=4, nvirt=8),
        "mrcisd_5e6o_v6": lambda: make_problem("mrcisd", seed=11, ksym=2, nact=6, nelec=5, nvirt=6),
        "open9": lambda: high_open_problem(nbf=12, seed=3, nelec=9, ksym=1, per=2),
        "open10": lambda: high_open_problem(nbf=14, seed=4, nelec=10, ksym=2, per=2),
        "two_words": lambda: make_problem("mrcis", seed=7, ksym=2, nact=4, nelec=4, nvirt=68),
    }


@pytest.mark.parametrize("name", list(_cases()))
def test_density1_matches_oracle(oracle_mod, name):
    p = _cases()[name]()
    O = oracle_mod.Oracle(p)
    c = _ctx(p)
    v = _unit(np.random.default_rng(5), 3, O.num_sefs())
    ref = O.density1(v)
    got = c.density1(v)
    assert got.shape == ref.shape
    err = np.abs(got - ref).max()
    assert err <= DENS_TOL, err
    tr = got[:, [q * (q + 1) // 2 + q for q in range(p.nbf)]].sum(1)
    assert np.abs(tr - p.nelec).max() <= 1e-11


def test_density1_root_batches(oracle_mod):
    """More roots than one pass of the pair kernel holds (the roots are done in batches)."""
    p = small_problem("fci_5e6o", 1, seed=4)
    O = oracle_mod.Oracle(p)
    c = _ctx(p)
    v = _unit(np.random.default_rng(6), 11, O.num_sefs())
    assert np.abs(c.density1(v) - O.density1(v)).max() <= DENS_TOL


def test_density1_of_davidson_roots(oracle_mod):
    """Densities of converged CI roots, and the groups rebuilt after new configurations."""
    p = small_problem("fci_6e8o", 4, seed=3)
    O = oracle_mod.Oracle(p)
    c = _ctx(p)
    c.build_hamiltonian(mixed=False)
    res = c.davidson(3, rtol=1e-8, want_vectors=True)
    got = c.density1(res.evecs)
    assert np.abs(got - O.density1(res.evecs)).max() <= DENS_TOL
    # the same context on another configuration space (same orbitals, odd electron count)
    from psoci_gb300.inputs import make_problem

    q = make_problem("mrcisd", seed=3, ksym=2, nact=4, nelec=3, nvirt=4)
    assert q.nbf == p.nbf
    Q = oracle_mod.Oracle(q)
    c.load_problem(q)
    c.build_determinants()
    w = _unit(np.random.default_rng(7), 2, Q.num_sefs())
    assert np.abs(c.density1(w) - Q.density1(w)).max() <= DENS_TOL


def test_density1_rejects_bad_calls():
    from psoci_gb300 import api

    p = small_problem("fci_4e6o", 1)
    c = api.Context(0)
    c.load_problem(p)
    c.nsef = 5  # pass the length check: the library itself must refuse (no determinants yet)
    with pytest.raises(api.PsociError):
        c.density1(np.zeros((1, 5)))
    c.build_determinants()
    with pytest.raises(ValueError):
        c.density1(np.zeros((1, c.nsef + 1)))
