"""Pin the oracle against the reference's own compute sources, built in this container.

Skipped where the reference tree is absent (the GPU host): there the committed golden
fixtures (test_oracle_golden.py) carry the same check.
"""
import os

import numpy as np
import pytest

from helpers import SMALL_CASES, high_open_problem, small_problem

from oracle import REFERENCE_TREE as REF_TREE  # noqa: E402
pytestmark = pytest.mark.skipif(not os.path.isdir(REF_TREE), reason="reference tree not present")


@pytest.fixture(scope="module")
def both():
    import oracle

    oracle.build(ref=True)
    return oracle


class _Quiet:
    """The reference prints its integral tables to stdout; silence fd 1."""

    def __enter__(self):
        self.devnull = os.open(os.devnull, os.O_WRONLY)
        self.saved = os.dup(1)
        os.dup2(self.devnull, 1)

    def __exit__(self, *a):
        os.dup2(self.saved, 1)
        os.close(self.devnull)
        os.close(self.saved)


@pytest.mark.parametrize("name,ksym", SMALL_CASES)
def test_h_bit_exact(both, name, ksym):
    p = small_problem(name, ksym, seed=9)
    with _Quiet():
        R = both.Reference(p)
        rr = R.build_lower(2)
    O = both.Oracle(p)
    ro = O.build_lower(2)
    assert (rr[0] == ro[0]).all() and (rr[1] == ro[1]).all()
    assert np.array_equal(rr[2], ro[2])


@pytest.mark.parametrize("nelec", [7, 8, 9, 10, 11])
def test_dets_high_open(both, nelec):
    for ksym in (1, 2, 3, 4):
        p = high_open_problem(nbf=13, seed=nelec, nelec=nelec, ksym=ksym, per=2)
        with _Quiet():
            R = both.Reference(p)
            dr = [R.config_dets(i) for i in range(p.nconf)]
        O = both.Oracle(p)
        for i in range(p.nconf):
            assert (dr[i] == O.config_dets(i)).all(), (nelec, ksym, i)


def test_integral_tables(both):
    p = small_problem("fci_6e8o", 2, seed=4)
    with _Quiet():
        R = both.Reference(p)
    O = both.Oracle(p)
    n = p.nbf
    for i in range(n):
        for j in range(n):
            assert R.fetch1e(i, j) == O.fetch1e(i, j)
    rng = np.random.default_rng(0)
    for _ in range(500):
        q = [int(x) for x in rng.integers(0, n, 4)]
        assert R.fetch2e(*q) == O.fetch2e(*q)


def test_blocks_status(both):
    """generateSOCIblocks status and zero blocks for pairs beyond a double excitation."""
    p = small_problem("fci_6e8o", 1, seed=5)
    with _Quiet():
        R = both.Reference(p)
    O = both.Oracle(p)
    rng = np.random.default_rng(1)
    for _ in range(300):
        i, j = sorted(int(x) for x in rng.integers(0, p.nconf, 2))[::-1]
        sr, br = R.block(i, j)
        so, bo = O.block(i, j)
        assert sr == so
        assert np.array_equal(br, bo)


@pytest.mark.parametrize("name,ksym", [("fci_4e6o", 2), ("fci_5e6o", 1), ("fci_6e8o", 3)])
def test_ciden_blocks_bit_exact(both, name, ksym):
    """generateSOCIblocksForCIDEN: status and +-1/0 SEF blocks for every pair within one move."""
    p = small_problem(name, ksym, seed=6)
    with _Quiet():
        R = both.Reference(p)
    O = both.Oracle(p)
    occ = p.occ.astype(int)
    connected = 0
    for i in range(p.nconf):
        moved = np.abs(occ[:i + 1] - occ[i]).sum(1)
        for j in np.nonzero(moved <= 2)[0]:
            sr, br = R.ciden_block(i, int(j))
            so, bo = O.ciden_block(i, int(j))
            assert sr == so, (i, j)
            assert np.array_equal(br, bo), (i, j)
            connected += sr != 0
    assert connected > p.nconf


def test_density1_bit_exact(both):
    """Packed spin-free 1-particle densities, FCI and MRCISD, even and odd electron counts."""
    from psoci_gb300.inputs import make_problem

    probs = [small_problem("fci_6e8o", 1, seed=2), small_problem("fci_5e6o", 2, seed=2),
             make_problem("mrcisd", seed=11, ksym=1, nact=6, nelec=4, nvirt=8),
             high_open_problem(nbf=12, seed=3, nelec=9, ksym=1, per=2)]
    rng = np.random.default_rng(5)
    for p in probs:
        with _Quiet():
            R = both.Reference(p)
        O = both.Oracle(p)
        v = rng.standard_normal((3, O.num_sefs()))
        v /= np.linalg.norm(v, axis=1, keepdims=True)
        dr = R.density1(v)
        do = O.density1(v)
        assert np.array_equal(dr, do)
        tr = do[:, [k * (k + 1) // 2 + k for k in range(p.nbf)]].sum(1)
        assert np.abs(tr - p.nelec).max() < 1e-12
