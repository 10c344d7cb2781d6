"""Repeated work on one context: the device-memory cache hands released buffers to later
allocations of the same context (exact sizes on a repeated step, up to 25% larger blocks
otherwise).  Results must not depend on what the buffers held before: repeated builds and
solves are bit-identical, and another problem after a first one (same orbital count, as a
context requires; reused blocks of other sizes) gives the same results as on a fresh context.
"""
import numpy as np
import pytest

from helpers import small_problem

pytestmark = pytest.mark.gpu


def _solve(c, p, mixed):
    c.load_problem(p)
    c.build_determinants()
    c.build_hamiltonian(mixed=mixed)
    rp, ci, va = c.get_hamiltonian()
    r = c.davidson(4, rtol=1e-8, mixed=mixed, refine=True, max_subspace=24, want_vectors=True)
    return rp, ci, va, np.array(r.evals), np.array(r.evecs)


@pytest.mark.parametrize("mixed", [False, True])
def test_repeated_steps_bit_identical(mixed):
    from psoci_gb300 import api

    p = small_problem("fci_6e8o", 1, seed=5)
    with api.Context(0) as c:
        a = _solve(c, p, mixed)
        for _ in range(2):
            b = _solve(c, p, mixed)
            for x, y in zip(a, b):
                assert np.array_equal(x, y)


def test_second_problem_matches_fresh_context():
    from psoci_gb300 import api

    big = small_problem("fci_6e8o", 1, seed=5)
    small = small_problem("fci_6e8o", 2, seed=7)
    with api.Context(0) as c:
        _solve(c, big, True)
        reused = _solve(c, small, True)
    with api.Context(0) as c:
        fresh = _solve(c, small, True)
    for x, y in zip(reused, fresh):
        assert np.array_equal(x, y)
