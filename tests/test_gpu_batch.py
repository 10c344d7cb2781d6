"""Batched Davidson over several symmetry blocks (psoci_davidson_batch) and the sigma autotuner.

Blocks of different sizes, electron parities and root counts solved together must give
each block's own roots: the oracle's spectrum within 1e-10 Eh (plain FP64) and 1e-7 Eh
(mixed precision with refinement).  Every mixed-sigma variant the autotuner chooses from
must reproduce the FP64 product within the mixed bar.
"""
import numpy as np
import pytest
import scipy.linalg as sla

from helpers import gpu_context, lower_to_full, small_problem

pytestmark = pytest.mark.gpu


def _blocks():
    from psoci_gb300.inputs import make_problem

    return [(small_problem("fci_6e8o", 1), 4), (small_problem("fci_5e6o", 2), 3),
            (make_problem("mrcisd", seed=11, ksym=1, nact=6, nelec=4, nvirt=8), 6),
            (small_problem("fci_6e8o", 3), 2)]


def test_batch_matches_oracle(oracle_mod):
    from psoci_gb300 import api

    blocks = _blocks()
    refs = []
    for p, k in blocks:
        O = oracle_mod.Oracle(p)
        rp, ci, va = O.build_lower(4)
        refs.append(sla.eigvalsh(lower_to_full(rp, ci, va, O.num_sefs()).toarray())[:k])
    ctxs = [gpu_context(p) for p, _ in blocks]
    for c in ctxs:
        c.build_hamiltonian(mixed=True)
    ks = [k for _, k in blocks]
    for mixed, tol in ((False, 1e-10), (True, 1e-7)):
        res = api.davidson_batch(ctxs, ks, rtol=1e-8, mixed=mixed, want_vectors=True)
        for r, ref, k in zip(res, refs, ks):
            assert len(r.evals) == k
            assert np.abs(r.evals - ref).max() <= tol, (r.evals, ref)
            assert r.evecs.shape[0] == k
    # the same blocks one at a time agree with the batch
    single = ctxs[2].davidson(ks[2], rtol=1e-8, mixed=False)
    batch = api.davidson_batch(ctxs, ks, rtol=1e-8, mixed=False)
    assert np.abs(single.evals - batch[2].evals).max() <= 1e-10
    for c in ctxs:
        c.close()


def test_sigma_variants():
    from psoci_gb300 import api

    p = small_problem("fci_6e8o", 1)
    c = gpu_context(p)
    c.build_hamiltonian(mixed=True)
    X = np.random.default_rng(3).standard_normal((c.nsef, 8))
    ref = c.sigma(X, prec=api.PREC_FP64)
    scale = np.abs(ref).max()
    outs = []
    for v in range(6):
        c.set_sigma_variant(v)
        for k in (8, 3):
            Y = c.sigma(X[:, :k], prec=api.PREC_MIXED)
            assert np.abs(Y - ref[:, :k]).max() <= 1e-5 * scale, (v, k)
        outs.append(c.sigma(X, prec=api.PREC_MIXED))
    for o in outs[1:]:
        assert np.abs(o - outs[0]).max() <= 1e-6 * scale
    choice, times = c.autotune_sigma(8)
    assert 0 <= choice < 6 and all(t > 0 for t in times)
    assert times[choice] == min(times)
    c.close()
