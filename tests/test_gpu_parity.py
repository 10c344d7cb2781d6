"""GPU path vs the oracle (C restatement of the reference), through the C ABI.

Bars: determinant bit-strings, phases and spin projections bit-exact; CSR structure
identical to the reference's lower triangle mirrored; element values within 1e-12 Eh
(the element kernel follows the reference's operation order, so they are usually
identical); FP64 sigma within 1e-12 relative; FP64 Davidson eigenvalues within 1e-10 Eh
of a dense/ARPACK solve of the oracle matrix; mixed-precision eigenvalues within 1e-7 Eh.
"""
import numpy as np
import pytest
import scipy.linalg as sla

from helpers import (SMALL_CASES, check_h_against_oracle, det_lists_to_bits, gpu_bits, gpu_context, high_open_problem,
                     lower_to_full, small_problem)

pytestmark = pytest.mark.gpu

H_TOL = 1e-12
SIGMA_RTOL = 1e-12
FF_RTOL = 1e-11
EIG_TOL_FP64 = 1e-10
EIG_TOL_MIXED = 1e-7


def _ctx(p):
    return gpu_context(p)


def _check_dets(c, O, p):
    g = c.get_determinants(p.nconf, p.nbf)
    cc = O.config_counts()
    assert (np.diff(g["detoff"]) == cc[:, 0]).all()
    assert (np.diff(g["sefoff"]) == cc[:, 1]).all()
    for i in range(p.nconf):
        ref = det_lists_to_bits(O.config_dets(i), p.nbf)
        d0 = g["detoff"][i]
        for d, (a, b, ms, ph) in enumerate(ref):
            assert gpu_bits(g["alpha"][d0 + d]) == a, (i, d)
            assert gpu_bits(g["beta"][d0 + d]) == b, (i, d)
            assert int(g["ms"][d0 + d]) == ms, (i, d)
            assert int(g["phase"][d0 + d]) == ph, (i, d)


def _check_h(c, O, p):
    return check_h_against_oracle(c, O, p, tol=H_TOL, nthreads=4)


@pytest.mark.parametrize("name,ksym", SMALL_CASES)
def test_dets_and_h_small(oracle_mod, name, ksym):
    p = small_problem(name, ksym)
    O = oracle_mod.Oracle(p)
    c = _ctx(p)
    _check_dets(c, O, p)
    _check_h(c, O, p)


@pytest.mark.parametrize("nelec,ksym", [(10, 1), (10, 2), (9, 1), (11, 4)])
def test_high_open_shells(oracle_mod, nelec, ksym):
    """8-11 open shells: the largest templates and the multi-word paths of the kernels."""
    p = high_open_problem(nbf=14, nelec=nelec, ksym=ksym, per=2)
    O = oracle_mod.Oracle(p)
    c = _ctx(p)
    _check_dets(c, O, p)
    _check_h(c, O, p)


def test_two_word_orbitals(oracle_mod):
    """nbf > 64: bit-strings span two 64-bit words."""
    from psoci_gb300.inputs import make_problem

    p = make_problem("mrcis", seed=7, ksym=2, nact=4, nelec=4, nvirt=68)
    assert p.nbf > 64
    O = oracle_mod.Oracle(p)
    c = _ctx(p)
    _check_dets(c, O, p)
    _check_h(c, O, p)


@pytest.mark.parametrize("kind,kw,ksym", [
    ("mrcisd", dict(nact=6, nelec=4, nvirt=8), 1),
    ("mrcisd", dict(nact=6, nelec=4, nvirt=8), 2),
    ("mrcisd", dict(nact=6, nelec=5, nvirt=6), 1),
    ("mrcis", dict(nact=8, nelec=6, nvirt=6), 3),
])
def test_mrci_lookup_screen(oracle_mod, kind, kw, ksym):
    """MRCI spaces take the lookup screen (at most two electrons above the active orbitals);
    the Hamiltonian must be the reference's all the same."""
    from psoci_gb300.inputs import make_problem

    p = make_problem(kind, seed=11, ksym=ksym, **kw)
    O = oracle_mod.Oracle(p)
    c = _ctx(p)
    _check_h(c, O, p)
    assert c.build_stats()["lookup_screen"] == 1


@pytest.mark.parametrize("name", ["fci_6e8o", "mrcis_6e8o_v40"])
def test_one_launch_evaluation_matches_two(name):
    """The element evaluation in two launches (connectivity masks, then elements; the default
    when they fit) and in one launch (the fallback for short memory) store the same matrix,
    bit for bit, with the mixed FP32 copy."""
    from psoci_gb300.inputs import named_workload

    p = small_problem(name, 1) if name == "fci_6e8o" else named_workload(name, seed=0, ksym=1)
    c = _ctx(p)
    c.build_hamiltonian(mixed=True)
    assert c.build_stats()["eval_launches"] == 2
    two = c.get_hamiltonian()
    c.set_eval_launches(1)
    c.build_hamiltonian(mixed=True)
    assert c.build_stats()["eval_launches"] == 1
    one = c.get_hamiltonian()
    for a, b in zip(two, one):
        assert a.shape == b.shape and np.array_equal(a, b)
    c.set_eval_launches(0)
    c.build_hamiltonian(mixed=True)
    assert c.build_stats()["eval_launches"] == 2
    with pytest.raises(Exception):
        c.set_eval_launches(3)


def test_fci_takes_all_pairs_screen(oracle_mod):
    p = small_problem("fci_6e8o", 1)
    c = _ctx(p)
    c.build_hamiltonian(mixed=True)
    assert c.build_stats()["lookup_screen"] == 0


def test_sigma_fp64_and_mixed(oracle_mod):
    p = small_problem("fci_6e8o", 1)
    O = oracle_mod.Oracle(p)
    c = _ctx(p)
    rp, ci, va = O.build_lower(4)
    c.build_hamiltonian(mixed=True)
    rng = np.random.default_rng(0)
    for k in (1, 3, 4, 5, 8, 11):
        X = rng.standard_normal((c.nsef, k))
        Yref = O.sigma_lower(rp, ci, va, X.T.copy()).T
        Y = c.sigma(X)
        scale = np.abs(Yref).max()
        assert np.abs(Y - Yref).max() <= SIGMA_RTOL * scale * 10
        Ym = c.sigma(X, prec=1)
        assert np.abs(Ym - Yref).max() <= 1e-5 * scale
        Yf = c.sigma(X, prec=2)  # float-float: about 47 significant bits
        assert np.abs(Yf - Yref).max() <= FF_RTOL * scale


@pytest.mark.parametrize("name,ksym", [("fci_6e8o", 1), ("fci_5e6o", 2)])
def test_davidson_fp64_and_mixed(oracle_mod, name, ksym):
    p = small_problem(name, ksym)
    O = oracle_mod.Oracle(p)
    rp, ci, va = O.build_lower(4)
    F = lower_to_full(rp, ci, va, O.num_sefs())
    ref = sla.eigvalsh(F.toarray())
    nroots = 4
    c = _ctx(p)
    c.build_hamiltonian(mixed=True)
    r64 = c.davidson(nroots, rtol=1e-8, mixed=False)
    assert np.abs(r64.evals - ref[:nroots]).max() <= EIG_TOL_FP64, (r64.evals, ref[:nroots])
    rmx = c.davidson(nroots, rtol=1e-8, mixed=True, refine=True)  # float-float refinement
    assert np.abs(rmx.evals - ref[:nroots]).max() <= EIG_TOL_MIXED
    assert rmx.refine_iters >= 1
    rm2 = c.davidson(nroots, rtol=1e-8, mixed=True, refine=2)  # FP64 refinement
    assert np.abs(rm2.evals - ref[:nroots]).max() <= EIG_TOL_MIXED
    r1 = c.davidson(nroots, rtol=1e-8, mixed=False, block=False)
    assert np.abs(r1.evals - ref[:nroots]).max() <= EIG_TOL_FP64


def test_end_to_end_solve(oracle_mod):
    from psoci_gb300 import api

    p = small_problem("fci_6e8o", 4)
    O = oracle_mod.Oracle(p)
    rp, ci, va = O.build_lower(4)
    ref = sla.eigvalsh(lower_to_full(rp, ci, va, O.num_sefs()).toarray())
    res = api.solve(p, nroots=6, mixed=True, rtol=1e-7)
    assert np.abs(res.evals - ref[:6]).max() <= EIG_TOL_MIXED


@pytest.mark.parametrize("name,ksym", [("fci_6e8o", 1), ("fci_5e6o", 2)])
def test_blocks_any_pair(oracle_mod, name, ksym):
    """psoci_blocks = generateSOCIblocks for arbitrary (A, B), both orders and the diagonal."""
    p = small_problem(name, ksym)
    O = oracle_mod.Oracle(p)
    c = _ctx(p)
    rng = np.random.default_rng(2)
    A = rng.integers(0, p.nconf, 400).astype(np.int32)
    B = rng.integers(0, p.nconf, 400).astype(np.int32)
    A[:20] = B[:20]
    got = c.blocks(A, B, p.nsef())
    for a, b, g in zip(A, B, got):
        st, ref = O.block(int(a), int(b))
        assert np.abs(g - ref).max() <= H_TOL, (a, b)


@pytest.mark.parametrize("kind,kw,ksym", [
    ("fci", dict(name="fci_6e8o"), 1),
    ("fci", dict(name="fci_5e6o"), 2),
    ("mrcisd", dict(nact=6, nelec=4, nvirt=8), 1),
])
def test_direct_sigma_matches_stored(oracle_mod, kind, kw, ksym):
    """Direct mode (no stored elements) against the stored FP64 CSR: same products and
    diagonal, and the same Davidson roots."""
    from psoci_gb300 import api
    from psoci_gb300.inputs import make_problem

    p = small_problem(kw["name"], ksym) if kind == "fci" else make_problem(kind, seed=11, ksym=ksym, **kw)
    c = _ctx(p)
    c.build_hamiltonian(mixed=False)
    d_ref = c.get_diag()
    X = np.random.default_rng(4).standard_normal((c.nsef, 11))
    Y_ref = c.sigma(X, prec=api.PREC_FP64)
    e_ref = c.davidson(4, rtol=1e-8, mixed=False).evals
    assert c.build_hamiltonian(direct=True) == 0
    assert np.abs(c.get_diag() - d_ref).max() <= H_TOL
    for prec, tol in ((api.PREC_FP64, SIGMA_RTOL), (api.PREC_MIXED, 1e-5)):
        Y = c.sigma(X, prec=prec)
        assert np.abs(Y - Y_ref).max() <= tol * np.abs(Y_ref).max(), prec
    e = c.davidson(4, rtol=1e-8, mixed=True).evals
    assert np.abs(e - e_ref).max() <= EIG_TOL_FP64
    with pytest.raises(api.PsociError):
        c.get_hamiltonian()
