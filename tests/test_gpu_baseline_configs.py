"""GPU parity at the benchmark configurations' own sizes, against the oracle (the C
restatement of the reference, pinned bit for bit to the reference's compiled sources).

* fci_6e12o — valence full CI, 12 orbitals, 6 electrons: 8,074 configurations and 33,814
  SEFs in each of the four double-group blocks (ksym 1-4).  Determinants bit-exact, CSR
  structure equal and element values within 1e-12 Eh; 4 roots with plain FP64 within 1e-10 Eh
  and mixed precision within 1e-7 Eh of ARPACK (tol 1e-13) on the oracle's matrix.
* mrcis_6e8o_v40 — CAS(6e,8o) plus singles into 40 virtuals: 20,944 configurations, 89,404
  SEFs.  The same bars for 8 roots, and for every spin-orbit splitting E_k - E_0.
* mrcisd_4e6o_v30 — CAS(4e,6o) plus singles and doubles into 30 virtuals: 32,775 SEFs, in
  direct mode (no stored elements): the direct sigma against the oracle's own lower-triangle
  sigma, and the Davidson roots against ARPACK.
"""
import numpy as np
import pytest
import scipy.sparse.linalg as spla

from helpers import check_h_against_oracle, det_lists_to_bits, gpu_bits, gpu_context, lower_to_full

pytestmark = pytest.mark.gpu

H_TOL = 1e-12
EIG_TOL_FP64 = 1e-10
EIG_TOL_MIXED = 1e-7
SIGMA_RTOL = 1e-12


def _arpack(F, k):
    w = spla.eigsh(F, k=k, which="SA", tol=1e-13, ncv=max(4 * k, 40))[0]
    return np.sort(w)


def _roots_and_splittings(c, F, nroots):
    ref = _arpack(F, nroots)
    r64 = c.davidson(nroots, rtol=1e-8, mixed=False)
    rmx = c.davidson(nroots, rtol=1e-8, mixed=True, refine=True)
    for res, tol in ((r64, EIG_TOL_FP64), (rmx, EIG_TOL_MIXED)):
        err = np.abs(res.evals - ref)
        assert err.max() <= tol, (err, res.evals, ref)
        split_err = np.abs((res.evals - res.evals[0]) - (ref - ref[0]))
        assert split_err.max() <= 2 * tol, split_err
    return ref, r64, rmx


@pytest.mark.parametrize("ksym", [1, 2, 3, 4])
def test_fci_6e12o_block(oracle_mod, ksym):
    from psoci_gb300.inputs import named_workload

    p = named_workload("fci_6e12o", seed=0, ksym=ksym)
    O = oracle_mod.Oracle(p)
    c = gpu_context(p)
    assert c.nsef == O.num_sefs()
    if ksym == 1:
        assert c.nsef == 33814
    # determinant tables: bit-strings, phases and spin projections of a sample of configurations
    g = c.get_determinants(p.nconf, p.nbf)
    cc = O.config_counts()
    assert (np.diff(g["detoff"]) == cc[:, 0]).all()
    assert (np.diff(g["sefoff"]) == cc[:, 1]).all()
    for i in np.random.default_rng(ksym).choice(p.nconf, 300, replace=False):
        d0 = g["detoff"][i]
        for d, (a, b, ms, ph) in enumerate(det_lists_to_bits(O.config_dets(int(i)), p.nbf)):
            assert gpu_bits(g["alpha"][d0 + d]) == a and gpu_bits(g["beta"][d0 + d]) == b
            assert int(g["ms"][d0 + d]) == ms and int(g["phase"][d0 + d]) == ph
    F = check_h_against_oracle(c, O, p, tol=H_TOL)
    rng = np.random.default_rng(5)
    X = rng.standard_normal((c.nsef, 8))
    Yref = F @ X
    scale = np.abs(Yref).max()
    assert np.abs(c.sigma(X) - Yref).max() <= SIGMA_RTOL * scale * 10
    assert np.abs(c.sigma(X, prec=1) - Yref).max() <= 1e-5 * scale
    assert np.abs(c.sigma(X, prec=2) - Yref).max() <= 1e-11 * scale
    _roots_and_splittings(c, F, 4)
    c.close()


def test_mrcis_6e8o_v40_eight_roots(oracle_mod):
    from psoci_gb300.inputs import named_workload

    p = named_workload("mrcis_6e8o_v40", seed=0, ksym=1)
    O = oracle_mod.Oracle(p)
    c = gpu_context(p)
    assert c.nsef == 89404
    F = check_h_against_oracle(c, O, p, tol=H_TOL)
    assert c.build_stats()["lookup_screen"] == 1
    ref, r64, rmx = _roots_and_splittings(c, F, 8)
    print("mrcis_6e8o_v40 roots:", r64.evals, "max |dE| fp64", np.abs(r64.evals - ref).max(), "mixed",
          np.abs(rmx.evals - ref).max())
    c.close()


def test_mrcisd_4e6o_v30_direct(oracle_mod):
    from psoci_gb300 import api
    from psoci_gb300.inputs import named_workload

    p = named_workload("mrcisd_4e6o_v30", seed=0, ksym=1)
    O = oracle_mod.Oracle(p)
    rp, ci, va = O.build_lower(0)
    n = O.num_sefs()
    assert n == 32775
    c = gpu_context(p)
    assert c.build_hamiltonian(direct=True) == 0
    assert np.abs(c.get_diag() - O.diag()).max() <= H_TOL
    X = np.random.default_rng(9).standard_normal((n, 8))
    Yref = O.sigma_lower(rp, ci, va, X.T.copy()).T
    scale = np.abs(Yref).max()
    # FP64 products, and FP32 element x FP32 input products with compensated sums
    for prec, tol in ((api.PREC_FP64, SIGMA_RTOL * 10), (api.PREC_MIXED, 1e-5)):
        Y = c.sigma(X, prec=prec)
        assert np.abs(Y - Yref).max() <= tol * scale, prec
    F = lower_to_full(rp, ci, va, n)
    ref = _arpack(F, 8)
    e = c.davidson(8, rtol=1e-8, mixed=False).evals
    assert np.abs(e - ref).max() <= EIG_TOL_FP64, (e, ref)
    em = c.davidson(8, rtol=1e-8, mixed=True, refine=True).evals
    assert np.abs(em - ref).max() <= EIG_TOL_MIXED, (em, ref)
    c.close()
