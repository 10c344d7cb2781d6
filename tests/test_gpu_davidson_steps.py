"""The step-level Davidson entry points (psoci_basis_*, psoci_subspace_*) through the C ABI:
the reference's loop written in Python against the one-call psoci_davidson and the oracle's
spectrum, the block variant of the same steps, and the call-order rules."""
import ctypes

import numpy as np
import pytest
import scipy.linalg as sla

from helpers import gpu_context, lower_to_full, small_problem

pytestmark = pytest.mark.gpu

PSOCI_OK, PSOCI_ERR_STATE, PSOCI_ERR_INVALID_ARG = 0, 3, 1


class Steps:
    def __init__(self, c):
        self.c, self.lib = c, c.lib

    def __call__(self, name, *args):
        st = getattr(self.lib, "psoci_" + name)(self.c.ctx, *args)
        return st

    def ok(self, name, *args):
        st = self(name, *args)
        assert st == PSOCI_OK, (name, st, self.lib.psoci_last_error(self.c.ctx))

    def existing(self):
        e = ctypes.c_int()
        self.ok("basis_info", ctypes.byref(e), None, None, None)
        return e.value


def reference_loop(S, nroots, maxsub, rtol, max_iter=400):
    """driver.PSOCI.splittest.C:1186-1311 (INCREMENTAL, NEWRNOMRS, DIAGGOP, MODIFIED_EXPAND)."""
    S.ok("basis_create", nroots, maxsub + 1)
    S.ok("basis_guess", 0)
    S.ok("basis_orthonormalize_all", None)
    S.ok("basis_compute_hv", 0, nroots, 0)
    evals = np.zeros(maxsub + 1)
    ev_p = evals.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    r = ctypes.c_double()
    coarse, cur_rtol, curroot, count, converged, nupd = 1e-3, 1e-3, 1, 0, False, nroots
    total, nsig = 0, nroots
    nap = ctypes.c_int()
    while count < max_iter and not converged:
        count += 1
        total += 1
        S.ok("subspace_generate_incremental", nupd)
        S.ok("subspace_diag", ev_p)
        converged, itest = True, curroot
        while itest <= nroots:
            S.ok("subspace_rnorm_single", itest, ctypes.byref(r))
            if r.value > cur_rtol:
                converged, curroot = False, itest
                break
            itest += 1
        if not converged:
            S.ok("basis_precondition_new", curroot, evals[curroot - 1], 1e-3)
            S.ok("basis_append_scratch", 0, ctypes.byref(nap))
            nsig += nap.value
            nupd = 1
        if converged and cur_rtol == coarse:
            converged, count, cur_rtol, curroot = False, 0, rtol, 1
            if S.existing() >= 2 * nroots:
                S.ok("basis_expand_replace", 2 * nroots)
            nupd = S.existing()
        if S.existing() > maxsub:
            S.ok("basis_expand_replace", 2 * nroots)
            nupd = S.existing()
    assert converged
    rn = np.zeros(nroots)
    S.ok("subspace_rnorms", rn.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    S.ok("basis_expand_replace", S.existing())
    vecs = np.zeros((nroots, S.c.nsef))
    S.ok("basis_vectors", nroots, vecs.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    return evals[:nroots].copy(), rn, vecs, total, nsig


@pytest.mark.parametrize("name,ksym", [("fci_6e8o", 1), ("fci_5e6o", 2)])
def test_reference_loop_matches_solve(oracle_mod, name, ksym):
    p = small_problem(name, ksym)
    O = oracle_mod.Oracle(p)
    rp, ci, va = O.build_lower(4)
    F = lower_to_full(rp, ci, va, O.num_sefs())
    ref = sla.eigvalsh(F.toarray())[:4]
    c = gpu_context(p)
    c.build_hamiltonian(mixed=True)
    S = Steps(c)
    ev, rn, vecs, iters, nsig = reference_loop(S, 4, 16, 1e-8)
    assert nsig >= iters
    assert np.abs(ev - ref).max() <= 1e-10
    assert (rn <= 1e-8).all()
    fast = c.davidson(4, rtol=1e-8, mixed=False)
    assert np.abs(ev - fast.evals).max() <= 1e-10
    # the expanded basis holds the eigenvectors: orthonormal, H v = E v
    assert np.abs(vecs @ vecs.T - np.eye(4)).max() <= 1e-10
    assert np.abs(F @ vecs.T - vecs.T * ev).max() <= 1e-7
    c.close()


def test_step_call_order(oracle_mod):
    p = small_problem("fci_4e6o", 1)
    c = gpu_context(p)
    S = Steps(c)
    assert S("basis_create", 2, 8) == PSOCI_ERR_STATE  # no Hamiltonian yet
    c.build_hamiltonian(mixed=False)
    assert S("basis_create", 2, 2) == PSOCI_ERR_INVALID_ARG  # room for no new vector
    S.ok("basis_create", 2, 8)
    S.ok("basis_guess", 1)
    assert S("subspace_generate_incremental", 2) == PSOCI_ERR_STATE  # products missing
    S.ok("basis_compute_hv", 0, 2, 0)
    assert S("subspace_diag", None) == PSOCI_ERR_STATE  # G not formed
    S.ok("subspace_generate_incremental", 2)
    r = ctypes.c_double()
    assert S("subspace_rnorm_single", 1, ctypes.byref(r)) == PSOCI_ERR_STATE  # no eigen-solve
    ev = np.zeros(8)
    S.ok("subspace_diag", ev.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    assert S("basis_precondition_new", 1, ev[0], 1e-3) == PSOCI_ERR_STATE  # no residual of root 1
    S.ok("subspace_rnorm_single", 1, ctypes.byref(r))
    assert S("basis_append_scratch", 0, None) == PSOCI_ERR_STATE  # nothing preconditioned
    S.ok("basis_precondition_new", 1, ev[0], 1e-3)
    n = ctypes.c_int()
    S.ok("basis_append_scratch", 0, ctypes.byref(n))
    assert n.value == 1 and S.existing() == 3
    c.build_hamiltonian(mixed=False)  # same space: the basis stays usable
    S.ok("subspace_generate_incremental", 1)
    c.lib.psoci_basis_destroy(c.ctx)
    assert S("basis_guess", 0) == PSOCI_ERR_STATE
    c.close()
