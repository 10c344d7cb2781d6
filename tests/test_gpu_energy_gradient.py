"""dE/d(integral tables) on the GPU (psoci_energy_gradient, the adjoint of the element
evaluation): the 1-particle and spin-orbit densities and the 8-fold packed 2-particle
density of CI vectors.

Checked against
* the oracle's unit-table gradient (one Hamiltonian per table entry, no adjoint logic) —
  every entry within 1e-11, plain FP64, on full-CI and MRCI spaces of both electron parities;
* the oracle's CIDEN 1-particle density (pinned to the reference's own density code):
  dE/dh_pp equals the occupation, dE/dh_pq (equal irreps) twice the density;
* central differences (step 1e-5) of the GPU eigenvalues themselves, through a
  torch.autograd.Function and torch.autograd.gradcheck, on the 12-orbital, 6-electron full CI
  (33,814 SEFs per block).
"""
import numpy as np
import pytest

from helpers import gpu_context, small_problem

pytestmark = pytest.mark.gpu


def _eigvecs(O, k):
    import scipy.linalg as sla

    from helpers import lower_to_full

    rp, ci, va = O.build_lower(4)
    F = lower_to_full(rp, ci, va, O.num_sefs()).toarray()
    w, v = sla.eigh(F)
    return w[:k], v[:, :k].T.copy()


def _case(name):
    from psoci_gb300.inputs import make_problem

    if name == "mrcisd_4e4o_v3":
        return make_problem("mrcisd", seed=11, ksym=2, nact=4, nelec=4, nvirt=3)
    if name == "mrcis_5e5o_v3":
        return make_problem("mrcis", seed=4, ksym=1, nact=5, nelec=5, nvirt=3)
    if name.startswith("open"):  # 7-9 open shells: configurations of more than 32 determinants
        from helpers import high_open_problem

        nbf, ne = {"open8": (9, 8), "open9": (10, 9)}[name]
        return high_open_problem(nbf=nbf, nelec=ne, per=2, seed=5)
    nm, ks = name.rsplit("_k", 1)
    return small_problem(nm, int(ks))


@pytest.mark.parametrize("name", ["fci_4e6o_k1", "fci_4e6o_k3", "fci_5e6o_k2", "mrcisd_4e4o_v3", "mrcis_5e5o_v3", "open8",
                                  "open9"])
def test_gradient_vs_unit_table_oracle(oracle_mod, name):
    from psoci_gb300 import api

    p = _case(name)
    O = oracle_mod.Oracle(p)
    _, v = _eigvecs(O, 3)
    v[2] = np.random.default_rng(1).standard_normal(v.shape[1])  # any vector, not only eigenvectors
    r1, r2 = O.energy_gradient(v)
    c = gpu_context(p)
    g1, g2 = c.energy_gradient(v)
    scale = max(np.abs(r1).max(), np.abs(r2).max())
    assert np.abs(g1 - r1).max() <= 1e-11 * scale, np.abs(g1 - r1).max()
    assert np.abs(g2 - r2).max() <= 1e-11 * scale, np.abs(g2 - r2).max()
    # mode 1: the derivatives of the non-zero integrals only
    n1, n2 = c.energy_gradient(v, nonzero_only=True)
    nz1, nz2 = p.one_packed() != 0, p.eri != 0
    assert np.abs(n1[:, nz1] - r1[:, nz1]).max() <= 1e-11 * scale
    assert np.abs(n2[:, nz2] - r2[:, nz2]).max() <= 1e-11 * scale
    assert (n1[:, ~nz1] == 0).all() and (n2[:, ~nz2] == 0).all()
    # FP32 sums within a configuration pair
    m1, m2 = c.energy_gradient(v, prec=api.PREC_MIXED)
    assert np.abs(m1 - r1).max() <= 1e-5 * scale and np.abs(m2 - r2).max() <= 1e-5 * scale
    c.close()


@pytest.mark.parametrize("name,ksym", [("fci_6e8o", 1), ("fci_5e6o", 2)])
def test_one_particle_part_is_ciden_density(oracle_mod, name, ksym):
    """dE/dh_pp = occupation, dE/dh_pq = 2 D_pq (p, q of one irrep): the spin-free part of the
    gradient is the reference's CIDEN density of the same vectors."""
    from psoci_gb300.inputs import tri

    p = small_problem(name, ksym)
    O = oracle_mod.Oracle(p)
    _, v = _eigvecs(O, 4)
    D = O.density1(v)
    c = gpu_context(p)
    g1, _ = c.energy_gradient(v)
    n = p.nbf
    for a in range(n):
        assert np.abs(g1[:, tri(a, a)] - D[:, tri(a, a)]).max() <= 1e-12
        for b in range(a):
            if p.irreps[a] == p.irreps[b]:
                assert np.abs(g1[:, tri(a, b)] - 2.0 * D[:, tri(a, b)]).max() <= 1e-12
    c.close()


def test_gradcheck_fci_6e12o():
    """torch.autograd.gradcheck of the lowest 4 eigenvalues of the 33,814-SEF full-CI block
    with respect to both tables (central differences, step 1e-5; the gradient's sums over
    configuration pairs are FP64 atomics, so repeated backward passes may differ in the last
    bits: nondet_tol 1e-10), plus central differences of
    single entries: a diagonal h, an off-diagonal h, a spin-orbit value, a Coulomb, an exchange
    and a symmetry-forbidden (zero) two-electron integral."""
    torch = pytest.importorskip("torch")
    from autograd_energy import EnergyFunction, Solver
    from psoci_gb300.inputs import canon_index, named_workload, tri

    p = named_workload("fci_6e12o", seed=0, ksym=1)
    S = Solver(p, 4)
    one = torch.tensor(p.one_packed(), dtype=torch.float64, requires_grad=True)
    eri = torch.tensor(p.eri, dtype=torch.float64, requires_grad=True)
    assert torch.autograd.gradcheck(lambda a, b: EnergyFunction.apply(a, b, S), (one, eri), eps=1e-5, atol=1e-6,
                                    rtol=1e-4, fast_mode=True, nondet_tol=1e-10)
    e0, v0 = S.solve(p.one_packed(), p.eri)
    g1, g2 = S.gradient(v0)
    irr = p.irreps
    so_pair = next((a, b) for a in range(p.nbf) for b in range(a) if irr[a] != irr[b])
    h_pair = next((a, b) for a in range(p.nbf) for b in range(a) if irr[a] == irr[b])
    zero = int(np.flatnonzero(p.eri == 0)[0])
    probes = [("one", tri(0, 0)), ("one", tri(*h_pair)), ("one", tri(*so_pair)), ("eri", canon_index(1, 1, 2, 2)),
              ("eri", canon_index(0, 1, 0, 1)), ("eri", zero)]
    h = 1e-5
    for tab, t in probes:
        ev = []
        for sgn in (1, -1):
            o, e = p.one_packed().copy(), p.eri.copy()
            (o if tab == "one" else e)[t] += sgn * h
            ev.append(S.solve(o, e)[0])
        fd = (ev[0] - ev[1]) / (2 * h)
        an = (g1 if tab == "one" else g2)[:, t]
        assert np.abs(fd - an).max() <= 1e-6, (tab, t, fd, an)


def test_gradient_feeds_natural_orbitals(oracle_mod):
    """The spin-free part of dE/dh (diagonal as it is, equal-irrep off-diagonal halved) is the
    CIDEN density, so its natural orbitals are those of psoci_density1."""
    from psoci_gb300 import api
    from psoci_gb300.inputs import tri

    p = small_problem("fci_6e8o", 1)
    O = oracle_mod.Oracle(p)
    _, v = _eigvecs(O, 2)
    c = gpu_context(p)
    g1, _ = c.energy_gradient(v)
    D = c.density1(v)
    n = p.nbf
    for r in range(2):
        d = np.zeros_like(g1[r])
        for a in range(n):
            d[tri(a, a)] = g1[r, tri(a, a)]
            for b in range(a):
                if p.irreps[a] == p.irreps[b]:
                    d[tri(a, b)] = 0.5 * g1[r, tri(a, b)]
        occ_g, _ = api.natural_orbitals(d, p.irreps)
        occ_d, _ = api.natural_orbitals(D[r], p.irreps)
        assert np.abs(np.sort(occ_g) - np.sort(occ_d)).max() <= 1e-10
        assert abs(occ_g.sum() - p.nelec) <= 1e-10
    c.close()
