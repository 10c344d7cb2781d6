"""Shared helpers for the parity tests."""
import numpy as np
import scipy.sparse as sp

from psoci_gb300.inputs import Problem, config_jsym, make_integrals, make_irreps, named_workload


def lower_to_full(rp, ci, va, n):
    """Full symmetric CSR (rows sorted by column) from lower-triangle storage."""
    L = sp.csr_matrix((va, ci, rp), shape=(n, n))
    D = sp.diags(L.diagonal())
    F = (L + L.T - D).tocsr()
    F.sort_indices()
    return F


def det_lists_to_bits(dets, nbf):
    """oracle/reference det rows -> (alpha bits, beta bits, ms, phase) as python ints."""
    out = []
    for row in dets:
        na, nb, ms, ph = int(row[0]), int(row[1]), int(row[2]), int(row[3])
        a = sum(1 << int(x) for x in row[6:6 + na])
        b = sum(1 << int(x) for x in row[6 + nbf:6 + nbf + nb])
        out.append((a, b, ms, ph))
    return out


def gpu_bits(words_row):
    v = 0
    for w, x in enumerate(words_row):
        v |= int(x) << (64 * w)
    return v


def high_open_problem(nbf=14, seed=5, nelec=10, ksym=1, per=2):
    """A small configuration list reaching 8-11 open shells."""
    rng = np.random.default_rng(seed)
    irr = make_irreps(nbf, rng)
    h, so, eri = make_integrals(nbf, irr, nbf, rng)
    occs = []
    for nopen in range(nelec % 2, min(nelec, 11) + 1, 2):
        ndbl = (nelec - nopen) // 2
        if ndbl + nopen > nbf:
            continue
        for _ in range(per):
            perm = rng.permutation(nbf)
            o = np.zeros(nbf, np.uint8)
            o[perm[:ndbl]] = 2
            o[perm[ndbl:ndbl + nopen]] = 1
            occs.append(o)
    occ = np.array(occs)
    js = config_jsym(occ, irr)
    return Problem(nbf=nbf, nelec=nelec, ksym=ksym, mx_open=int((occ == 1).sum(1).max()), jsym=js, occ=occ, h=h,
                   so=so, eri=eri, irreps=irr)


# problems small enough for the oracle to finish in seconds
SMALL_CASES = [
    ("fci_4e6o", 1), ("fci_4e6o", 2), ("fci_4e6o", 3), ("fci_4e6o", 4),
    ("fci_5e6o", 1), ("fci_5e6o", 2),
    ("fci_6e8o", 1), ("fci_6e8o", 4),
]


def small_problem(name, ksym, seed=3):
    return named_workload(name, seed=seed, ksym=ksym)


def gpu_context(p):
    """A GPU context with the problem loaded and its determinants built."""
    from psoci_gb300 import api

    c = api.Context(0)
    c.load_problem(p)
    c.build_determinants()
    return c


def check_h_against_oracle(c, O, p, tol=1e-12, mixed=True, nthreads=0):
    """Build H on the GPU and compare it with the oracle's lower triangle mirrored: equal
    row pointers and columns, values and diagonal within tol.  Returns the full oracle CSR."""
    rp, ci, va = O.build_lower(nthreads)
    n = O.num_sefs()
    F = lower_to_full(rp, ci, va, n)
    c.build_hamiltonian(mixed=mixed)
    grp, gci, gva = c.get_hamiltonian()
    assert c.nnz == F.nnz
    assert (grp == F.indptr).all()
    assert (gci == F.indices).all()
    diff = np.abs(gva - F.data).max() if F.nnz else 0.0
    assert diff <= tol, diff
    d = c.get_diag()
    assert np.abs(d - O.diag()).max() <= tol
    return F
