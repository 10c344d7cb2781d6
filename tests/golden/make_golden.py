"""Generate tests/golden/*.npz from the reference's own compute sources.

Runs the reference harness (oracle/_ref/libpsoci_ref.so: PsociConfigs, PsociDeterminants,
PsociIntegrals and PsociHamiltonian compiled unchanged against a single-process GA/MPI
shim) on small seeded synthetic problems and stores, per problem:

* the inputs (occupations, jsym, nbf, nelec, ksym, mx_open, h, so, packed eri);
* per-configuration ndet / nsef / nopen and the full determinant table
  (nalpha, nbeta, spin projection, phase, sums, sorted alpha / beta lists);
* the lower-triangle Hamiltonian in CSR as packSefsef keeps it;
* the lowest eigenvalues of the assembled symmetric matrix (dense LAPACK);
* two seeded unit vectors and their packed 1-particle densities from the reference's
  CIDEN element path (generateSOCIblocksForCIDEN + transformSEFSEFtoMOGET).

Needs the reference tree (only in the build container).  Usage:
    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np
import scipy.linalg as sla

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

import oracle  # noqa: E402
from helpers import high_open_problem, lower_to_full  # noqa: E402
from psoci_gb300.inputs import make_problem, named_workload  # noqa: E402

CASES = {
    "fci_4e6o_k1": lambda: named_workload("fci_4e6o", seed=11, ksym=1),
    "fci_4e6o_k2": lambda: named_workload("fci_4e6o", seed=11, ksym=2),
    "fci_5e6o_k1": lambda: named_workload("fci_5e6o", seed=12, ksym=1),
    "fci_5e6o_s22": lambda: named_workload("fci_5e6o", seed=22, ksym=2),
    "mrcis_4e4o_v6_k3": lambda: make_problem("mrcis", seed=13, ksym=3, nact=4, nelec=4, nvirt=6),
    "open10_k1": lambda: high_open_problem(nbf=12, seed=14, nelec=10, ksym=1, per=1),
    "open11_k2": lambda: high_open_problem(nbf=12, seed=15, nelec=11, ksym=2, per=1),
}


def main():
    oracle.build(ref=True)
    devnull = os.open(os.devnull, os.O_WRONLY)
    saved = os.dup(1)
    for name, mk in CASES.items():
        p = mk()
        os.dup2(devnull, 1)  # the reference prints its integral tables
        try:
            R = oracle.Reference(p)
            counts = R.config_counts()
            dets = np.concatenate([R.config_dets(i) for i in range(p.nconf)], 0)
            rp, ci, va = R.build_lower(4)
            n = int(counts[:, 1].sum())
            dvec = np.random.default_rng(7).standard_normal((2, n))
            dvec /= np.linalg.norm(dvec, axis=1, keepdims=True)
            dens = R.density1(dvec)
        finally:
            os.dup2(saved, 1)
        F = lower_to_full(rp, ci, va, n)
        nev = min(8, n)
        ev = sla.eigvalsh(F.toarray())[:nev]
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), nbf=p.nbf, nelec=p.nelec, ksym=p.ksym,
                            mx_open=p.mx_open, jsym=p.jsym, occ=p.occ, h=p.h, so=p.so, eri=p.eri, counts=counts,
                            dets=dets.astype(np.int16), rowptr=rp, cols=ci, vals=va, evals=ev, dvec=dvec, dens=dens)
        print(f"{name}: nconf={p.nconf} N={n} nnz_lower={len(ci)} ev0={ev[0]:.10f}")


if __name__ == "__main__":
    main()
