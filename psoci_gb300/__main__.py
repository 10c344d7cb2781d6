"""Solve one double-group symmetry block of a named synthetic workload on one GPU.

  python -m psoci_gb300 --workload mrcisd_6e8o_v24 [--roots 8] [--rtol 1e-5] [--fp64]
                        [--no-davidson] [--sigma K] [--density] [--gradient] [--direct] [--verbose 1]

Determinants -> Hamiltonian (CSR) -> block Davidson; prints the sizes and the total
energies in the layout of the reference driver's "Eigenvalue" lines.  ``--sigma K`` also
applies H to K random vectors once (the Davidson's inner product, on its own);
``--density`` forms the 1-particle densities of the converged roots and prints the
natural-orbital occupations of the first root (diagonal blocks of one orbital label);
``--gradient`` forms dE/d(integral tables) of the converged roots (1-, 2-particle and
spin-orbit densities, derivatives of the non-zero integrals); ``--direct`` stores no matrix
elements (every product evaluates them again).
"""
from __future__ import annotations

import argparse
import time

import numpy as np

from . import api
from .inputs import named_workload


def main(argv=None):
    ap = argparse.ArgumentParser(prog="python -m psoci_gb300")
    ap.add_argument("--workload", default="mrcis_6e8o_v40")
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--ksym", type=int, default=1)
    ap.add_argument("--roots", type=int, default=8)
    ap.add_argument("--rtol", type=float, default=1e-5)
    ap.add_argument("--fp64", action="store_true", help="FP64 elements in sigma (default: FP32 copy)")
    ap.add_argument("--no-davidson", action="store_true")
    ap.add_argument("--sigma", type=int, default=0, help="apply H to this many random vectors once")
    ap.add_argument("--density", action="store_true", help="1-particle densities of the roots")
    ap.add_argument("--gradient", action="store_true", help="energy gradients of the roots")
    ap.add_argument("--direct", action="store_true", help="direct mode: no stored elements")
    ap.add_argument("--eval-launches", type=int, default=0, choices=(0, 1),
                    help="1: the H build's element evaluation in one launch (default 0: two when they fit)")
    ap.add_argument("--max-subspace", type=int, default=48)
    ap.add_argument("--device", type=int, default=0)
    ap.add_argument("--verbose", type=int, default=0)
    a = ap.parse_args(argv)
    p = named_workload(a.workload, seed=a.seed, ksym=a.ksym)
    mixed = not a.fp64
    with api.Context(a.device, verbose=a.verbose) as c:
        c.load_problem(p)
        c.set_eval_launches(a.eval_launches)
        t0 = time.perf_counter()
        c.build_determinants()
        nnz = c.build_hamiltonian(mixed=mixed, direct=a.direct)
        tb = time.perf_counter() - t0
        print(f"workload {a.workload}: configurations {p.nconf}, SEFs {c.nsef}, stored elements {nnz}, "
              f"build {tb:.3f} s")
        if a.verbose:
            b = c.build_stats()
            print("build phases (CUDA events, ms): " + ", ".join(
                f"{k[:-3]} {b[k]:.2f}" for k in ("screen_ms", "evaluate_ms", "rows_ms", "assemble_ms", "total_ms")))
        if a.sigma:
            X = np.random.default_rng(0).standard_normal((c.nsef, a.sigma))
            Y = c.sigma(X, prec=api.PREC_MIXED if mixed else api.PREC_FP64)
            print(f"sigma on {a.sigma} vectors: |HX|_max {np.abs(Y).max():.6e}")
        if not a.no_davidson:
            r = c.davidson(a.roots, rtol=a.rtol, mixed=mixed, refine=True, max_subspace=a.max_subspace,
                           want_vectors=a.density or a.gradient)
            ecore = c.core_energy()
            for i, e in enumerate(r.evals):
                print(f"Eigenvalue {i + 1:4d} Total energy (au) {e + ecore:20.12f} Electronic (au) {e:20.12f}")
            print(f"iterations {r.iterations}, sigma vectors {r.sigma_calls}, {r.seconds:.3f} s")
            if a.gradient:
                t0 = time.perf_counter()
                g1, g2 = c.energy_gradient(r.evecs, nonzero_only=True)
                tg = time.perf_counter() - t0
                diag = [q * (q + 1) // 2 + q for q in range(p.nbf)]
                print(f"energy gradient of {len(r.evals)} roots: {tg:.3f} s; traces of dE/dh_pp "
                      + np.array2string(g1[:, diag].sum(1), precision=10))
            if a.density:
                for rep in range(2):  # the first call also forms the configuration groups
                    t0 = time.perf_counter()
                    d = c.density1(r.evecs)
                    td = time.perf_counter() - t0
                    print(f"density1 of {len(r.evals)} roots ({'with' if rep == 0 else 'groups kept'}): "
                          f"{td * 1e3:.2f} ms")
                occ, _ = api.natural_orbitals(d[0], p.irreps)
                tr = d[:, [q * (q + 1) // 2 + q for q in range(p.nbf)]].sum(1)
                print(f"traces {np.array2string(tr, precision=10)}; largest NO occupations, root 1: "
                      + " ".join(f"{x:.6f}" for x in np.sort(occ)[::-1][:8]))


if __name__ == "__main__":
    main()
