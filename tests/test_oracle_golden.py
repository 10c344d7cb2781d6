"""The oracle (C restatement) against golden fixtures produced by the reference's own code.

The fixtures in tests/golden/ were generated by tests/golden/make_golden.py from the
reference's compute sources compiled unchanged (oracle/_ref).  Determinant tables and the
lower-triangle CSR structure must match bit for bit; element values are compared exactly
as well (same operation order, IEEE arithmetic, no contraction).
"""
import glob
import os

import numpy as np
import pytest
import scipy.linalg as sla

from helpers import lower_to_full
from psoci_gb300.inputs import Problem

GOLD = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz")))


def load(path):
    z = np.load(path)
    p = Problem(nbf=int(z["nbf"]), nelec=int(z["nelec"]), ksym=int(z["ksym"]), mx_open=int(z["mx_open"]),
                jsym=z["jsym"], occ=z["occ"], h=z["h"], so=z["so"], eri=z["eri"])
    return p, z


def test_fixtures_present():
    assert len(GOLD) >= 7


@pytest.mark.parametrize("path", GOLD, ids=[os.path.basename(g)[:-4] for g in GOLD])
def test_oracle_matches_golden(oracle_mod, path):
    p, z = load(path)
    O = oracle_mod.Oracle(p)
    assert (O.config_counts() == z["counts"]).all()
    dets = np.concatenate([O.config_dets(i) for i in range(p.nconf)], 0)
    assert (dets == z["dets"].astype(np.int32)).all()
    rp, ci, va = O.build_lower(2)
    assert (rp == z["rowptr"]).all()
    assert (ci == z["cols"]).all()
    assert np.array_equal(va, z["vals"]), np.abs(va - z["vals"]).max()
    F = lower_to_full(rp, ci, va, len(rp) - 1)
    ev = sla.eigvalsh(F.toarray())[:len(z["evals"])]
    assert np.abs(ev - z["evals"]).max() < 1e-10


def test_fixture_covers_all_template_classes():
    """Together the fixtures exercise even/odd electron counts and 0..11 open shells."""
    seen = set()
    for path in GOLD:
        _, z = load(path)
        for no in np.unique(z["counts"][:, 2]):
            seen.add((int(z["nelec"]) % 2, int(no)))
    assert {(1, 11), (0, 10), (0, 6), (1, 5), (0, 0)} <= seen


@pytest.mark.parametrize("path", GOLD, ids=[os.path.basename(g)[:-4] for g in GOLD])
def test_density1_matches_golden(oracle_mod, path):
    """The CIDEN 1-particle density of two seeded unit vectors, bit for bit."""
    p, z = load(path)
    d = oracle_mod.Oracle(p).density1(z["dvec"])
    assert np.array_equal(d, z["dens"]), np.abs(d - z["dens"]).max()
    tr = d[:, [k * (k + 1) // 2 + k for k in range(p.nbf)]].sum(1)
    assert np.abs(tr - p.nelec).max() < 1e-12
