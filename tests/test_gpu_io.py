"""GPU tests of the host-facing pieces: the C++ driver, the H checkpoint and vector restart."""
import os
import re
import subprocess

import numpy as np
import pytest
import scipy.linalg as sla

from helpers import lower_to_full, small_problem

pytestmark = pytest.mark.gpu


def _ref_evals(oracle_mod, p, k):
    O = oracle_mod.Oracle(p)
    rp, ci, va = O.build_lower(4)
    return sla.eigvalsh(lower_to_full(rp, ci, va, O.num_sefs()).toarray())[:k]


def test_cpp_driver(tmp_path, oracle_mod):
    from psoci_gb300 import build, inputs

    build.build()
    p = small_problem("fci_6e8o", 1)
    cfg, ints = str(tmp_path / "configs"), str(tmp_path / "ints.bin")
    inputs.write_config_file(cfg, p)
    inputs.write_integral_file(ints, p)
    vec = str(tmp_path / "vectors.txt")
    out = subprocess.run([build.DRIVER, "-c", cfg, "-m", ints, "-n", "4", "-F", "1e-7", "-p", "1", "-v", vec],
                         capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    ev = [float(m.group(1)) for m in re.finditer(r"Electronic \(au\) (\S+)", out.stdout)]
    ref = _ref_evals(oracle_mod, p, 4)
    assert len(ev) == 4 and np.abs(np.array(ev) - ref).max() <= 1e-7
    assert os.path.exists(vec)
    # restart from the written vectors converges immediately
    out2 = subprocess.run([build.DRIVER, "-c", cfg, "-m", ints, "-n", "4", "-F", "1e-7", "-p", "0", "-v", vec, "-r"],
                          capture_output=True, text=True, timeout=300)
    assert out2.returncode == 0, out2.stderr
    iters = int(re.search(r"Number of total iterations is (\d+)", out2.stdout).group(1))
    assert iters <= 3
    # -N: natural-orbital occupations of each root, from its density through the C++ mirror
    out3 = subprocess.run([build.DRIVER, "-c", cfg, "-m", ints, "-n", "2", "-F", "1e-8", "-p", "0", "-v", vec, "-N"],
                          capture_output=True, text=True, timeout=300)
    assert out3.returncode == 0, out3.stderr
    rows = re.findall(r"NO occupations root (\d+) (.*)", out3.stdout)
    assert [int(r[0]) for r in rows] == [0, 1]
    for _, vals in rows:
        occ = np.array([float(x) for x in vals.split()])
        assert occ.max() <= 2.0 + 1e-9 and occ.min() >= -1e-9 and (np.diff(occ) <= 1e-12).all()


def test_hamiltonian_checkpoint(tmp_path):
    from psoci_gb300 import api

    p = small_problem("fci_5e6o", 2)
    path = str(tmp_path / "h.bin")
    with api.Context(0) as c:
        c.load_problem(p)
        c.build_determinants()
        c.build_hamiltonian(mixed=True)
        ref = c.get_hamiltonian()
        c.save_hamiltonian(path)
        e0 = c.davidson(3, rtol=1e-8, mixed=False).evals
    with api.Context(0) as c:
        c.load_problem(p)
        c.build_determinants()
        c.load_hamiltonian(path)
        got = c.get_hamiltonian()
        for a, b in zip(ref, got):
            assert np.array_equal(a, b)
        assert np.abs(c.davidson(3, rtol=1e-8, mixed=True).evals - e0).max() < 1e-9
    # corrupt payload, truncated file, other configurations
    data = bytearray(open(path, "rb").read())
    data[-100] ^= 0xFF
    bad = str(tmp_path / "bad.bin")
    open(bad, "wb").write(bytes(data))
    short = str(tmp_path / "short.bin")
    open(short, "wb").write(bytes(data[: len(data) // 3]))
    other = small_problem("fci_5e6o", 2, seed=99)
    with api.Context(0) as c:
        c.load_problem(p)
        c.build_determinants()
        for f in (bad, short, str(tmp_path / "missing.bin")):
            with pytest.raises(api.PsociError) as e:
                c.load_hamiltonian(f)
            assert e.value.status == 9
    with api.Context(0) as c:
        q = other
        q.occ = q.occ[::-1].copy()
        q.jsym = q.jsym[::-1].copy()
        c.load_problem(q)
        c.build_determinants()
        with pytest.raises(api.PsociError):
            c.load_hamiltonian(path)


def test_restart_guess():
    from psoci_gb300 import api

    p = small_problem("fci_6e8o", 4)
    with api.Context(0) as c:
        c.load_problem(p)
        c.build_determinants()
        c.build_hamiltonian(mixed=True)
        r1 = c.davidson(4, rtol=1e-7, mixed=False, want_vectors=True)
        c.set_guess(r1.evecs)
        r2 = c.davidson(4, rtol=1e-7, mixed=False)
        assert r2.iterations <= 2
        assert np.abs(r2.evals - r1.evals).max() < 1e-10
        c.set_guess(None)


def test_bad_inputs_rejected():
    from psoci_gb300 import api

    p = small_problem("fci_4e6o", 1)
    with api.Context(0) as c:
        occ = p.occ.copy()
        occ[0, 0] = 3
        with pytest.raises(api.PsociError):
            c.set_configs(p.nbf, p.nelec, p.ksym, p.mx_open, p.jsym, occ)
        with pytest.raises(api.PsociError):
            c.set_configs(p.nbf, p.nelec + 1, p.ksym, p.mx_open, p.jsym, p.occ)
        with pytest.raises(api.PsociError):  # sigma before any H
            c.sigma(np.zeros((3, 1)))


def test_bad_inputs_reported_in_order_on_large_lists():
    """Large configuration lists are checked on all host cores; the lowest failing
    configuration is the one reported, with its own message."""
    from psoci_gb300 import api
    from psoci_gb300.inputs import named_workload

    p = named_workload("mrcisd_6e8o_v16", seed=1, ksym=1)
    assert p.nconf > 40000
    with api.Context(0) as c:
        occ = p.occ.copy()
        occ[40000, 3] = 3
        nel = occ[30001].astype(int)
        q = int(np.nonzero(nel == 0)[0][0])
        occ[30001, q] = 1  # one electron too many
        with pytest.raises(api.PsociError, match="configuration 30001 holds"):
            c.set_configs(p.nbf, p.nelec, p.ksym, p.mx_open, p.jsym, occ)
        occ[30001, q] = 0
        with pytest.raises(api.PsociError, match="configuration 40000 orbital 3 occupation 3"):
            c.set_configs(p.nbf, p.nelec, p.ksym, p.mx_open, p.jsym, occ)
        c.set_configs(p.nbf, p.nelec, p.ksym, p.mx_open, p.jsym, p.occ)


def test_cpp_reference_loop(tmp_path, oracle_mod):
    """-L: the reference's own Davidson loop (one vector per iteration, coarse then final
    tolerance, collapse to 2 x roots) through the step-level PsociGAbasis / PsociGAsubspace
    methods of the C++ mirror, against the one-call solve and the oracle's spectrum."""
    from psoci_gb300 import build, inputs

    build.build()
    p = small_problem("fci_6e8o", 1)
    cfg, ints = str(tmp_path / "configs"), str(tmp_path / "ints.bin")
    inputs.write_config_file(cfg, p)
    inputs.write_integral_file(ints, p)
    ref = _ref_evals(oracle_mod, p, 4)
    runs = {}
    for name, extra in (("solve", ["-p", "0"]), ("loop", ["-L"])):
        vec = str(tmp_path / f"v_{name}.txt")
        out = subprocess.run([build.DRIVER, "-c", cfg, "-m", ints, "-n", "4", "-F", "1e-8", "-x", "4", "-v", vec] + extra,
                             capture_output=True, text=True, timeout=300)
        assert out.returncode == 0, out.stderr
        ev = np.array([float(m.group(1)) for m in re.finditer(r"Electronic \(au\) (\S+)", out.stdout)])
        iters = int(re.search(r"Number of total iterations is (\d+)", out.stdout).group(1))
        coll = int(re.search(r"Number of SUBSPACE contractions is (\d+)", out.stdout).group(1))
        runs[name] = (ev, iters, coll, vec)
    ev_s, _, _, _ = runs["solve"]
    ev_l, it_l, coll_l, vec_l = runs["loop"]
    assert len(ev_l) == 4
    assert np.abs(ev_l - ev_s).max() <= 1e-10, (ev_l, ev_s)
    assert np.abs(ev_l - ref).max() <= 1e-10
    assert it_l > 4 and coll_l >= 1  # one vector per iteration, with collapses
    # the loop's vectors restart the loop: already converged at the coarse and final tolerance
    out = subprocess.run([build.DRIVER, "-c", cfg, "-m", ints, "-n", "4", "-F", "1e-8", "-v", vec_l, "-r", "-L"],
                         capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    assert int(re.search(r"Number of total iterations is (\d+)", out.stdout).group(1)) <= 3
