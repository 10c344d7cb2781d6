"""Synthetic inputs and the PSOCI configuration-file format (host logic, no GPU)."""
import numpy as np
import pytest

from psoci_gb300 import inputs


def test_named_workload_sizes():
    """SEF counts of the benchmark workloads (nsef per config from PsociDeterminants.C:954)."""
    want = {"fci_6e12o": (8074, 33814), "mrcis_6e8o_v40": (20944, 89404), "mrcisd_4e6o_v30": (11355, 32775)}
    for name, (nconf, nsef) in want.items():
        p = inputs.named_workload(name, seed=1, ksym=1)
        assert p.nconf == nconf
        assert p.num_sefs() == nsef


def test_closed_shells_only_in_matching_parity_block():
    p1 = inputs.named_workload("fci_4e6o", seed=0, ksym=1)
    p2 = inputs.named_workload("fci_4e6o", seed=0, ksym=2)
    closed1 = int(((p1.occ == 1).sum(1) == 0).sum())
    closed2 = int(((p2.occ == 1).sum(1) == 0).sum())
    assert closed1 > 0 and closed2 == 0


def test_integral_symmetry_rules():
    rng = np.random.default_rng(3)
    nbf = 8
    irr = inputs.make_irreps(nbf, rng)
    h, so, eri = inputs.make_integrals(nbf, irr, 4, rng)
    assert np.allclose(h, h.T) and np.allclose(so, -so.T)
    same = irr[:, None] == irr[None, :]
    assert (h[~same] == 0).all() and (so[same] == 0).all()
    # packed eri: zero unless the four irreps XOR to zero
    n1 = nbf * (nbf + 1) // 2
    assert eri.shape == (n1 * (n1 + 1) // 2,)
    i, j = np.tril_indices(nbf)
    pairs = list(zip(i, j))
    t = 0
    for a in range(n1):
        for b in range(a + 1):
            p, q = pairs[a]
            r, s = pairs[b]
            if ((irr[p] - 1) ^ (irr[q] - 1) ^ (irr[r] - 1) ^ (irr[s] - 1)) != 0:
                assert eri[t] == 0.0
            t += 1


def test_config_file_round_trip(tmp_path):
    p = inputs.named_workload("fci_5e6o", seed=2, ksym=3)
    f = tmp_path / "configs"
    inputs.write_config_file(str(f), p)
    nbf, nelec, ksym, mx, js, occ = inputs.read_config_file(str(f))
    assert (nbf, nelec, ksym, mx) == (p.nbf, p.nelec, p.ksym, p.mx_open)
    assert (js == p.jsym).all() and (occ == p.occ).all()


def test_config_file_all_open_shell_rule(tmp_path):
    """The reference rejects configurations without a doubly occupied orbital
    (PsociConfigs.C:247); this reader accepts them unless asked not to."""
    f = tmp_path / "configs"
    f.write_text("t\n4 2 1 2 2\n1 1100\n1 2000\n")
    inputs.read_config_file(str(f))
    with pytest.raises(ValueError):
        inputs.read_config_file(str(f), allow_all_open=False)


@pytest.mark.parametrize("bad", ["t\n4 2 1 3 2\n1 1100\n1 2000\n", "t\n4 2 1 1 2\n1 1110\n", "t\n4 2 1 1 2\n1 11a0\n",
                                 "t\n"])
def test_config_file_rejects_corrupt(tmp_path, bad):
    f = tmp_path / "configs"
    f.write_text(bad)
    with pytest.raises(ValueError):
        inputs.read_config_file(str(f))
