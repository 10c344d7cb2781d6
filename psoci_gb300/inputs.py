"""Seeded synthetic PSOCI inputs: orbital irreps, integrals and configuration spaces.

The reference reads Columbus SIFS integrals and a PSOCI configuration file
(``PsociConfigs.C:126-302``: title; ``nbf nelec ksym ncfgs nopen``; ``jsym occstring``
lines).  No molecular data ships with it, so every workload here is synthetic, with
the distributions the benchmark configurations name:

* orbital irreps in {1..4}; the product rule is XOR on ``label-1`` so a
  configuration's ``jsym = 1 + XOR(irrep-1 over singly occupied orbitals)``;
* ``h_pp ~ U(-5,-1)`` (reference / active orbitals), ``U(0.2,3)`` (virtuals);
  ``h_pq ~ N(0, 0.05)`` symmetric, only between orbitals of equal irrep;
* spin-orbit ``SO_pq ~ N(0, 5e-3)``, real antisymmetric, only between orbitals of
  different irrep.  The reference stores h and SO in one packed triangle and lets SO
  records overwrite (``PsociIntegrals.C:505-535``), so the two supports must be
  disjoint;
* ``(pq|rs) = 0.5 exp(-|p-q|-|r-s|) U(0.5,1)``, 8-fold symmetric, zero unless the
  four irreps XOR to zero; ``(pp|qq) ~ U(0.3,0.8)``.

Closed-shell configurations belong only to ksym blocks with ``jsym%2 == ksym%2``
(``PsociHamiltonian.C:1489-1495``); other blocks drop them.
"""
from __future__ import annotations

import dataclasses
import itertools
from typing import Optional

import numpy as np


def tri(i, j):
    """0-based packed position of (max(i,j), min(i,j)) in a lower triangle."""
    a = np.maximum(i, j)
    b = np.minimum(i, j)
    return a * (a + 1) // 2 + b


def canon_index(i, j, k, l):
    """0-based position of (ij|kl) in the canonical 8-fold packed two-electron table."""
    return tri(tri(i, j), tri(k, l))


def n_eri(nbf: int) -> int:
    n1 = nbf * (nbf + 1) // 2
    return n1 * (n1 + 1) // 2


@dataclasses.dataclass
class Problem:
    """One double-group symmetry block: configurations plus integrals."""

    nbf: int
    nelec: int
    ksym: int
    mx_open: int
    jsym: np.ndarray  # int32 [nconf], 1-based
    occ: np.ndarray  # uint8 [nconf, nbf], 0/1/2
    h: np.ndarray  # float64 [nbf, nbf] symmetric
    so: np.ndarray  # float64 [nbf, nbf] antisymmetric
    eri: np.ndarray  # float64 [n_eri(nbf)] canonical packed
    ecore: float = 0.0
    irreps: Optional[np.ndarray] = None
    name: str = ""
    seed: int = 0

    @property
    def nconf(self) -> int:
        return int(self.occ.shape[0])

    def nopen(self) -> np.ndarray:
        return (self.occ == 1).sum(axis=1).astype(np.int32)

    def nsef(self) -> np.ndarray:
        k = np.maximum(self.nopen() - 1, 0)
        return ((1 << (k // 2)) ** 2).astype(np.int64)

    def ndet(self) -> np.ndarray:
        k = np.maximum(self.nopen() - 1, 0)
        return (1 << k).astype(np.int64)

    def num_sefs(self) -> int:
        return int(self.nsef().sum())

    def one_packed(self) -> np.ndarray:
        """Packed 1-e table as the reference holds it (SO overwrites h off the diagonal)."""
        n = self.nbf
        i, j = np.tril_indices(n)
        out = np.zeros(n * (n + 1) // 2)
        hv = self.h[i, j]
        sv = np.where(i != j, self.so[i, j], 0.0)
        out[tri(i, j)] = np.where(sv != 0.0, sv, hv)
        return out


# ----------------------------------------------------------------------------------
# integrals
# ----------------------------------------------------------------------------------
def make_irreps(nbf: int, rng: np.random.Generator, nirrep: int = 4) -> np.ndarray:
    return rng.integers(1, nirrep + 1, size=nbf).astype(np.int32)


def make_integrals(nbf: int, irreps: np.ndarray, n_ref: int, rng: np.random.Generator):
    """h, so, packed eri.  Orbitals [0, n_ref) are reference (occupied/active) orbitals."""
    irr = irreps.astype(np.int64) - 1
    h = np.zeros((nbf, nbf))
    diag = np.where(np.arange(nbf) < n_ref, rng.uniform(-5.0, -1.0, nbf), rng.uniform(0.2, 3.0, nbf))
    off = rng.normal(0.0, 0.05, (nbf, nbf))
    off = np.tril(off, -1)
    same = irr[:, None] == irr[None, :]
    h = np.where(same, off + off.T, 0.0)
    h[np.diag_indices(nbf)] = diag
    s = rng.normal(0.0, 5e-3, (nbf, nbf))
    s = np.tril(s, -1)
    so = np.where(~same, s - s.T, 0.0)

    n1 = nbf * (nbf + 1) // 2
    n2 = n1 * (n1 + 1) // 2
    # pair tables
    pi, pj = np.tril_indices(nbf)
    pair_i = np.empty(n1, np.int64)
    pair_j = np.empty(n1, np.int64)
    pair_i[tri(pi, pj)] = pi
    pair_j[tri(pi, pj)] = pj
    P = np.arange(n2, dtype=np.int64)
    IJ = ((np.sqrt(8.0 * P + 1.0) - 1.0) // 2).astype(np.int64)
    # fix rounding at the boundaries
    IJ = np.where(IJ * (IJ + 1) // 2 > P, IJ - 1, IJ)
    IJ = np.where((IJ + 1) * (IJ + 2) // 2 <= P, IJ + 1, IJ)
    KL = P - IJ * (IJ + 1) // 2
    i, j, k, l = pair_i[IJ], pair_j[IJ], pair_i[KL], pair_j[KL]
    allowed = (irr[i] ^ irr[j] ^ irr[k] ^ irr[l]) == 0
    u = rng.uniform(0.5, 1.0, n2)
    val = 0.5 * np.exp(-np.abs(i - j) - np.abs(k - l)) * u
    coul = (i == j) & (k == l)
    val = np.where(coul, rng.uniform(0.3, 0.8, n2), val)
    eri = np.where(allowed, val, 0.0)
    return h, so, eri


# ----------------------------------------------------------------------------------
# configuration spaces
# ----------------------------------------------------------------------------------
def occupations(norb: int, nel: int) -> np.ndarray:
    """All 0/1/2 occupation vectors of ``nel`` electrons in ``norb`` orbitals,
    ordered lexicographically with 2 > 1 > 0 (aufbau-first)."""
    if nel < 0 or nel > 2 * norb:
        return np.zeros((0, norb), np.uint8)
    out = []

    def rec(prefix, left, pos):
        if pos == norb:
            if left == 0:
                out.append(prefix.copy())
            return
        rem = norb - pos - 1
        for o in (2, 1, 0):
            if o <= left and left - o <= 2 * rem:
                prefix.append(o)
                rec(prefix, left - o, pos + 1)
                prefix.pop()

    rec([], nel, 0)
    return np.array(out, dtype=np.uint8).reshape(-1, norb)


def config_jsym(occ: np.ndarray, irreps: np.ndarray) -> np.ndarray:
    irr = irreps.astype(np.int64) - 1
    x = np.zeros(occ.shape[0], np.int64)
    for p in range(occ.shape[1]):
        x ^= np.where(occ[:, p] == 1, irr[p], 0)
    return (x + 1).astype(np.int32)


def fci_space(nbf: int, nelec: int) -> np.ndarray:
    return occupations(nbf, nelec)


def mrci_space(nact: int, nelec: int, nvirt: int, level: int) -> np.ndarray:
    """Full-CI reference of ``nelec`` in ``nact`` orbitals plus all single (level 1)
    or single and double (level 2) excitations into ``nvirt`` virtuals."""
    blocks = [np.concatenate([occupations(nact, nelec), np.zeros((len(occupations(nact, nelec)), nvirt), np.uint8)], 1)]
    if level >= 1:
        act = occupations(nact, nelec - 1)
        for a in range(nvirt):
            v = np.zeros((len(act), nvirt), np.uint8)
            v[:, a] = 1
            blocks.append(np.concatenate([act, v], 1))
    if level >= 2:
        act = occupations(nact, nelec - 2)
        for b in range(nvirt):
            for a in range(b + 1):
                v = np.zeros((len(act), nvirt), np.uint8)
                if a == b:
                    v[:, a] = 2
                else:
                    v[:, a] = 1
                    v[:, b] = 1
                blocks.append(np.concatenate([act, v], 1))
    return np.concatenate(blocks, 0)


def select_block(occ: np.ndarray, jsym: np.ndarray, ksym: int):
    """Drop closed-shell configurations whose jsym parity differs from ksym's."""
    closed = (occ == 1).sum(axis=1) == 0
    keep = ~closed | ((jsym % 2) == (ksym % 2))
    return occ[keep], jsym[keep]


def make_problem(kind: str, seed: int = 0, ksym: int = 1, **kw) -> Problem:
    """Named synthetic workloads.

    ``fci``    : full CI, kw ``nbf`` (12), ``nelec`` (6)
    ``mrcis``  : kw ``nact`` (8), ``nelec`` (6), ``nvirt`` (40)
    ``mrcisd`` : kw ``nact`` (8 or 6), ``nelec``, ``nvirt``
    """
    rng = np.random.default_rng(seed)
    if kind == "fci":
        nbf = kw.get("nbf", 12)
        nelec = kw.get("nelec", 6)
        occ = fci_space(nbf, nelec)
        n_ref = nbf
    elif kind in ("mrcis", "mrcisd"):
        nact = kw.get("nact", 8)
        nelec = kw.get("nelec", 6)
        nvirt = kw.get("nvirt", 40)
        nbf = nact + nvirt
        occ = mrci_space(nact, nelec, nvirt, 1 if kind == "mrcis" else 2)
        n_ref = nact
    else:
        raise ValueError(f"unknown workload kind {kind!r}")
    irreps = make_irreps(nbf, rng, kw.get("nirrep", 4))
    h, so, eri = make_integrals(nbf, irreps, n_ref, rng)
    if kw.get("no_so", False):
        so[:] = 0.0
    jsym = config_jsym(occ, irreps)
    occ, jsym = select_block(occ, jsym, ksym)
    limit = kw.get("max_configs")
    if limit is not None:
        occ, jsym = occ[:limit], jsym[:limit]
    mx_open = int((occ == 1).sum(axis=1).max()) if len(occ) else 0
    ecore = float(kw.get("ecore", 0.0))
    return Problem(nbf=nbf, nelec=nelec, ksym=ksym, mx_open=mx_open, jsym=np.ascontiguousarray(jsym, np.int32),
                   occ=np.ascontiguousarray(occ, np.uint8), h=h, so=so, eri=eri, ecore=ecore, irreps=irreps,
                   name=f"{kind}:{kw}", seed=seed)


# ----------------------------------------------------------------------------------
# PSOCI configuration file (PsociConfigs.C:126-302 format)
# ----------------------------------------------------------------------------------
def write_config_file(path: str, p: Problem, title: str = "psoci-gb300 synthetic") -> None:
    with open(path, "w") as f:
        f.write(title + "\n")
        f.write(f"{p.nbf} {p.nelec} {p.ksym} {p.nconf} {p.mx_open}\n")
        for js, row in zip(p.jsym, p.occ):
            f.write(f"{int(js)} {''.join(str(int(x)) for x in row)}\n")


def read_config_file(path: str, allow_all_open: bool = True):
    """Parse a PSOCI configuration file.  Returns (nbf, nelec, ksym, mx_open, jsym, occ).

    The reference rejects configurations with no doubly occupied orbital
    (``PsociConfigs.C:247``: ``!(ielec-iopen) % 2``); ``allow_all_open`` (default)
    accepts them, ``False`` reproduces the rejection as a ValueError.
    """
    with open(path) as f:
        lines = [ln.rstrip("\n") for ln in f]
    if len(lines) < 2:
        raise ValueError("configuration file too short")
    hdr = lines[1].split()
    if len(hdr) < 5:
        raise ValueError("bad header line: expected nbf nelec ksym ncfgs nopen")
    nbf, nelec, ksym, ncfg, nopen_hdr = (int(x) for x in hdr[:5])
    body = [ln.split() for ln in lines[2:] if ln.strip()]
    if len(body) != ncfg:
        raise ValueError(f"header says {ncfg} configurations, file holds {len(body)}")
    jsym = np.empty(ncfg, np.int32)
    occ = np.empty((ncfg, nbf), np.uint8)
    for t, parts in enumerate(body):
        if len(parts) != 2 or len(parts[1]) != nbf or any(ch not in "012" for ch in parts[1]):
            raise ValueError(f"bad configuration line {t + 3}")
        jsym[t] = int(parts[0])
        occ[t] = np.frombuffer(parts[1].encode(), np.uint8) - ord("0")
        ne = int(occ[t].sum())
        if ne != nelec:
            raise ValueError(f"configuration {t + 1} holds {ne} electrons, header says {nelec}")
        nop = int((occ[t] == 1).sum())
        if not allow_all_open and nop == ne:
            raise ValueError(f"configuration {t + 1} has no doubly occupied orbital (reference rejects it)")
    mx_open = int((occ == 1).sum(axis=1).max())
    return nbf, nelec, ksym, mx_open, jsym, occ


def write_integral_file(path: str, p: Problem) -> None:
    """Binary integral file for the C++ driver: "PSOCIINT", int32 nbf, float64 ecore,
    packed one-electron table (SO folded in), canonical two-electron table."""
    with open(path, "wb") as f:
        f.write(b"PSOCIINT")
        f.write(np.int32(p.nbf).tobytes())
        f.write(np.float64(p.ecore).tobytes())
        f.write(np.ascontiguousarray(p.one_packed(), np.float64).tobytes())
        f.write(np.ascontiguousarray(p.eri, np.float64).tobytes())


def named_workload(name: str, seed: int = 0, ksym: int = 1) -> Problem:
    """The workloads the benchmark configurations name."""
    table = {
        # valence full CI: 12 orbitals, 6 electrons
        "fci_6e12o": ("fci", dict(nbf=12, nelec=6)),
        # MRCIS: CAS(6e,8o) reference + singles into 40 virtuals
        "mrcis_6e8o_v40": ("mrcis", dict(nact=8, nelec=6, nvirt=40)),
        # MRCISD: CAS(4e,6o) reference + singles and doubles into 30 virtuals
        "mrcisd_4e6o_v30": ("mrcisd", dict(nact=6, nelec=4, nvirt=30)),
        # the same space with 16 and 24 virtuals (263,004 / 568,204 SEFs): profiler captures
        "mrcisd_6e8o_v16": ("mrcisd", dict(nact=8, nelec=6, nvirt=16)),
        "mrcisd_6e8o_v24": ("mrcisd", dict(nact=8, nelec=6, nvirt=24)),
        # 66 orbitals (two-word bit-strings, like the 72-orbital benchmark space), 124,815 SEFs
        "mrcisd_4e6o_v60": ("mrcisd", dict(nact=6, nelec=4, nvirt=60)),
        # scaled MRCISD: CAS(6e,8o) + singles and doubles into 64 virtuals (~3.8M SEFs)
        "mrcisd_6e8o_v64": ("mrcisd", dict(nact=8, nelec=6, nvirt=64)),
        # the same into 112 virtuals (11.6M SEFs, 120 orbitals): about 8.4e9 stored elements
        # (135 GB with the FP32 copy, plus the build's working set); the direct-mode case
        "mrcisd_6e8o_v112": ("mrcisd", dict(nact=8, nelec=6, nvirt=112)),
        # small cases for tests
        "fci_4e6o": ("fci", dict(nbf=6, nelec=4)),
        "fci_5e6o": ("fci", dict(nbf=6, nelec=5)),
        "fci_6e8o": ("fci", dict(nbf=8, nelec=6)),
    }
    kind, kw = table[name]
    return make_problem(kind, seed=seed, ksym=ksym, **kw)
