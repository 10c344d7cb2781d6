"""Oracle for PSOCI's Hamiltonian-build / sigma path — TEST INFRASTRUCTURE ONLY.

Two CPU implementations live here, both used only as checkers (tests/, the smoke
check) and as the timed CPU baseline (bench.py):

* ``Oracle``    — ctypes wrapper of ``psoci_oracle.c``, a plain-C restatement of the
                  reference algorithm (builds anywhere, including the GPU host);
* ``Reference`` — ctypes wrapper of ``_ref/libpsoci_ref.so``: the reference's own
                  compute sources compiled unchanged (only where the reference tree
                  is present).

The psoci_gb300 package never imports this module.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
# The reference's source tree: read by the reference build (Makefile target ``ref``) and by the
# tests that compare with it; absent on hosts without it.  One environment variable sets it.
REFERENCE_TREE = os.environ.get("PSOCI_REFERENCE_TREE", "/root/reference/psociRestart-Cori")
REF_DIR = os.path.join(HERE, "_ref")
ORACLE_SO = os.path.join(REF_DIR, "liboracle.so")
REF_SO = os.path.join(REF_DIR, "libpsoci_ref.so")

_c_int_p = ctypes.POINTER(ctypes.c_int)
_c_long_p = ctypes.POINTER(ctypes.c_long)
_c_dbl_p = ctypes.POINTER(ctypes.c_double)
_c_u8_p = ctypes.POINTER(ctypes.c_ubyte)


def _p(a, t):
    return a.ctypes.data_as(t)


def build(ref: bool = True) -> None:
    """Compile the C restatement (always) and the reference harness (when present)."""
    targets = ["oracle"] + (["ref"] if ref else [])
    subprocess.run(["make", "-s", "-f", os.path.join(HERE, "Makefile"), f"REFDIR={REFERENCE_TREE}"] + targets,
                   check=True, cwd=HERE)


def reference_tree_present() -> bool:
    return os.path.isdir(REFERENCE_TREE)


def ref_available() -> bool:
    return os.path.exists(REF_SO)


class _Base:
    prefix = ""

    def _fn(self, name, restype, argtypes):
        f = getattr(self.lib, self.prefix + name)
        f.restype = restype
        f.argtypes = argtypes
        return f


class Oracle(_Base):
    """C restatement of the reference (psoci_oracle.c)."""

    prefix = "orc_"

    def __init__(self, prob):
        if not os.path.exists(ORACLE_SO):
            build(ref=False)
        self.lib = ctypes.CDLL(ORACLE_SO)
        self.p = prob
        create = self._fn("create", ctypes.c_void_p,
                          [ctypes.c_int] * 5 + [_c_int_p, _c_u8_p, _c_dbl_p, _c_dbl_p, _c_dbl_p])
        self._keep = [np.ascontiguousarray(prob.jsym, np.int32), np.ascontiguousarray(prob.occ, np.uint8),
                      np.ascontiguousarray(prob.h, np.float64), np.ascontiguousarray(prob.so, np.float64),
                      np.ascontiguousarray(prob.eri, np.float64)]
        js, oc, h, so, eri = self._keep
        self.ctx = create(prob.nbf, prob.nelec, prob.ksym, prob.mx_open, prob.nconf, _p(js, _c_int_p),
                          _p(oc, _c_u8_p), _p(h, _c_dbl_p), _p(so, _c_dbl_p), _p(eri, _c_dbl_p))
        self._destroy = self._fn("destroy", None, [ctypes.c_void_p])

    def __del__(self):
        try:
            self._destroy(self.ctx)
        except Exception:
            pass

    def num_sefs(self):
        return self._fn("num_sefs", ctypes.c_long, [ctypes.c_void_p])(self.ctx)

    def config_counts(self):
        out = np.zeros(3 * self.p.nconf, np.int32)
        self._fn("config_counts", None, [ctypes.c_void_p, _c_int_p])(self.ctx, _p(out, _c_int_p))
        return out.reshape(-1, 3)

    def config_dets(self, i):
        nd = int(self.config_counts()[i, 0]) if not hasattr(self, "_cc") else int(self._cc[i, 0])
        out = np.zeros((nd, 6 + 2 * self.p.nbf), np.int32)
        self._fn("config_dets", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, _c_int_p])(self.ctx, i, _p(out, _c_int_p))
        return out

    def fetch1e(self, i, j):
        return self._fn("fetch1e", ctypes.c_double, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int])(self.ctx, i, j)

    def fetch2e(self, i, j, k, l):
        return self._fn("fetch2e", ctypes.c_double, [ctypes.c_void_p] + [ctypes.c_int] * 4)(self.ctx, i, j, k, l)

    def block(self, i, j):
        ns = self.p.nsef()
        out = np.zeros(int(ns[i] * ns[j]))
        st = self._fn("block", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, _c_dbl_p])(
            self.ctx, i, j, _p(out, _c_dbl_p))
        return st, out.reshape(int(ns[i]), int(ns[j]))

    def build_lower(self, nthreads=0):
        """Lower-triangle CSR (rowptr int64, cols int32, vals float64) in reference order."""
        nthreads = nthreads or os.cpu_count() or 1
        nnz = self._fn("build_lower", ctypes.c_long, [ctypes.c_void_p, ctypes.c_int])(self.ctx, nthreads)
        n = self.num_sefs()
        rp = np.zeros(n + 1, np.int64)
        ci = np.zeros(max(nnz, 1), np.int32)
        va = np.zeros(max(nnz, 1), np.float64)
        self._fn("copy_lower", None, [ctypes.c_void_p, _c_long_p, _c_int_p, _c_dbl_p])(
            self.ctx, _p(rp, _c_long_p), _p(ci, _c_int_p), _p(va, _c_dbl_p))
        return rp, ci[:nnz], va[:nnz]

    def build_rows(self, rows, nthreads=0):
        """Lower-triangle rows of the given configurations only; returns the stored count."""
        nthreads = nthreads or os.cpu_count() or 1
        r = np.ascontiguousarray(rows, np.int32)
        f = self._fn("build_rows", ctypes.c_long, [ctypes.c_void_p, ctypes.c_int, _c_int_p, ctypes.c_int])
        return f(self.ctx, nthreads, _p(r, _c_int_p), len(r))

    def sample_rows(self):
        """CSR of the rows kept by the last build_rows: the sampled configurations' SEF rows
        in order, each the reference's lower-triangle row (rowptr, cols, vals)."""
        nr, nz = ctypes.c_long(), ctypes.c_long()
        self._fn("sample_counts", None, [ctypes.c_void_p, _c_long_p, _c_long_p])(self.ctx, ctypes.byref(nr),
                                                                                   ctypes.byref(nz))
        rp = np.zeros(nr.value + 1, np.int64)
        ci = np.zeros(max(nz.value, 1), np.int32)
        va = np.zeros(max(nz.value, 1), np.float64)
        self._fn("copy_sample", None, [ctypes.c_void_p, _c_long_p, _c_int_p, _c_dbl_p])(
            self.ctx, _p(rp, _c_long_p), _p(ci, _c_int_p), _p(va, _c_dbl_p))
        return rp, ci[:nz.value], va[:nz.value]

    def ciden_block(self, i, j):
        ns = self.p.nsef()
        out = np.zeros(int(ns[i] * ns[j]))
        st = self._fn("ciden_block", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, _c_dbl_p])(
            self.ctx, i, j, _p(out, _c_dbl_p))
        return st, out.reshape(int(ns[i]), int(ns[j]))

    def density1(self, vecs):
        """Packed 1-particle densities (k x nbf(nbf+1)/2) of root-major vectors (k x N)."""
        v = np.ascontiguousarray(np.atleast_2d(vecs), np.float64)
        out = np.zeros((v.shape[0], self.p.nbf * (self.p.nbf + 1) // 2))
        self._fn("density1", None, [ctypes.c_void_p, ctypes.c_int, _c_dbl_p, _c_dbl_p])(
            self.ctx, v.shape[0], _p(v, _c_dbl_p), _p(out, _c_dbl_p))
        return out

    def density1_rows(self, vecs, rows):
        """The reference's pair loop restricted to rows I (pairs J <= I), for timing samples."""
        v = np.ascontiguousarray(np.atleast_2d(vecs), np.float64)
        r = np.ascontiguousarray(rows, np.int32)
        out = np.zeros((v.shape[0], self.p.nbf * (self.p.nbf + 1) // 2))
        self._fn("density1_rows", None, [ctypes.c_void_p, ctypes.c_int, _c_dbl_p, ctypes.c_int, _c_int_p, _c_dbl_p])(
            self.ctx, v.shape[0], _p(v, _c_dbl_p), len(r), _p(r, _c_int_p), _p(out, _c_dbl_p))
        return out

    def energy_gradient(self, vecs, nonzero_only=False, nthreads=0):
        """dE_r / d(packed one-electron table) [k, nbf(nbf+1)/2] and dE_r / d(canonical
        two-electron table) [k, NNDAF(NNDAF(nbf))] of E_r = v_r^T H v_r, one unit-table
        build per entry (see psoci_oracle.c)."""
        nthreads = nthreads or os.cpu_count() or 1
        v = np.ascontiguousarray(np.atleast_2d(vecs), np.float64)
        n1 = self.p.nbf * (self.p.nbf + 1) // 2
        g1 = np.zeros((v.shape[0], n1))
        g2 = np.zeros((v.shape[0], n1 * (n1 + 1) // 2))
        self._fn("energy_gradient", None, [ctypes.c_void_p, ctypes.c_int, _c_dbl_p, ctypes.c_int, _c_dbl_p, _c_dbl_p,
                                           ctypes.c_int])(self.ctx, v.shape[0], _p(v, _c_dbl_p), int(nonzero_only),
                                                          _p(g1, _c_dbl_p), _p(g2, _c_dbl_p), nthreads)
        return g1, g2

    def diag(self):
        d = np.zeros(self.num_sefs())
        self._fn("diag", None, [ctypes.c_void_p, _c_dbl_p])(self.ctx, _p(d, _c_dbl_p))
        return d

    def sigma_lower(self, rp, ci, va, x, nthreads=0):
        """y = H x from lower storage; x is [k, n] (vector-major) float64."""
        nthreads = nthreads or os.cpu_count() or 1
        x = np.ascontiguousarray(np.atleast_2d(x), np.float64)
        y = np.zeros_like(x)
        f = self._fn("sigma_lower", None, [ctypes.c_long, _c_long_p, _c_int_p, _c_dbl_p, ctypes.c_int, _c_dbl_p,
                                           _c_dbl_p, ctypes.c_int])
        f(x.shape[1], _p(rp, _c_long_p), _p(ci, _c_int_p), _p(va, _c_dbl_p), x.shape[0], _p(x, _c_dbl_p),
          _p(y, _c_dbl_p), nthreads)
        return y


def sigma_lower_rows(rp, ci, va, x, nthreads=0):
    """y = H x for one vector from lower storage, rows over threads (the timed CPU sigma)."""
    lib = ctypes.CDLL(ORACLE_SO)
    f = lib.orc_sigma_lower_rows
    f.restype = None
    f.argtypes = [ctypes.c_long, _c_long_p, _c_int_p, _c_dbl_p, _c_dbl_p, _c_dbl_p, ctypes.c_int]
    x = np.ascontiguousarray(x, np.float64)
    y = np.zeros_like(x)
    f(len(rp) - 1, _p(rp, _c_long_p), _p(ci, _c_int_p), _p(va, _c_dbl_p), _p(x, _c_dbl_p), _p(y, _c_dbl_p),
      nthreads or os.cpu_count() or 1)
    return y


def davidson_ref(rp, ci, va, diag, nroots, rtol, maxsub=0, max_iter=1000, nthreads=0):
    """The reference's Davidson loop on the CPU (see psoci_oracle.c): returns (evals, rnorms,
    {"iterations", "sigma_vectors", "collapses"}, converged)."""
    lib = ctypes.CDLL(ORACLE_SO)
    f = lib.orc_davidson_ref
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_long, _c_long_p, _c_int_p, _c_dbl_p, _c_dbl_p, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                  ctypes.c_int, ctypes.c_int, _c_dbl_p, _c_dbl_p, _c_long_p]
    ev = np.zeros(nroots)
    rn = np.zeros(nroots)
    st = np.zeros(3, np.int64)
    d = np.ascontiguousarray(diag, np.float64)
    rc = f(len(rp) - 1, _p(rp, _c_long_p), _p(ci, _c_int_p), _p(va, _c_dbl_p), _p(d, _c_dbl_p), nroots,
           maxsub or 4 * nroots, rtol, max_iter, nthreads or os.cpu_count() or 1, _p(ev, _c_dbl_p), _p(rn, _c_dbl_p),
           _p(st, _c_long_p))
    return ev, rn, {"iterations": int(st[0]), "sigma_vectors": int(st[1]), "collapses": int(st[2])}, rc == 0


class Reference(_Base):
    """The reference's own compute sources (compiled unchanged), via oracle/ref_harness.cpp.
    Process-global state: one problem at a time."""

    prefix = "ref_"

    def __init__(self, prob):
        if not os.path.exists(REF_SO):
            build(ref=True)
        if not os.path.exists(REF_SO):
            raise RuntimeError("reference harness unavailable (reference tree absent)")
        self.lib = ctypes.CDLL(REF_SO)
        self.p = prob
        self._occ = np.ascontiguousarray(prob.occ, np.uint8)
        self._fn("set_integrals", ctypes.c_int, [ctypes.c_int, _c_dbl_p, _c_dbl_p, _c_dbl_p, ctypes.c_double])(
            prob.nbf, _p(np.ascontiguousarray(prob.h), _c_dbl_p), _p(np.ascontiguousarray(prob.so), _c_dbl_p),
            _p(np.ascontiguousarray(prob.eri), _c_dbl_p), prob.ecore)
        js = np.ascontiguousarray(prob.jsym, np.int32)
        self._fn("set_configs", ctypes.c_int, [ctypes.c_int] * 5 + [_c_int_p, _c_u8_p])(
            prob.nbf, prob.nelec, prob.ksym, prob.mx_open, prob.nconf, _p(js, _c_int_p), _p(self._occ, _c_u8_p))

    def num_sefs(self):
        return self._fn("num_sefs", ctypes.c_long, [])()

    def config_counts(self):
        out = np.zeros(3 * self.p.nconf, np.int32)
        self._fn("config_counts", None, [_c_int_p])(_p(out, _c_int_p))
        return out.reshape(-1, 3)

    def config_dets(self, i):
        nd = int(self.p.ndet()[i])
        out = np.zeros((nd, 6 + 2 * self.p.nbf), np.int32)
        self._fn("config_dets", ctypes.c_int, [ctypes.c_int, _c_int_p])(i, _p(out, _c_int_p))
        return out

    def fetch1e(self, i, j):
        return self._fn("fetch1e", ctypes.c_double, [ctypes.c_int, ctypes.c_int])(i, j)

    def fetch2e(self, i, j, k, l):
        return self._fn("fetch2e", ctypes.c_double, [ctypes.c_int] * 4)(i, j, k, l)

    def block(self, i, j):
        ns = self.p.nsef()
        out = np.zeros(int(ns[i] * ns[j]))
        st = self._fn("block", ctypes.c_int, [ctypes.c_int, ctypes.c_int, _c_dbl_p])(i, j, _p(out, _c_dbl_p))
        return st, out.reshape(int(ns[i]), int(ns[j]))

    def ciden_block(self, i, j):
        ns = self.p.nsef()
        out = np.zeros(int(ns[i] * ns[j]))
        st = self._fn("ciden_block", ctypes.c_int, [ctypes.c_int, ctypes.c_int, _c_dbl_p])(i, j, _p(out, _c_dbl_p))
        return st, out.reshape(int(ns[i]), int(ns[j]))

    def density1(self, vecs):
        v = np.ascontiguousarray(np.atleast_2d(vecs), np.float64)
        out = np.zeros((v.shape[0], self.p.nbf * (self.p.nbf + 1) // 2))
        self._fn("density1", None, [_c_u8_p, ctypes.c_int, _c_dbl_p, _c_dbl_p])(
            _p(self._occ, _c_u8_p), v.shape[0], _p(v, _c_dbl_p), _p(out, _c_dbl_p))
        return out

    def build_lower(self, nthreads=0):
        nthreads = nthreads or os.cpu_count() or 1
        f = self._fn("build_lower", ctypes.c_long, [_c_u8_p, ctypes.c_int, _c_long_p, _c_int_p, _c_dbl_p])
        n = self.num_sefs()
        rp = np.zeros(n + 1, np.int64)
        nnz = f(_p(self._occ, _c_u8_p), nthreads, _p(rp, _c_long_p), None, None)
        ci = np.zeros(max(nnz, 1), np.int32)
        va = np.zeros(max(nnz, 1), np.float64)
        f(_p(self._occ, _c_u8_p), nthreads, _p(rp, _c_long_p), _p(ci, _c_int_p), _p(va, _c_dbl_p))
        return rp, ci[:nnz], va[:nnz]


def lower_to_full_scipy(rp, ci, va, n):
    """Symmetric scipy CSR from lower-triangle storage."""
    import scipy.sparse as sp

    L = sp.csr_matrix((va, ci, rp), shape=(n, n))
    D = sp.diags(L.diagonal())
    return (L + L.T - D).tocsr()
