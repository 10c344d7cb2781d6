"""Python host side over the C ABI of libpsoci_gpu.so (include/psoci_gpu.h).

``Context`` owns one ``psoci_ctx`` (one GPU, one stream) and exposes the entry points with
numpy arguments.  There is no CPU fallback: if the native library is missing, or no CUDA
device is present, construction raises ``PsociError``.
"""
from __future__ import annotations

import ctypes
import dataclasses
import os
from typing import Optional

import numpy as np

from . import build as _build

PSOCI_OK = 0
STATUS = {
    0: "ok", 1: "invalid argument", 2: "unsupported", 3: "call order", 4: "cuda error", 5: "out of device memory",
    6: "device wait timed out", 7: "not converged", 8: "non-finite value", 9: "i/o error",
}
PREC_FP64, PREC_MIXED, PREC_FF = 0, 1, 2
HMODE_CSR_FP64, HMODE_CSR_BOTH, HMODE_DIRECT = 0, 1, 2


class PsociError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


class _Opts(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int), ("verbose", ctypes.c_int)]


class DavOpts(ctypes.Structure):
    _fields_ = [("nroots", ctypes.c_int), ("max_subspace", ctypes.c_int), ("max_iter", ctypes.c_int),
                ("rtol", ctypes.c_double), ("prec", ctypes.c_int), ("refine", ctypes.c_int), ("block", ctypes.c_int),
                ("precond_min", ctypes.c_double)]


class BuildInfo(ctypes.Structure):
    _fields_ = [("candidates", ctypes.c_int64), ("pairs", ctypes.c_int64), ("segments", ctypes.c_int64),
                ("nnz", ctypes.c_int64), ("nnz_lower", ctypes.c_int64), ("slab_slots", ctypes.c_int64),
                ("evaluations", ctypes.c_int), ("fast", ctypes.c_int), ("lookup_screen", ctypes.c_int),
                ("eval_launches", ctypes.c_int),
                ("screen_ms", ctypes.c_double), ("evaluate_ms", ctypes.c_double), ("rows_ms", ctypes.c_double),
                ("assemble_ms", ctypes.c_double), ("total_ms", ctypes.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class DavStats(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int), ("sigma_calls", ctypes.c_int), ("collapses", ctypes.c_int),
                ("refine_iters", ctypes.c_int), ("seconds", ctypes.c_double), ("sigma_seconds", ctypes.c_double)]


# every entry point of include/psoci_gpu.h: name -> (restype, argtypes)
_P = ctypes.c_void_p
_I64P = ctypes.POINTER(ctypes.c_int64)
_I32P = ctypes.POINTER(ctypes.c_int32)
_U64P = ctypes.POINTER(ctypes.c_uint64)
_U8P = ctypes.POINTER(ctypes.c_uint8)
_DP = ctypes.POINTER(ctypes.c_double)
_IP = ctypes.POINTER(ctypes.c_int)
SIGNATURES = {
    "psoci_create": (ctypes.c_int, [ctypes.POINTER(_P), ctypes.POINTER(_Opts)]),
    "psoci_destroy": (None, [_P]),
    "psoci_status_str": (ctypes.c_char_p, [ctypes.c_int]),
    "psoci_last_error": (ctypes.c_char_p, [_P]),
    "psoci_set_integrals": (ctypes.c_int, [_P, ctypes.c_int, _DP, _DP, ctypes.c_double]),
    "psoci_set_configs": (ctypes.c_int, [_P, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                         _I32P, _U8P]),
    "psoci_build_determinants": (ctypes.c_int, [_P]),
    "psoci_get_counts": (ctypes.c_int, [_P, _I64P, _I64P, _IP, _IP]),
    "psoci_get_determinants": (ctypes.c_int, [_P, _U64P, _U64P, _U8P, _I32P, _I64P, _I64P]),
    "psoci_build_hamiltonian": (ctypes.c_int, [_P, ctypes.c_int, _I64P]),
    "psoci_blocks": (ctypes.c_int, [_P, ctypes.c_int, _I32P, _I32P, _DP]),
    "psoci_get_hamiltonian": (ctypes.c_int, [_P, _I64P, _I32P, _DP]),
    "psoci_get_diag": (ctypes.c_int, [_P, _DP]),
    "psoci_get_rows": (ctypes.c_int, [_P, ctypes.c_int, _I64P, _I64P, _I32P, _DP]),
    "psoci_sigma": (ctypes.c_int, [_P, ctypes.c_int, _DP, _DP, ctypes.c_int]),
    "psoci_sigma_device": (ctypes.c_int, [_P, ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                          ctypes.c_int, ctypes.c_int]),
    "psoci_davidson": (ctypes.c_int, [_P, ctypes.POINTER(DavOpts), _DP, _DP, _DP, ctypes.POINTER(DavStats)]),
    "psoci_core_energy": (ctypes.c_double, [_P]),
    "psoci_stream": (ctypes.c_void_p, [_P]),
    "psoci_launch_count": (ctypes.c_ulonglong, []),
    "psoci_build_stats": (ctypes.c_int, [_P, ctypes.POINTER(BuildInfo)]),
    "psoci_sigma_mixed_noalloc": (ctypes.c_int, [_P, ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                                 ctypes.c_int]),
    "psoci_set_guess": (ctypes.c_int, [_P, ctypes.c_int, _DP]),
    "psoci_density1": (ctypes.c_int, [_P, ctypes.c_int, _DP, _DP]),
    "psoci_density1_device": (ctypes.c_int, [_P, ctypes.c_int, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p]),
    "psoci_tsprod": (ctypes.c_int, [_P, ctypes.c_int, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                    ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]),
    "psoci_autotune_sigma": (ctypes.c_int, [_P, ctypes.c_int, _IP, ctypes.POINTER(ctypes.c_float)]),
    "psoci_set_eval_launches": (ctypes.c_int, [_P, ctypes.c_int]),
    "psoci_davidson_batch": (ctypes.c_int, [ctypes.POINTER(_P), ctypes.c_int, ctypes.POINTER(DavOpts),
                                            ctypes.POINTER(_DP), ctypes.POINTER(_DP), ctypes.POINTER(_DP),
                                            ctypes.POINTER(DavStats), _IP]),
    "psoci_energy_gradient": (ctypes.c_int, [_P, ctypes.c_int, _DP, ctypes.c_int, ctypes.c_int, _DP, _DP]),
    "psoci_energy_gradient_device": (ctypes.c_int, [_P, ctypes.c_int, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int,
                                                    ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]),
    "psoci_natural_orbitals": (ctypes.c_int, [ctypes.c_int, _DP, _I32P, _DP, _DP, _I32P]),
    "psoci_subspace_eigen": (ctypes.c_int, [ctypes.c_int, _DP, ctypes.c_int, _DP, _DP, ctypes.c_int]),
    "psoci_write_vectors": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_int, ctypes.c_int64, ctypes.c_int, _DP,
                                           ctypes.c_char_p]),
    "psoci_read_vectors": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_int, ctypes.c_int64, ctypes.c_int, _DP, _IP]),
    "psoci_basis_create": (ctypes.c_int, [_P, ctypes.c_int, ctypes.c_int]),
    "psoci_basis_destroy": (None, [_P]),
    "psoci_basis_guess": (ctypes.c_int, [_P, ctypes.c_int]),
    "psoci_basis_orthonormalize_all": (ctypes.c_int, [_P, _IP]),
    "psoci_basis_compute_hv": (ctypes.c_int, [_P, ctypes.c_int, ctypes.c_int, ctypes.c_int]),
    "psoci_subspace_generate_incremental": (ctypes.c_int, [_P, ctypes.c_int]),
    "psoci_subspace_diag": (ctypes.c_int, [_P, _DP]),
    "psoci_subspace_rnorm_single": (ctypes.c_int, [_P, ctypes.c_int, _DP]),
    "psoci_subspace_rnorms": (ctypes.c_int, [_P, _DP]),
    "psoci_basis_precondition_new": (ctypes.c_int, [_P, ctypes.c_int, ctypes.c_double, ctypes.c_double]),
    "psoci_basis_append_scratch": (ctypes.c_int, [_P, ctypes.c_int, _IP]),
    "psoci_basis_expand_replace": (ctypes.c_int, [_P, ctypes.c_int]),
    "psoci_basis_info": (ctypes.c_int, [_P, _IP, _IP, _IP, _IP]),
    "psoci_basis_vectors": (ctypes.c_int, [_P, ctypes.c_int, _DP]),
    "psoci_save_hamiltonian": (ctypes.c_int, [_P, ctypes.c_char_p]),
    "psoci_load_hamiltonian": (ctypes.c_int, [_P, ctypes.c_char_p]),
}

_lib = None


def load_library(build_if_missing: bool = True) -> ctypes.CDLL:
    """Load libpsoci_gpu.so (building it in-tree when absent or stale)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if build_if_missing:
        path = _build.build()
    if not os.path.exists(path):
        raise PsociError(4, f"native library {path} is missing; run psoci_gb300.build.build()")
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def _ptr(a: np.ndarray, t):
    return a.ctypes.data_as(t)


@dataclasses.dataclass
class DavidsonResult:
    evals: np.ndarray
    evecs: Optional[np.ndarray]
    rnorms: np.ndarray
    iterations: int
    sigma_calls: int
    collapses: int
    refine_iters: int
    seconds: float
    sigma_seconds: float


class Context:
    """One GPU context: integrals, configurations, determinants, H, Davidson."""

    def __init__(self, device: int = 0, verbose: int = 0):
        self.lib = load_library()
        self.ctx = _P()
        opts = _Opts(device, verbose)
        st = self.lib.psoci_create(ctypes.byref(self.ctx), ctypes.byref(opts))
        if st != PSOCI_OK:
            raise PsociError(st, "psoci_create failed (no CUDA device?)")
        self.nsef = 0
        self.nnz = 0
        self.nbf = 0

    def close(self):
        if getattr(self, "ctx", None):
            self.lib.psoci_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, st: int, what: str):
        if st != PSOCI_OK:
            msg = self.lib.psoci_last_error(self.ctx)
            raise PsociError(st, f"{what}: {msg.decode() if msg else ''}")

    # -- inputs ------------------------------------------------------------------------
    def set_integrals(self, nbf: int, one_packed: np.ndarray, eri_packed: np.ndarray, ecore: float = 0.0):
        one = np.ascontiguousarray(one_packed, np.float64)
        eri = np.ascontiguousarray(eri_packed, np.float64)
        self._check(self.lib.psoci_set_integrals(self.ctx, nbf, _ptr(one, _DP), _ptr(eri, _DP), float(ecore)),
                    "set_integrals")

    def set_configs(self, nbf, nelec, ksym, mx_open, jsym, occ):
        js = np.ascontiguousarray(jsym, np.int32)
        oc = np.ascontiguousarray(occ, np.uint8)
        self._check(self.lib.psoci_set_configs(self.ctx, nbf, nelec, ksym, mx_open, len(js), _ptr(js, _I32P),
                                               _ptr(oc, _U8P)), "set_configs")
        self.nbf = nbf

    def load_problem(self, p):
        """Integrals and configurations of an inputs.Problem."""
        self.set_integrals(p.nbf, p.one_packed(), p.eri, p.ecore)
        self.set_configs(p.nbf, p.nelec, p.ksym, p.mx_open, p.jsym, p.occ)

    # -- determinants --------------------------------------------------------------------
    def build_determinants(self):
        self._check(self.lib.psoci_build_determinants(self.ctx), "build_determinants")
        nsef, ndet = ctypes.c_int64(), ctypes.c_int64()
        ms, md = ctypes.c_int(), ctypes.c_int()
        self._check(self.lib.psoci_get_counts(self.ctx, ctypes.byref(nsef), ctypes.byref(ndet), ctypes.byref(ms),
                                              ctypes.byref(md)), "get_counts")
        self.nsef, self.ndet = nsef.value, ndet.value
        return self.nsef, self.ndet

    def get_determinants(self, nconf: int, nbf: int):
        words = (nbf + 63) // 64
        a = np.zeros(self.ndet * words, np.uint64)
        b = np.zeros(self.ndet * words, np.uint64)
        ph = np.zeros(self.ndet, np.uint8)
        ms = np.zeros(self.ndet, np.int32)
        do = np.zeros(nconf + 1, np.int64)
        so = np.zeros(nconf + 1, np.int64)
        self._check(self.lib.psoci_get_determinants(self.ctx, _ptr(a, _U64P), _ptr(b, _U64P), _ptr(ph, _U8P),
                                                    _ptr(ms, _I32P), _ptr(do, _I64P), _ptr(so, _I64P)),
                    "get_determinants")
        return dict(alpha=a.reshape(-1, words), beta=b.reshape(-1, words), phase=ph, ms=ms, detoff=do, sefoff=so)

    # -- Hamiltonian ---------------------------------------------------------------------
    def build_hamiltonian(self, mixed: bool = True, direct: bool = False) -> int:
        """Stored CSR (FP64, plus an FP32 copy when mixed), or with direct=True no stored
        elements: every sigma evaluates them again (returns 0)."""
        nnz = ctypes.c_int64()
        mode = HMODE_DIRECT if direct else (HMODE_CSR_BOTH if mixed else HMODE_CSR_FP64)
        self._check(self.lib.psoci_build_hamiltonian(self.ctx, mode, ctypes.byref(nnz)), "build_hamiltonian")
        self.nnz = nnz.value
        return self.nnz

    def blocks(self, A, B, nsef_per_config):
        """Reference sefsef blocks for pairs (A[q], B[q]); returns a list of 2-D arrays."""
        A = np.ascontiguousarray(A, np.int32)
        B = np.ascontiguousarray(B, np.int32)
        ns = np.asarray(nsef_per_config)
        sizes = ns[A] * ns[B]
        out = np.zeros(max(int(sizes.sum()), 1))
        self._check(self.lib.psoci_blocks(self.ctx, len(A), _ptr(A, _I32P), _ptr(B, _I32P), _ptr(out, _DP)), "blocks")
        res, o = [], 0
        for a, b in zip(A, B):
            n = int(ns[a] * ns[b])
            res.append(out[o:o + n].reshape(int(ns[a]), int(ns[b])))
            o += n
        return res

    def get_hamiltonian(self):
        rp = np.zeros(self.nsef + 1, np.int64)
        ci = np.zeros(max(self.nnz, 1), np.int32)
        va = np.zeros(max(self.nnz, 1), np.float64)
        self._check(self.lib.psoci_get_hamiltonian(self.ctx, _ptr(rp, _I64P), _ptr(ci, _I32P), _ptr(va, _DP)),
                    "get_hamiltonian")
        return rp, ci[:self.nnz], va[:self.nnz]

    def get_rows(self, rows):
        """Selected rows of the stored CSR (both triangles): (rowptr [len(rows)+1], cols, vals)."""
        r = np.ascontiguousarray(rows, np.int64)
        rp = np.zeros(len(r) + 1, np.int64)
        self._check(self.lib.psoci_get_rows(self.ctx, len(r), _ptr(r, _I64P), _ptr(rp, _I64P), None, None), "get_rows")
        ci = np.zeros(max(int(rp[-1]), 1), np.int32)
        va = np.zeros(max(int(rp[-1]), 1), np.float64)
        self._check(self.lib.psoci_get_rows(self.ctx, len(r), _ptr(r, _I64P), _ptr(rp, _I64P), _ptr(ci, _I32P),
                                            _ptr(va, _DP)), "get_rows")
        return rp, ci[:rp[-1]], va[:rp[-1]]

    def get_diag(self):
        d = np.zeros(self.nsef)
        self._check(self.lib.psoci_get_diag(self.ctx, _ptr(d, _DP)), "get_diag")
        return d

    # -- sigma ---------------------------------------------------------------------------
    def sigma(self, X: np.ndarray, prec: int = PREC_FP64) -> np.ndarray:
        """Y = H X for X of shape [N, k] (row-major), host memory."""
        X = np.ascontiguousarray(X, np.float64)
        if X.ndim == 1:
            X = X[:, None]
        Y = np.zeros_like(X)
        self._check(self.lib.psoci_sigma(self.ctx, X.shape[1], _ptr(X, _DP), _ptr(Y, _DP), prec), "sigma")
        return Y

    def sigma_device(self, dX_ptr: int, ldx: int, dY_ptr: int, ldy: int, k: int, prec: int = PREC_FP64):
        self._check(self.lib.psoci_sigma_device(self.ctx, k, ctypes.c_void_p(dX_ptr), ldx, ctypes.c_void_p(dY_ptr), ldy,
                                                prec), "sigma_device")

    # -- Davidson ------------------------------------------------------------------------
    def davidson(self, nroots: int, rtol: float = 1e-6, mixed: bool = False, refine: bool = True,
                 block: bool = True, max_subspace: int = 0, max_iter: int = 1000, want_vectors: bool = False,
                 precond_min: float = 1e-3) -> DavidsonResult:
        o = DavOpts(nroots, max_subspace, max_iter, rtol, PREC_MIXED if mixed else PREC_FP64, int(refine), int(block),
                    precond_min)
        ev = np.zeros(nroots)
        rn = np.zeros(nroots)
        vec = np.zeros((nroots, self.nsef)) if want_vectors else None
        stats = DavStats()
        st = self.lib.psoci_davidson(self.ctx, ctypes.byref(o), _ptr(ev, _DP),
                                     _ptr(vec, _DP) if vec is not None else None, _ptr(rn, _DP), ctypes.byref(stats))
        self._check(st, "davidson")
        return DavidsonResult(ev, vec, rn, stats.iterations, stats.sigma_calls, stats.collapses, stats.refine_iters,
                              stats.seconds, stats.sigma_seconds)

    def density1(self, vecs) -> np.ndarray:
        """Spin-free 1-particle densities of CI vectors [k, N] (root-major): array
        [k, nbf(nbf+1)/2], packed lower triangle (index p(p+1)/2 + q, p >= q)."""
        v = np.ascontiguousarray(np.atleast_2d(vecs), np.float64)
        if v.shape[1] != self.nsef:
            raise ValueError(f"density1: vectors of length {v.shape[1]}, expected {self.nsef}")
        out = np.zeros((v.shape[0], self.nbf * (self.nbf + 1) // 2))
        self._check(self.lib.psoci_density1(self.ctx, v.shape[0], _ptr(v, _DP), _ptr(out, _DP)), "density1")
        return out

    def density1_device(self, dV_ptr: int, ldv: int, dD_ptr: int, k: int):
        """density1 on device pointers (root-major vectors, stride ldv); asynchronous on
        the context's stream."""
        self._check(self.lib.psoci_density1_device(self.ctx, k, ctypes.c_void_p(dV_ptr), ldv,
                                                   ctypes.c_void_p(dD_ptr)), "density1_device")

    def tsprod_device(self, method: int, n: int, dA: int, lda: int, m: int, dB: int, ldb: int, k: int, dC: int):
        """C (m x k) = A^T B on device pointers by method 0 (float-float), 1 (FP64 FMA) or 2
        (FP64 tensor-core MMA)."""
        self._check(self.lib.psoci_tsprod(self.ctx, method, n, ctypes.c_void_p(dA), lda, m, ctypes.c_void_p(dB), ldb,
                                          k, ctypes.c_void_p(dC)), "tsprod")

    def autotune_sigma(self, k: int = 8):
        """Pick the fastest mixed-sigma variant for this Hamiltonian: (choice, ms per variant)."""
        ch = ctypes.c_int()
        t = (ctypes.c_float * 6)()
        self._check(self.lib.psoci_autotune_sigma(self.ctx, k, ctypes.byref(ch), t), "autotune_sigma")
        return ch.value, [float(x) for x in t]

    def set_eval_launches(self, launches: int):
        """1: evaluate the H build's elements in one launch; 0: automatic (two when they fit)."""
        self._check(self.lib.psoci_set_eval_launches(self.ctx, launches), "set_eval_launches")

    def set_sigma_variant(self, v: int):
        """Install mixed-sigma variant v (0..5) without timing."""
        ch = ctypes.c_int(v)
        self._check(self.lib.psoci_autotune_sigma(self.ctx, 0, ctypes.byref(ch), None), "autotune_sigma")

    def energy_gradient(self, vecs, nonzero_only: bool = False, prec: int = PREC_FP64):
        """dE_r/d(packed one-electron table) [k, nbf(nbf+1)/2] and dE_r/d(canonical two-electron
        table) [k, NNDAF(NNDAF(nbf))] for CI vectors [k, N] (root-major): the 1-particle and
        spin-orbit densities and the 8-fold packed 2-particle density of each root."""
        v = np.ascontiguousarray(np.atleast_2d(vecs), np.float64)
        if v.shape[1] != self.nsef:
            raise ValueError(f"energy_gradient: vectors of length {v.shape[1]}, expected {self.nsef}")
        n1 = self.nbf * (self.nbf + 1) // 2
        g1 = np.zeros((v.shape[0], n1))
        g2 = np.zeros((v.shape[0], n1 * (n1 + 1) // 2))
        self._check(self.lib.psoci_energy_gradient(self.ctx, v.shape[0], _ptr(v, _DP), int(nonzero_only), prec,
                                                   _ptr(g1, _DP), _ptr(g2, _DP)), "energy_gradient")
        return g1, g2

    def energy_gradient_device(self, dV_ptr: int, ldv: int, k: int, dG1_ptr: int, dG2_ptr: int,
                               nonzero_only: bool = False, prec: int = PREC_FP64):
        self._check(self.lib.psoci_energy_gradient_device(self.ctx, k, ctypes.c_void_p(dV_ptr), ldv, int(nonzero_only),
                                                          prec, ctypes.c_void_p(dG1_ptr), ctypes.c_void_p(dG2_ptr)),
                    "energy_gradient_device")

    def core_energy(self) -> float:
        return self.lib.psoci_core_energy(self.ctx)

    def set_guess(self, vecs):
        """Restart vectors for the next davidson(): array [k, N] (or None to clear)."""
        if vecs is None:
            self._check(self.lib.psoci_set_guess(self.ctx, 0, None), "set_guess")
            return
        v = np.ascontiguousarray(np.atleast_2d(vecs), np.float64)
        self._check(self.lib.psoci_set_guess(self.ctx, v.shape[0], _ptr(v, _DP)), "set_guess")

    def save_hamiltonian(self, path: str):
        self._check(self.lib.psoci_save_hamiltonian(self.ctx, path.encode()), "save_hamiltonian")

    def load_hamiltonian(self, path: str):
        self._check(self.lib.psoci_load_hamiltonian(self.ctx, path.encode()), "load_hamiltonian")
        nnz = ctypes.c_int64()
        # the stored count is not exposed separately: read it back from the CSR row pointers
        rp = np.zeros(self.nsef + 1, np.int64)
        self._check(self.lib.psoci_get_hamiltonian(self.ctx, _ptr(rp, _I64P), None, None), "get_hamiltonian")
        self.nnz = int(rp[-1])
        del nnz

    def stream_handle(self) -> int:
        """cudaStream_t of this context (for CUDA events on the launching stream)."""
        return int(self.lib.psoci_stream(self.ctx) or 0)

    def build_stats(self) -> dict:
        """Counters and CUDA-event phase times (ms) of the last Hamiltonian build."""
        b = BuildInfo()
        self._check(self.lib.psoci_build_stats(self.ctx, ctypes.byref(b)), "build_stats")
        return b.as_dict()

    def launch_count(self) -> int:
        """Kernels the library has launched in this process so far (all contexts)."""
        return int(self.lib.psoci_launch_count())


def davidson_batch(contexts, nroots, rtol: float = 1e-6, mixed: bool = True, refine: bool = True,
                   max_subspace=0, max_iter: int = 1000, want_vectors: bool = False, precond_min: float = 1e-3):
    """Solve several symmetry blocks (one Context each, Hamiltonians built) at once:
    nroots[b] roots of block b.  Returns a list of DavidsonResult (vectors when asked)."""
    lib = load_library()
    nb = len(contexts)
    ms = list(max_subspace) if isinstance(max_subspace, (list, tuple)) else [max_subspace] * nb
    opts = (DavOpts * nb)(*[DavOpts(int(nroots[b]), int(ms[b]), max_iter, rtol, PREC_MIXED if mixed else PREC_FP64,
                                    int(refine), 1, precond_min) for b in range(nb)])
    ctxs = (_P * nb)(*[c.ctx for c in contexts])
    ev = [np.zeros(int(nroots[b])) for b in range(nb)]
    rn = [np.zeros(int(nroots[b])) for b in range(nb)]
    vec = [np.zeros((int(nroots[b]), contexts[b].nsef)) for b in range(nb)] if want_vectors else None
    pev = (_DP * nb)(*[_ptr(a, _DP) for a in ev])
    prn = (_DP * nb)(*[_ptr(a, _DP) for a in rn])
    pvec = (_DP * nb)(*[_ptr(a, _DP) for a in vec]) if vec is not None else None
    stats = (DavStats * nb)()
    bst = (ctypes.c_int * nb)()
    st = lib.psoci_davidson_batch(ctxs, nb, opts, pev, pvec, prn, stats, bst)
    if st != PSOCI_OK:
        bad = [b for b in range(nb) if bst[b] != PSOCI_OK]
        raise PsociError(st, f"davidson_batch: blocks {bad} failed: " +
                         "; ".join(lib.psoci_last_error(contexts[b].ctx).decode() for b in bad))
    return [DavidsonResult(ev[b], vec[b] if vec is not None else None, rn[b], stats[b].iterations,
                           stats[b].sigma_calls, stats[b].collapses, stats[b].refine_iters, stats[b].seconds,
                           stats[b].sigma_seconds) for b in range(nb)]


def natural_orbitals(dens_packed, orb_sym):
    """Natural orbitals of one packed density [nbf(nbf+1)/2] per symmetry block.

    Returns (occupations [nbf], blocks): blocks is a list, in ascending label order, of
    dicts {"sym", "orbitals", "occupations", "vectors"}; vectors[i] holds natural orbital i
    over the block's orbitals, occupations largest first."""
    lib = load_library()
    d = np.ascontiguousarray(dens_packed, np.float64).ravel()
    sym = np.ascontiguousarray(orb_sym, np.int32).ravel()
    nbf = len(sym)
    if len(d) != nbf * (nbf + 1) // 2:
        raise ValueError(f"natural_orbitals: density of length {len(d)} for {nbf} orbitals")
    _, counts = np.unique(sym, return_counts=True)
    occ = np.zeros(nbf)
    vecs = np.zeros(int((counts.astype(np.int64) ** 2).sum()))
    order = np.zeros(nbf, np.int32)
    st = lib.psoci_natural_orbitals(nbf, _ptr(d, _DP), _ptr(sym, _I32P), _ptr(occ, _DP), _ptr(vecs, _DP),
                                    _ptr(order, _I32P))
    if st != PSOCI_OK:
        raise PsociError(st, "natural_orbitals")
    blocks, e, v = [], 0, 0
    for n in counts:
        n = int(n)
        orbs = order[e:e + n].copy()
        blocks.append(dict(sym=int(sym[orbs[0]]), orbitals=orbs, occupations=occ[e:e + n].copy(),
                           vectors=vecs[v:v + n * n].reshape(n, n).copy()))
        e += n
        v += n * n
    return occ, blocks


def subspace_eigen(G):
    """Eigenpairs of a symmetric matrix as the Davidson solver's Rayleigh-Ritz step computes
    them: (w ascending [n], Y [n, n] with column c = eigenvector c)."""
    lib = load_library()
    g = np.ascontiguousarray(G, np.float64)
    n = g.shape[0]
    if g.ndim != 2 or g.shape[1] != n or n < 1:
        raise ValueError(f"subspace_eigen: square matrix expected, got {g.shape}")
    w = np.zeros(n)
    Y = np.zeros((n, n))
    st = lib.psoci_subspace_eigen(n, _ptr(g, _DP), n, _ptr(w, _DP), _ptr(Y, _DP), n)
    if st != PSOCI_OK:
        raise PsociError(st, "subspace_eigen")
    return w, Y


def write_vectors(path: str, vecs: np.ndarray, binary: bool = False, title: str = ""):
    """CI vectors [nroots, nbasis] to a file in the reference's PsociVector layout."""
    lib = load_library()
    v = np.ascontiguousarray(np.atleast_2d(vecs), np.float64)
    st = lib.psoci_write_vectors(path.encode(), int(binary), v.shape[1], v.shape[0], _ptr(v, _DP), title.encode())
    if st != PSOCI_OK:
        raise PsociError(st, f"write_vectors {path}")


def read_vectors(path: str, nbasis: int, max_roots: int, binary: bool = False) -> np.ndarray:
    lib = load_library()
    out = np.zeros((max_roots, nbasis))
    n = ctypes.c_int()
    st = lib.psoci_read_vectors(path.encode(), int(binary), nbasis, max_roots, _ptr(out, _DP), ctypes.byref(n))
    if st != PSOCI_OK:
        raise PsociError(st, f"read_vectors {path}")
    return out[:n.value]


def solve(problem, nroots: int = 8, mixed: bool = True, rtol: float = 1e-6, device: int = 0, verbose: int = 0,
          **kw) -> DavidsonResult:
    """End to end: host inputs -> determinants -> H -> Davidson -> eigenvalues on the host."""
    with Context(device, verbose) as c:
        c.load_problem(problem)
        c.build_determinants()
        c.build_hamiltonian(mixed=mixed)
        return c.davidson(nroots, rtol=rtol, mixed=mixed, **kw)
