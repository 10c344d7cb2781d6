"""The allocation-free mixed sigma (psoci_sigma_mixed_noalloc) against psoci_sigma_device.

psoci_sigma_mixed_noalloc exists for callers that cannot call cudaMalloc while they run: host
programs whose own allocator owns the whole GPU memory budget, and loops that must not take an
allocation's implicit synchronisation.  It stages its FP32 inputs in a fixed 16 MiB device
array instead of a buffer grown on demand.  Both entry points run the same kernels, so their
outputs must agree.  Three calls in a row (8, 3 and 11 vectors: the row stride of the staged
copy changes between calls, and 11 vectors take two chunks through the one array) check that
the shared array's old contents do not leak into the next result.  The rejections (no FP32
copy, direct mode, more SEFs than the array holds) are checked too.  This file is collected
last on purpose.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PSOCI_ERR_UNSUPPORTED, PSOCI_ERR_STATE = 2, 3


def _noalloc(lib):
    f = lib.psoci_sigma_mixed_noalloc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int]
    return f


def test_noalloc_sigma_matches_sigma_device():
    torch = pytest.importorskip("torch")
    from helpers import small_problem
    from psoci_gb300 import api

    lib = api.load_library()
    f = _noalloc(lib)
    p = small_problem("fci_6e8o", 1)
    with api.Context(0) as c:
        c.load_problem(p)
        c.build_determinants()
        c.build_hamiltonian(mixed=True)
        n = c.nsef
        gen = torch.Generator(device="cpu").manual_seed(0)
        for k in (8, 3, 11):  # calls in a row: different widths, strides and inputs
            X = torch.randn(n, k, dtype=torch.float64, generator=gen).to("cuda:0")
            Y_ref = torch.zeros(n, k, dtype=torch.float64, device="cuda:0")
            Y_new = torch.full((n, k), float("nan"), dtype=torch.float64, device="cuda:0")
            torch.cuda.synchronize()
            c.sigma_device(X.data_ptr(), k, Y_ref.data_ptr(), k, k, api.PREC_MIXED)
            st = f(c.ctx, k, ctypes.c_void_p(X.data_ptr()), k, ctypes.c_void_p(Y_new.data_ptr()), k)
            assert st == 0, lib.psoci_last_error(c.ctx)
            torch.cuda.synchronize()
            ref, new = Y_ref.cpu().numpy(), Y_new.cpu().numpy()
            scale = np.abs(ref).max()
            assert np.isfinite(new).all()
            assert np.abs(new - ref).max() <= 1e-12 * scale, k


def test_noalloc_sigma_rejections():
    torch = pytest.importorskip("torch")
    from helpers import small_problem
    from psoci_gb300 import api
    from psoci_gb300.inputs import named_workload

    lib = api.load_library()
    f = _noalloc(lib)
    p = small_problem("fci_6e8o", 1)
    with api.Context(0) as c:
        c.load_problem(p)
        c.build_determinants()
        X = torch.zeros(c.nsef, 4, dtype=torch.float64, device="cuda:0")
        Y = torch.zeros_like(X)
        c.build_hamiltonian(mixed=False)  # no FP32 copy
        assert f(c.ctx, 4, ctypes.c_void_p(X.data_ptr()), 4, ctypes.c_void_p(Y.data_ptr()), 4) == PSOCI_ERR_STATE
        c.build_hamiltonian(direct=True)  # nothing stored
        assert f(c.ctx, 4, ctypes.c_void_p(X.data_ptr()), 4, ctypes.c_void_p(Y.data_ptr()), 4) == PSOCI_ERR_STATE
    big = named_workload("mrcisd_6e8o_v24", seed=1)  # 568,204 SEFs > 524,288
    with api.Context(0) as c:
        c.load_problem(big)
        c.build_determinants()
        c.build_hamiltonian(mixed=True)
        assert c.nsef > 524288
        X = torch.zeros(c.nsef, 1, dtype=torch.float64, device="cuda:0")
        Y = torch.zeros_like(X)
        st = f(c.ctx, 1, ctypes.c_void_p(X.data_ptr()), 1, ctypes.c_void_p(Y.data_ptr()), 1)
        assert st == PSOCI_ERR_UNSUPPORTED
        assert b"524288" in lib.psoci_last_error(c.ctx)
