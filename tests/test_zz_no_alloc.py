"""The allocation-free mixed sigma (psoci_sigma_mixed_noalloc) against psoci_sigma_device.

psoci_sigma_mixed_noalloc exists for callers that cannot call cudaMalloc while they run (work
issued inside a stream capture, hosts whose allocator owns the whole GPU memory budget, loops
that must not take an allocation's implicit synchronisation).  It stages its FP32 inputs in a
fixed 16 MiB device array instead of a buffer grown on demand.  Both entry points run the same
kernels, so their outputs must agree; two calls in a row check that the shared array's old
contents do not leak into the next result.  This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_noalloc_sigma_matches_sigma_device():
    torch = pytest.importorskip("torch")
    from helpers import small_problem
    from psoci_gb300 import api

    lib = api.load_library()
    f = lib.psoci_sigma_mixed_noalloc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int]

    p = small_problem("fci_6e8o", 1)
    with api.Context(0) as c:
        c.load_problem(p)
        c.build_determinants()
        c.build_hamiltonian(mixed=True)
        n = c.nsef
        gen = torch.Generator(device="cpu").manual_seed(0)
        for k in (8, 5):  # two calls in a row, different widths and inputs
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
            assert np.abs(new - ref).max() <= 1e-12 * scale
