"""The tall-skinny projection C = A^T B (psoci_tsprod) by its three methods — float-float on the
FP32 pipe (the Davidson's own), FP64 FMA, FP64 tensor-core MMA — against numpy, for the shapes
the Davidson meets (up to 40 basis vectors against up to 8 new ones, rows not a multiple of
the kernels' tiles)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,m,k", [(1, 1, 1), (1003, 8, 8), (54321, 40, 8), (70001, 17, 3), (300000, 33, 5)])
def test_tsprod_methods(n, m, k):
    torch = pytest.importorskip("torch")
    from psoci_gb300 import api

    rng = np.random.default_rng(n + m + k)
    lda, ldb = m + 3, k + 1
    A = rng.standard_normal((n, lda))
    B = rng.standard_normal((n, ldb))
    ref = A[:, :m].T @ B[:, :k]
    scale = np.abs(A[:, :m]).sum(0).max() * np.abs(B[:, :k]).max()
    dA = torch.from_numpy(A).cuda()
    dB = torch.from_numpy(B).cuda()
    with api.Context(0) as c:
        for method, tol in ((0, 1e-12), (1, 1e-13), (2, 1e-13)):
            dC = torch.full((m, k), float("nan"), dtype=torch.float64, device="cuda")
            c.tsprod_device(method, n, dA.data_ptr(), lda, m, dB.data_ptr(), ldb, k, dC.data_ptr())
            C = dC.cpu().numpy()
            assert np.isfinite(C).all(), method
            assert np.abs(C - ref).max() <= tol * scale, (method, np.abs(C - ref).max() / scale)
