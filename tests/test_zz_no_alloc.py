"""tnad_svd_noalloc: the allocation-free SVD entry point.

Some callers cannot call cudaMalloc — a host framework that owns all device
memory through its own allocator, or a latency-critical loop where an
allocation would synchronise the device.  For them tnad_svd_noalloc works on
caller-supplied device buffers and a fixed static scratch array (matrices up to
256×256).  This test calls it through the C ABI twice in a row and checks both
results against the regular entry point tnad_svd (same Jacobi kernels) at the
FP64 tolerance the other SVD tests use.  It is collected last (file name), runs
alone in a fresh process as well as after the other tests.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc_svd(tn, A_dev, m, n, torch):
    lib = tn._lib.load()
    U = torch.zeros(m * n, dtype=torch.float64, device="cuda")
    S = torch.zeros(n, dtype=torch.float64, device="cuda")
    V = torch.zeros(n * n, dtype=torch.float64, device="cuda")
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = lib.tnad_svd_noalloc(tn.ptr(A_dev.data_ptr()), m, n, tn.ptr(U.data_ptr()), tn.ptr(S.data_ptr()),
                              tn.ptr(V.data_ptr()), stream)
    torch.cuda.synchronize()
    assert rc == 0, rc
    f = lambda t, shape: t.cpu().numpy().reshape(shape, order="F")
    return f(U, (m, n)), S.cpu().numpy(), f(V, (n, n))


@pytest.mark.parametrize("m,n", [(200, 200), (96, 61)])
def test_svd_noalloc_matches_tnad_svd_twice(tn, m, n):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(m + n)
    for call in range(2):  # the second call reuses the scratch left by the first
        A = rng.standard_normal((m, n))
        A_dev = torch.tensor(A.ravel(order="F"), device="cuda")
        U, S, V = _noalloc_svd(tn, A_dev, m, n, torch)
        U_r, S_r, V_r = tn.svd(A)  # the regular entry point
        assert np.max(np.abs(S - S_r)) <= 1e-13 * S_r[0]
        assert np.allclose(U @ np.diag(S) @ V.T, A, atol=1e-12 * np.abs(A).max() * n)
        # same kernels in the same order: the factors agree column by column
        assert np.max(np.abs(U - U_r)) <= 1e-12
        assert np.max(np.abs(V - V_r)) <= 1e-12


def test_svd_noalloc_rejects_sizes_beyond_its_scratch(tn):
    torch = pytest.importorskip("torch")
    lib = tn._lib.load()
    buf = torch.zeros(300 * 300, dtype=torch.float64, device="cuda")
    p = tn.ptr(buf.data_ptr())
    assert lib.tnad_svd_noalloc(p, 300, 300, p, p, p, None) == -2  # TNAD_ERR_SHAPE
