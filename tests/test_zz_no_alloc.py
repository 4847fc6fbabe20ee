"""tnad_svd_noalloc: the allocation-free SVD entry point.

Some callers cannot call cudaMalloc — a host framework that owns all device
memory through its own allocator, or a latency-critical loop where an
allocation would synchronise the device.  For them tnad_svd_noalloc works on
caller-supplied device buffers and a fixed static scratch array (matrices up to
256×256).  This test calls it through the C ABI twice in a row per case and
checks both results against LAPACK's singular values and the orthogonality of
U and V (an independent check), and against the regular entry point tnad_svd
(same Jacobi kernels) at the FP64 tolerance the other SVD tests use.  The cases
cover a full-rank square matrix, a tall one, a rank-deficient one (whose null
columns go through the weak-column completion and its scratch slots) and a call
on a non-default stream.  The file is collected last (its name), and runs alone
in a fresh process as well as after the other tests.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc_svd(tn, A_dev, m, n, torch, stream=None):
    lib = tn._lib.load()
    U = torch.zeros(m * n, dtype=torch.float64, device="cuda")
    S = torch.zeros(n, dtype=torch.float64, device="cuda")
    V = torch.zeros(n * n, dtype=torch.float64, device="cuda")
    st = stream if stream is not None else torch.cuda.current_stream()
    st.wait_stream(torch.cuda.current_stream())  # A, U, S, V were written on the current stream
    rc = lib.tnad_svd_noalloc(tn.ptr(A_dev.data_ptr()), m, n, tn.ptr(U.data_ptr()), tn.ptr(S.data_ptr()),
                              tn.ptr(V.data_ptr()), C.c_void_p(st.cuda_stream))
    torch.cuda.synchronize()
    assert rc == 0, rc
    f = lambda t, shape: t.cpu().numpy().reshape(shape, order="F")
    return f(U, (m, n)), S.cpu().numpy(), f(V, (n, n))


def _matrix(kind, m, n, rng):
    A = rng.standard_normal((m, n))
    if kind == "rank_deficient":
        A[:, 30:] = A[:, : n - 30]  # repeated columns: rank 30, n − 30 null directions
    return A


@pytest.mark.parametrize("kind,m,n,own_stream", [("full", 200, 200, False), ("full", 96, 61, False),
                                                 ("rank_deficient", 96, 61, False), ("full", 150, 120, True)])
def test_svd_noalloc_matches_lapack_and_tnad_svd_twice(tn, kind, m, n, own_stream):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(m + n + len(kind))
    stream = torch.cuda.Stream() if own_stream else None
    for call in range(2):  # the second call reuses the scratch left by the first
        A = _matrix(kind, m, n, rng)
        A_dev = torch.tensor(A.ravel(order="F"), device="cuda")
        U, S, V = _noalloc_svd(tn, A_dev, m, n, torch, stream)
        # independent checks: LAPACK's singular values, orthogonal factors, reconstruction
        S_lapack = np.linalg.svd(A, compute_uv=False)
        assert np.max(np.abs(S - S_lapack)) <= 1e-13 * S_lapack[0], (call, np.max(np.abs(S - S_lapack)))
        assert np.max(np.abs(U.T @ U - np.eye(n))) <= 1e-13 * n, call
        assert np.max(np.abs(V.T @ V - np.eye(n))) <= 1e-13 * n, call
        assert np.allclose(U @ np.diag(S) @ V.T, A, atol=1e-12 * np.abs(A).max() * n)
        # the regular entry point: same kernels in the same order, so the factors
        # agree column by column
        U_r, S_r, V_r = tn.svd(A)
        assert np.max(np.abs(S - S_r)) <= 1e-13 * S_r[0]
        assert np.max(np.abs(U - U_r)) <= 1e-12
        assert np.max(np.abs(V - V_r)) <= 1e-12


def test_svd_noalloc_rejects_sizes_beyond_its_scratch(tn):
    torch = pytest.importorskip("torch")
    lib = tn._lib.load()
    buf = torch.zeros(300 * 300, dtype=torch.float64, device="cuda")
    p = tn.ptr(buf.data_ptr())
    assert lib.tnad_svd_noalloc(p, 300, 300, p, p, p, None) == -2  # TNAD_ERR_SHAPE
    assert lib.tnad_svd_noalloc(p, 300, 200, p, p, p, None) == -2
    assert lib.tnad_svd_noalloc(p, 100, 120, p, p, p, None) == -1  # m < n: TNAD_ERR_ARG
