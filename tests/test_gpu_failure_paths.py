"""Failure paths of libtnad on the GPU, made to happen without faulting it.

The environment variable TNAD_TEST_FAULT, read when a context is created, arms
one fault for that context's next call of the affected kind:

* ``tc_withhold`` — the next tensor-core GEMM never issues the TMA loads of
  its first K slice and waits at most 20 ms on its mbarriers.  Every wait on
  that stage runs out; the kernel records the error, drains the copies it did
  issue, frees its TMEM and returns, and the host reports TNAD_ERR_TIMEOUT.
* ``jacobi_cap`` — the next Jacobi SVD may run one FP64 sweep only, so a
  matrix that needs more returns TNAD_ERR_NOT_CONVERGED.

In both cases the same context must then work normally: the next call succeeds
with the correct result.
"""
import ctypes as C
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _context_with_fault(tn, fault):
    os.environ["TNAD_TEST_FAULT"] = fault
    try:
        return tn._lib.Context(0)
    finally:
        del os.environ["TNAD_TEST_FAULT"]


def _gemm(c, tn, A, B, prec):
    M, K = A.shape
    N = B.shape[1]
    out = tn.fzeros((M, N))
    rc = c.lib.tnad_gemm(c.h, prec, b"N", b"N", M, N, K, 1.0, tn.ptr(A), M, tn.ptr(B), K, 0.0, tn.ptr(out), M)
    return rc, out


def test_tensor_core_gemm_bounded_wait_returns_timeout_and_context_recovers(tn):
    rng = np.random.default_rng(5)
    A = np.asfortranarray(rng.standard_normal((256, 384)))
    B = np.asfortranarray(rng.standard_normal((384, 192)))
    c = _context_with_fault(tn, "tc_withhold")
    try:
        rc, _ = _gemm(c, tn, A, B, tn._lib.PREC_TF32X3)
        assert rc == -8, (rc, c.lib.tnad_last_error(c.h))  # TNAD_ERR_TIMEOUT
        assert b"mbarrier" in c.lib.tnad_last_error(c.h)
        rc, out = _gemm(c, tn, A, B, tn._lib.PREC_TF32X3)
        assert rc == 0, c.lib.tnad_last_error(c.h)
        assert np.linalg.norm(out - A @ B) <= 1e-5 * np.linalg.norm(A @ B)
    finally:
        c.close()


def test_jacobi_sweep_cap_returns_not_converged_and_context_recovers(tn):
    A = np.asfortranarray(np.random.default_rng(6).standard_normal((64, 64)))
    c = _context_with_fault(tn, "jacobi_cap")
    try:
        U, S, V = tn.fzeros((64, 64)), tn.fzeros((64,)), tn.fzeros((64, 64))
        rc = c.lib.tnad_svd(c.h, tn.ptr(A), 64, 64, tn.ptr(U), tn.ptr(S), tn.ptr(V))
        assert rc == -4, (rc, c.lib.tnad_last_error(c.h))  # TNAD_ERR_NOT_CONVERGED
        assert b"sweep cap" in c.lib.tnad_last_error(c.h)
        rc = c.lib.tnad_svd(c.h, tn.ptr(A), 64, 64, tn.ptr(U), tn.ptr(S), tn.ptr(V))
        assert rc == 0, c.lib.tnad_last_error(c.h)
        assert np.max(np.abs(S - np.linalg.svd(A, compute_uv=False))) <= 1e-13 * S[0]
    finally:
        c.close()


def test_unarmed_contexts_ignore_unknown_fault_names(tn):
    c = _context_with_fault(tn, "no_such_fault")
    try:
        A = np.asfortranarray(np.random.default_rng(7).standard_normal((256, 384)))
        B = np.asfortranarray(np.random.default_rng(8).standard_normal((384, 192)))
        rc, out = _gemm(c, tn, A, B, tn._lib.PREC_TF32X3)
        assert rc == 0 and np.linalg.norm(out - A @ B) <= 1e-5 * np.linalg.norm(A @ B)
    finally:
        c.close()
