"""Symmetric SVD of the CTMRG corner (src/ctmrg.jl:134-136) on the GPU: FP32
Jacobi sweeps with the eigenvalue rule, polished to FP64 by the product
refinement (or by FP64 Jacobi sweeps where the refinement does not converge),
against LAPACK on seeded symmetric matrices with the spectra the path meets:

* exact ±λ pairs with the spectral profile of the D=4 N(0,1) workloads' corner
  (|λ| from 1 down to ~1e-5, every singular value shared by two eigenvalues)
  — refinement;
* a zero-padded rank-deficient matrix (the first CTMRG steps from the :raw
  environment) — refinement, with the null space as one unresolved group;
* a graded spectrum down to the rounding floor (the uniform-tensor D=2/D=3
  workloads) — FP32 cannot separate its small eigenvalues, so the refinement
  gives up and the FP64 sweeps finish.

Tolerances: LAPACK's own accuracy is ~n·ε·‖A‖ for eigenvalues and residuals;
the tests allow 1e-12 of ‖A‖ (2e-12 with the tensor-core products, whose
terms are accurate to ~2^-47 of the row and column scales).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _orth(n, rng):
    q, r = np.linalg.qr(rng.standard_normal((n, n)))
    return q * np.sign(np.diag(r))


# log10 of |λ|/|λ_1| against the fraction of the spectrum, read off the
# converged enlarged corner of the D=4, χ=64 N(0,1) workload (every value twice)
_CORNER_F = [0.0, 0.03, 0.0625, 0.125, 0.25, 0.5, 0.75, 0.9, 0.95, 0.98, 0.99, 1.0]
_CORNER_L = [0.0, -1.04, -1.31, -1.63, -2.01, -2.50, -2.96, -3.45, -3.72, -4.07, -4.31, -5.25]


def corner_like(n, seed):
    """±λ pairs with the spectral profile of the D=4, χ=64 corner, random eigenvectors."""
    rng = np.random.default_rng(seed)
    f = (np.arange(n // 2) + 0.5) / (n // 2)
    mags = 10.0 ** (np.interp(f, _CORNER_F, _CORNER_L) + 0.02 * rng.standard_normal(n // 2))
    lam = np.concatenate([mags, -mags])
    Q = _orth(n, rng)
    A = (Q * lam) @ Q.T
    return 0.5 * (A + A.T), lam


def rank_deficient(n, r, seed):
    rng = np.random.default_rng(seed)
    P = _orth(n, rng)[:, :r]
    lam = rng.standard_normal(r)
    A = (P * lam) @ P.T
    return 0.5 * (A + A.T), np.concatenate([lam, np.zeros(n - r)])


def graded(n, seed):
    rng = np.random.default_rng(seed)
    lam = 10.0 ** (-14.0 * np.arange(n) / n) * rng.choice([-1.0, 1.0], n)
    Q = _orth(n, rng)
    A = (Q * lam) @ Q.T
    return 0.5 * (A + A.T), lam


def check_svd(A, U, S, V, tol):
    n = A.shape[0]
    nA = np.linalg.norm(A, 2)
    ref = np.sort(np.abs(np.linalg.eigvalsh(A)))[::-1]
    assert np.all(np.diff(S) <= 0.0)
    assert np.max(np.abs(S - ref)) <= tol * nA
    assert np.max(np.abs(V.T @ V - np.eye(n))) <= tol * 10
    assert np.max(np.abs(U.T @ U - np.eye(n))) <= tol * 10
    # A·V = U·diag(S), column by column, and U = V·sign(λ)
    assert np.max(np.abs(A @ V - U * S)) <= tol * nA
    assert np.allclose(np.abs(U), np.abs(V), atol=0.0, rtol=0.0)


@pytest.mark.parametrize("n", [256, 512, 1024])
@pytest.mark.parametrize("tc", [False, True])
def test_corner_spectrum_with_pm_pairs_is_refined(tn, n, tc):
    A, _ = corner_like(n, n + 1)
    r0, f0 = tn.solver_stats()
    U, S, V = tn.svd_symmetric(A, tensor_cores=tc)
    r1, f1 = tn.solver_stats()
    assert (r1 - r0, f1 - f0) == (1, 0)
    check_svd(A, U, S, V, 2e-12 if tc else 1e-12)


def test_rank_deficient_is_refined(tn):
    A, _ = rank_deficient(1024, 256, 3)
    r0, f0 = tn.solver_stats()
    U, S, V = tn.svd_symmetric(A)
    r1, f1 = tn.solver_stats()
    assert (r1 - r0, f1 - f0) == (1, 0)
    check_svd(A, U, S, V, 1e-12)


def test_graded_spectrum_falls_back_to_sweeps(tn):
    A, _ = graded(324, 5)
    r0, f0 = tn.solver_stats()
    U, S, V = tn.svd_symmetric(A)
    r1, f1 = tn.solver_stats()
    assert r1 - r0 + f1 - f0 == 1
    check_svd(A, U, S, V, 1e-12)


def test_two_calls_in_a_row_agree(tn):
    A, _ = corner_like(512, 11)
    U1, S1, V1 = tn.svd_symmetric(A, tensor_cores=True)
    U2, S2, V2 = tn.svd_symmetric(A, tensor_cores=True)
    assert np.array_equal(S1, S2) and np.array_equal(U1, U2) and np.array_equal(V1, V2)
