"""CPU checks of the symmetric corner SVD's algorithm (oracle/eig_refine_oracle.py,
the NumPy restatement of csrc/jacobi.cu's eigenvalue-rule FP32 sweeps and
csrc/eig_refine.cu's product refinement) against LAPACK:

* the spectra the GPU refines (±λ pairs with the D=4 corner's profile; a null
  space) come out at LAPACK accuracy;
* a graded spectrum is handed back (where the GPU falls back to FP64 sweeps);
* the CTMRG energy gradient (the reference's unrolled reverse with svd_back,
  src/trg.jl:72-105) does not depend on which of the two decompositions of the
  corner is used: the restated one agrees with LAPACK's to 1e-10.
"""
import numpy as np
import pytest

from test_gpu_eig_refine import corner_like, graded, rank_deficient


@pytest.fixture(scope="module")
def er():
    from oracle import eig_refine_oracle

    return eig_refine_oracle


def _check(A, out, tol=1e-13):
    assert out is not None
    U, S, V = out
    ref = np.sort(np.abs(np.linalg.eigvalsh(A)))[::-1]
    n = A.shape[0]
    assert np.max(np.abs(S - ref)) <= tol * ref[0]
    assert np.max(np.abs(V.T @ V - np.eye(n))) <= 1e-13
    assert np.max(np.abs(A @ V - U * S)) <= tol * ref[0]


def test_corner_spectrum_is_refined_to_lapack_accuracy(er):
    A, _ = corner_like(256, 4)
    _check(A, er.svd_symmetric(A))


def test_null_space_stays_one_unsolved_group(er):
    A, _ = rank_deficient(256, 64, 5)
    _check(A, er.svd_symmetric(A))


def test_graded_spectrum_is_handed_back(er):
    A, _ = graded(256, 6)
    assert er.svd_symmetric(A) is None


def test_ctmrg_gradient_does_not_depend_on_the_corner_decomposition(er, orc):
    """Three CTMRG steps at D=4, χ=16 (n = 256) and the energy gradient, with
    LAPACK's SVD and with the restated GPU decomposition of every corner."""
    torch = pytest.importorskip("torch")

    class RestatedSVD(torch.autograd.Function):
        @staticmethod
        def forward(ctx, A):
            out = er.svd_symmetric(A.detach().numpy())
            assert out is not None
            U, S, V = (torch.from_numpy(np.ascontiguousarray(x)) for x in out)
            ctx.save_for_backward(U, S, V)
            ctx.set_materialize_grads(False)
            return U, S, V

        @staticmethod
        def backward(ctx, dU, dS, dV):
            U, S, V = ctx.saved_tensors
            return orc.svd_back(U, S, V, dU, dS, dV)

    bulk = orc.ipeps_normal_maxabs(4, 2, 0)
    h = orc.hamiltonian_heisenberg()
    e0, g0, _ = orc.energy_and_grad(h, bulk, 16, 0.0, 2)
    lapack_svd = orc.svd
    orc.svd = lambda A: RestatedSVD.apply(A)
    try:
        e1, g1, _ = orc.energy_and_grad(h, bulk, 16, 0.0, 2)
    finally:
        orc.svd = lapack_svd
    assert abs(e1 - e0) <= 1e-13 * abs(e0)
    assert np.linalg.norm(g1 - g0) <= 1e-10 * np.linalg.norm(g0)
