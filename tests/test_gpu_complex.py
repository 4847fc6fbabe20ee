"""ComplexF64 SVD and SVD adjoint on the GPU (tnad_svd_z, tnad_svd_back_z)
against LAPACK, the oracle's complex restatement of svd_back
(src/trg.jl:72-105 with the imaginary-diagonal term of :85), and the
reference's own complex SVD tests (test/svd.jl:15-101) run through the GPU
decomposition and adjoint."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

SHAPES = [(6, 3), (3, 6), (3, 3), (50, 40), (40, 50), (1, 4)]


def _crandn(rng, shape):
    return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)


@pytest.mark.parametrize("m,n", SHAPES)
def test_complex_svd_matches_lapack(tn, m, n):
    rng = np.random.default_rng(m * 100 + n)
    A = _crandn(rng, (m, n))
    U, S, V = tn.svd_complex(A)
    k = min(m, n)
    assert U.shape == (m, k) and V.shape == (n, k) and S.shape == (k,)
    assert np.max(np.abs(S - np.linalg.svd(A, compute_uv=False))) <= 1e-13 * S[0]
    assert np.allclose(U @ np.diag(S) @ V.conj().T, A, atol=1e-12 * np.abs(A).max() * max(m, n))
    assert np.allclose(U.conj().T @ U, np.eye(k), atol=1e-13 * k)
    assert np.allclose(V.conj().T @ V, np.eye(k), atol=1e-13 * k)


@pytest.mark.parametrize("m,n", SHAPES)
def test_complex_svd_back_matches_oracle(tn, orc, m, n):
    rng = np.random.default_rng(7 * m + n)
    A = _crandn(rng, (m, n))
    U, S, Vh = np.linalg.svd(A, full_matrices=False)
    V = Vh.conj().T
    k = min(m, n)
    dU, dS, dV = _crandn(rng, (m, k)), rng.standard_normal(k), _crandn(rng, (n, k))
    got = tn.svd_back_complex(U, S, V, dU, dS, dV)
    ref = orc.svd_back(*(torch.as_tensor(x) for x in (U, S, V, dU, dS, dV))).numpy()
    assert np.max(np.abs(got - ref)) <= 1e-12 * np.abs(ref).max()
    got_u = tn.svd_back_complex(U, S, V, dU=dU)
    ref_u = orc.svd_back(torch.as_tensor(U), torch.as_tensor(S), torch.as_tensor(V), torch.as_tensor(dU), None,
                         None).numpy()
    assert np.max(np.abs(got_u - ref_u)) <= 1e-12 * np.abs(ref_u).max()


def _herm(n, seed):
    rng = np.random.default_rng(seed)
    H = _crandn(rng, (n, n))
    return H + H.conj().T


def _loss_and_grad(tn, which, A):
    """A loss of test/svd.jl through the GPU SVD, and its gradient (Zygote's
    convention ∂L/∂Re A + i·∂L/∂Im A) through the GPU adjoint."""
    U, S, V = tn.svd_complex(A)
    m, n = A.shape
    dU = dS = dV = None
    if which == "U":
        H = _herm(m, 2)
        psi = U[:, 0]
        L = float(np.real(psi.conj() @ H @ psi))
        dU = np.zeros_like(U)
        dU[:, 0] = 2 * H @ psi
    elif which == "V":
        H = _herm(n, 2)
        psi = V[:, 0]
        L = float(np.real(psi.conj() @ H @ psi))
        dV = np.zeros_like(V)
        dV[:, 0] = 2 * H @ psi
    elif which == "UV":
        L = float(np.real(np.conj(U[0, 0]) * V[0, 0]))
        dU, dV = np.zeros_like(U), np.zeros_like(V)
        dU[0, 0] = V[0, 0]          # ∂/∂Re u + i∂/∂Im u of Re(conj(u)·v) is v
        dV[0, 0] = U[0, 0]          # and of v it is u
    else:
        L = float(S.sum())
        dS = np.ones_like(S)
    return L, tn.svd_back_complex(U, S, V, dU, dS, dV)


@pytest.mark.parametrize("shape", [(6, 3), (3, 6), (3, 3)])
@pytest.mark.parametrize("which", ["U", "V", "UV", "S"])
def test_reference_complex_svd_gradient_checks_on_gpu(tn, shape, which):
    """test/svd.jl:6-13's first-order check f(A) − f(A − η·g) ≈ η·Σ|g|² (rtol
    1e-2, atol 1e-8, η = 1e-5), with f and g from the GPU."""
    rng = np.random.default_rng(10 * shape[0] + shape[1] + 100 * ["U", "V", "UV", "S"].index(which))
    A = _crandn(rng, shape)
    L, g = _loss_and_grad(tn, which, A)
    L2, _ = _loss_and_grad(tn, which, A - 1e-5 * g)
    dy, dy_expect = L - L2, 1e-5 * float(np.sum(np.abs(g) ** 2))
    assert abs(dy - dy_expect) <= 1e-8 + 1e-2 * abs(dy_expect), (dy, dy_expect)


def test_reference_imag_diag_case_on_gpu(tn):
    """test/svd.jl:69-86: the fixed 2×2 A, the gradient entry [2,1] against a
    central difference in its real and imaginary parts (atol 1e-3)."""
    A = np.array([[-1 + 1j, 2 + 1j], [1 - 2j, 3 + 0.8j]])
    da = np.array([[0, 0], [1, 0]], dtype=complex)
    f = lambda x: _loss_and_grad(tn, "UV", x)[0]
    nd = (f(A + 1e-4 * da) - f(A - 1e-4 * da)) / 2e-4 + 1j * (f(A + 1e-4j * da) - f(A - 1e-4j * da)) / 2e-4
    _, g = _loss_and_grad(tn, "UV", A)
    assert abs(g[1, 0] - nd) <= 1e-3, (g[1, 0], nd)
