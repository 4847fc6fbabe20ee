"""The CPU oracle pinned against the reference's published values and tests.

These are the checks that make the oracle trustworthy before it is used to
check the GPU path (restatements of test/trg.jl, test/svd.jl, test/ctmrg.jl,
test/fixedpoint.jl, test/autodiff.jl, test/exampletensors.jl and the README).
"""
import json
from pathlib import Path

import numpy as np
import pytest
import torch

GOLD = json.loads((Path(__file__).parent / "golden" / "reference_values.json").read_text())


def test_trg_readme_chi20(orc):
    z, g = orc.trg_dbeta(0.5, 20, 20)
    assert abs(z - GOLD["trg_ising_b0.5_chi20_n20"]["value"]) < 1e-14
    assert abs(g - GOLD["trg_ising_b0.5_chi20_n20_dbeta"]["value"]) < 1e-12


def test_trg_test_value_and_userguide_gradient(orc):
    z, _ = orc.trg_dbeta(0.4, 5, 5)
    assert abs(z - GOLD["trg_ising_b0.4_chi5_n5"]["value"]) < 1e-14
    _, g = orc.trg_dbeta(0.5, 5, 5)
    assert abs(g - GOLD["trg_ising_b0.5_chi5_n5_dbeta"]["value"]) < 1e-13


def test_trg_gradient_vs_num_grad(orc):
    # test/trg.jl:19: num_grad(foo, 0.4, δ=1e-6) ≈ gradient
    f = lambda b: float(orc.trg(orc.model_tensor_ising(b), 5, 5))
    _, g = orc.trg_dbeta(0.4, 5, 5)
    fd = (f(0.4 + 5e-7) - f(0.4 - 5e-7)) / 1e-6
    assert abs(fd - g) < 1e-6 * abs(g)


def test_trg_svd_reconstructs(orc):
    # test/trg.jl:6-10
    rng = np.random.default_rng(0)
    t = torch.as_tensor(rng.standard_normal((10, 10, 10, 10)))
    u, v = orc.trg_svd(t, 100, 0)
    r = torch.einsum("ija,akl->ijkl", u, v)
    assert torch.allclose(r, t, atol=1e-11)


def test_hamiltonian_heisenberg_readme(orc):
    h = orc.hamiltonian_heisenberg()
    want = np.array(GOLD["heisenberg_h"]["value"])  # [k][l][i][j]
    for k in range(2):
        for l in range(2):
            assert np.array_equal(h[:, :, k, l], want[k][l])


def test_model_tensor_readme_and_tensorfromclassical(orc):
    a = orc.model_tensor_ising(0.5).numpy()
    want = np.array(GOLD["ising_model_tensor_b0.5"]["value"])
    for k in range(2):
        for l in range(2):
            assert np.allclose(a[:, :, k, l], want[k][l], atol=5e-6)
    # test/exampletensors.jl:6-9
    b = 0.37
    assert np.allclose(orc.model_tensor_ising(b).numpy(), orc.tensorfromclassical(np.array([[b, -b], [-b, b]])))


def _taylor_check(f, A, eta=1e-5):
    """gradient_check of test/svd.jl:6-13 (real restatement)."""
    x = A.clone().requires_grad_(True)
    (g,) = torch.autograd.grad(f(x), x)
    dy_expect = eta * float((g * g).sum())
    dy = float(f(A)) - float(f(A - eta * g))
    return np.isclose(dy, dy_expect, rtol=1e-2, atol=1e-8)


@pytest.mark.parametrize("M,N", [(6, 3), (3, 6), (3, 3)])
def test_svd_adjoint_taylor(orc, M, N):
    rng = np.random.default_rng(2)
    H = rng.standard_normal((max(M, N), max(M, N)))
    H = torch.as_tensor(H + H.T)

    def loss_u(A):
        U, S, V = orc.svd(A)
        psi = U[:, 0]
        return psi @ H[:M, :M] @ psi

    def loss_v(A):
        U, S, V = orc.svd(A)
        psi = V[:, 0]
        return psi @ H[:N, :N] @ psi

    def loss_uv(A):
        U, S, V = orc.svd(A)
        return U[0, 0] * V[0, 0]

    def loss_s(A):
        return orc.svd(A)[1].sum()

    A = torch.as_tensor(rng.standard_normal((M, N)))
    for f in (loss_u, loss_v, loss_uv, loss_s):
        assert _taylor_check(f, A)


def test_norm_adjoint(orc):
    # test/autodiff.jl:6-8
    rng = np.random.default_rng(1)
    a = torch.as_tensor(rng.standard_normal((10, 10))).requires_grad_(True)
    (g,) = torch.autograd.grad(orc.norm(a), a)
    fd = np.zeros((10, 10))
    an = a.detach().numpy()
    for i in range(10):
        for j in range(10):
            p, m = an.copy(), an.copy()
            p[i, j] += 5e-6
            m[i, j] -= 5e-6
            fd[i, j] = (np.linalg.norm(p) - np.linalg.norm(m)) / 1e-5
    assert np.allclose(g.numpy(), fd, atol=1e-8)


def test_stopfunction_semantics(orc):
    """maxit bounds the loop at maxit+1 steps; ‖vals₁ − Inf‖ = Inf ≤ Inf stops after one step."""
    a = orc.model_tensor_ising(0.4)
    C, T = orc.init_random(2, 4, np.random.default_rng(0))
    assert orc.ctmrg(a, C, T, tol=0.0, maxit=3).steps == 4
    assert orc.ctmrg(a, C, T, tol=0.0, maxit=0).steps == 1
    assert orc.ctmrg(a, C, T, tol=float("inf"), maxit=10).steps == 1


@pytest.mark.parametrize("beta,chi,atol", [(0.0, 2, 1e-6), (1.0, 2, 1e-8), (0.2, 10, 1e-4), (0.4, 10, 1e-3),
                                           (0.6, 4, 1e-8), (0.8, 2, 1e-8)])
def test_magnetisation_vs_onsager(orc, beta, chi, atol):
    # test/ctmrg.jl:37-42 (isapprox default rtol ~1.5e-8 for the ≈ cases).  The Julia seed
    # stream cannot be reproduced; near βc (β=0.4) 100 steps from a random start leave a
    # seed-dependent residual of up to ~1e-3, so a fixed NumPy seed is used.
    m = orc.magnetisation(beta, chi, np.random.default_rng(2))
    exact = orc.magofbeta(beta)
    assert abs(m - exact) <= max(atol, 1.5e-8 * abs(exact))


def test_energy_gradient_vs_fd(orc):
    h = orc.hamiltonian_heisenberg()
    A = orc.ipeps_uniform(2, 2, 0)
    e, g, _ = orc.energy_and_grad(h, A, 6, 1e-10, 100)
    for idx in [(0, 0, 0, 0, 0), (1, 0, 1, 0, 1), (1, 1, 1, 1, 0)]:
        p, m = A.copy(), A.copy()
        p[idx] += 1e-5
        m[idx] -= 1e-5
        fd = (float(orc.energy(h, torch.as_tensor(p), 6, 1e-10, 100)) -
              float(orc.energy(h, torch.as_tensor(m), 6, 1e-10, 100))) / 2e-5
        assert abs(fd - g[idx]) < 1e-7


def test_non_interacting_product_state(orc):
    # test/variationalipeps.jl:15-20 (seeded NumPy stand-in for the Julia RNG)
    rng = np.random.default_rng(3)
    h = orc.diaglocalhamiltonian([1.0, -1.0])
    a = 1e-12 * rng.standard_normal((2, 2, 2, 2, 2))
    a[0, 0, 0, 0, 1] = rng.standard_normal()
    e = float(orc.energy(h, torch.as_tensor(a), 4, 1e-12, 100))
    assert abs(e / 2 - (-1.0)) < 1e-8


def test_heisenberg_readme_random_energy_range(orc):
    # README.md:104-109: a random symmetrised D=2 iPEPS has E ≈ -0.5 (random input)
    h = orc.hamiltonian_heisenberg()
    e = float(orc.energy(h, torch.as_tensor(orc.ipeps_uniform(2, 2, 0)), 20, 1e-6, 100))
    assert -0.7 < e < -0.3


# ----------------------------------------------------------------- complex SVD adjoint
def _gradient_check(f, x, eta=1e-5):
    """test/svd.jl:6-13: f(x) − f(x − η·g) ≈ η·Σ|g|² (rtol 1e-2, atol 1e-8)."""
    import torch

    xt = torch.as_tensor(x).clone().requires_grad_(True)
    (g,) = torch.autograd.grad(f(xt), xt)
    dy = float(f(torch.as_tensor(x))) - float(f(torch.as_tensor(x) - eta * g))
    dy_expect = eta * float((g.abs() ** 2).sum())
    return abs(dy - dy_expect) <= 1e-8 + 1e-2 * abs(dy_expect)


def _complex_losses(orc, seed):
    import torch

    def loss_u(A):
        U, S, V = orc.svd(A)
        H = torch.as_tensor(_herm(A.shape[0], seed))
        psi = U[:, 0]
        return (psi.conj() @ H @ psi).real

    def loss_v(A):
        U, S, V = orc.svd(A)
        H = torch.as_tensor(_herm(A.shape[1], seed))
        psi = V[:, 0]
        return (psi.conj() @ H @ psi).real

    def loss_uv(A):
        U, S, V = orc.svd(A)
        return (U[0, 0].conj() * V[0, 0]).real

    def loss_s(A):
        U, S, V = orc.svd(A)
        return S.sum()

    return {"U": loss_u, "V": loss_v, "UV": loss_uv, "S": loss_s}


def _herm(n, seed):
    rng = np.random.default_rng(seed)
    H = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    return H + H.conj().T


@pytest.mark.parametrize("shape", [(6, 3), (3, 6), (3, 3)])
@pytest.mark.parametrize("which", ["U", "V", "UV", "S"])
def test_oracle_complex_svd_adjoint_taylor(orc, shape, which):
    """test/svd.jl:15-101 (svd grad U, V, U+V, S on complex (6,3), (3,6), (3,3))
    on the oracle's complex restatement of svd_back."""
    rng = np.random.default_rng(10 * shape[0] + shape[1] + 100 * ["U", "V", "UV", "S"].index(which))
    a = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    assert _gradient_check(_complex_losses(orc, 2)[which], a)


def test_oracle_complex_svd_adjoint_imag_diag(orc):
    """test/svd.jl:69-86: the fixed 2×2 complex A, gradient of Re(conj(U[1,1])·V[1,1])
    against a central difference in Re and Im of A[2,1] (atol 1e-3)."""
    import torch

    loss = _complex_losses(orc, 2)["UV"]
    A = np.array([[-1 + 1j, 2 + 1j], [1 - 2j, 3 + 0.8j]])
    da = np.array([[0, 0], [1, 0]], dtype=complex)
    f = lambda x: float(loss(torch.as_tensor(x)))
    nd = (f(A + 1e-4 * da) - f(A - 1e-4 * da)) / 2e-4 + 1j * (f(A + 1e-4j * da) - f(A - 1e-4j * da)) / 2e-4
    At = torch.as_tensor(A).clone().requires_grad_(True)
    (g,) = torch.autograd.grad(loss(At), At)
    assert abs(complex(g[1, 0]) - nd) <= 1e-3
    assert _gradient_check(loss, A)
