"""The reference's ComplexF64 tests restated against the CPU oracle.

test/trg.jl:22-28 and test/variationalipeps.jl:136-175 check that TRG, CTMRG,
the energy and their gradients accept complex tensors: a real tensor embedded
as complex, or multiplied by a global phase, gives the real result, and an
optimisation from a complex start reaches the real minimum.  The oracle follows
the reference's conjugations (adjoint(cpmat), conj(z) in the projections,
corner', conj(edge) in the edge symmetrisation, conj(bulk) in the double layer,
v' in trg_svd) and Zygote's convention for the gradient of a real function of
a complex array (∂/∂Re + i ∂/∂Im).  Julia's Random.seed!(2) streams cannot be
reproduced; the tensors come from NumPy's default_rng(2).
"""
import numpy as np
import pytest


def test_trg_complex_embedding(orc):
    """test/trg.jl:22-28 (β, χ, niter = 0.4, 12, 3)."""
    torch = pytest.importorskip("torch")
    beta, chi, niter = 0.4, 12, 3
    a = orc.model_tensor_ising(beta)
    z_real = orc.trg(a, chi, niter)
    z_cplx = orc.trg(a.to(torch.complex128), chi, niter)
    assert abs(float(z_real) - float(z_cplx.real)) <= 1e-13 * abs(float(z_real))
    assert abs(float(z_cplx.imag)) <= 1e-14
    b = torch.tensor(beta, dtype=torch.float64, requires_grad=True)
    (g_real,) = torch.autograd.grad(orc.trg(orc.model_tensor_ising(b), chi, niter), b)
    b2 = torch.tensor(beta, dtype=torch.float64, requires_grad=True)
    (g_cplx,) = torch.autograd.grad(orc.trg(orc.model_tensor_ising(b2).to(torch.complex128), chi, niter).real, b2)
    assert abs(float(g_real) - float(g_cplx)) <= 1e-12 * abs(float(g_real))


@pytest.fixture(scope="module")
def sym_ipeps(orc):
    rng = np.random.default_rng(2)
    a = orc.indexperm_symmetrize(orc.as_t(rng.standard_normal((2, 2, 2, 2, 2)))).numpy()
    return a, np.exp(1j * rng.random() * 2 * np.pi)


def test_energy_of_complex_embedding_and_global_phase(orc, sym_ipeps):
    """test/variationalipeps.jl:136-145 (χ=4, tol=1e-12, maxit=100)."""
    a, phi = sym_ipeps
    h = orc.hamiltonian_heisenberg()
    e_real = complex(orc.energy(h, orc.as_t(a), 4, 1e-12, 100))
    e_cplx = complex(orc.energy(h, orc.as_t(a + 0j), 4, 1e-12, 100))
    e_phase = complex(orc.energy(h, orc.as_t(a * phi), 4, 1e-12, 100))
    assert abs(e_cplx - e_real) <= 1e-13 and abs(e_phase - e_real) <= 1e-13


def test_gradient_of_real_energy_for_complex_tensors(orc, sym_ipeps):
    """test/variationalipeps.jl:147-155: the gradient of real(energy) at the complex
    embedding is the real gradient; at a·ϕ it is ϕ times it (the energy is
    invariant under a global phase)."""
    a, phi = sym_ipeps
    h = orc.hamiltonian_heisenberg()
    _, g_real, _ = orc.energy_and_grad(h, a, 4, 1e-12, 100)
    _, g_cplx, _ = orc.energy_and_grad(h, a + 0j, 4, 1e-12, 100)
    _, g_phase, _ = orc.energy_and_grad(h, a * phi, 4, 1e-12, 100)
    scale = np.abs(g_real).max()
    assert np.abs(g_cplx - g_real).max() <= 1e-12 * scale
    assert np.abs(g_phase - phi * g_real).max() <= 1e-12 * scale


def test_optimisation_from_a_complex_start_reaches_the_real_minimum(orc):
    """test/variationalipeps.jl:157-175 (χ=20, tol=1e-12, maxit=100, f_tol=1e-6;
    L-BFGS(m=10) for the complex start), atol 1e-3."""
    rng = np.random.default_rng(2)
    h = orc.hamiltonian_heisenberg()
    a = orc.indexperm_symmetrize(orc.as_t(rng.standard_normal((2, 2, 2, 2, 2)))).numpy()
    e_real, _ = orc.optimiseipeps(a, h, 20, 1e-12, 100, f_tol=1e-6, iters=200, m=20)
    start = rng.standard_normal((2, 2, 2, 2, 2)) + 1j * rng.standard_normal((2, 2, 2, 2, 2))
    ac = orc.indexperm_symmetrize(orc.as_t(start)).numpy()
    e_cplx, x = orc.optimiseipeps(ac, h, 20, 1e-12, 100, f_tol=1e-6, iters=200, m=10)
    assert np.iscomplexobj(x)
    assert abs(e_real - e_cplx) <= 1e-3
