"""GPU parity of libtnad (plain FP64 path) against the CPU oracle and the
reference's published values.  Every call goes through the C ABI.

Gauge: the projector z = u[:, 1:χ] is defined up to column signs (and rotations
inside degenerate multiplets), so environments are compared through
gauge-invariant quantities (singular values, energies, traces of products,
input gradients), never element by element.
"""
import json
from pathlib import Path

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

GOLD = json.loads((Path(__file__).parent / "golden" / "reference_values.json").read_text())
RTOL_FP64 = 1e-10  # the plain FP64 path's parity bar (relative)


def rel(a, b):
    a, b = np.asarray(a, dtype=float), np.asarray(b, dtype=float)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


# ----------------------------------------------------------------- decompositions
@pytest.mark.parametrize("m,n", [(1, 1), (7, 7), (50, 50), (80, 61), (200, 200)])
def test_svd_matches_lapack(tn, m, n):
    rng = np.random.default_rng(m * 1000 + n)
    A = rng.standard_normal((m, n))
    U, S, V = tn.svd(A)
    S_ref = np.linalg.svd(A, compute_uv=False)
    assert rel(S, S_ref) < 1e-13
    assert np.allclose(U @ np.diag(S) @ V.T, A, atol=1e-12 * np.abs(A).max() * n)
    assert np.allclose(U.T @ U, np.eye(n), atol=1e-13 * n)
    assert np.allclose(V.T @ V, np.eye(n), atol=1e-13 * n)


def test_svd_rank_deficient_and_zero_columns(tn):
    rng = np.random.default_rng(1)
    B = rng.standard_normal((30, 4))
    A = B @ rng.standard_normal((4, 30))  # rank 4
    A[:, 7] = 0.0
    U, S, V = tn.svd(A)
    assert np.allclose(U.T @ U, np.eye(30), atol=1e-12)
    assert np.allclose(U @ np.diag(S) @ V.T, A, atol=1e-11)
    assert np.all(S[4:] < 1e-12 * S[0])


def test_svd_back_matches_oracle(tn, orc):
    rng = np.random.default_rng(3)
    for m, n in [(12, 12), (20, 9)]:
        A = rng.standard_normal((m, n))
        U, S, Vh = np.linalg.svd(A, full_matrices=False)
        V = Vh.T
        dU, dS, dV = rng.standard_normal((m, n)), rng.standard_normal(n), rng.standard_normal((n, n))
        got = tn.svd_back(U, S, V, dU, dS, dV)
        ref = orc.svd_back(*(torch.as_tensor(x) for x in (U, S, V, dU, dS, dV))).numpy()
        assert rel(got, ref) < 1e-12
        got_u = tn.svd_back(U, S, V, dU=dU)
        ref_u = orc.svd_back(torch.as_tensor(U), torch.as_tensor(S), torch.as_tensor(V), torch.as_tensor(dU), None,
                             None).numpy()
        assert rel(got_u, ref_u) < 1e-12


# ----------------------------------------------------------------- TRG
def test_trg_readme_values(tn):
    lnZ, g = tn.trg_beta(0.5, 20, 20)
    assert abs(lnZ - GOLD["trg_ising_b0.5_chi20_n20"]["value"]) < 1e-12
    assert abs(g - GOLD["trg_ising_b0.5_chi20_n20_dbeta"]["value"]) < 1e-9


def test_trg_test_values(tn):
    assert abs(tn.trg(tn.model_tensor(tn.Ising(), 0.4), 5, 5) - GOLD["trg_ising_b0.4_chi5_n5"]["value"]) < 1e-12
    _, g = tn.trg_beta(0.5, 5, 5)
    assert abs(g - GOLD["trg_ising_b0.5_chi5_n5_dbeta"]["value"]) < 1e-10


@pytest.mark.parametrize("beta,chi,niter", [(0.3, 8, 6), (0.44, 12, 8), (0.6, 16, 10), (0.5, 20, 20)])
def test_trg_matches_oracle(tn, orc, beta, chi, niter):
    """ln Z and d ln Z/dβ against the oracle at the FP64 bar (1e-10 relative),
    including the README configuration β = 0.5, χ = 20, niter = 20."""
    lnZ, g = tn.trg_beta(beta, chi, niter)
    z_ref, g_ref = orc.trg_dbeta(beta, chi, niter)
    assert abs(lnZ - z_ref) < RTOL_FP64 * abs(z_ref)
    assert abs(g - g_ref) < RTOL_FP64 * abs(g_ref)


def test_trg_gradient_vs_num_grad(tn):
    # test/trg.jl:19
    f = lambda b: tn.trg(tn.model_tensor(tn.Ising(), b), 5, 5)
    _, g = tn.trg_beta(0.4, 5, 5)
    assert abs(tn.num_grad(f, 0.4, delta=1e-6) - g) < 1e-6 * abs(g)


def test_trg_svd_reconstructs(tn):
    # test/trg.jl:6-10
    t = np.random.default_rng(0).standard_normal((10, 10, 10, 10))
    u, v = tn.trg_svd(t, 100, 0)
    assert np.allclose(np.einsum("ija,akl->ijkl", u, v), t, atol=1e-11)


# ----------------------------------------------------------------- CTMRG
def _sym_bulk(orc, D, seed):
    A = orc.symmetrized(orc.ipeps_uniform(D, 2, seed))
    _, a = orc.double_layer(torch.as_tensor(A))
    return a.numpy()


def _invariants(C, T):
    C, T = np.asarray(C), np.asarray(T)
    ev = np.sort(np.abs(np.linalg.eigvalsh((C + C.T) / 2)))
    inv = [np.trace(np.linalg.matrix_power(C, 4))]
    inv.append(sum(np.trace(T[:, j, :] @ C @ T[:, j, :] @ C) for j in range(T.shape[1])))
    return ev, np.array(inv)


def test_init_raw_matches_oracle(tn, orc):
    a = _sym_bulk(orc, 2, 0)
    for chi in (2, 4, 9):
        C0, T0 = orc.init_raw(torch.as_tensor(a), chi)
        rt = tn.SquareCTMRGRuntime(a, "raw", chi)
        assert np.array_equal(rt.corner, C0.numpy()) or rel(rt.corner, C0.numpy()) < 1e-15
        assert rel(rt.edge, T0.numpy()) < 1e-15


def test_ctmrgstep_matches_oracle(tn, orc):
    a = _sym_bulk(orc, 2, 1)
    C, T = orc.init_random(4, 6, np.random.default_rng(7))
    rt = tn.SquareCTMRGRuntime(a, C.numpy(), T.numpy())
    rt2, vals = tn.ctmrgstep(rt)
    Cr, Tr, vr = orc.ctmrgstep(torch.as_tensor(a), C, T)
    assert rel(vals, vr.numpy()) < 1e-11
    ev, inv = _invariants(rt2.corner, rt2.edge)
    ev_r, inv_r = _invariants(Cr.numpy(), Tr.numpy())
    assert rel(ev, ev_r) < 1e-11
    assert rel(inv, inv_r) < 1e-11


def test_ctmrgstep_backward_matches_oracle(tn, orc):
    a = _sym_bulk(orc, 2, 2)
    C, T = orc.init_random(4, 6, np.random.default_rng(8))

    def f(Cn, Tn):  # gauge-invariant scalar of the new environment
        t = torch.einsum("ijk,jl->ilk", Tn, torch.eye(Tn.shape[1], dtype=Tn.dtype))
        val = torch.trace(torch.linalg.matrix_power(Cn, 4))
        for j in range(Tn.shape[1]):
            val = val + torch.trace(t[:, j, :] @ Cn @ t[:, j, :] @ Cn)
        return val

    at = torch.as_tensor(a).clone().requires_grad_(True)
    Ct = C.clone().requires_grad_(True)
    Tt = T.clone().requires_grad_(True)
    Cn, Tn, _ = orc.ctmrgstep(at, Ct, Tt)
    ga_r, gC_r, gT_r = torch.autograd.grad(f(Cn, Tn), (at, Ct, Tt))
    # cotangents in the GPU's own gauge
    rt = tn.SquareCTMRGRuntime(a, C.numpy(), T.numpy())
    rt2, _ = tn.ctmrgstep(rt)
    Cg = torch.as_tensor(rt2.corner).requires_grad_(True)
    Tg = torch.as_tensor(rt2.edge).requires_grad_(True)
    dC, dT = torch.autograd.grad(f(Cg, Tg), (Cg, Tg))
    ga, gC, gT = tn.ctmrgstep_backward(rt, dC.numpy(), dT.numpy())
    assert rel(ga, ga_r.numpy()) < 1e-9
    assert rel(gC, gC_r.numpy()) < 1e-9
    assert rel(gT, gT_r.numpy()) < 1e-9


def test_ctmrg_stop_semantics(tn, orc):
    a = _sym_bulk(orc, 2, 3)
    C, T = orc.init_random(4, 5, np.random.default_rng(1))
    rt = tn.SquareCTMRGRuntime(a, C.numpy(), T.numpy())
    assert tn.ctmrg(rt, 0.0, 3).steps == 4
    assert tn.ctmrg(rt, 0.0, 0).steps == 1
    assert tn.ctmrg(rt, float("inf"), 10).steps == 1
    r1 = tn.ctmrg(rt, 1e-9, 200)
    r2 = orc.ctmrg(torch.as_tensor(a), C, T, 1e-9, 200)
    assert r1.steps == r2.steps
    assert rel(_invariants(r1.corner, r1.edge)[1], _invariants(r2.corner.numpy(), r2.edge.numpy())[1]) < 1e-9


@pytest.mark.parametrize("beta,chi,atol", [(0.0, 2, 1e-6), (1.0, 2, 1e-8), (0.2, 10, 1e-4), (0.6, 4, 1e-8),
                                           (0.8, 2, 1e-8)])
def test_magnetisation_vs_onsager(tn, beta, chi, atol):
    # test/ctmrg.jl:37-42 on the GPU CTMRG
    m = tn.magnetisation(tn.Ising(), beta, chi, rng=np.random.default_rng(2))
    exact = tn.magofbeta(tn.Ising(), beta)
    assert abs(m - exact) <= max(atol, 1.5e-8 * abs(exact))


# ----------------------------------------------------------------- energy
def test_symmetrize_matches_oracle(tn, orc):
    A = np.random.default_rng(4).standard_normal((3, 3, 3, 3, 2))
    got = tn.indexperm_symmetrize(tn.SquareIPEPS(A)).bulk
    assert rel(got, orc.symmetrized(A)) < 1e-14


def test_expectationvalue_matches_oracle(tn, orc):
    A = torch.as_tensor(orc.symmetrized(orc.ipeps_uniform(2, 2, 5)))
    ap, a = orc.double_layer(A)
    C, T = orc.init_random(4, 7, np.random.default_rng(3))
    h = orc.hamiltonian_heisenberg()
    ref = float(orc.expectationvalue(torch.as_tensor(h), ap, C, T))
    got = tn.expectationvalue(h, ap.numpy(), tn.CTMRGRuntime(a.numpy(), C.numpy(), T.numpy()))
    assert abs(got - ref) < 1e-13 * abs(ref)


def test_energy_cfg2_heisenberg_D2_chi20(tn, orc):
    """Heisenberg, D=2, χ=20, tol=1e-6, maxit=100 (FP64)."""
    h = tn.hamiltonian(tn.Heisenberg())
    A = orc.ipeps_uniform(2, 2, 0)
    r = tn._energy(h, tn.SquareIPEPS(A), 20, 1e-6, 100)
    e_ref, steps_ref = orc.energy(h, torch.as_tensor(A), 20, 1e-6, 100, return_steps=True)
    # the first steps project onto the null space of a rank-16 corner (χ=20): the
    # completion is implementation-defined in LAPACK too, so parity is on E at tol 1e-6
    assert abs(r.E - float(e_ref)) < 1e-6
    # converged: identical to the oracle at the FP64 bar
    e_c = tn.energy(h, tn.SquareIPEPS(A), 20, 1e-12, 300)
    e_cr = float(orc.energy(h, torch.as_tensor(A), 20, 1e-12, 300))
    assert abs(e_c - e_cr) < RTOL_FP64 * abs(e_cr)


@pytest.mark.parametrize("D,chi,seed", [(2, 8, 11), (2, 12, 11), (2, 20, 0)])
def test_energy_and_gradient_match_oracle(tn, orc, D, chi, seed):
    """Plain FP64 path at tol 1e-12: energy and the full unrolled gradient
    against the oracle's (the reference's Zygote gradient restated) at the FP64
    bar, 1e-10 relative.  (2, 20, seed 0) is the D=2, χ=20 Heisenberg workload."""
    h = tn.hamiltonian(tn.Heisenberg())
    A = orc.ipeps_uniform(D, 2, seed)
    E, g = tn.energy_and_gradient(h, tn.SquareIPEPS(A), chi, 1e-12, 200)
    E_r, g_r, _ = orc.energy_and_grad(h, A, chi, 1e-12, 200)
    assert abs(E - E_r) < RTOL_FP64 * abs(E_r)
    assert rel(g, g_r) < RTOL_FP64


def test_energy_gradient_fd_cfg3_D3_chi36(tn, orc):
    """D=3 (d=9), χ=36: the GPU gradient against the oracle's at tol 1e-12 (FP64
    bar, 1e-10 relative) and, at tol 1e-10, against a central difference (step 1e-5)."""
    h = tn.hamiltonian(tn.Heisenberg())
    A = orc.ipeps_uniform(3, 2, 0)
    E12, g12 = tn.energy_and_gradient(h, tn.SquareIPEPS(A), 36, 1e-12, 200)
    E12_r, g12_r, _ = orc.energy_and_grad(h, A, 36, 1e-12, 200)
    assert abs(E12 - E12_r) < RTOL_FP64 * abs(E12_r)
    assert rel(g12, g12_r) < RTOL_FP64
    E, g = tn.energy_and_gradient(h, tn.SquareIPEPS(A), 36, 1e-10, 100)
    E_r, g_r, _ = orc.energy_and_grad(h, A, 36, 1e-10, 100)
    assert abs(E - E_r) < 1e-9 * abs(E_r)
    assert rel(g, g_r) < RTOL_FP64
    idx = (1, 0, 2, 1, 1)
    p, m = A.copy(), A.copy()
    p[idx] += 1e-5
    m[idx] -= 1e-5
    fd = (tn.energy(h, tn.SquareIPEPS(p), 36, 1e-10, 100) - tn.energy(h, tn.SquareIPEPS(m), 36, 1e-10, 100)) / 2e-5
    assert abs(fd - g[idx]) < 1e-6 * max(1.0, abs(g[idx]))


def test_nonfinite_input_is_an_error(tn):
    h = tn.hamiltonian(tn.Heisenberg())
    A = np.ones((2, 2, 2, 2, 2))
    A[0, 0, 0, 0, 0] = np.nan
    with pytest.raises(tn.TnadError):
        tn.energy(h, tn.SquareIPEPS(A), 4, 1e-8, 10)


def test_shape_errors(tn):
    with pytest.raises(tn.DimensionMismatch):
        tn.energy(tn.hamiltonian(tn.Heisenberg()), np.zeros((2, 3, 2, 2, 2)), 4, 1e-8, 10)
    with pytest.raises(tn.DimensionMismatch):
        tn.trg(np.zeros((2, 2, 3, 2)), 4, 2)


@pytest.mark.parametrize("budget", [0, 200_000])
def test_unrolled_gradient_recomputes_steps_beyond_the_tape_budget(tn, orc, budget):
    """Unrolled reverse with a tape budget too small for the per-step
    decompositions (none kept, or only the first few): the missing steps are
    recomputed from the (C, T) checkpoints and the gradient is unchanged."""
    h = tn.hamiltonian(tn.Heisenberg())
    A = orc.ipeps_uniform(2, 2, 5)
    full = tn.default_opts(prec=0, solver=0, adjoint=0)
    E0, g0 = tn.energy_and_gradient(h, tn.SquareIPEPS(A), 12, 1e-12, 200, full)
    small = tn.default_opts(prec=0, solver=0, adjoint=0, tape_budget=budget)
    E1, g1 = tn.energy_and_gradient(h, tn.SquareIPEPS(A), 12, 1e-12, 200, small)
    assert E1 == E0
    assert rel(g1, g0) < 1e-12
