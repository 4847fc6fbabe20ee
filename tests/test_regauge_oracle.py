"""The re-gauged fixed-point adjoint, restated on the CPU (oracle/regauge_oracle.py).

Pins the method the device adjoint uses (csrc/fixedpoint.cu) without a GPU:
Γ undoes a gauge transformation of an environment whose corner spectrum comes
in ±λ pairs; Γ's pullback, as the GEMM sequence the device runs, matches a
central difference; and on a D=4 N(0,1) site tensor the polar-aligned CTMRG
cycles between gauge-equivalent environments while Γ∘f has the converged
environment as its fixed point, with an implicit gradient equal to the
derivative of the converged energy.
"""
import numpy as np
import pytest
import torch

from oracle import regauge_oracle as ro
from oracle import tnad_oracle as o


def paired_env(rng, chi, d):
    Q, _ = np.linalg.qr(rng.standard_normal((chi, chi)))
    half = np.sort(rng.uniform(0.05, 1.0, chi // 2))
    lam = np.concatenate([half, -half])
    C = Q @ np.diag(lam) @ Q.T
    T = rng.standard_normal((chi, d, chi))
    T = T + T.transpose(2, 1, 0)
    return torch.as_tensor(C / np.linalg.norm(C)), torch.as_tensor(T / np.linalg.norm(T))


def test_regauge_undoes_a_gauge_transformation():
    rng = np.random.default_rng(0)
    C, T = paired_env(rng, 12, 3)
    G, _ = np.linalg.qr(rng.standard_normal((12, 12)))
    G = torch.as_tensor(G)
    Cy = G @ C @ G.T
    Ty = torch.einsum("ia,adb,jb->idj", G, T, G)
    Cg, Tg, _ = ro.regauge(Cy, Ty, C, T)
    assert float((Cg - C).norm()) < 1e-12
    assert float((Tg - T).norm()) < 1e-12


def test_regauge_pullback_matches_central_difference():
    rng = np.random.default_rng(1)
    chi, d = 10, 4
    C, T = paired_env(rng, chi, d)
    G, _ = np.linalg.qr(np.eye(chi) + 0.1 * rng.standard_normal((chi, chi)))
    G = torch.as_tensor(G)
    Cy = G @ C @ G.T
    Ty = torch.einsum("ia,adb,jb->idj", G, T, G)
    _, _, s = ro.regauge(Cy, Ty, C, T)
    lam, W0 = ro._eig_desc(Cy)
    _, Wr = ro._eig_desc(C)
    dC = rng.standard_normal((chi, chi))
    dC = dC + dC.T
    dT = rng.standard_normal((chi, d, chi))
    dT = dT + dT.transpose(2, 1, 0)
    bC = rng.standard_normal((chi, chi))
    bT = rng.standard_normal((chi, d, chi))

    def L(eps):
        Cg, Tg, _ = ro.regauge(Cy + eps * torch.as_tensor(dC), Ty + eps * torch.as_tensor(dT), C, T, s, W0)
        return float((Cg * torch.as_tensor(bC)).sum() + (Tg * torch.as_tensor(bT)).sum())

    fd = (L(1e-6) - L(-1e-6)) / 2e-6
    W = (W0 * s[None, :]).numpy()
    gC, gT = ro.regauge_vjp(Cy.numpy(), Ty.numpy(), W, lam.numpy(), Wr.numpy(), bC, bT)
    an = float(np.sum(gC * dC) + np.sum(gT * dT))
    assert abs(an - fd) <= 1e-6 * abs(fd)


def test_aligned_ctmrg_cycles_and_the_regauged_adjoint_is_the_energy_derivative():
    """D=4 N(0,1) site tensor (NumPy seed 0, max-abs normalised), χ=16, 100 steps."""
    torch.set_num_threads(min(8, torch.get_num_threads()))
    A = o.ipeps_normal_maxabs(4, 2, 0)
    h = o.hamiltonian_heisenberg()
    E, g, info = ro.implicit_gradient(h, A, 16, 100)
    # the aligned step alone does not return x* (period-2 gauge cycle) ...
    assert info["residual_f"] > 1e-4, info
    # ... but the re-gauged step does
    assert info["residual_g"] < 1e-10, info

    def energy(x):
        _, a = o.double_layer(o.indexperm_symmetrize(torch.as_tensor(x)))
        ap, _ = o.double_layer(o.indexperm_symmetrize(torch.as_tensor(x)))
        C, T, _ = ro.aligned_ctmrg(a, 16, 100)[-1]
        return float(o.expectationvalue(torch.as_tensor(h), ap, C, T))

    # the aligned iteration converges to the reference CTMRG's energy (src/ctmrg.jl step)
    assert abs(E - float(o.energy(h, torch.as_tensor(A), 16, 1e-12, 300))) < 1e-10
    v = np.random.default_rng(1).standard_normal(A.shape)
    v /= np.linalg.norm(v)
    step = 1e-4
    fd = (energy(A + step * v) - energy(A - step * v)) / (2 * step)
    assert abs(float(np.sum(g * v)) - fd) <= 1e-6 * abs(fd), (float(np.sum(g * v)), fd, info)
