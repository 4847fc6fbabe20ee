"""Mixed path: TF32X3 tensor-core contractions + subspace solver + FP64 ladder,
differentiated by the implicit fixed-point adjoint.  Checked against the CPU
oracle (FP64, unrolled Zygote-equivalent gradient) and the converged-energy
fixtures of tests/golden/estar.json."""
import json
from pathlib import Path

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

ESTAR = json.loads((Path(__file__).parent / "golden" / "estar.json").read_text())


def rel(a, b):
    a, b = np.asarray(a, dtype=float), np.asarray(b, dtype=float)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def test_mixed_energy_D2(tn, orc):
    h = tn.hamiltonian(tn.Heisenberg())
    A = orc.ipeps_uniform(2, 2, 11)
    E = tn.energy(h, tn.SquareIPEPS(A), 12, 1e-10, 200, opts=tn.mixed_opts())
    E_r = float(orc.energy(h, torch.as_tensor(A), 12, 1e-12, 300))
    assert abs(E - E_r) < 1e-9


def test_mixed_energy_and_fixedpoint_gradient_D3_chi36(tn, orc):
    """cfg3: D=3, χ=36, tol 1e-10.  Gradient error against the oracle's unrolled
    gradient is bounded by the 3xTF32 adjoint contractions (1e-5 relative)."""
    h = tn.hamiltonian(tn.Heisenberg())
    A = orc.ipeps_uniform(3, 2, 0)
    st = {}
    E, g = tn.energy_and_gradient(h, tn.SquareIPEPS(A), 36, 1e-10, 200, opts=tn.mixed_opts(), stats=st)
    E_r, g_r, _ = orc.energy_and_grad(h, A, 36, 1e-10, 100)
    assert abs(E - E_r) < 1e-9
    assert rel(g, g_r) < 1e-5, st
    assert st["fp_iters"] >= 1
    # the implicit adjoint's premise holds here: x* is a fixed point of the aligned step
    assert st["fixed_point_residual"] < 1e-6, st


def test_mixed_gradient_D4_chi32_matches_difference_quotient(tn):
    """D=4 N(0,1) site tensor, χ=32: the converged iteration cycles between
    gauge-equivalent environments (x* → G·x*·Gᵀ → x*), which the energy does not
    see.  The adjoint differentiates the step followed by the re-gauge onto x*,
    whose fixed point x* is; its gradient matches a central difference of the
    plain FP64 energy along a random direction and on one component."""
    h = tn.hamiltonian(tn.Heisenberg())
    A = tn.site_tensor("normal_maxabs", 4, 2, 0)
    st = {}
    _, g = tn.energy_and_gradient(h, tn.SquareIPEPS(A), 32, 1e-9, 400, opts=tn.mixed_opts(), stats=st)
    assert st["fixed_point_residual"] < 1e-6, st
    plain = tn.default_opts()
    rng = np.random.default_rng(1)
    d = rng.standard_normal(A.shape)
    d /= np.linalg.norm(d)
    e = np.zeros(A.shape)
    e[1, 0, 1, 1, 1] = 1.0
    for v, step in ((d, 1e-4), (e, 1e-5)):
        Ep = tn.energy(h, tn.SquareIPEPS(np.asfortranarray(A + step * v)), 32, 1e-11, 400, plain)
        Em = tn.energy(h, tn.SquareIPEPS(np.asfortranarray(A - step * v)), 32, 1e-11, 400, plain)
        fd = (Ep - Em) / (2 * step)
        gv = float(np.sum(g * v))
        # difference-quotient error: O(step²) plus ~1e-12/step from the stop rule
        assert abs(gv - fd) <= 1e-4 * abs(fd) + 2e-7, (gv, fd, st)


def test_plain_gradient_D4_chi32_matches_difference_quotient(tn):
    """The plain FP64 path (full symmetric Jacobi SVD each step, unrolled reverse:
    the reference's semantics) on the same D=4 tensor.  M's spectrum comes in ±λ
    pairs, so its singular values are pairwise degenerate; the decomposition must
    still be an SVD (U = A·V/σ on those columns) for svd_back to hold."""
    h = tn.hamiltonian(tn.Heisenberg())
    A = tn.site_tensor("normal_maxabs", 4, 2, 0)
    plain = tn.default_opts()
    _, g = tn.energy_and_gradient(h, tn.SquareIPEPS(A), 32, 1e-9, 400, opts=plain)
    idx, step = (1, 0, 1, 1, 1), 1e-5
    p, m = A.copy(), A.copy()
    p[idx] += step
    m[idx] -= step
    fd = (tn.energy(h, tn.SquareIPEPS(p), 32, 1e-11, 400, plain) -
          tn.energy(h, tn.SquareIPEPS(m), 32, 1e-11, 400, plain)) / (2 * step)
    assert abs(g[idx] - fd) <= 1e-4 * abs(fd) + 2e-7, (g[idx], fd)


def test_plain_fixedpoint_adjoint_matches_unrolled(tn, orc):
    h = tn.hamiltonian(tn.Heisenberg())
    A = orc.ipeps_uniform(2, 2, 7)
    o = tn.default_opts(adjoint=1, fp_tol=1e-12)
    E, g = tn.energy_and_gradient(h, tn.SquareIPEPS(A), 10, 1e-12, 300, opts=o)
    E_r, g_r, _ = orc.energy_and_grad(h, A, 10, 1e-12, 300)
    assert abs(E - E_r) < 1e-10 * abs(E_r)
    assert rel(g, g_r) < 1e-7


@pytest.mark.parametrize("name", ["heisenberg_D4_chi64"])
def test_mixed_reaches_1e8_of_oracle_Estar(tn, orc, name):
    """The headline target: |E − E*| ≤ 1e-8 at D=4, χ=64 on the mixed path."""
    w = ESTAR[name]
    A = orc.ipeps_normal_maxabs(w["D"], 2, w["seed"])
    h = tn.hamiltonian(tn.Heisenberg())
    st = {}
    E, g = tn.energy_and_gradient(h, tn.SquareIPEPS(A), w["chi"], 3e-8, 400, opts=tn.mixed_opts(), stats=st)
    assert abs(E - w["E_star"]) <= 1e-8, (E, w["E_star"], st)
    assert np.all(np.isfinite(g))


def _unit_direction(shape, seed):
    v = np.random.default_rng(seed).standard_normal(shape)
    return v / np.linalg.norm(v)


def test_mixed_D4_chi100_reaches_1e8_and_its_gradient_matches_a_difference_quotient(tn):
    """The large-environment configuration at χ = 100 (enlarged corner
    1600×1600, D = 4 N(0,1) tensor, seed 0): |E − E*| ≤ 1e-8 against the
    oracle's converged energy (tests/golden/estar.json), and the implicit-adjoint
    gradient along a random unit direction against a central difference
    (step 1e-4) of mixed-path energies converged to the stop rule 1e-10."""
    w = ESTAR["heisenberg_D4_chi100"]
    A = tn.site_tensor(w["recipe"], w["D"], 2, w["seed"])
    h = tn.hamiltonian(tn.Heisenberg())
    st = {}
    E, g = tn.energy_and_gradient(h, tn.SquareIPEPS(A), 100, 3e-8, 400, opts=tn.mixed_opts(), stats=st)
    assert abs(E - w["E_star"]) <= 1e-8, (E, w["E_star"], st)
    assert st["fixed_point_residual"] < 1e-5, st
    v, step = _unit_direction(A.shape, 1), 1e-4
    Ep = tn.energy(h, tn.SquareIPEPS(np.asfortranarray(A + step * v)), 100, 1e-10, 400, tn.mixed_opts())
    Em = tn.energy(h, tn.SquareIPEPS(np.asfortranarray(A - step * v)), 100, 1e-10, 400, tn.mixed_opts())
    fd = (Ep - Em) / (2 * step)
    gv = float(np.sum(g * v))
    assert abs(gv - fd) <= 1e-4 * abs(fd) + 2e-7, (gv, fd, st)


def test_mixed_path_beyond_one_cta_polar_factor_chi130(tn):
    """χ = 130 (above the 128 that the one-CTA Newton–Schulz polar factor holds):
    the gauge alignment and the fixed-point adjoint take the multi-CTA polar
    factor.  D = 3 uniform tensor: mixed energy against the plain FP64 path at
    the same χ, and the gradient along a random direction against a central
    difference of plain FP64 energies."""
    h = tn.hamiltonian(tn.Heisenberg())
    A = tn.site_tensor("uniform", 3, 2, 0)
    st = {}
    E, g = tn.energy_and_gradient(h, tn.SquareIPEPS(A), 130, 1e-10, 300, opts=tn.mixed_opts(), stats=st)
    plain = tn.default_opts()
    E_p = tn.energy(h, tn.SquareIPEPS(A), 130, 1e-11, 300, plain)
    assert abs(E - E_p) <= 1e-8, (E, E_p, st)
    v, step = _unit_direction(A.shape, 2), 1e-4
    Ep = tn.energy(h, tn.SquareIPEPS(np.asfortranarray(A + step * v)), 130, 1e-11, 300, plain)
    Em = tn.energy(h, tn.SquareIPEPS(np.asfortranarray(A - step * v)), 130, 1e-11, 300, plain)
    fd = (Ep - Em) / (2 * step)
    gv = float(np.sum(g * v))
    assert abs(gv - fd) <= 1e-4 * abs(fd) + 2e-7, (gv, fd, st)
