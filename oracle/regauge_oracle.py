"""CPU restatement of the re-gauged fixed-point adjoint (no reference counterpart).

TEST INFRASTRUCTURE ONLY.  Only ``tests/`` may import this module, as the
checker of the method libtnad's implicit adjoint uses (csrc/fixedpoint.cu); the
product never calls it.

The reference differentiates CTMRG by unrolling the loop (src/fixedpoint.jl:11-15
under Zygote).  The implicit adjoint instead differentiates one step at the
converged environment x* = (C*, T*), which needs x* to be a fixed point of the
map it differentiates.  For site tensors whose corner spectrum comes in ±λ pairs
(N(0,1) D=4 tensors) the polar-aligned step (the subspace solver's projector
z ← z·polar(zᵀ·z_prev)) converges to a period-2 cycle x* → G·x*·Gᵀ → x* of
gauge-equivalent environments.  The re-gauge Γ maps the step's output back
onto x*'s gauge:

    Γ(y) = Rᵀ·y·R,   R = W·W*ᵀ,

with W, W* the eigenvectors of C_y and C* ordered by λ (signed, so ±λ pairs
never tie) and W's column signs chosen so that y's T matches T* in that basis
(a spanning tree from the largest |λ*|).  Γ(G·x*·Gᵀ) = x*, and Γ∘f has x* as
its fixed point.

* ``aligned_ctmrg``: the polar-aligned CTMRG step iterated with the exact top-χ
  eigenvectors of M = cp + cpᵀ (ordered by |θ|), as the subspace solver's
  converged iteration computes it;
* ``regauge``: Γ, optionally with the signs held fixed (differentiable);
* ``regauge_vjp``: the pullback of Γ as the GEMM sequence the device runs;
* ``implicit_gradient``: dE/dA from (I − (∂g/∂x)ᵀ)λ = ∂E/∂x with g = Γ∘f,
  torch autograd for the step and SciPy GMRES for the solve.
"""
from __future__ import annotations

import numpy as np
import torch

from oracle import tnad_oracle as o


def _polar(X: torch.Tensor) -> torch.Tensor:
    U, _, Vh = torch.linalg.svd(X)
    return U @ Vh


class _TopEig(torch.autograd.Function):
    """Eigenvectors of the k largest |θ| of a symmetric M, with the pullback
    M̄ = W·(F ∘ Wᵀ·Ū)·W_kᵀ (F_ij = 1/(θ_j − θ_i)), symmetrised."""

    @staticmethod
    def forward(ctx, M, k):
        th, W = torch.linalg.eigh(M)
        idx = torch.argsort(th.abs(), descending=True)
        th, W = th[idx], W[:, idx]
        ctx.save_for_backward(th, W)
        ctx.k = k
        return W[:, :k].clone()

    @staticmethod
    def backward(ctx, Ub):
        th, W = ctx.saved_tensors
        k = ctx.k
        G = W.T @ Ub
        dif = th[None, :k] - th[:, None]
        F = torch.where(dif.abs() > 0, 1.0 / torch.where(dif == 0, torch.ones_like(dif), dif), torch.zeros_like(dif))
        F[torch.arange(k), torch.arange(k)] = 0.0
        Mb = W @ (G * F) @ W[:, :k].T
        return 0.5 * (Mb + Mb.T), None


def aligned_step(a, C, T, zref=None):
    """One CTMRG step (src/ctmrg.jl:126-153) with the projector's columns the
    top-χ eigenvectors of M, rotated onto zref by the polar factor."""
    chi, D = C.shape[0], a.shape[0]
    n = chi * D
    cp = o.enlarged_corner(a, C, T)
    M = o.reshape_f(cp, (n, n))
    M = M + M.T
    z = _TopEig.apply(M, chi)
    if zref is not None:
        with torch.no_grad():
            O = _polar(z.T @ zref)
        z = z @ O
    zt = o.reshape_f(z, (chi, D, chi))
    w = torch.einsum("abcd,abi->icd", cp, zt)
    Cn = torch.einsum("icd,cdj->ij", w, zt)
    Tn = o.project_edge(a, T, zt)
    Cn = Cn + Cn.T
    Tn = Tn + Tn.permute(2, 1, 0)
    return Cn / Cn.norm(), Tn / Tn.norm(), z


def aligned_ctmrg(a, chi: int, steps: int):
    """Iterate ``aligned_step`` from the :raw start; returns [(C, T, z)] per step."""
    hist = []
    with torch.no_grad():
        C, T = o.init_raw(a, chi)
        z = None
        for _ in range(steps):
            C, T, z = aligned_step(a, C, T, z)
            hist.append((C, T, z))
    return hist


def _eig_desc(C):
    lam, W = torch.linalg.eigh(C)
    idx = torch.argsort(lam, descending=True)
    return lam[idx], W[:, idx]


def _tree_signs(That, That_ref, lam_ref):
    chi = That.shape[0]
    c = torch.einsum("adb,adb->ab", That, That_ref)
    order = torch.argsort(lam_ref.abs(), descending=True).tolist()
    s = torch.zeros(chi, dtype=That.dtype)
    s[order[0]] = 1.0
    done = [order[0]]
    for a_ in order[1:]:
        b = max(done, key=lambda b_: abs(float(c[a_, b_])))
        s[a_] = s[b] * (-1.0 if float(c[a_, b]) < 0.0 else 1.0)
        done.append(a_)
    return s


def regauge(Cy, Ty, Cref, Tref, s=None, W_align=None):
    """Γ(y) onto the gauge of (Cref, Tref); returns (C̃, T̃, s).  With s given the
    map is smooth (differentiable by autograd).  W_align: eigenvectors whose
    column signs the eigensolver's output is first matched to (so that repeated
    evaluations near one point use the same signs)."""
    lam_r, W_r = _eig_desc(Cref)
    lam, W = _eig_desc(Cy)
    if W_align is not None:
        sg = torch.sign((W * W_align).sum(0))
        W = W * torch.where(sg == 0, torch.ones_like(sg), sg)[None, :]
    if s is None:
        with torch.no_grad():
            Th = torch.einsum("xa,xdy,yb->adb", W, Ty, W)
            Th_r = torch.einsum("xa,xdy,yb->adb", W_r, Tref, W_r)
            s = _tree_signs(Th, Th_r, lam_r)
    W = W * s[None, :]
    R = W @ W_r.T
    return R.T @ Cy @ R, torch.einsum("ai,adb,bj->idj", R, Ty, R), s


def regauge_vjp(Cy, Ty, W, lam, Wr, dC, dT):
    """(C̄_y, T̄_y) for the cotangent (dC, dT) of Γ(y), as the device computes it
    (column-major views of T: χ×(dχ) and (χd)×χ).  W: signed eigenvectors of
    C_y (eigenvalues lam), Wr: those of the reference, both λ-descending."""
    chi, d = Ty.shape[0], Ty.shape[1]
    cd = chi * d

    def view(X, shape):
        return np.reshape(X, shape, order="F")

    R = W @ Wr.T
    P = view(Ty, (cd, chi)) @ R
    Q = R.T @ view(Ty, (chi, cd))
    dTm = view(dT, (chi, cd))
    X1 = R @ dTm
    dTy = view(view(X1, (cd, chi)) @ R.T, (chi, d, chi))
    Rb = view(P, (chi, cd)) @ dTm.T + view(Q, (cd, chi)).T @ view(dT, (cd, chi))
    K = W.T @ (Rb @ Wr)
    lb = np.sum(Wr * (dC @ Wr), axis=0)
    dif = lam[None, :] - lam[:, None]
    F = np.zeros_like(dif)
    off = ~np.eye(chi, dtype=bool) & (dif != 0.0)
    F[off] = 1.0 / dif[off]
    A = F * K + np.diag(lb)
    return W @ A @ W.T, dTy


def implicit_gradient(h, A0, chi: int, steps: int, tol: float = 1e-10):
    """dE/dA at the end of ``steps`` aligned steps from :raw, by the implicit
    adjoint of g = Γ∘f.  Returns (E, grad, info) with info = fixed-point
    residuals of f and of g, and the GMRES product count."""
    import scipy.sparse.linalg as sla

    A0 = torch.as_tensor(np.asarray(A0, dtype=np.float64))
    h = torch.as_tensor(np.asarray(h, dtype=np.float64))

    def layers(A):
        return o.double_layer(o.indexperm_symmetrize(A))

    with torch.no_grad():
        _, a = layers(A0)
    Cs, Ts, zs = aligned_ctmrg(a, chi, steps)[-1]
    with torch.no_grad():
        C1, T1, _ = aligned_step(a, Cs, Ts, zs)
        Cg, Tg, s = regauge(C1, T1, Cs, Ts)

    def res(x, y):
        return float(torch.sqrt(((x[0] - y[0]) ** 2).sum() + ((x[1] - y[1]) ** 2).sum()) / np.sqrt(2.0))

    info = {"residual_f": res((C1, T1), (Cs, Ts)), "residual_g": res((Cg, Tg), (Cs, Ts))}
    A = A0.clone().requires_grad_(True)
    ap, a_ = layers(A)
    xC = Cs.clone().requires_grad_(True)
    xT = Ts.clone().requires_grad_(True)
    E = o.expectationvalue(h, ap, xC, xT)
    gC, gT, gA = torch.autograd.grad(E, (xC, xT, A), retain_graph=True)
    xbar = torch.cat([gC.reshape(-1), gT.reshape(-1)]).numpy()
    Cn, Tn, _ = aligned_step(a_, xC, xT, zs)
    fC, fT, _ = regauge(Cn, Tn, Cs, Ts, s)
    fout = torch.cat([fC.reshape(-1), fT.reshape(-1)])
    count = [0]

    def mv(v):
        count[0] += 1
        g = torch.autograd.grad(fout, (xC, xT), grad_outputs=torch.as_tensor(v), retain_graph=True)
        return v - torch.cat([g[0].reshape(-1), g[1].reshape(-1)]).numpy()

    n = xbar.size
    lam, _ = sla.gmres(sla.LinearOperator((n, n), matvec=mv, dtype=np.float64), xbar, rtol=tol, restart=40,
                       maxiter=20)
    grad = torch.autograd.grad(fout, A, grad_outputs=torch.as_tensor(lam))[0] + gA
    info["gmres_products"] = count[0]
    return float(E.detach()), grad.numpy(), info
