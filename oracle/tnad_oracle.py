"""CPU oracle for the TensorNetworkAD contraction-and-truncation path.

TEST INFRASTRUCTURE ONLY.  Only ``tests/``, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` may import this
module, and only as the checker or as the timed CPU restatement of the
reference.  The product (``libtnad`` and the Python host mirror) never calls it.

This is a line-by-line FP64 restatement of the Julia reference (which cannot run
here: Julia, OMEinsum, Zygote and Optim are absent), in ComplexF64 where the
input is complex, with the reference's conjugations.  Every array keeps the
reference's index order and every reshape is column-major (``reshape_f``), as in
Julia.  Gradients come from torch autograd, which reproduces Zygote's generic
adjoints (einsum, permutedims, reshape, maximum, log); the two custom adjoints
of the reference are restated exactly:

* the SVD adjoint ``svd_back`` (src/trg.jl:72-105, Lorentzian eta = 1e-40);
* the norm adjoint  ``Δ·A/(‖A‖+eps(0f0))``      (src/autodiff.jl:23-29).

Multi-tensor einsums of the reference are evaluated as pairwise contractions in
a cheap order (OMEinsum's order only changes rounding).  ``tp`` of
src/ctmrg.jl:131 is never materialised; the edge update of :140 is contracted
as T·z -> ·a -> ·z, which is the same sum.

Parity pins (checked in tests/test_oracle_golden.py):
  trg(model_tensor(Ising(),0.5),20,20) = 1.0257933734351765     README.md:59-60
  d/dβ of the same                     = 1.7455677143228514     README.md:69-70
  trg(model_tensor(Ising(),0.4),5,5)   = 0.8919788686747141     test/trg.jl:18
  d/dβ trg(.., 5, 5) at β=0.5          = 1.7502426939979507     docs/src/userguide.md:25-28
  hamiltonian(Heisenberg())            = printed tensor         README.md:83-100
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np
import torch

DT = torch.float64

# ---------------------------------------------------------------------------
# helpers
# ---------------------------------------------------------------------------


def reshape_f(x: torch.Tensor, shape) -> torch.Tensor:
    """Column-major (Julia) reshape of a tensor stored in Julia index order."""
    shape = tuple(int(s) for s in shape)
    xr = x.permute(*reversed(range(x.ndim)))
    return xr.reshape(tuple(reversed(shape))).permute(*reversed(range(len(shape))))


def ein(spec: str, *ops):
    return torch.einsum(spec, *ops)


def as_t(x) -> torch.Tensor:
    """FP64 tensor, or complex128 for complex input (ComplexF64 in the reference)."""
    if isinstance(x, torch.Tensor):
        return x if x.is_complex() else x.to(DT)
    if np.iscomplexobj(x):
        return torch.as_tensor(np.asarray(x, dtype=np.complex128))
    return torch.as_tensor(np.asarray(x, dtype=np.float64))


class _Norm(torch.autograd.Function):
    """LinearAlgebra.norm with the reference's adjoint (src/autodiff.jl:23-29)."""

    @staticmethod
    def forward(ctx, a):
        n = torch.linalg.vector_norm(a)
        ctx.save_for_backward(a, n)
        return n

    @staticmethod
    def backward(ctx, g):
        a, n = ctx.saved_tensors
        eps0f0 = float(np.nextafter(np.float32(0), np.float32(1)))  # eps(0f0)
        return g * a / (n + eps0f0)


def norm(a):
    return _Norm.apply(a)


def svd_back(U, S, V, dU, dS, dV, eta: float = 1e-40):
    """Restatement of svd_back (src/trg.jl:72-105), real or complex U, V."""
    if dU is None and dS is None and dV is None:
        return None
    S2 = S * S
    Sinv = S / (S2 + eta)
    F = S2[None, :] - S2[:, None]           # F[i,j] = s_j^2 - s_i^2   (:78)
    F = F / (F * F + eta)                    # (:79)
    cplx = U.is_complex()
    res = torch.zeros(S.shape[0], S.shape[0], dtype=U.dtype)
    if dU is not None:
        UdU = U.conj().T @ dU                # (:83)
        J = F * UdU                          # (:84)
        res = res + (J + J.conj().T) * S[None, :]   # (:85) (J+J')*Diagonal(S)
        if cplx:                                    # (:85) + Diagonal(1im*imag(diag(UdU)) .* Sinv)
            res = res + torch.diag(1j * torch.diagonal(UdU).imag * Sinv)
    if dV is not None:
        K = F * (V.conj().T @ dV)            # (:88-89)
        res = res + S[:, None] * (K + K.conj().T)   # (:90)
    if dS is not None:
        res = res + torch.diag(dS).to(res.dtype)    # (:93)
    out = U @ res @ V.conj().T               # (:96)
    if dU is not None and U.shape[0] != U.shape[1]:
        out = out + ((dU - U @ (U.conj().T @ dU)) * Sinv[None, :]) @ V.conj().T          # (:98-99)
    if dV is not None and V.shape[0] != V.shape[1]:
        dVh = dV.conj().T
        out = out + (U * Sinv[None, :]) @ (dVh - (dVh @ V) @ V.conj().T)                 # (:102-103)
    return out


class _SVD(torch.autograd.Function):
    """LinearAlgebra.svd (thin) with the Zygote adjoint of src/trg.jl:77-83."""

    @staticmethod
    def forward(ctx, A):
        U, S, Vh = torch.linalg.svd(A, full_matrices=False)
        V = Vh.conj().T.contiguous()
        ctx.save_for_backward(U, S, V)
        ctx.set_materialize_grads(False)
        return U, S, V

    @staticmethod
    def backward(ctx, dU, dS, dV):
        U, S, V = ctx.saved_tensors
        return svd_back(U, S, V, dU, dS, dV)


def svd(A):
    return _SVD.apply(A)


# ---------------------------------------------------------------------------
# Hamiltonians and example tensors (src/hamiltonianmodels.jl, src/exampletensors.jl)
# ---------------------------------------------------------------------------

SX = np.array([[0.0, 1.0], [1.0, 0.0]])
SY = np.array([[0.0, -1.0j], [1.0j, 0.0]])
SZ = np.array([[1.0, 0.0], [0.0, -1.0]])
ID2 = np.eye(2)


def _outer(a, b):
    return np.einsum("ij,kl->ijkl", a, b)


def hamiltonian_tfising(hx: float) -> np.ndarray:
    """hamiltonian(::TFIsing)  src/hamiltonianmodels.jl:28-33."""
    return -2 * _outer(SZ, SZ) - hx / 2 * _outer(SX, ID2) - hx / 2 * _outer(ID2, SX)


def hamiltonian_heisenberg(Jz=1.0, Jx=1.0, Jy=1.0) -> np.ndarray:
    """hamiltonian(::Heisenberg)  src/hamiltonianmodels.jl:53-59 (sublattice rotation)."""
    h = Jz * _outer(SZ, SZ) - Jx * _outer(SX, SX) - Jy * _outer(SY, SY)
    h = np.einsum("ijcd,kc,ld->ijkl", h, SX, SX.conj().T)
    return np.real(h / 2)


def diaglocalhamiltonian(diag) -> np.ndarray:
    """src/variationalipeps.jl:15-20."""
    diag = np.asarray(diag, dtype=np.float64)
    n = diag.shape[0]
    h = np.diag(diag)
    idn = np.eye(n)
    return h.reshape(n, n, 1, 1) * idn.reshape(1, 1, n, n) + h.reshape(1, 1, n, n) * idn.reshape(n, n, 1, 1)


def _ising_q(beta):
    beta = as_t(beta)
    cb, sb = torch.sqrt(torch.cosh(beta)), torch.sqrt(torch.sinh(beta))
    q = torch.stack([torch.stack([cb + sb, cb - sb]), torch.stack([cb - sb, cb + sb])]) / math.sqrt(2)
    return q


def model_tensor_ising(beta) -> torch.Tensor:
    """model_tensor(::Ising, β)  src/exampletensors.jl:30-35; differentiable in β."""
    a = torch.zeros(2, 2, 2, 2, dtype=DT)
    a[0, 0, 0, 0] = 1.0
    a[1, 1, 1, 1] = 1.0
    q = _ising_q(beta)
    return ein("abcd,ai,bj,ck,dl->ijkl", a, q, q, q, q)


def mag_tensor_ising(beta) -> torch.Tensor:
    """mag_tensor(::Ising, β)  src/exampletensors.jl:43-48."""
    a = torch.zeros(2, 2, 2, 2, dtype=DT)
    a[0, 0, 0, 0] = 1.0
    a[1, 1, 1, 1] = -1.0
    q = _ising_q(beta)
    return ein("abcd,ai,bj,ck,dl->ijkl", a, q, q, q, q)


def tensorfromclassical(ham) -> np.ndarray:
    """src/exampletensors.jl:17-21 (matrix square root of exp.(ham))."""
    import scipy.linalg
    w = np.exp(np.asarray(ham, dtype=np.float64))
    q = np.real(scipy.linalg.sqrtm(w))
    return np.einsum("ij,ik,il,im->jklm", q, q, q, q)


ISING_BETA_C = math.log(1 + math.sqrt(2)) / 2


def magofbeta(beta: float) -> float:
    """Onsager/Yang magnetisation  src/exampletensors.jl:77."""
    return (1 - math.sinh(2 * beta) ** -4) ** (1 / 8) if beta > ISING_BETA_C else 0.0


# ---------------------------------------------------------------------------
# TRG  (src/trg.jl:13-44)
# ---------------------------------------------------------------------------


def _searchsortedfirst_rev(s: torch.Tensor, tol: float) -> int:
    """Julia searchsortedfirst(s, tol, rev=true) for descending s (1-based)."""
    cnt = int((s > tol).sum().item())
    return cnt + 1


def trg_svd(t, dmax, tol):
    """src/trg.jl:33-44."""
    d1, d2, d3, d4 = t.shape
    tmat = reshape_f(t, (d1 * d2, d3 * d4))
    u, s, v = svd(tmat)
    dmax = min(_searchsortedfirst_rev(s.detach(), tol), dmax, s.shape[0])
    FS = s[:dmax]
    sq = torch.sqrt(FS)
    uu = reshape_f(u[:, :dmax] * sq[None, :], (d1, d2, dmax))
    vv = reshape_f(v.conj().T[:dmax, :] * sq[:, None], (dmax, d3, d4))  # copy(v')[1:dmax, :]
    return uu, vv


def trg(a, chi: int, niter: int, tol: float = 1e-16):
    """trg(a, χ, niter; tol)  src/trg.jl:13-30.  Returns lnZ per site (0-d tensor)."""
    a = as_t(a) if not isinstance(a, torch.Tensor) else a
    lnZ = torch.zeros((), dtype=DT)
    for n in range(1, niter + 1):
        maxval = a.abs().max()
        a = a / maxval
        lnZ = lnZ + 2.0 ** (1 - n) * torch.log(maxval)
        dr_ul = ein("urdl->drul", a)
        ld_ru = ein("urdl->ldru", a)
        dr, ul = trg_svd(dr_ul, chi, tol)
        ld, ru = trg_svd(ld_ru, chi, tol)
        x = ein("npu,por->nuor", dr, ld)
        y = ein("dom,lmn->doln", ul, ru)
        a = ein("nuor,doln->urdl", x, y)
    trace = ein("ijij->", a)
    lnZ = lnZ + torch.log(trace) / 2.0 ** niter
    return lnZ


def trg_dbeta(beta: float, chi: int, niter: int, tol: float = 1e-16):
    """(lnZ, d lnZ/dβ) for the Ising model, as README.md:57-73."""
    b = torch.tensor(float(beta), dtype=DT, requires_grad=True)
    z = trg(model_tensor_ising(b), chi, niter, tol)
    (g,) = torch.autograd.grad(z, b)
    return float(z.detach()), float(g)


# ---------------------------------------------------------------------------
# fixed point + CTMRG  (src/fixedpoint.jl, src/ctmrg.jl)
# ---------------------------------------------------------------------------


@dataclass
class CTMRGResult:
    corner: torch.Tensor
    edge: torch.Tensor
    steps: int
    vals: torch.Tensor


def init_raw(bulk: torch.Tensor, chi: int):
    """_initializect_square(bulk, Val(:raw), χ)  src/ctmrg.jl:74-86 (no gradient)."""
    bulk = bulk.detach()
    D = bulk.shape[0]
    corner = torch.zeros(chi, chi, dtype=bulk.dtype)
    edge = torch.zeros(chi, D, chi, dtype=bulk.dtype)
    cinit = bulk.sum(dim=(2, 3))
    tinit = bulk.sum(dim=3)
    m = min(D, chi)
    corner[:m, :m] = cinit[:m, :m]
    edge[:m, :, :m] = tinit[:m, :, :m]
    return corner, edge


def init_random(D: int, chi: int, rng: np.random.Generator):
    """_initializect_square(bulk, Val(:random), χ)  src/ctmrg.jl:66-72 (NumPy RNG)."""
    corner = torch.as_tensor(rng.standard_normal((chi, chi)))
    edge = torch.as_tensor(rng.standard_normal((chi, D, chi)))
    corner = corner + corner.conj().T
    edge = edge + edge.conj().permute(2, 1, 0)
    return corner, edge


def enlarged_corner(bulk, corner, edge):
    """cp = ein"ad,iba,dcl,jkcb -> ijlk"(corner, edge, edge, bulk)  src/ctmrg.jl:130."""
    x1 = ein("ad,iba->ibd", corner, edge)
    x2 = ein("ibd,dcl->ibcl", x1, edge)
    return ein("ibcl,jkcb->ijlk", x2, bulk)


def project_edge(bulk, edge, z):
    """ein"abjcd,abi,dck -> ijk"(tp, conj(z), z) with tp = ein"iam,jkla -> ijklm"(edge, bulk)
    (src/ctmrg.jl:131,140), contracted without materialising tp."""
    y1 = ein("aed,abi->edbi", edge, z.conj())
    y2 = ein("edbi,bjce->dijc", y1, bulk)
    return ein("dijc,dck->ijk", y2, z)


def ctmrgstep(bulk, corner, edge):
    """One CTMRG step  src/ctmrg.jl:126-153.  Returns (corner, edge, vals)."""
    D, chi = bulk.shape[0], corner.shape[0]
    cp = enlarged_corner(bulk, corner, edge)
    cpmat = reshape_f(cp, (chi * D, chi * D))
    cpmat = cpmat + cpmat.conj().T                      # cpmat += adjoint(cpmat)
    u, s, v = svd(cpmat)
    z = reshape_f(u[:, :chi], (chi, D, chi))
    w = ein("abcd,abi->icd", cp, z.conj())               # ein"abcd,abi,cdj -> ij"(cp, conj(z), z)
    corner_n = ein("icd,cdj->ij", w, z)
    edge_n = project_edge(bulk, edge, z)
    vals = (s / s[0]).detach()
    corner_n = corner_n + corner_n.conj().T              # corner += corner'
    edge_n = edge_n + edge_n.conj().permute(2, 1, 0)     # edge += ein"ijk -> kji"(conj(edge))
    corner_n = corner_n / norm(corner_n)
    edge_n = edge_n / norm(edge_n)
    return corner_n, edge_n, vals


def ctmrg(bulk, corner, edge, tol: float, maxit: int) -> CTMRGResult:
    """ctmrg(rt; tol, maxit)  src/ctmrg.jl:110-117 driven by fixedpoint/StopFunction
    (src/fixedpoint.jl:11-41).

    StopFunction starts with counter = -1, so the state after k steps is tested
    with counter k: the loop stops at the first k >= 1 with counter > maxit
    (k = maxit+1) or ‖vals_k − vals_{k−1}‖₂ ≤ tol (vals_0 = Inf never passes).
    """
    chi, D = corner.shape[0], bulk.shape[0]
    oldvals = torch.full((chi * D,), float("inf"), dtype=DT)
    counter = 0  # state 0 (the guess) has been tested: counter -1 -> 0
    k = 0
    vals = oldvals
    while True:
        corner, edge, vals = ctmrgstep(bulk, corner, edge)
        k += 1
        counter += 1
        if counter > maxit:
            break
        diff = torch.linalg.vector_norm(vals - oldvals)
        if bool(diff <= tol):
            break
        oldvals = vals
    return CTMRGResult(corner, edge, k, vals)


# ---------------------------------------------------------------------------
# iPEPS, energy  (src/ipeps.jl, src/variationalipeps.jl)
# ---------------------------------------------------------------------------


def indexperm_symmetrize(x: torch.Tensor) -> torch.Tensor:
    """src/ipeps.jl:32-39."""
    x = x + x.permute(0, 3, 2, 1, 4)
    x = x + x.permute(2, 1, 0, 3, 4)
    x = x + x.permute(1, 0, 3, 2, 4)
    x = x + x.permute(3, 2, 1, 0, 4)
    return x / norm(x)


def double_layer(A: torch.Tensor):
    """ap and a of src/variationalipeps.jl:32-34."""
    d, s = A.shape[0], A.shape[4]
    D = d * d
    ap = ein("abcdx,ijkly->aibjckdlxy", A, A.conj())
    ap = reshape_f(ap, (D, D, D, D, s, s))
    a = ein("ijklaa->ijkl", ap)
    return ap, a


def expectationvalue(h, ap, corner, edge):
    """src/variationalipeps.jl:49-56."""
    ap = ap / norm(ap)
    w1 = ein("ab,ica->icb", corner, edge)
    w2 = ein("icb,bde->icde", w1, edge)
    r = ein("eg,gfk->efk", corner, edge)
    v = ein("icde,cjfdlm->iejflm", w2, ap)
    l = ein("iejflm,efk->ijklm", v, r)
    G = ein("abcij,abckl->ijkl", l, l)
    e = (G * h).sum()
    t = ein("ijkaa->ijk", l)
    n = (t * t).sum()
    return e / n


def energy(h, bulk, chi: int, tol: float, maxit: int, return_steps: bool = False):
    """energy(h, ipeps; χ, tol, maxit)  src/variationalipeps.jl:28-40."""
    h = as_t(h)
    A = indexperm_symmetrize(bulk)
    ap, a = double_layer(A)
    corner, edge = init_raw(a, chi)
    res = ctmrg(a, corner, edge, tol, maxit)
    e = expectationvalue(h, ap, res.corner, res.edge)
    return (e, res.steps) if return_steps else e


def energy_and_grad(h, bulk, chi: int, tol: float, maxit: int):
    """(E, dE/dbulk, steps): Zygote.gradient(x -> energy(h, IPEPS(x); ...), bulk)."""
    x = as_t(bulk).clone().requires_grad_(True)
    e, steps = energy(h, x, chi, tol, maxit, return_steps=True)
    if e.is_complex():  # Zygote.gradient(x -> real(energy(...)), bulk): ∂/∂Re + i ∂/∂Im
        e = e.real
    (g,) = torch.autograd.grad(e, x)
    return float(e.detach()), g.numpy(), steps


def optimiseipeps(bulk, h, chi: int, tol: float, maxit: int, f_tol: float = 1e-6, iters: int = 200, m: int = 20):
    """optimiseipeps (src/variationalipeps.jl:67-75) with SciPy L-BFGS(m) in place of Optim."""
    import scipy.optimize

    shape = np.asarray(bulk).shape
    cplx = np.iscomplexobj(bulk)
    size = int(np.prod(shape))

    def unpack(x):
        return x[:size].reshape(shape) + 1j * x[size:].reshape(shape) if cplx else x.reshape(shape)

    def fg(x):
        # a complex tensor is optimised over (Re, Im); Zygote's gradient of a real
        # function of a complex array is ∂/∂Re + i ∂/∂Im
        e, g, _ = energy_and_grad(h, unpack(x), chi, tol, maxit)
        return e, (np.concatenate([g.real.ravel(), g.imag.ravel()]) if cplx else g.ravel())

    b = np.asarray(bulk)
    x0 = np.concatenate([b.real.ravel(), b.imag.ravel()]) if cplx else np.asarray(b, dtype=np.float64).ravel()
    r = scipy.optimize.minimize(fg, x0, jac=True, method="L-BFGS-B",
                                options=dict(maxcor=m, maxiter=iters, ftol=f_tol, gtol=1e-10))
    return float(r.fun), unpack(r.x)


def magnetisation(beta: float, chi: int, rng: np.random.Generator, tol=1e-6, maxit=100):
    """magnetisation(::Ising, β, χ)  src/exampletensors.jl:57-69 (random init from NumPy RNG)."""
    a = model_tensor_ising(beta)
    m = mag_tensor_ising(beta)
    corner, edge = init_random(a.shape[0], chi, rng)
    res = ctmrg(a, corner, edge, tol, maxit)
    c, t = res.corner, res.edge
    ctc = ein("ia,ajb,bk->ijk", c, t, c)
    env = ein("alc,ckd,bjd,bia->ijkl", ctc, t, ctc, t)
    mag = (env * m).sum()
    nrm = (env * a).sum()
    return float(abs(mag / nrm))


# ---------------------------------------------------------------------------
# seeded synthetic inputs (the reference's own RNG streams are Julia-only)
# ---------------------------------------------------------------------------


def ipeps_uniform(D: int, s: int, seed: int) -> np.ndarray:
    """Uniform [0,1) site tensor of shape (D,D,D,D,s) from NumPy default_rng(seed)."""
    rng = np.random.default_rng(seed)
    return np.asfortranarray(rng.random((D, D, D, D, s)))


def ipeps_normal_maxabs(D: int, s: int, seed: int) -> np.ndarray:
    """N(0,1) site tensor normalised to max|.| = 1 (large-environment workload)."""
    rng = np.random.default_rng(seed)
    x = rng.standard_normal((D, D, D, D, s))
    return x / np.abs(x).max()


def symmetrized(bulk) -> np.ndarray:
    return indexperm_symmetrize(as_t(bulk)).numpy()
