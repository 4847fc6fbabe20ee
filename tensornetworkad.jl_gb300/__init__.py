"""GB300-native TensorNetworkAD: the reference's Julia API mirrored over libtnad.

Names, argument meaning and errors follow under-Peter/TensorNetworkAD.jl:

    model_tensor(Ising(), β)                      src/exampletensors.jl:30-35
    trg(a, χ, niter; tol)                         src/trg.jl:13-30
    SquareCTMRGRuntime(bulk, env, χ), ctmrg(rt)   src/ctmrg.jl:23-117
    SquareIPEPS, indexperm_symmetrize             src/ipeps.jl
    energy(h, ipeps; χ, tol, maxit)               src/variationalipeps.jl:28-40
    expectationvalue, optimiseipeps               src/variationalipeps.jl:49-75
    hamiltonian(Ising/TFIsing/Heisenberg)         src/hamiltonianmodels.jl
    num_grad                                      src/autodiff.jl:44-63

Zygote's role (reverse-mode through trg/ctmrg/energy) is played by
``trg_gradient``, ``energy_and_gradient`` and the torch autograd functions in
``autodiff``; every forward and backward runs in libtnad on the GPU.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from . import _lib as L
from ._lib import DimensionMismatch, TnadError, ctx, default_opts, farr, fzeros, ptr  # noqa: F401

import ctypes as C

# ---------------------------------------------------------------------------
# models and Hamiltonians (host arithmetic, tiny)
# ---------------------------------------------------------------------------


class HamiltonianModel:
    pass


class Ising(HamiltonianModel):
    pass


@dataclass
class TFIsing(HamiltonianModel):
    hx: float


@dataclass
class Heisenberg(HamiltonianModel):
    Jz: float = 1.0
    Jx: float = 1.0
    Jy: float = 1.0


_SX = np.array([[0.0, 1.0], [1.0, 0.0]])
_SYSY = np.array([[0.0, -1.0], [1.0, 0.0]])  # i·σy is real: σy⊗σy = −(iσy)⊗(iσy)
_SZ = np.array([[1.0, 0.0], [0.0, -1.0]])
_ID = np.eye(2)


def _outer(a, b):
    return np.einsum("ij,kl->ijkl", a, b)


def hamiltonian(model: HamiltonianModel) -> np.ndarray:
    """Two-site operator h[i,j,k,l] (src/hamiltonianmodels.jl:28-33, 53-59)."""
    if isinstance(model, TFIsing):
        hx = model.hx
        h = -2 * _outer(_SZ, _SZ) - hx / 2 * _outer(_SX, _ID) - hx / 2 * _outer(_ID, _SX)
    elif isinstance(model, Heisenberg):
        h = model.Jz * _outer(_SZ, _SZ) - model.Jx * _outer(_SX, _SX) + model.Jy * _outer(_SYSY, _SYSY)
        h = np.einsum("ijcd,kc,ld->ijkl", h, _SX, _SX.T)
        h = h / 2
    else:
        raise TypeError(f"no hamiltonian for {type(model).__name__}")
    return np.asfortranarray(h)


def diaglocalhamiltonian(diag) -> np.ndarray:
    """src/variationalipeps.jl:15-20."""
    diag = np.asarray(diag, dtype=np.float64)
    n = diag.shape[0]
    h, idn = np.diag(diag), np.eye(n)
    return np.asfortranarray(h.reshape(n, n, 1, 1) * idn.reshape(1, 1, n, n) + h.reshape(1, 1, n, n) * idn.reshape(n, n, 1, 1))


def model_tensor(model: HamiltonianModel, beta: float, with_derivative: bool = False):
    """model_tensor(::Ising, β) (src/exampletensors.jl:30-35); optionally ∂a/∂β."""
    if not isinstance(model, Ising):
        raise TypeError("model_tensor is defined for Ising()")
    a, da = fzeros((2, 2, 2, 2)), fzeros((2, 2, 2, 2))
    rc = L.load().tnad_model_tensor_ising(float(beta), ptr(a), ptr(da))
    if rc != 0:
        raise TnadError(rc, "model_tensor")
    return (a, da) if with_derivative else a


ISING_BETA_C = math.log(1 + math.sqrt(2)) / 2


def magofbeta(model: Ising, beta: float) -> float:
    """Analytic magnetisation (src/exampletensors.jl:77)."""
    return (1 - math.sinh(2 * beta) ** -4) ** (1 / 8) if beta > ISING_BETA_C else 0.0


# ---------------------------------------------------------------------------
# TRG
# ---------------------------------------------------------------------------


def trg(a, chi: int, niter: int, tol: float = 1e-16) -> float:
    """ln Z per site (src/trg.jl:13-30), computed by libtnad."""
    lnZ, _ = _trg(a, chi, niter, tol, record=False)
    return lnZ


def _trg(a, chi, niter, tol, record):
    a = farr(a)
    d = a.shape[0]
    if a.shape != (d, d, d, d):
        raise DimensionMismatch(f"trg needs a d×d×d×d tensor, got {a.shape}")
    c = ctx()
    out = C.c_double()
    tp = L.VP()
    c.check(c.lib.tnad_trg(c.h, ptr(a), d, int(chi), int(niter), float(tol), C.byref(out),
                           C.byref(tp) if record else None))
    return out.value, (L.Tape(c, tp, "trg") if record else None)


def trg_gradient(a, chi: int, niter: int, tol: float = 1e-16, dlnZ: float = 1.0):
    """(lnZ, ∂lnZ/∂a): the Zygote gradient of trg (src/trg.jl:13-30, 55-61, 72-105)."""
    a = farr(a)
    lnZ, tp = _trg(a, chi, niter, tol, record=True)
    g = fzeros(a.shape)
    c = tp.c
    c.check(c.lib.tnad_trg_backward(c.h, tp.h, float(dlnZ), ptr(g)))
    return lnZ, g


def trg_beta(beta: float, chi: int, niter: int, tol: float = 1e-16):
    """(lnZ, d lnZ/dβ) for trg(model_tensor(Ising(), β), χ, niter) (README.md:57-73)."""
    a, da = model_tensor(Ising(), beta, with_derivative=True)
    lnZ, g = trg_gradient(a, chi, niter, tol)
    return lnZ, float(np.sum(g * da))


def trg_svd(t, chi: int, tol: float):
    """trg_svd(t, χ, tol) (src/trg.jl:33-44) → (u: d1×d2×k, v: k×d3×d4)."""
    t = farr(t)
    d1, d2, d3, d4 = t.shape
    kmax = min(chi, d1 * d2, d3 * d4)
    u, v = fzeros((d1 * d2 * kmax,)), fzeros((kmax * d3 * d4,))
    k = C.c_int()
    c = ctx()
    c.check(c.lib.tnad_trg_svd(c.h, ptr(t), d1, d2, d3, d4, int(chi), float(tol), ptr(u), ptr(v), C.byref(k)))
    k = k.value
    return (u[: d1 * d2 * k].reshape((d1, d2, k), order="F"), v[: k * d3 * d4].reshape((k, d3, d4), order="F"))


def svd(A):
    """FP64 one-sided Jacobi SVD on the GPU: (U, S, V) with A = U·diag(S)·Vᵀ (thin, m ≥ n)."""
    A = farr(A)
    m, n = A.shape
    if m < n:
        V, S, U = svd(A.T)
        return U, S, V
    U, S, V = fzeros((m, n)), fzeros((n,)), fzeros((n, n))
    c = ctx()
    c.check(c.lib.tnad_svd(c.h, ptr(A), m, n, ptr(U), ptr(S), ptr(V)))
    return U, S, V


def svd_symmetric(A, tensor_cores: bool = False):
    """SVD of a symmetric matrix (the cpmat of src/ctmrg.jl:134-136) through its
    eigendecomposition on the GPU: (U, S, V), S = |λ| descending, U = V·sign(λ).
    ``tensor_cores`` runs the refinement's FP64 products on the tensor cores."""
    A = farr(A)
    n = A.shape[0]
    if A.shape != (n, n):
        raise DimensionMismatch(f"svd_symmetric needs a square matrix, got {A.shape}")
    U, S, V = fzeros((n, n)), fzeros((n,)), fzeros((n, n))
    c = ctx()
    prec = L.PREC_FP64_TC if tensor_cores else L.PREC_FP64
    c.check(c.lib.tnad_svd_sym(c.h, prec, ptr(A), n, ptr(U), ptr(S), ptr(V)))
    return U, S, V


def solver_stats():
    """(refined, fell_back): symmetric SVDs of this thread's context that took the
    product refinement / fell back to FP64 Jacobi sweeps."""
    c = ctx()
    r, f = C.c_int64(), C.c_int64()
    c.check(c.lib.tnad_ctx_solver_stats(c.h, C.byref(r), C.byref(f)))
    return int(r.value), int(f.value)


def svd_complex(A):
    """Thin SVD of a complex matrix on the GPU: (U, S, V) with A = U·diag(S)·Vᴴ."""
    A = L.zarr(A)
    m, n = A.shape
    k = min(m, n)
    U, V = np.zeros((m, k), np.complex128, order="F"), np.zeros((n, k), np.complex128, order="F")
    S = fzeros((k,))
    c = ctx()
    c.check(c.lib.tnad_svd_z(c.h, L.zptr(A), m, n, L.zptr(U), ptr(S), L.zptr(V)))
    return U, S, V


def svd_back_complex(U, S, V, dU=None, dS=None, dV=None, eta: float = 1e-40):
    """Complex SVD adjoint (src/trg.jl:72-105, with the imaginary-diagonal term of :85) on the GPU."""
    U, V, S = L.zarr(U), L.zarr(V), farr(S)
    m, n = U.shape[0], V.shape[0]
    dA = np.zeros((m, n), np.complex128, order="F")
    c = ctx()
    c.check(c.lib.tnad_svd_back_z(c.h, L.zptr(U), ptr(S), L.zptr(V), m, n,
                                  L.zptr(None if dU is None else L.zarr(dU)), ptr(None if dS is None else farr(dS)),
                                  L.zptr(None if dV is None else L.zarr(dV)), float(eta), L.zptr(dA)))
    return dA


def svd_back(U, S, V, dU=None, dS=None, dV=None, eta: float = 1e-40):
    """SVD adjoint (src/trg.jl:72-105) on the GPU."""
    U, S, V = farr(U), farr(S), farr(V)
    m, n = U.shape
    dA = fzeros((m, n))
    c = ctx()
    c.check(c.lib.tnad_svd_back(c.h, ptr(U), ptr(S), ptr(V), m, n, ptr(None if dU is None else farr(dU)),
                                ptr(None if dS is None else farr(dS)), ptr(None if dV is None else farr(dV)),
                                float(eta), ptr(dA)))
    return dA


# ---------------------------------------------------------------------------
# lattices, runtimes, iPEPS
# ---------------------------------------------------------------------------


class AbstractLattice:
    pass


class SquareLattice(AbstractLattice):
    pass


@dataclass
class CTMRGRuntime:
    """bulk d×d×d×d, corner χ×χ, edge χ×d×χ (src/ctmrg.jl:23-34)."""
    bulk: np.ndarray
    corner: np.ndarray
    edge: np.ndarray
    lattice: type = SquareLattice
    steps: int = 0

    @property
    def chi(self) -> int:
        return self.corner.shape[0]

    @property
    def D(self) -> int:
        return self.bulk.shape[0]


def getchi(rt: CTMRGRuntime) -> int:
    return rt.chi


def getD(rt: CTMRGRuntime) -> int:
    return rt.D


def SquareCTMRGRuntime(bulk, env, chi: int = None, *, rng: np.random.Generator | None = None, corner=None,
                       edge=None) -> CTMRGRuntime:
    """SquareCTMRGRuntime(bulk, Val(:raw)|Val(:random), χ) (src/ctmrg.jl:62-86), or (bulk, corner, edge)."""
    bulk = farr(bulk)
    d = bulk.shape[0]
    if bulk.shape != (d, d, d, d):
        raise DimensionMismatch(f"bulk must be d×d×d×d, got {bulk.shape}")
    if isinstance(env, np.ndarray):  # SquareCTMRGRuntime(bulk, corner, edge)
        return CTMRGRuntime(bulk, farr(env), farr(chi))
    if env == "raw":
        Cc, Tt = fzeros((chi, chi)), fzeros((chi, d, chi))
        c = ctx()
        c.check(c.lib.tnad_init_raw(c.h, ptr(bulk), d, int(chi), ptr(Cc), ptr(Tt)))
        return CTMRGRuntime(bulk, Cc, Tt)
    if env == "random":
        rng = rng or np.random.default_rng()
        Cc = rng.standard_normal((chi, chi))
        Tt = rng.standard_normal((chi, d, chi))
        Cc = Cc + Cc.T
        Tt = Tt + Tt.transpose(2, 1, 0)
        return CTMRGRuntime(bulk, farr(Cc), farr(Tt))
    raise ValueError("env must be 'raw' or 'random'")


def ctmrg(rt: CTMRGRuntime, tol: float, maxit: int, opts: L.Opts | None = None) -> CTMRGRuntime:
    """ctmrg(rt; tol, maxit) (src/ctmrg.jl:110-117) on the GPU."""
    out, _ = _ctmrg(rt, tol, maxit, opts, record=False)
    return out


def _ctmrg(rt, tol, maxit, opts, record):
    d, chi = rt.D, rt.chi
    Cc, Tt = fzeros((chi, chi)), fzeros((chi, d, chi))
    steps = C.c_int()
    tp = L.VP()
    c = ctx()
    o = opts or default_opts()
    c.check(c.lib.tnad_ctmrg(c.h, ptr(rt.bulk), d, chi, ptr(farr(rt.corner)), ptr(farr(rt.edge)), float(tol),
                             int(maxit), C.byref(o), ptr(Cc), ptr(Tt), C.byref(steps),
                             C.byref(tp) if record else None))
    return CTMRGRuntime(rt.bulk, Cc, Tt, rt.lattice, steps.value), (L.Tape(c, tp, "ctmrg") if record else None)


def ctmrg_gradient(rt: CTMRGRuntime, tol: float, maxit: int, dC, dT, opts=None):
    """Pullback of ctmrg w.r.t. the bulk (the initial environment gets none: src/autodiff.jl:4-5)."""
    out, tp = _ctmrg(rt, tol, maxit, opts, record=True)
    g = fzeros(rt.bulk.shape)
    c = tp.c
    c.check(c.lib.tnad_ctmrg_backward(c.h, tp.h, ptr(farr(dC)), ptr(farr(dT)), ptr(g)))
    return out, g


def ctmrgstep(rt: CTMRGRuntime):
    """One ctmrgstep (src/ctmrg.jl:126-153): (runtime', vals)."""
    d, chi = rt.D, rt.chi
    Cc, Tt, vals = fzeros((chi, chi)), fzeros((chi, d, chi)), fzeros((chi * d,))
    c = ctx()
    c.check(c.lib.tnad_ctmrgstep(c.h, ptr(rt.bulk), d, chi, ptr(farr(rt.corner)), ptr(farr(rt.edge)), ptr(Cc),
                                 ptr(Tt), ptr(vals)))
    return CTMRGRuntime(rt.bulk, Cc, Tt, rt.lattice), vals


def ctmrgstep_backward(rt: CTMRGRuntime, dC, dT):
    d, chi = rt.D, rt.chi
    ga, gC, gT = fzeros(rt.bulk.shape), fzeros((chi, chi)), fzeros((chi, d, chi))
    c = ctx()
    c.check(c.lib.tnad_ctmrgstep_backward(c.h, ptr(rt.bulk), d, chi, ptr(farr(rt.corner)), ptr(farr(rt.edge)),
                                          ptr(farr(dC)), ptr(farr(dT)), ptr(ga), ptr(gC), ptr(gT)))
    return ga, gC, gT


@dataclass
class IPEPS:
    bulk: np.ndarray
    lattice: type = SquareLattice


def SquareIPEPS(bulk) -> IPEPS:
    """SquareIPEPS (src/ipeps.jl:17-22): bulk must be d×d×d×d×s."""
    bulk = farr(bulk)
    if bulk.ndim != 5 or not (bulk.shape[0] == bulk.shape[1] == bulk.shape[2] == bulk.shape[3]):
        raise DimensionMismatch(f"size of tensor error, should be `(d, d, d, d, s)`, got {bulk.shape}.")
    return IPEPS(bulk)


def getd(ipeps: IPEPS) -> int:
    return ipeps.bulk.shape[0]


def gets(ipeps: IPEPS) -> int:
    return ipeps.bulk.shape[4]


def indexperm_symmetrize(ipeps: IPEPS) -> IPEPS:
    """src/ipeps.jl:32-39 on the GPU."""
    A = ipeps.bulk
    D, s = A.shape[0], A.shape[4]
    out = fzeros(A.shape)
    c = ctx()
    c.check(c.lib.tnad_symmetrize(c.h, ptr(A), D, s, ptr(out)))
    return SquareIPEPS(out)


def expectationvalue(h, ap, rt: CTMRGRuntime) -> float:
    """src/variationalipeps.jl:49-56."""
    ap = farr(ap)
    d, s = ap.shape[0], ap.shape[4]
    E = C.c_double()
    c = ctx()
    c.check(c.lib.tnad_expectationvalue(c.h, ptr(farr(h)), ptr(ap), d, s, rt.chi, ptr(farr(rt.corner)),
                                        ptr(farr(rt.edge)), C.byref(E)))
    return E.value


@dataclass
class EnergyResult:
    E: float
    steps: int
    corner: np.ndarray | None = None
    edge: np.ndarray | None = None
    tape: object = None


def _energy(h, ipeps, chi, tol, maxit, opts=None, record=False, env=None, want_env=False):
    bulk = ipeps.bulk if isinstance(ipeps, IPEPS) else farr(ipeps)
    if bulk.ndim != 5 or not (bulk.shape[0] == bulk.shape[1] == bulk.shape[2] == bulk.shape[3]):
        raise DimensionMismatch(f"size of tensor error, should be `(d, d, d, d, s)`, got {bulk.shape}.")
    D, s = bulk.shape[0], bulk.shape[4]
    d = D * D
    o = opts or default_opts()
    Ci = Ti = None
    if env is not None:
        Ci, Ti = farr(env[0]), farr(env[1])
        o.warm_start = 1
    Co = To = None
    if want_env:
        Co, To = fzeros((chi, chi)), fzeros((chi, d, chi))
    E = C.c_double()
    steps = C.c_int()
    tp = L.VP()
    c = ctx()
    c.check(c.lib.tnad_energy(c.h, ptr(farr(h)), ptr(bulk), D, s, int(chi), float(tol), int(maxit), C.byref(o),
                              ptr(Ci), ptr(Ti), C.byref(E), C.byref(steps), ptr(Co), ptr(To),
                              C.byref(tp) if record else None))
    return EnergyResult(E.value, steps.value, Co, To, L.Tape(c, tp, "energy") if record else None)


def energy(h, ipeps, chi: int, tol: float, maxit: int, opts=None) -> float:
    """energy(h, ipeps; χ, tol, maxit) (src/variationalipeps.jl:28-40) on the GPU."""
    return _energy(h, ipeps, chi, tol, maxit, opts).E


def energy_and_gradient(h, ipeps, chi: int, tol: float, maxit: int, opts=None, env=None, stats: dict | None = None):
    """(E, ∂E/∂bulk): Zygote.gradient of energy (src/variationalipeps.jl:71-73).

    ``stats`` (optional dict) receives the solver diagnostics of tnad_energy_stats."""
    r = _energy(h, ipeps, chi, tol, maxit, opts, record=True, env=env)
    bulk = ipeps.bulk if isinstance(ipeps, IPEPS) else farr(ipeps)
    g = fzeros(bulk.shape)
    c = r.tape.c
    c.check(c.lib.tnad_energy_backward(c.h, r.tape.h, 1.0, ptr(g)))
    if stats is not None:
        stats.update(tape_stats(r.tape))
    return r.E, g


def tape_stats(tape) -> dict:
    vals = [C.c_int() for _ in range(4)] + [C.c_double(), C.c_double()]
    rc = tape.c.lib.tnad_energy_stats(tape.h, *[C.byref(v) for v in vals])
    if rc != 0:
        raise TnadError(rc, "tnad_energy_stats")
    keys = ["steps", "fp64_steps", "switch_step", "fp_iters", "last_diff", "fp_residual"]
    out = {k: v.value for k, v in zip(keys, vals)}
    r = C.c_double()
    if tape.c.lib.tnad_energy_fixed_point_residual(tape.h, C.byref(r)) == 0:
        out["fixed_point_residual"] = r.value
    return out


def mixed_opts(ladder_tol: float = 1e-5, fp_tol: float = 1e-9, fp_maxit: int = 200, fp64_tc: int = 1,
               **kw) -> L.Opts:
    """Options of the mixed path: TF32X3 contractions with the FP64 polishing ladder
    (whose FP64 products run as tensor-core FP64 emulation when fp64_tc = 1), the
    warm-started subspace solver, and the implicit fixed-point adjoint."""
    return default_opts(prec=L.PREC_LADDER, solver=L.SOLVER_SUBSPACE, adjoint=L.ADJOINT_FIXEDPOINT, stop_rule=1,
                        ladder_tol=ladder_tol, fp_tol=fp_tol, fp_maxit=fp_maxit, fp64_tc=fp64_tc, **kw)


def optimiseipeps(ipeps: IPEPS, h, chi: int, tol: float, maxit: int, f_tol: float = 1e-6, iterations: int = 1000,
                  m: int = 20, callback=None, opts=None, driver: str = "scipy", g_tol: float = 1e-10,
                  stats: dict | None = None):
    """optimiseipeps (src/variationalipeps.jl:67-75): L-BFGS(m) on energy with the GPU gradient;
    returns (minimum, minimizer).

    driver="scipy": SciPy's L-BFGS-B on the host plays Optim's LBFGS(m = 20), one
    library call per evaluation.  driver="device": the L-BFGS of the library
    (tnad_optimiseipeps), iterate and pairs on the device, Armijo backtracking;
    ``stats`` receives its iteration and evaluation counts.
    """
    if driver == "device":
        A = farr(ipeps.bulk).copy(order="F")
        D, s = A.shape[0], A.shape[4]
        E, it, ev = C.c_double(), C.c_int(), C.c_int()
        o = opts or default_opts()
        c = ctx()
        c.check(c.lib.tnad_optimiseipeps(c.h, ptr(farr(h)), ptr(A), D, s, int(chi), float(tol), int(maxit),
                                         C.byref(o), int(m), int(iterations), float(f_tol), float(g_tol),
                                         C.byref(E), C.byref(it), C.byref(ev)))
        if stats is not None:
            stats.update(iterations=it.value, evaluations=ev.value)
        return E.value, A
    import scipy.optimize

    shape = ipeps.bulk.shape

    def fg(x):
        e, g = energy_and_gradient(h, SquareIPEPS(x.reshape(shape, order="F")), chi, tol, maxit, opts)
        return e, np.asarray(g).ravel(order="F")

    r = scipy.optimize.minimize(fg, np.asarray(ipeps.bulk).ravel(order="F"), jac=True, method="L-BFGS-B",
                                callback=callback,
                                options=dict(maxcor=m, maxiter=iterations, ftol=f_tol, gtol=1e-12))
    return float(r.fun), r.x.reshape(shape, order="F")


def num_grad(f, K, delta: float = 1e-5, dist=None):
    """(f(K+δ/2) − f(K−δ/2))/δ, elementwise for arrays (src/autodiff.jl:44-63).

    dist: the ``torch.distributed`` module itself, with its default process
    group initialised (one rank per GPU).  The elements are then independent
    units: each rank differentiates a contiguous share of them and every rank
    returns the gathered array."""
    if np.isscalar(K):
        return (f(K + delta / 2) - f(K - delta / 2)) / delta
    K = np.asarray(K, dtype=np.float64)
    idx = list(np.ndindex(K.shape))
    rank, world = 0, 1
    if dist is not None and dist.is_initialized():
        rank, world = dist.get_rank(), dist.get_world_size()
    part = []
    for i in idx[len(idx) * rank // world:len(idx) * (rank + 1) // world]:
        kp, km = K.copy(), K.copy()
        kp[i] += delta / 2
        km[i] -= delta / 2
        part.append((f(kp) - f(km)) / delta)
    if world > 1:
        parts = [None] * world
        dist.all_gather_object(parts, part)
        part = [v for p in parts for v in p]
    return np.asarray(part, dtype=np.float64).reshape(K.shape)


def mag_tensor(model: Ising, beta: float) -> np.ndarray:
    """mag_tensor(::Ising, β) (src/exampletensors.jl:43-48)."""
    cb, sb = math.sqrt(math.cosh(beta)), math.sqrt(math.sinh(beta))
    q = np.array([[cb + sb, cb - sb], [cb - sb, cb + sb]]) / math.sqrt(2)
    a = np.zeros((2, 2, 2, 2))
    a[0, 0, 0, 0], a[1, 1, 1, 1] = 1.0, -1.0
    return np.asfortranarray(np.einsum("abcd,ai,bj,ck,dl->ijkl", a, q, q, q, q))


def magnetisation(model: Ising, beta: float, chi: int, rng: np.random.Generator | None = None, tol=1e-6,
                  maxit=100) -> float:
    """magnetisation(::Ising, β, χ) (src/exampletensors.jl:57-69): CTMRG on the GPU from a random env."""
    a = model_tensor(model, beta)
    m = mag_tensor(model, beta)
    rt = ctmrg(SquareCTMRGRuntime(a, "random", chi, rng=rng), tol, maxit)
    c, t = rt.corner, rt.edge
    ctc = np.einsum("ia,ajb,bk->ijk", c, t, c)
    env = np.einsum("alc,ckd,bjd,bia->ijkl", ctc, t, ctc, t)
    return abs(float(np.sum(env * m)) / float(np.sum(env * a)))


__all__ = [
    "svd_symmetric", "solver_stats",
    "Ising", "TFIsing", "Heisenberg", "hamiltonian", "diaglocalhamiltonian", "model_tensor", "mag_tensor",
    "magnetisation", "magofbeta", "trg", "trg_gradient", "trg_beta", "trg_svd", "svd", "svd_back",
    "AbstractLattice", "SquareLattice", "CTMRGRuntime", "SquareCTMRGRuntime", "ctmrg", "ctmrg_gradient",
    "ctmrgstep", "ctmrgstep_backward", "IPEPS", "SquareIPEPS", "indexperm_symmetrize", "expectationvalue",
    "energy", "energy_and_gradient", "optimiseipeps", "num_grad", "DimensionMismatch", "TnadError",
]


# ---------------------------------------------------------------------------
# building blocks exposed for tests and callers
# ---------------------------------------------------------------------------


def site_tensor(recipe: str, D: int, s: int, seed: int) -> np.ndarray:
    """Seeded synthetic site tensors of the benchmark workloads (NumPy default_rng):
    "uniform" — entries uniform in [0, 1); "normal_maxabs" — N(0, 1) entries divided by
    the largest |entry|."""
    rng = np.random.default_rng(seed)
    if recipe == "uniform":
        return np.asfortranarray(rng.random((D, D, D, D, s)))
    if recipe == "normal_maxabs":
        x = rng.standard_normal((D, D, D, D, s))
        return np.asfortranarray(x / np.abs(x).max())
    raise ValueError(f"unknown site-tensor recipe {recipe!r}")


def gemm(A, B, ta="N", tb="N", alpha=1.0, beta=0.0, Cin=None, prec=L.PREC_FP64):
    """alpha·op(A)·op(B) + beta·C on the GPU (column-major, FP64 or 3xTF32)."""
    A, B = farr(A), farr(B)
    M = A.shape[1] if ta == "T" else A.shape[0]
    K = A.shape[0] if ta == "T" else A.shape[1]
    N = B.shape[0] if tb == "T" else B.shape[1]
    Cm = fzeros((M, N)) if Cin is None else farr(Cin).copy(order="F")
    c = ctx()
    c.check(c.lib.tnad_gemm(c.h, int(prec), ta.encode(), tb.encode(), M, N, K, float(alpha), ptr(A),
                            A.shape[0], ptr(B), B.shape[0], float(beta), ptr(Cm), M))
    return Cm


def contract(spec: str, A, B, prec=L.PREC_FP64):
    """Pairwise einsum "la,lb->lc" on the GPU."""
    lhs, lc = spec.replace(" ", "").split("->")
    la, lb = lhs.split(",")
    A, B = farr(A), farr(B)
    dims = {**dict(zip(la, A.shape)), **dict(zip(lb, B.shape))}
    out = fzeros(tuple(dims[ch] for ch in lc))
    da = (C.c_int64 * len(la))(*A.shape)
    db = (C.c_int64 * len(lb))(*B.shape)
    c = ctx()
    c.check(c.lib.tnad_contract(c.h, int(prec), ptr(A), la.encode(), da, ptr(B), lb.encode(), db, ptr(out),
                                lc.encode()))
    return out
