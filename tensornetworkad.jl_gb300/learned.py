"""Learned CTMRG warm start (no reference counterpart).

A 3-layer perceptron (width 512 by default, BF16 tensor-core products with FP32
accumulation) predicts, from the symmetrised site tensor, the gauge-fixed
environment that plain CTMRG converges to: the corner spectrum λ (χ values)
and the edge tensor Tg (χ×D²×χ).  ``energy`` with ``warm_start=WARM_LEARNED``
then starts CTMRG from C = diag(λ̂), T = T̂; the CTMRG residual judges the
prediction and a :raw restart replaces it whenever the residual does not fall
from step 2 to step 4.

Everything numeric runs in libtnad on the GPU: target gauge fixing
(tnad_env_gauge_fix), features (tnad_warm_start_features), training
(tnad_mlp_train_step: forward, MSE backward, AdamW) and inference.  This module
only drives those calls: it draws site tensors, collects targets from CTMRG,
standardises them, schedules the learning rate and folds the standardisation
into the last layer.
"""
from __future__ import annotations

import ctypes as C
import math
import time
from dataclasses import dataclass

import numpy as np

from . import _lib as L
from ._lib import ctx, farr, fptr, ptr

ROOT_SEED = 0x5EED


def n_in_of(D: int, s: int) -> int:
    return D ** 4 * s


def n_out_of(D: int, chi: int) -> int:
    return chi + chi * D * D * chi


class WarmStartNet:
    """The warm-start network for site tensors D×D×D×D×s at bond dimension χ."""

    def __init__(self, D: int, s: int, chi: int, width: int = 512, seed: int = 0):
        self.D, self.s, self.chi, self.width = D, s, chi, width
        self.n_in, self.n_out = n_in_of(D, s), n_out_of(D, chi)
        self.c = ctx()
        self.h = L.VP()
        self.c.check(self.c.lib.tnad_mlp_create(self.c.h, self.n_in, width, self.n_out, int(seed), C.byref(self.h)))
        self.n_params = int(self.c.lib.tnad_mlp_param_count(self.h))

    def __del__(self):
        try:
            if self.h:
                self.c.lib.tnad_ctx_set_warm_start(self.c.h, None, 0, 0, 0)
                self.c.lib.tnad_mlp_free(self.h)
                self.h = L.VP()
        except Exception:
            pass

    # ---- parameters ----
    def get_params(self) -> np.ndarray:
        P = np.zeros(self.n_params, np.float32)
        self.c.check(self.c.lib.tnad_mlp_get_params(self.c.h, self.h, fptr(P)))
        return P

    def set_params(self, P) -> None:
        P = np.asfortranarray(np.asarray(P, np.float32))
        assert P.size == self.n_params
        self.c.check(self.c.lib.tnad_mlp_set_params(self.c.h, self.h, fptr(P)))

    # ---- compute ----
    def forward(self, X) -> np.ndarray:
        X = np.asfortranarray(np.asarray(X, np.float32).reshape(self.n_in, -1, order="F"))
        Y = np.zeros((self.n_out, X.shape[1]), np.float32, order="F")
        self.c.check(self.c.lib.tnad_mlp_forward(self.c.h, self.h, fptr(X), X.shape[1], fptr(Y), 0))
        return Y

    def gradient(self, X, Y):
        """(loss, ∂loss/∂params) of loss = mean((net(X) − Y)²)."""
        X = np.asfortranarray(np.asarray(X, np.float32))
        Y = np.asfortranarray(np.asarray(Y, np.float32))
        G = np.zeros(self.n_params, np.float32)
        loss = C.c_float()
        self.c.check(self.c.lib.tnad_mlp_gradient(self.c.h, self.h, fptr(X), fptr(Y), X.shape[1], C.byref(loss),
                                                  fptr(G), 0))
        return float(loss.value), G

    def train_step(self, idx, lr: float, weight_decay: float = 0.0, X=None, Y=None, want_loss: bool = False):
        """One AdamW step on columns idx of (X, Y) (None: the resident set)."""
        idx = np.ascontiguousarray(np.asarray(idx, np.int32))
        loss = C.c_float()
        if X is None:
            xp = yp = fptr(None)
            n = 0
        else:
            X = np.asfortranarray(np.asarray(X, np.float32))
            Y = np.asfortranarray(np.asarray(Y, np.float32))
            xp, yp, n = fptr(X), fptr(Y), X.shape[1]
        self.c.check(self.c.lib.tnad_mlp_train_step(
            self.c.h, self.h, xp, yp, n, idx.ctypes.data_as(C.POINTER(C.c_int32)), idx.size, float(lr),
            float(weight_decay), C.byref(loss) if want_loss else None, 0))
        return float(loss.value) if want_loss else None

    def set_data(self, X, Y) -> None:
        X = np.asfortranarray(np.asarray(X, np.float32))
        Y = np.asfortranarray(np.asarray(Y, np.float32))
        assert X.shape[0] == self.n_in and Y.shape[0] == self.n_out and X.shape[1] == Y.shape[1]
        self.c.check(self.c.lib.tnad_mlp_set_data(self.c.h, self.h, fptr(X), fptr(Y), X.shape[1]))

    def fit(self, X, Y, steps: int = 3000, batch: int = 128, lr: float = 1e-3, weight_decay: float = 1e-4,
            warmup: int = 100, seed: int = 0, log_every: int = 0) -> dict:
        """Train on (X, Y) (n_in×N, n_out×N raw targets) with AdamW and a cosine
        learning-rate decay, on standardised targets (Y − μ)/σ (μ per output, σ
        one scale); afterwards μ and σ are folded into the last layer, so the
        network predicts raw targets."""
        X = np.asarray(X, np.float32)
        Y = np.asarray(Y, np.float64)
        mu = Y.mean(axis=1)
        sigma = float(np.sqrt(np.mean((Y - mu[:, None]) ** 2))) or 1.0
        Yn = ((Y - mu[:, None]) / sigma).astype(np.float32)
        self.set_data(X, Yn)
        N = X.shape[1]
        rng = np.random.default_rng(seed)
        hist = []
        t0 = time.perf_counter()
        perm, pos = rng.permutation(N), 0
        for k in range(steps):
            if pos + batch > N:
                perm, pos = rng.permutation(N), 0
            idx = perm[pos:pos + min(batch, N)]
            pos += batch
            f = min(1.0, (k + 1) / warmup) * 0.5 * (1.0 + math.cos(math.pi * k / steps))
            want = bool(log_every) and (k % log_every == 0 or k == steps - 1)
            l = self.train_step(idx, lr * max(f, 0.01), weight_decay, want_loss=want)
            if want:
                hist.append((k, l))
        loss_end = self.train_step(perm[:min(batch, N)], 0.0, 0.0, want_loss=True)
        secs = time.perf_counter() - t0
        self.c.check(self.c.lib.tnad_mlp_set_data(self.c.h, self.h, fptr(None), fptr(None), 0))
        # fold y = σ·(W3 h + b3) + μ into W3, b3
        P = self.get_params().astype(np.float64)
        ow = self.n_params - self.n_out - self.n_out * self.width
        ob = self.n_params - self.n_out
        W3 = P[ow:ob].reshape(self.n_out, self.width, order="F")
        P[ow:ob] = (sigma * W3).ravel(order="F")
        P[ob:] = sigma * P[ob:] + mu
        self.set_params(P.astype(np.float32))
        return dict(loss_std=loss_end, history=hist, seconds=secs, steps=steps, batch=batch, mu=mu, sigma=sigma)

    # ---- warm start ----
    def attach(self) -> None:
        """Make this network the predictor of energy(..., warm_start=WARM_LEARNED)."""
        self.c.check(self.c.lib.tnad_ctx_set_warm_start(self.c.h, self.h, self.D, self.s, self.chi))

    def predict_env(self, A):
        """(C, T) predicted for site tensor A (D×D×D×D×s) by the attached network."""
        d = self.D * self.D
        Cm, Tm = np.zeros((self.chi, self.chi), order="F"), np.zeros((self.chi, d, self.chi), order="F")
        self.c.check(self.c.lib.tnad_warm_start_env(self.c.h, ptr(farr(A)), self.D, self.s, self.chi, ptr(Cm),
                                                    ptr(Tm)))
        return Cm, Tm


def features(A, D: int, s: int) -> np.ndarray:
    """Network input of site tensor A (tnad_warm_start_features)."""
    c = ctx()
    x = np.zeros(n_in_of(D, s), np.float32)
    c.check(c.lib.tnad_warm_start_features(c.h, ptr(farr(A)), D, s, fptr(x)))
    return x


def gauge_fix(Cm, Tm):
    """(λ, Tg) of a symmetric environment (tnad_env_gauge_fix)."""
    c = ctx()
    Cm, Tm = farr(Cm), farr(Tm)
    chi, d = Tm.shape[0], Tm.shape[1]
    lam = np.zeros(chi)
    Tg = np.zeros((chi, d, chi), order="F")
    c.check(c.lib.tnad_env_gauge_fix(c.h, ptr(Cm), ptr(Tm), chi, d, ptr(lam), ptr(Tg)))
    return lam, Tg


def target_of(Cm, Tm) -> np.ndarray:
    lam, Tg = gauge_fix(Cm, Tm)
    return np.concatenate([lam, Tg.ravel(order="F")])


def warm_start_status() -> int:
    """1: the last WARM_LEARNED energy call kept the prediction; -1: rejected; 0: unused."""
    c = ctx()
    return int(c.lib.tnad_ctx_warm_start_status(c.h))


def random_site_tensor(D: int, s: int, rng: np.random.Generator) -> np.ndarray:
    """Site tensor with entries uniform in [-1, 1] (energy symmetrises and normalises it)."""
    return np.asfortranarray(rng.uniform(-1.0, 1.0, size=(D, D, D, D, s)))


@dataclass
class Sample:
    A: np.ndarray
    x: np.ndarray
    y: np.ndarray
    steps: int
    E: float


def make_samples(tensors, h, chi: int, tol: float, maxit: int, opts=None, threads: int = 1) -> list[Sample]:
    """Run CTMRG (through energy) on each site tensor and keep the gauge-fixed
    converged environment as the target.  With threads > 1 the runs go to that
    many host threads, each with its own libtnad context and CUDA stream, so
    that several CTMRG runs share the GPU."""
    from . import _energy

    def one(A):
        D, s = A.shape[0], A.shape[4]
        r = _energy(h, A, chi, tol, maxit, opts, want_env=True)
        return Sample(A, features(A, D, s), target_of(r.corner, r.edge).astype(np.float32), r.steps, r.E)

    if threads <= 1:
        return [one(A) for A in tensors]
    from concurrent.futures import ThreadPoolExecutor

    with ThreadPoolExecutor(max_workers=threads) as ex:
        return list(ex.map(one, tensors))


def heisenberg_trajectory(D: int, chi: int, Jz: float, rng: np.random.Generator, evals: int, tol: float,
                          maxit: int, opts=None) -> list[np.ndarray]:
    """Site tensors visited by L-BFGS (optimiseipeps) on the Heisenberg model
    with coupling Jz, from a uniform [-1, 1] start: one per gradient evaluation."""
    import scipy.optimize

    from . import Heisenberg, SquareIPEPS, energy_and_gradient, hamiltonian

    h = hamiltonian(Heisenberg(Jz=Jz))
    A0 = random_site_tensor(D, 2, rng)
    seen = []

    def fg(x):
        A = x.reshape(A0.shape, order="F")
        seen.append(np.asfortranarray(A.copy()))
        e, g = energy_and_gradient(h, SquareIPEPS(A), chi, tol, maxit, opts)
        return e, np.asarray(g).ravel(order="F")

    scipy.optimize.minimize(fg, A0.ravel(order="F"), jac=True, method="L-BFGS-B",
                            options=dict(maxcor=20, maxfun=evals, maxiter=evals, gtol=1e-12, ftol=1e-12))
    return seen[:evals]


def shard_range(n: int, rank: int, world: int) -> range:
    """Contiguous share of n independent units (site tensors) for one rank."""
    lo = n * rank // world
    return range(lo, n * (rank + 1) // world)


def gather_shards(part: list, dist=None) -> list:
    """Concatenate every rank's share in rank order (identity without a process group)."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return list(part)
    parts = [None] * dist.get_world_size()
    dist.all_gather_object(parts, list(part))
    return [x for p in parts for x in p]


def stack(samples: list[Sample]):
    X = np.stack([s.x for s in samples], axis=1).astype(np.float32)
    Y = np.stack([s.y for s in samples], axis=1).astype(np.float32)
    return np.asfortranarray(X), np.asfortranarray(Y)


def compare_starts(tensors, h, chi: int, tol: float, maxit: int, opts_factory) -> dict:
    """CTMRG steps and wall time to tol from the learned start and from :raw,
    per site tensor (energy forward, the attached network)."""
    from . import _energy

    res = dict(cold_steps=[], warm_steps=[], cold_s=[], warm_s=[], dE=[], status=[])
    for A in tensors:
        o = opts_factory()
        o.warm_start = L.WARM_NONE
        t0 = time.perf_counter()
        rc = _energy(h, A, chi, tol, maxit, o)
        t1 = time.perf_counter()
        o = opts_factory()
        o.warm_start = L.WARM_LEARNED
        rw = _energy(h, A, chi, tol, maxit, o)
        t2 = time.perf_counter()
        res["cold_steps"].append(rc.steps)
        res["warm_steps"].append(rw.steps)
        res["cold_s"].append(t1 - t0)
        res["warm_s"].append(t2 - t1)
        res["dE"].append(abs(rw.E - rc.E))
        res["status"].append(warm_start_status())
    return {k: np.asarray(v) for k, v in res.items()}
