"""NumPy restatement of the GPU path for the symmetric SVD of the CTMRG corner.

TEST INFRASTRUCTURE ONLY: imported by ``tests/`` as the CPU check of the
algorithm in ``tensornetworkad.jl_gb300/csrc/jacobi.cu`` (FP32 sweeps with the
eigenvalue rule) and ``csrc/eig_refine.cu`` (the product refinement).  The
product path never calls it.

The reference decomposes the symmetrised enlarged corner with
``LinearAlgebra.svd`` (src/ctmrg.jl:134-136); the GPU computes it as an
eigendecomposition M = X·diag(λ)·Xᵀ returned as S = |λ| (descending), V = X,
U = X·sign(λ).  This module restates, step for step:

* ``jacobi_eig_fp32``: one-sided Jacobi in float32 in the circle-method order,
  each rotation diagonalising the 2×2 block of VᵀMV (the eigenvalue rule), stop
  once at most 16n pairs rotated in a sweep (absolute threshold 2ε₃₂‖M‖_F);
* three FP64 Newton–Schulz steps on V;
* ``refine``: the Ogita–Aishima iteration with the GPU's groups (strongly
  coupled pairs as intervals of the |λ|-sorted order, η = 0.05), its noise
  level max(4nε‖M‖_F, 8·max|S_ij|), Rayleigh–Ritz inside groups of ≤ 64
  columns, a Newton–Schulz step after every update, its stop rule and its
  give-up rules (``None`` where the GPU falls back to FP64 Jacobi sweeps).
"""
from __future__ import annotations

import numpy as np

EPS64 = np.finfo(np.float64).eps
EPS32 = np.finfo(np.float32).eps
ETA = 0.05
MAX_GROUP = 64
MAX_IT = 8
MAX_START_OFF = 1e-4


def _pairs(r: int, NP: int):
    k = np.arange(NP // 2)
    p = np.where(k == 0, NP - 1, (r + k) % (NP - 1))
    q = np.where(k == 0, r, (r - k + (NP - 1)) % (NP - 1))
    return np.minimum(p, q), np.maximum(p, q)


def jacobi_eig_fp32(A: np.ndarray, max_sweeps: int = 30) -> np.ndarray:
    """FP32 eigenvalue-rule Jacobi (one-sided storage W = A·V); returns V (float64)."""
    n = A.shape[0]
    W = A.astype(np.float32)
    V = np.eye(n, dtype=np.float32)
    NP = n + (n & 1)
    thr = np.float32(2.0 * EPS32 * np.sqrt(np.sum(A.astype(np.float64) ** 2)))
    for _ in range(max_sweeps):
        rot = 0
        for r in range(NP - 1):
            p, q = _pairs(r, NP)
            ok = (p < n) & (q < n)
            p, q = p[ok], q[ok]
            x, y, vx, vy = W[:, p], W[:, q], V[:, p], V[:, q]
            a = np.sum(vx * x, axis=0)
            b = np.sum(vy * y, axis=0)
            g = np.float32(0.5) * (np.sum(vx * y, axis=0) + np.sum(vy * x, axis=0))
            do = (g != 0) & (np.abs(g) > thr)
            zeta = np.where(do, (b - a) / (2 * np.where(do, g, 1)), 0).astype(np.float32)
            t = (np.sign(zeta) + (zeta == 0)) / (np.abs(zeta) + np.sqrt(1 + zeta * zeta))
            cs = np.where(do, 1 / np.sqrt(1 + t * t), 1).astype(np.float32)
            sn = np.where(do, cs * t, 0).astype(np.float32)
            W[:, p], W[:, q] = cs * x - sn * y, sn * x + cs * y
            V[:, p], V[:, q] = cs * vx - sn * vy, sn * vx + cs * vy
            rot += int(do.sum())
        if rot <= 16 * n:
            break
    return V.astype(np.float64)


def newton_schulz(X: np.ndarray, steps: int) -> np.ndarray:
    n = X.shape[1]
    for _ in range(steps):
        X = X @ (1.5 * np.eye(n) - 0.5 * (X.T @ X))
    return X


def _groups(lam, S, G, noise):
    """Group ids per column, and the groups to solve (lists of columns)."""
    n = len(lam)
    al = np.abs(lam)
    order = np.lexsort((np.arange(n), -al))   # |λ| descending, ties by index
    pos = np.empty(n, int)
    pos[order] = np.arange(n)
    den = ETA * np.abs(lam[:, None] - lam[None, :])
    strong = (np.abs(S - lam[:, None] * G) > den) | (np.abs(S - lam[None, :] * G) > den)
    np.fill_diagonal(strong, False)
    cover = np.zeros(n + 1, int)
    for i in range(n):
        ks = np.nonzero(strong[:, i])[0]
        lo = min(pos[i], pos[ks].min()) if len(ks) else pos[i]
        hi = max(pos[i], pos[ks].max()) if len(ks) else pos[i]
        if hi > lo:
            cover[lo] += 1
            cover[hi] -= 1
    linked = np.cumsum(cover[:n]) > 0            # sorted r linked to r + 1
    head = np.ones(n, bool)
    head[1:] = ~linked[:-1]
    gid_sorted = np.cumsum(head) - 1
    gid = np.empty(n, int)
    gid[order] = gid_sorted
    solve = []
    for h in np.nonzero(head)[0]:
        e = h + 1
        while e < n and not head[e]:
            e += 1
        if e - h >= 2 and al[order[h]] > noise:
            solve.append(order[h:e])
    return gid, solve


def refine(A: np.ndarray, X: np.ndarray):
    """The product refinement of eig_refine.cu; (X, λ) or None where the GPU gives up."""
    n = A.shape[0]
    fro = np.sqrt(np.sum(A * A))
    prev_off = 0.0
    for it in range(MAX_IT):
        AX = A @ X
        S = X.T @ AX
        G = X.T @ X
        lam = np.diag(S) / np.diag(G)
        off = S.copy()
        np.fill_diagonal(off, 0.0)
        mo = np.abs(off).max()
        mr = np.abs(np.eye(n) - G).max()
        if not (np.isfinite(mo) and np.isfinite(mr)):
            return None
        noise = max(4.0 * n * EPS64 * fro, 8.0 * mo)
        gid, solve = _groups(lam, S, G, noise)
        if any(len(g) > MAX_GROUP for g in solve):
            return None
        off_rel = mo / fro
        if (it == 0 and off_rel > MAX_START_OFF) or (it > 0 and off_rel > 4.0 * prev_off):
            return None
        prev_off = off_rel
        done = it >= 1 and off_rel <= 1e-10 and mr <= 1e-8 and not solve
        for cols in solve:   # Rayleigh–Ritz inside the group; S, G, X follow
            blk = 0.5 * (S[np.ix_(cols, cols)] + S[np.ix_(cols, cols)].T)
            _, Q = np.linalg.eigh(blk)
            S[:, cols] = S[:, cols] @ Q
            S[cols, :] = Q.T @ S[cols, :]
            G[:, cols] = G[:, cols] @ Q
            G[cols, :] = Q.T @ G[cols, :]
            X[:, cols] = X[:, cols] @ Q
        if solve:
            lam = np.diag(S) / np.diag(G)
        R = np.eye(n) - G
        same = gid[:, None] == gid[None, :]
        dl = lam[None, :] - lam[:, None]
        safe = np.where(same | (dl == 0), 1.0, dl)
        E = np.where(same | (dl == 0), 0.5 * R, (S + lam[None, :] * R) / safe)
        np.fill_diagonal(E, 0.5 * np.diag(R))
        X = newton_schulz(X + X @ E, 1)
        if done:
            return X, np.einsum("ij,ij->j", X, A @ X)
    return None


def svd_symmetric(A: np.ndarray):
    """(U, S, V) as the GPU returns them, or None where it falls back to FP64 sweeps."""
    X = newton_schulz(jacobi_eig_fp32(A), 3)
    out = refine(A, X)
    if out is None:
        return None
    X, lam = out
    order = np.lexsort((np.arange(len(lam)), -np.abs(lam)))
    X, lam = X[:, order], lam[order]
    sg = np.where(lam < 0, -1.0, 1.0)
    return X * sg[None, :], np.abs(lam), X
