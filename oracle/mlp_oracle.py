"""CPU oracle for the learned CTMRG warm start (no reference counterpart).

TEST INFRASTRUCTURE ONLY.  Only ``tests/`` may import this module, as the
checker of libtnad's warm-start kernels; the product never calls it.

The reference (TensorNetworkAD.jl) has no learned component, so this oracle is
a direct NumPy statement of what the kernels are specified to compute:

* ``bf16``: round-to-nearest-even of FP32 to BF16 (the operand rounding of the
  tensor-core products);
* ``gemm_bf16``: op(A)·op(B) of BF16-rounded FP32 operands, summed in FP64
  (the kernel accumulates in FP32 within chunks of 512 products, so the two
  differ by FP32 accumulation rounding only);
* ``mlp_forward`` / ``mlp_gradient``: the 3-layer perceptron and the gradient
  of the mean squared error, with every product taken through ``gemm_bf16``
  at the same places as the GPU;
* ``adamw_step``: AdamW (β = 0.9, 0.999, ε = 1e-8, decoupled weight decay on
  the weight matrices only), in FP32;
* ``features``, ``gauge_fix``, ``build_env``: the network's input, target and
  output maps.

The parameter vector layout is W1 (width×n_in) | b1 | W2 | b2 | W3 (n_out×width)
| b3 with column-major matrices, as in the C ABI.
"""
from __future__ import annotations

import numpy as np


def bf16(x) -> np.ndarray:
    """FP32 → BF16 (round to nearest, ties to even), returned as FP32."""
    x = np.ascontiguousarray(np.asarray(x, dtype=np.float32))
    u = x.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return (r & 0xFFFFFFFF).astype(np.uint32).view(np.float32).reshape(x.shape)


def gemm_bf16(ta: str, tb: str, A, B, alpha=1.0, beta=0.0, C=None) -> np.ndarray:
    a = bf16(A.T if ta == "T" else A).astype(np.float64)
    b = bf16(B.T if tb == "T" else B).astype(np.float64)
    r = alpha * (a @ b)
    if C is not None and beta != 0.0:
        r = r + beta * np.asarray(C, dtype=np.float64)
    return r.astype(np.float32)


def layout(n_in: int, width: int, n_out: int):
    rows = [n_in, width, width, n_out]
    offs, off = [], 0
    for l in range(3):
        ow = off
        off += rows[l + 1] * rows[l]
        ob = off
        off += rows[l + 1]
        offs.append((ow, ob))
    return rows, offs, off


def unpack(P: np.ndarray, n_in: int, width: int, n_out: int):
    rows, offs, _ = layout(n_in, width, n_out)
    Ws, bs = [], []
    for l, (ow, ob) in enumerate(offs):
        Ws.append(P[ow:ow + rows[l + 1] * rows[l]].reshape(rows[l + 1], rows[l], order="F"))
        bs.append(P[ob:ob + rows[l + 1]])
    return Ws, bs


def mlp_forward(P, X, n_in, width, n_out):
    """Layer outputs [H1, H2, Y] for X (n_in × B), FP32."""
    Ws, bs = unpack(np.asarray(P, np.float32), n_in, width, n_out)
    H, h = [], np.asarray(X, np.float32)
    for l in range(3):
        z = gemm_bf16("N", "N", Ws[l], h) + bs[l][:, None]
        h = np.maximum(z, np.float32(0)) if l < 2 else z
        H.append(h.astype(np.float32))
    return H


def mlp_gradient(P, X, Y, n_in, width, n_out):
    """(loss, gradient) of mean((net(X) − Y)²), products through gemm_bf16."""
    P = np.asarray(P, np.float32)
    X = np.asarray(X, np.float32)
    Ws, _ = unpack(P, n_in, width, n_out)
    H = mlp_forward(P, X, n_in, width, n_out)
    n = H[2].size
    r = (H[2] - np.asarray(Y, np.float32)).astype(np.float32)
    loss = float(np.sum(r.astype(np.float64) ** 2) / n)
    d = (np.float32(2.0 / n) * r).astype(np.float32)
    rows, offs, total = layout(n_in, width, n_out)
    G = np.zeros(total, np.float32)
    for l in (2, 1, 0):
        inp = H[l - 1] if l > 0 else X
        ow, ob = offs[l]
        G[ow:ow + rows[l + 1] * rows[l]] = gemm_bf16("N", "T", d, inp).ravel(order="F")
        G[ob:ob + rows[l + 1]] = d.astype(np.float64).sum(axis=1).astype(np.float32)
        if l > 0:
            d = gemm_bf16("T", "N", Ws[l], d)
            d = np.where(H[l - 1] > 0, d, np.float32(0)).astype(np.float32)
    return loss, G


def adamw_step(P, G, M1, M2, t, lr, wd, n_in, width, n_out, b1=0.9, b2=0.999, eps=1e-8):
    """One AdamW step in FP32; returns (P, M1, M2) after step number t (1-based)."""
    P = np.asarray(P, np.float32).copy()
    rows, offs, total = layout(n_in, width, n_out)
    bias = np.zeros(total, bool)
    for l, (_, ob) in enumerate(offs):
        bias[ob:ob + rows[l + 1]] = True
    f = np.float32
    P = np.where(bias, P, P - f(lr) * f(wd) * P).astype(np.float32)
    M1 = (f(b1) * M1 + (f(1) - f(b1)) * G).astype(np.float32)
    M2 = (f(b2) * M2 + (f(1) - f(b2)) * G * G).astype(np.float32)
    bc1, bc2 = f(1.0 - 0.9 ** t), f(1.0 - 0.999 ** t)
    P = (P - f(lr) * (M1 / bc1) / (np.sqrt(M2 / bc2) + f(eps))).astype(np.float32)
    return P, M1, M2


def features(As: np.ndarray) -> np.ndarray:
    """Network input: the symmetrised, normalised site tensor times the sign of
    its first largest-|·| entry (column-major flattening), FP32."""
    v = np.asarray(As, np.float64).ravel(order="F")
    k = int(np.argmax(np.abs(v)))
    return (np.sign(v[k]) if v[k] != 0 else 1.0) * v


def gauge_fix(C: np.ndarray, T: np.ndarray):
    """(λ, Tg): C = W·diag(λ)·Wᵀ with |λ| descending; Tg = Wᵀ·T·W on both χ
    legs with column signs s_0 = 1 and, for a ≥ 1, s_a making the largest
    |Tg[a,i,b]| over i and b < a positive (first in (b, i) order on ties)."""
    chi, d = T.shape[0], T.shape[1]
    lam, W = np.linalg.eigh(0.5 * (C + C.T))
    order = np.argsort(-np.abs(lam), kind="stable")
    lam, W = lam[order], W[:, order]
    Tg = np.einsum("xa,xiy,yb->aib", W, T, W)
    s = np.ones(chi)
    for a in range(1, chi):
        blk = Tg[a, :, :a]  # (i, b)
        mags = np.abs(blk).T.ravel()  # order k = i + d·b
        k = int(np.argmax(mags))
        i, b = k % d, k // d
        s[a] = -s[b] if (mags[k] > 0 and blk[i, b] < 0) else s[b]
    Tg = Tg * s[:, None, None] * s[None, None, :]
    return lam, Tg


def build_env(y: np.ndarray, chi: int, d: int):
    """Network output [λ̂ | T̂] → (C, T) = (diag(λ̂)/‖λ̂‖, sym(T̂)/‖sym(T̂)‖)."""
    y = np.asarray(y, np.float64)
    lam = y[:chi]
    Th = y[chi:].reshape(chi, d, chi, order="F")
    Ts = 0.5 * (Th + Th.transpose(2, 1, 0))
    C = np.diag(lam / np.linalg.norm(lam))
    return C, Ts / np.linalg.norm(Ts)
