"""Learned warm start: the BF16 tensor-core GEMM, the network's forward and
backward kernels, AdamW, the target gauge fix and the warm start itself,
against the NumPy oracle (oracle/mlp_oracle.py) and against cold starts."""
import numpy as np
import pytest

from oracle import mlp_oracle as mo

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def wl(tn):
    import importlib

    return importlib.import_module(tn.__name__ + ".learned")


def _rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - np.asarray(b, np.float64)) /
                 max(np.linalg.norm(np.asarray(b, np.float64)), 1e-300))


@pytest.mark.parametrize("ta,tb,M,N,K", [("N", "N", 512, 256, 162), ("N", "T", 1040, 96, 37),
                                         ("T", "N", 96, 37, 1040), ("N", "N", 11700, 64, 512),
                                         ("T", "N", 512, 64, 11700), ("N", "T", 200, 130, 2000)])
def test_gemm_bf16_matches_rounded_operands(tn, ta, tb, M, N, K):
    """BF16 tcgen05 GEMM = product of the BF16-rounded operands up to FP32
    accumulation rounding (relative 1e-5 of the result norm)."""
    import ctypes as C

    rng = np.random.default_rng(M + N + K)
    A = np.asfortranarray(rng.standard_normal((K, M) if ta == "T" else (M, K)).astype(np.float32))
    B = np.asfortranarray(rng.standard_normal((N, K) if tb == "T" else (K, N)).astype(np.float32))
    Cin = np.asfortranarray(rng.standard_normal((M, N)).astype(np.float32))
    out = Cin.copy(order="F")
    c = tn.ctx()
    c.check(c.lib.tnad_gemm_bf16(c.h, ta.encode(), tb.encode(), M, N, K, C.c_float(0.75), tn._lib.fptr(A),
                                 A.shape[0], tn._lib.fptr(B), B.shape[0], C.c_float(-0.5), tn._lib.fptr(out), M))
    ref = mo.gemm_bf16(ta, tb, A, B, 0.75, -0.5, Cin)
    assert _rel(out, ref) <= 1e-5
    # and it is a BF16 product: far from the FP32 product of the unrounded operands
    exact = 0.75 * (A.T if ta == "T" else A).astype(np.float64) @ (B.T if tb == "T" else B).astype(np.float64) \
        - 0.5 * Cin
    assert 1e-4 < _rel(out, exact) < 2e-2


@pytest.mark.parametrize("n_in,width,n_out,B", [(50, 96, 300, 37), (162, 512, 11700, 64)])
def test_mlp_forward_and_gradient_match_oracle(wl, n_in, width, n_out, B):
    rng = np.random.default_rng(n_in)
    net = wl.WarmStartNet.__new__(wl.WarmStartNet)
    # a bare network of the requested shape (not tied to a (D, s, χ))
    import ctypes as C

    net.c = wl.ctx()
    net.h = wl.L.VP()
    net.c.check(net.c.lib.tnad_mlp_create(net.c.h, n_in, width, n_out, 7, C.byref(net.h)))
    net.n_in, net.n_out, net.width = n_in, n_out, width
    net.n_params = int(net.c.lib.tnad_mlp_param_count(net.h))
    assert net.n_params == mo.layout(n_in, width, n_out)[2]
    P = net.get_params()
    # He-uniform init, zero biases
    Ws, bs = mo.unpack(P, n_in, width, n_out)
    for l, W in enumerate(Ws):
        bound = np.sqrt(6.0 / W.shape[1])
        assert np.abs(W).max() <= bound and np.abs(W).max() > 0.9 * bound
        assert abs(W.mean()) < 0.05 * bound
        assert not bs[l].any()
    # non-zero biases so that their gradients and the ReLU masks are exercised
    P = P.copy()
    for l in range(3):
        ob = mo.layout(n_in, width, n_out)[1][l][1]
        P[ob:ob + (width if l < 2 else n_out)] = 0.1 * rng.standard_normal(width if l < 2 else n_out)
    net.set_params(P)
    X = np.asfortranarray(rng.standard_normal((n_in, B)).astype(np.float32))
    Y = np.asfortranarray(rng.standard_normal((n_out, B)).astype(np.float32))
    Yg = net.forward(X)
    Yo = mo.mlp_forward(P, X, n_in, width, n_out)[2]
    assert _rel(Yg, Yo) <= 2e-3
    loss, G = net.gradient(X, Y)
    lo, Go = mo.mlp_gradient(P, X, Y, n_in, width, n_out)
    assert abs(loss - lo) <= 1e-4 * lo
    rows, offs, _ = mo.layout(n_in, width, n_out)
    for l, (ow, ob) in enumerate(offs):
        nw = rows[l + 1] * rows[l]
        assert _rel(G[ow:ow + nw], Go[ow:ow + nw]) <= 5e-3, f"dW{l + 1}"
        assert _rel(G[ob:ob + rows[l + 1]], Go[ob:ob + rows[l + 1]]) <= 5e-3, f"db{l + 1}"
    # the gradient is the gradient: directional derivative of the FP64 loss
    v = rng.standard_normal(P.size).astype(np.float32)
    v /= np.linalg.norm(v)

    def f64_loss(p):
        Ws_, bs_ = mo.unpack(p, n_in, width, n_out)
        h = X.astype(np.float64)
        for k in range(3):
            z = Ws_[k].astype(np.float64) @ h + bs_[k][:, None]
            h = np.maximum(z, 0) if k < 2 else z
        return np.mean((h - Y) ** 2)

    eps = 1e-2
    fd = (f64_loss(P + eps * v) - f64_loss(P - eps * v)) / (2 * eps)
    assert abs(fd - float(G.astype(np.float64) @ v)) <= 3e-2 * abs(fd) + 1e-6
    net.c.lib.tnad_mlp_free(net.h)
    net.h = wl.L.VP()


def test_adamw_step_matches_oracle(wl):
    n_in, width, n_out, N = 32, 64, 100, 20
    rng = np.random.default_rng(3)
    import ctypes as C

    c = wl.ctx()
    h = wl.L.VP()
    c.check(c.lib.tnad_mlp_create(c.h, n_in, width, n_out, 11, C.byref(h)))
    try:
        X = np.asfortranarray(rng.standard_normal((n_in, N)).astype(np.float32))
        Y = np.asfortranarray(rng.standard_normal((n_out, N)).astype(np.float32))
        n = mo.layout(n_in, width, n_out)[2]
        P0 = np.zeros(n, np.float32)
        c.check(c.lib.tnad_mlp_get_params(c.h, h, wl.fptr(P0)))
        idx = np.array([3, 17, 0, 9, 9, 12], np.int32)
        M1 = np.zeros(n, np.float32)
        M2 = np.zeros(n, np.float32)
        P = P0.copy()
        for t in (1, 2):
            loss = C.c_float()
            c.check(c.lib.tnad_mlp_train_step(c.h, h, wl.fptr(X), wl.fptr(Y), N,
                                              idx.ctypes.data_as(C.POINTER(C.c_int32)), idx.size, C.c_float(1e-3),
                                              C.c_float(0.1), C.byref(loss), 0))
            _, Go = mo.mlp_gradient(P, X[:, idx], Y[:, idx], n_in, width, n_out)
            P, M1, M2 = mo.adamw_step(P, Go, M1, M2, t, 1e-3, 0.1, n_in, width, n_out)
        Pg = np.zeros(n, np.float32)
        c.check(c.lib.tnad_mlp_get_params(c.h, h, wl.fptr(Pg)))
        # Adam's normalised step is ≈ lr per coordinate; a coordinate whose
        # gradient is within rounding of 0 may move differently, so compare the
        # update P − P0 in norm
        assert _rel(Pg - P0, P - P0) <= 2e-2
        assert np.max(np.abs(Pg - P)) <= 4.5e-3
    finally:
        c.lib.tnad_mlp_free(h)


def _sym_env(rng, chi, d):
    Q, _ = np.linalg.qr(rng.standard_normal((chi, chi)))
    lam = np.sort(rng.uniform(0.05, 1.0, chi))[::-1] * np.where(rng.random(chi) < 0.2, -1, 1)
    Cm = Q @ np.diag(lam) @ Q.T
    T = rng.standard_normal((chi, d, chi))
    T = 0.5 * (T + T.transpose(2, 1, 0))
    return np.asfortranarray(Cm), np.asfortranarray(T), lam


def test_gauge_fix_matches_oracle_and_is_gauge_invariant(wl):
    rng = np.random.default_rng(5)
    chi, d = 20, 4
    Cm, T, _ = _sym_env(rng, chi, d)
    lam, Tg = wl.gauge_fix(Cm, T)
    lo, To = mo.gauge_fix(Cm, T)
    assert np.max(np.abs(lam - lo)) <= 1e-12
    assert np.max(np.abs(Tg - To)) <= 1e-10
    assert np.allclose(Tg, Tg.transpose(2, 1, 0), atol=1e-12)
    # any orthogonal change of the environment's gauge gives the same target
    Q, _ = np.linalg.qr(rng.standard_normal((chi, chi)))
    C2 = np.asfortranarray(Q.T @ Cm @ Q)
    T2 = np.asfortranarray(np.einsum("xa,xiy,yb->aib", Q, T, Q))
    lam2, Tg2 = wl.gauge_fix(C2, T2)
    assert np.max(np.abs(lam2 - lam)) <= 1e-12
    assert np.max(np.abs(Tg2 - Tg)) <= 1e-10


def test_features_match_oracle(tn, wl, orc):
    import torch

    rng = np.random.default_rng(8)
    A = rng.uniform(-1, 1, (3, 3, 3, 3, 2))
    x = wl.features(A, 3, 2)
    As = orc.indexperm_symmetrize(torch.tensor(A)).numpy()
    assert np.max(np.abs(x - mo.features(As))) <= 1e-7
    # A and −A (same double layer, same environment) give the same input
    assert np.array_equal(wl.features(-A, 3, 2), x)


def test_learned_warm_start_saves_ctmrg_steps(tn, wl):
    """Trained on CTMRG environments of 384 random site tensors (D=2, χ=16),
    the network's start needs fewer plain FP64 CTMRG steps in total than :raw
    on 32 held-out tensors (5% at least); a network that predicts nothing is
    rejected before the first step and the cold start runs instead.

    Random tensors can have more than one CTMRG fixed point, and a start other
    than :raw can land on another one: the share of held-out tensors where both
    runs reach the same fixed point is bounded from below.  The gain comes
    mostly from the slow tensors; on quick ones both starts are close."""
    D, s, chi, tol, maxit = 2, 2, 16, 1e-9, 300
    h = tn.hamiltonian(tn.Heisenberg())
    rng = np.random.default_rng(2024)
    plain = lambda: tn.default_opts(prec=0, solver=0, adjoint=1)  # noqa: E731  reference CTMRG
    train = wl.make_samples([wl.random_site_tensor(D, s, rng) for _ in range(384)], h, chi, tol, maxit,
                            tn.mixed_opts(), threads=8)
    X, Y = wl.stack(train)
    net = wl.WarmStartNet(D, s, chi, width=512, seed=1)
    info = net.fit(X, Y, steps=2500, batch=64, lr=1e-3, weight_decay=1e-4)
    net.attach()
    held = [wl.random_site_tensor(D, s, rng) for _ in range(32)]
    r = wl.compare_starts(held, h, chi, tol, maxit, plain)
    same = r["dE"] <= 1e-7
    print(f"\nloss {info['loss_std']:.4f}  steps cold {r['cold_steps'].sum()} warm {r['warm_steps'].sum()}"
          f"  same fixed point {same.mean():.2f}  kept {np.mean(r['status'] == 1):.2f}")
    assert np.isfinite(info["loss_std"]) and info["loss_std"] < 0.3
    assert np.all(r["status"] != 0)
    assert same.mean() >= 0.75
    assert r["warm_steps"].sum() <= 0.95 * r["cold_steps"].sum()
    # a network that predicts nothing (all parameters zero) is rejected before
    # the first step and the cold start runs: same steps, same energy
    net.set_params(np.zeros(net.n_params, np.float32))
    r3 = wl.compare_starts(held[:3], h, chi, tol, maxit, plain)
    assert np.all(r3["status"] == -1)
    assert np.array_equal(r3["warm_steps"], r3["cold_steps"])
    assert np.all(r3["dE"] == 0.0)
