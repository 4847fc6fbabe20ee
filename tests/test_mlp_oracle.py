"""The warm-start network's CPU oracle (oracle/mlp_oracle.py) pinned against
PyTorch on the CPU: BF16 rounding against torch's float32 → bfloat16
conversion, the forward and gradient against torch autograd in FP64 on the
same BF16-rounded operands, AdamW against torch.optim.AdamW, and the gauge
fix against its defining properties."""
import numpy as np
import pytest

from oracle import mlp_oracle as mo

torch = pytest.importorskip("torch")


def test_bf16_rounding_matches_torch():
    rng = np.random.default_rng(0)
    x = np.concatenate([rng.standard_normal(10000).astype(np.float32) * 10.0 ** rng.integers(-8, 8, 10000),
                        np.array([1.0 + 2.0 ** -8, 1.0 + 3 * 2.0 ** -8, -1.0 - 2.0 ** -8, 0.0, -0.0], np.float32)])
    ref = torch.from_numpy(x).to(torch.bfloat16).to(torch.float32).numpy()
    assert np.array_equal(mo.bf16(x), ref)  # round to nearest, ties to even


def _torch_loss(P, X, Y, n_in, width, n_out):
    """FP64 torch restatement of the network on BF16-rounded weights and input
    (activations are not re-rounded, so this is the BF16 network up to the
    rounding of the intermediate operands)."""
    rows, offs, _ = mo.layout(n_in, width, n_out)
    p = torch.tensor(P.astype(np.float64), requires_grad=True)
    h = torch.tensor(mo.bf16(X).astype(np.float64))
    for l, (ow, ob) in enumerate(offs):
        W = p[ow:ow + rows[l + 1] * rows[l]].reshape(rows[l], rows[l + 1]).T  # column-major view
        b = p[ob:ob + rows[l + 1]]
        z = W @ h + b[:, None]
        h = torch.relu(z) if l < 2 else z
    loss = torch.mean((h - torch.tensor(Y.astype(np.float64))) ** 2)
    (g,) = torch.autograd.grad(loss, p)
    return float(loss.detach()), g.numpy()


def test_mlp_gradient_matches_torch_autograd():
    n_in, width, n_out, B = 20, 48, 30, 16
    rng = np.random.default_rng(1)
    total = mo.layout(n_in, width, n_out)[2]
    P = mo.bf16(rng.standard_normal(total).astype(np.float32) * 0.3)  # BF16-exact weights
    X = rng.standard_normal((n_in, B)).astype(np.float32)
    Y = rng.standard_normal((n_out, B)).astype(np.float32)
    loss, G = mo.mlp_gradient(P, X, Y, n_in, width, n_out)
    tl, tg = _torch_loss(P, X, Y, n_in, width, n_out)
    assert abs(loss - tl) <= 2e-2 * tl  # activations rounded to BF16 in the oracle only
    assert np.linalg.norm(G - tg) <= 3e-2 * np.linalg.norm(tg)


def test_adamw_matches_torch():
    n_in, width, n_out = 6, 8, 5
    rows, offs, total = mo.layout(n_in, width, n_out)
    rng = np.random.default_rng(2)
    P = rng.standard_normal(total).astype(np.float32)
    grads = [rng.standard_normal(total).astype(np.float32) for _ in range(3)]
    bias = np.zeros(total, bool)
    for l, (_, ob) in enumerate(offs):
        bias[ob:ob + rows[l + 1]] = True
    pw = torch.tensor(P[~bias], requires_grad=True)
    pb = torch.tensor(P[bias], requires_grad=True)
    opt = torch.optim.AdamW([{"params": [pw], "weight_decay": 0.1}, {"params": [pb], "weight_decay": 0.0}],
                            lr=1e-2, betas=(0.9, 0.999), eps=1e-8)
    Pm, M1, M2 = P.copy(), np.zeros(total, np.float32), np.zeros(total, np.float32)
    for t, g in enumerate(grads, start=1):
        pw.grad = torch.tensor(g[~bias])
        pb.grad = torch.tensor(g[bias])
        opt.step()
        Pm, M1, M2 = mo.adamw_step(Pm, g, M1, M2, t, 1e-2, 0.1, n_in, width, n_out)
    assert np.max(np.abs(Pm[~bias] - pw.detach().numpy())) <= 1e-6
    assert np.max(np.abs(Pm[bias] - pb.detach().numpy())) <= 1e-6


def test_gauge_fix_is_canonical():
    rng = np.random.default_rng(3)
    chi, d = 12, 4
    Q, _ = np.linalg.qr(rng.standard_normal((chi, chi)))
    lam = np.sort(rng.uniform(0.05, 1.0, chi))[::-1] * np.where(rng.random(chi) < 0.3, -1, 1)
    C = Q @ np.diag(lam) @ Q.T
    T = rng.standard_normal((chi, d, chi))
    T = 0.5 * (T + T.transpose(2, 1, 0))
    l1, T1 = mo.gauge_fix(C, T)
    assert np.allclose(np.abs(l1), np.sort(np.abs(lam))[::-1])
    # any orthogonal gauge change of the environment gives the same target
    R, _ = np.linalg.qr(rng.standard_normal((chi, chi)))
    l2, T2 = mo.gauge_fix(R.T @ C @ R, np.einsum("xa,xiy,yb->aib", R, T, R))
    assert np.allclose(l1, l2, atol=1e-12) and np.allclose(T1, T2, atol=1e-10)
    # the sign rule: for a ≥ 1 the largest |Tg[a, i, b]| over i and b < a is positive
    for a in range(1, chi):
        blk = T1[a, :, :a]
        i, b = np.unravel_index(np.argmax(np.abs(blk)), blk.shape)
        assert blk[i, b] > 0
    # and the inverse map of the network output gives a normalised symmetric environment
    Cb, Tb = mo.build_env(np.concatenate([l1, T1.ravel(order="F")]), chi, d)
    assert np.isclose(np.linalg.norm(Cb), 1.0) and np.isclose(np.linalg.norm(Tb), 1.0)
    assert np.allclose(Tb, Tb.transpose(2, 1, 0))
