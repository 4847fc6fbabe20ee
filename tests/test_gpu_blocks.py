"""GPU building blocks (GEMM kernels, pairwise contraction engine) against NumPy."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHAPES = [(1, 1, 1), (12, 12, 12), (33, 17, 5), (64, 64, 64), (130, 70, 300), (4, 4, 5000), (1024, 64, 64),
          (256, 1024, 96),
          # matrix-vector products (the Gram–Schmidt steps of GMRES) and small split-K products
          (4000, 1, 31), (31, 1, 70000), (33, 1, 5000), (1, 1, 3000), (64, 64, 48), (96, 96, 40)]


@pytest.mark.parametrize("M,N,K", SHAPES)
@pytest.mark.parametrize("ta,tb", [("N", "N"), ("T", "N"), ("N", "T"), ("T", "T")])
def test_gemm_f64(tn, M, N, K, ta, tb):
    rng = np.random.default_rng(M + 7 * N + 13 * K)
    A = rng.standard_normal((K, M) if ta == "T" else (M, K))
    B = rng.standard_normal((N, K) if tb == "T" else (K, N))
    C0 = rng.standard_normal((M, N))
    got = tn.gemm(A, B, ta, tb, alpha=0.7, beta=-1.3, Cin=C0)
    ref = 0.7 * ((A.T if ta == "T" else A) @ (B.T if tb == "T" else B)) - 1.3 * C0
    assert np.max(np.abs(got - ref)) <= 1e-13 * max(1.0, np.abs(ref).max()) * np.sqrt(K)


SPECS = ["ad,iba->ibd", "ibd,dcl->ibcl", "ibcl,jkcb->ijlk", "abcd,abi->icd", "icd,cdj->ij", "aed,abi->edbi",
         "edbi,bjce->dijc", "dijc,dck->ijk", "ijk,dck->dijc", "dijc,bjce->edbi", "abcij,abckl->ijkl",
         "npu,por->nuor", "nuor,doln->urdl", "abc,abc->"]


@pytest.mark.parametrize("spec", SPECS)
def test_contract_engine(tn, spec):
    rng = np.random.default_rng(len(spec))
    lhs, lc = spec.split("->")
    la, lb = lhs.split(",")
    ext = {ch: 2 + (ord(ch) % 4) for ch in set(la + lb)}
    A = rng.standard_normal(tuple(ext[ch] for ch in la))
    B = rng.standard_normal(tuple(ext[ch] for ch in lb))
    got = tn.contract(spec, A, B)
    ref = np.einsum(spec, A, B)
    assert np.allclose(got, ref, rtol=1e-13, atol=1e-13)


@pytest.mark.parametrize("M,N,K", [(128, 64, 32), (256, 128, 96), (1024, 64, 64), (1024, 1024, 64), (300, 200, 77),
                                   (4096, 256, 256), (1024, 1024, 1024)])
@pytest.mark.parametrize("ta,tb", [("N", "N"), ("T", "N"), ("N", "T"), ("T", "T")])
def test_gemm_tf32x3_tcgen05(tn, M, N, K, ta, tb):
    """3xTF32 on tcgen05: x = x_hi + x_lo with 11-bit TF32 pieces represents x to
    2^-22; the tensor cores' FP32 accumulation adds error growing with the K
    chunk (128 here, chunks summed in FP64).  Tolerance 2e-5 of the operand
    scale (|Σ a·b| ~ √K for N(0,1) entries)."""
    rng = np.random.default_rng(M + 3 * N + 5 * K)
    A = rng.standard_normal((K, M) if ta == "T" else (M, K))
    B = rng.standard_normal((N, K) if tb == "T" else (K, N))
    C0 = rng.standard_normal((M, N))
    got = tn.gemm(A, B, ta, tb, alpha=0.5, beta=0.25, Cin=C0, prec=1)
    ref = 0.5 * ((A.T if ta == "T" else A) @ (B.T if tb == "T" else B)) + 0.25 * C0
    scale = 0.5 * np.sqrt(K)  # |Σ a·b| for N(0,1) operands
    assert np.max(np.abs(got - ref)) <= 2e-5 * scale


@pytest.mark.parametrize("M,N,K", [(128, 64, 256), (300, 200, 77), (1024, 64, 1024), (64, 1024, 4096),
                                   (1024, 1024, 256), (256, 96, 40000), (200, 130, 1000)])
@pytest.mark.parametrize("ta,tb", [("N", "N"), ("T", "N"), ("N", "T"), ("T", "T")])
def test_gemm_fp64_tensor_core_emulation(tn, M, N, K, ta, tb):
    """FP64-accurate products from six BF16 slices per operand on tcgen05.  The
    error bound of the scheme is about √K·2^-48·max_k|A_ik|·max_k|B_kj|; for
    these N(0,1)-shaped rows that is below 2^-44·(|A|·|B|)_ij, the bound asserted
    per entry (an FP64 DFMA product is at ~√K·2^-53 of the same quantity; the
    FP64 BLAS product used as reference is at that level too).  Rows and
    columns are scaled over twelve orders of magnitude (per-row/column scaling
    of the slices), one row is zero, and K = 40000 exercises the split over CTAs
    beyond one CTA's 32768 K values."""
    rng = np.random.default_rng(M + 3 * N + 5 * K + (ta == "T") + 2 * (tb == "T"))
    A = rng.standard_normal((M, K)) * np.exp(rng.uniform(-14, 14, (M, 1)))
    B = rng.standard_normal((K, N)) * np.exp(rng.uniform(-14, 14, (1, N)))
    zr = min(3, M - 1)
    A[zr, :] = 0.0
    Aop, Bop = (np.asfortranarray(A.T) if ta == "T" else A), (np.asfortranarray(B.T) if tb == "T" else B)
    C0 = rng.standard_normal((M, N))
    got = tn.gemm(Aop, Bop, ta, tb, alpha=0.75, beta=-0.5, Cin=C0, prec=3)
    ref = 0.75 * (A @ B) - 0.5 * C0
    bound = 2.0 ** -44 * 0.75 * (np.abs(A) @ np.abs(B)) + 2.0 ** -50 * np.abs(C0)
    ratio = np.abs(got - ref) / bound
    assert float(ratio.max()) <= 1.0, float(ratio.max())
    assert np.all(got[zr, :] == -0.5 * C0[zr, :])


def test_gemm_fp64_tensor_core_emulation_matches_dfma(tn):
    """Against the DFMA GEMM on an N(0,1) product: both FP64-accurate."""
    rng = np.random.default_rng(11)
    A, B = rng.standard_normal((1024, 512)), rng.standard_normal((512, 96))
    g_tc = tn.gemm(A, B, prec=3)
    g_64 = tn.gemm(A, B, prec=0)
    assert np.max(np.abs(g_tc - g_64)) <= 1e-13 * np.sqrt(512)


def test_gemm_fp64_tensor_core_emulation_propagates_nonfinite(tn):
    rng = np.random.default_rng(12)
    A, B = rng.standard_normal((256, 300)), rng.standard_normal((300, 128))
    A[5, 7] = np.nan
    B[9, 70] = np.inf
    got = tn.gemm(A, B, prec=3)
    assert np.all(np.isnan(got[5, :])) and np.all(np.isnan(got[:, 70]))
    ok = np.ones(got.shape, bool)
    ok[5, :] = False
    ok[:, 70] = False
    Af, Bf = np.where(np.isfinite(A), A, 0.0), np.where(np.isfinite(B), B, 0.0)
    ref, den = Af @ Bf, np.abs(Af) @ np.abs(Bf)
    assert np.max(np.abs(got[ok] - ref[ok]) / den[ok]) <= 2.0 ** -44
