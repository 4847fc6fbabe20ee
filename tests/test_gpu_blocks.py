"""GPU building blocks (GEMM kernels, pairwise contraction engine) against NumPy."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHAPES = [(1, 1, 1), (12, 12, 12), (33, 17, 5), (64, 64, 64), (130, 70, 300), (4, 4, 5000), (1024, 64, 64),
          (256, 1024, 96)]


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
