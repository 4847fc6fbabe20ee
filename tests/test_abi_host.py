"""CPU-only checks of the C ABI library and the host mirror (no compute calls)."""
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent


def header_symbols():
    txt = (ROOT / "include" / "tnad.h").read_text()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(tnad_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol(tn):
    import ctypes

    lib = ctypes.CDLL(str(tn._lib.LIB_PATH))
    syms = header_symbols()
    assert len(syms) >= 20
    for s in syms:
        assert hasattr(lib, s), s
    # the ctypes binding declares exactly the header's functions
    assert sorted(tn._lib.exported_symbols()) == syms


def test_library_has_no_driver_link_dependency(tn):
    import subprocess

    out = subprocess.run(["ldd", str(tn._lib.LIB_PATH)], capture_output=True, text=True).stdout
    assert "libcuda.so" not in out


def test_model_tensor_host_matches_oracle(tn, orc):
    for b in (0.1, 0.5, 1.3):
        a, da = tn.model_tensor(tn.Ising(), b, with_derivative=True)
        assert np.allclose(a, orc.model_tensor_ising(b).numpy(), rtol=1e-14, atol=1e-15)
        fd = (tn.model_tensor(tn.Ising(), b + 1e-6) - tn.model_tensor(tn.Ising(), b - 1e-6)) / 2e-6
        assert np.allclose(da, fd, atol=1e-8)


def test_hamiltonians_match_oracle(tn, orc):
    assert np.array_equal(tn.hamiltonian(tn.Heisenberg()), orc.hamiltonian_heisenberg())
    assert np.array_equal(tn.hamiltonian(tn.Heisenberg(2.0, 2.0, 1.0)), orc.hamiltonian_heisenberg(2.0, 2.0, 1.0))
    assert np.array_equal(tn.hamiltonian(tn.TFIsing(1.0)), orc.hamiltonian_tfising(1.0))
    assert np.array_equal(tn.diaglocalhamiltonian([0.3, 0.1, -0.43]), orc.diaglocalhamiltonian([0.3, 0.1, -0.43]))


def test_square_ipeps_dimension_mismatch(tn):
    # test/ctmrg.jl:18-26
    sq = tn.SquareIPEPS(np.random.default_rng(0).standard_normal((3, 3, 3, 3, 2)))
    assert tn.getd(sq) == 3 and tn.gets(sq) == 2
    with pytest.raises(tn.DimensionMismatch):
        tn.SquareIPEPS(np.zeros((3, 3, 4, 3, 2)))
    assert isinstance(tn.SquareLattice(), tn.AbstractLattice)


def test_num_grad(tn):
    # src/autodiff.jl:44-63 doctests
    assert abs(tn.num_grad(lambda x: x * x, 3.0) - 6.0) < 1e-8
    g = tn.num_grad(lambda m: np.trace(m), np.random.default_rng(0).random((2, 2)))
    assert np.allclose(g, np.eye(2))


def test_no_cpu_fallback_without_gpu(tn):
    """Without a CUDA device, creating a context fails loudly (no silent CPU path)."""
    import torch

    if torch.cuda.is_available():
        pytest.skip("GPU present")
    with pytest.raises(tn.TnadError):
        tn._lib.Context(0)


def test_site_tensor_recipes_match_the_oracle_fixtures(tn, orc):
    """The package's seeded workload inputs are the oracle's (the E* fixtures were made from those)."""
    assert np.array_equal(tn.site_tensor("uniform", 3, 2, 0), orc.ipeps_uniform(3, 2, 0))
    assert np.array_equal(tn.site_tensor("normal_maxabs", 4, 2, 0), orc.ipeps_normal_maxabs(4, 2, 0))
