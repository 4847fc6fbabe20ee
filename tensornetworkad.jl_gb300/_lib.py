"""ctypes binding of libtnad (include/tnad.h).

This is the binding a Python caller of the C ABI uses; the Julia shim binds the
same symbols with ``ccall``.  Arrays cross the boundary as Fortran-ordered
float64 NumPy arrays, i.e. in Julia's column-major layout.  There is no CPU
fallback: if the shared library or a CUDA device is missing, calls raise.
"""
from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "libtnad.so"

TNAD_OK = 0
ERRORS = {
    -1: "TNAD_ERR_ARG", -2: "TNAD_ERR_SHAPE", -3: "TNAD_ERR_CUDA", -4: "TNAD_ERR_NOT_CONVERGED",
    -5: "TNAD_ERR_NONFINITE", -6: "TNAD_ERR_NOMEM", -7: "TNAD_ERR_STATE", -8: "TNAD_ERR_TIMEOUT",
}
PREC_FP64, PREC_TF32X3, PREC_LADDER, PREC_FP64_TC = 0, 1, 2, 3
WARM_NONE, WARM_GIVEN, WARM_LEARNED = 0, 1, 2
SOLVER_FULL_SVD, SOLVER_SUBSPACE = 0, 1
ADJOINT_UNROLLED, ADJOINT_FIXEDPOINT = 0, 1


class TnadError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class DimensionMismatch(ValueError):
    """Julia's DimensionMismatch (raised by SquareIPEPS, src/ipeps.jl:17-22)."""


class Opts(C.Structure):
    _fields_ = [
        ("prec", C.c_int32), ("solver", C.c_int32), ("adjoint", C.c_int32), ("device_ptrs", C.c_int32),
        ("warm_start", C.c_int32), ("stop_rule", C.c_int32), ("fp_maxit", C.c_int32), ("fp64_tc", C.c_int32),
        ("fp_tol", C.c_double), ("ladder_tol", C.c_double), ("tape_budget", C.c_int64),
    ]


DP = C.POINTER(C.c_double)
FP = C.POINTER(C.c_float)
VP = C.c_void_p
IP = C.POINTER(C.c_int)

# name: (restype, argtypes) — exactly the declarations of include/tnad.h
SIGNATURES = {
    "tnad_ctx_create": (C.c_int, [C.POINTER(VP), C.c_int]),
    "tnad_ctx_destroy": (None, [VP]),
    "tnad_last_error": (C.c_char_p, [VP]),
    "tnad_version": (C.c_int, []),
    "tnad_opts_default": (None, [C.POINTER(Opts)]),
    "tnad_ctx_workspace_bytes": (C.c_int64, [VP]),
    "tnad_ctx_kernel_launches": (C.c_int64, [VP]),
    "tnad_ctx_kernel_timer": (C.c_int, [VP, C.c_char_p]),
    "tnad_ctx_kernel_timer_read": (C.c_int, [VP, C.POINTER(C.c_int64), DP, DP]),
    "tnad_ctx_stream": (VP, [VP]),
    "tnad_tape_free": (None, [VP]),
    "tnad_gemm": (C.c_int, [VP, C.c_int, C.c_char, C.c_char, C.c_int64, C.c_int64, C.c_int64, C.c_double, DP,
                            C.c_int64, DP, C.c_int64, C.c_double, DP, C.c_int64]),
    "tnad_contract": (C.c_int, [VP, C.c_int, DP, C.c_char_p, C.POINTER(C.c_int64), DP, C.c_char_p,
                                C.POINTER(C.c_int64), DP, C.c_char_p]),
    "tnad_model_tensor_ising": (C.c_int, [C.c_double, DP, DP]),
    "tnad_trg": (C.c_int, [VP, DP, C.c_int, C.c_int, C.c_int, C.c_double, DP, C.POINTER(VP)]),
    "tnad_trg_backward": (C.c_int, [VP, VP, C.c_double, DP]),
    "tnad_trg_svd": (C.c_int, [VP, DP, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, DP, DP, IP]),
    "tnad_svd": (C.c_int, [VP, DP, C.c_int, C.c_int, DP, DP, DP]),
    "tnad_svd_noalloc": (C.c_int, [DP, C.c_int, C.c_int, DP, DP, DP, VP]),
    "tnad_svd_sym": (C.c_int, [VP, C.c_int, DP, C.c_int, DP, DP, DP]),
    "tnad_ctx_solver_stats": (C.c_int, [VP, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    "tnad_svd_back": (C.c_int, [VP, DP, DP, DP, C.c_int, C.c_int, DP, DP, DP, C.c_double, DP]),
    "tnad_svd_z": (C.c_int, [VP, DP, C.c_int, C.c_int, DP, DP, DP]),
    "tnad_svd_back_z": (C.c_int, [VP, DP, DP, DP, C.c_int, C.c_int, DP, DP, DP, C.c_double, DP]),
    "tnad_ctmrgstep": (C.c_int, [VP, DP, C.c_int, C.c_int, DP, DP, DP, DP, DP]),
    "tnad_ctmrgstep_backward": (C.c_int, [VP, DP, C.c_int, C.c_int, DP, DP, DP, DP, DP, DP, DP]),
    "tnad_init_raw": (C.c_int, [VP, DP, C.c_int, C.c_int, DP, DP]),
    "tnad_ctmrg": (C.c_int, [VP, DP, C.c_int, C.c_int, DP, DP, C.c_double, C.c_int, C.POINTER(Opts), DP, DP, IP,
                             C.POINTER(VP)]),
    "tnad_ctmrg_backward": (C.c_int, [VP, VP, DP, DP, DP]),
    "tnad_symmetrize": (C.c_int, [VP, DP, C.c_int, C.c_int, DP]),
    "tnad_expectationvalue": (C.c_int, [VP, DP, DP, C.c_int, C.c_int, C.c_int, DP, DP, DP]),
    "tnad_energy": (C.c_int, [VP, DP, DP, C.c_int, C.c_int, C.c_int, C.c_double, C.c_int, C.POINTER(Opts), DP, DP,
                              DP, IP, DP, DP, C.POINTER(VP)]),
    "tnad_energy_backward": (C.c_int, [VP, VP, C.c_double, DP]),
    "tnad_optimiseipeps": (C.c_int, [VP, DP, DP, C.c_int, C.c_int, C.c_int, C.c_double, C.c_int, C.POINTER(Opts),
                                     C.c_int, C.c_int, C.c_double, C.c_double, DP, IP, IP]),
    "tnad_energy_stats": (C.c_int, [VP, IP, IP, IP, IP, DP, DP]),
    "tnad_energy_fixed_point_residual": (C.c_int, [VP, DP]),
    "tnad_mlp_create": (C.c_int, [VP, C.c_int, C.c_int, C.c_int, C.c_uint64, C.POINTER(VP)]),
    "tnad_gemm_bf16": (C.c_int, [VP, C.c_char, C.c_char, C.c_int64, C.c_int64, C.c_int64, C.c_float, FP, C.c_int64,
                                 FP, C.c_int64, C.c_float, FP, C.c_int64]),
    "tnad_mlp_free": (None, [VP]),
    "tnad_mlp_param_count": (C.c_int64, [VP]),
    "tnad_mlp_get_params": (C.c_int, [VP, VP, FP]),
    "tnad_mlp_set_params": (C.c_int, [VP, VP, FP]),
    "tnad_mlp_forward": (C.c_int, [VP, VP, FP, C.c_int, FP, C.c_int]),
    "tnad_mlp_gradient": (C.c_int, [VP, VP, FP, FP, C.c_int, FP, FP, C.c_int]),
    "tnad_mlp_set_data": (C.c_int, [VP, VP, FP, FP, C.c_int64]),
    "tnad_mlp_train_step": (C.c_int, [VP, VP, FP, FP, C.c_int64, C.POINTER(C.c_int32), C.c_int, C.c_float,
                                      C.c_float, FP, C.c_int]),
    "tnad_env_gauge_fix": (C.c_int, [VP, DP, DP, C.c_int, C.c_int, DP, DP]),
    "tnad_ctx_set_warm_start": (C.c_int, [VP, VP, C.c_int, C.c_int, C.c_int]),
    "tnad_warm_start_features": (C.c_int, [VP, DP, C.c_int, C.c_int, FP]),
    "tnad_warm_start_env": (C.c_int, [VP, DP, C.c_int, C.c_int, C.c_int, DP, DP]),
    "tnad_ctx_warm_start_status": (C.c_int, [VP]),
}

_lib = None
_lock = threading.Lock()


def load() -> C.CDLL:
    """Load libtnad.so (raises if it has not been built)."""
    global _lib
    with _lock:
        if _lib is None:
            if not LIB_PATH.exists():
                raise ImportError(f"libtnad.so not built at {LIB_PATH}; run build.py or __graft_entry__.build()")
            lib = C.CDLL(str(LIB_PATH))
            for name, (res, args) in SIGNATURES.items():
                f = getattr(lib, name)
                f.restype = res
                f.argtypes = args
            _lib = lib
    return _lib


def exported_symbols() -> list[str]:
    return list(SIGNATURES)


def default_opts(**kw) -> Opts:
    o = Opts()
    load().tnad_opts_default(C.byref(o))
    for k, v in kw.items():
        setattr(o, k, v)
    return o


class Context:
    """One libtnad context (one CUDA stream + device workspace) per host thread."""

    def __init__(self, device: int = 0):
        self.lib = load()
        self.h = VP()
        rc = self.lib.tnad_ctx_create(C.byref(self.h), device)
        if rc != TNAD_OK:
            raise TnadError(rc, "tnad_ctx_create failed (no CUDA device?)")

    def check(self, rc: int):
        if rc != TNAD_OK:
            raise TnadError(rc, self.lib.tnad_last_error(self.h).decode())

    @property
    def launches(self) -> int:
        return int(self.lib.tnad_ctx_kernel_launches(self.h))

    def close(self):
        if self.h:
            self.lib.tnad_ctx_destroy(self.h)
            self.h = VP()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_tls = threading.local()


def ctx(device: int = 0) -> Context:
    c = getattr(_tls, "ctx", None)
    if c is None:
        c = Context(device)
        _tls.ctx = c
    return c


class Tape:
    """Owns a tnad_tape (freed on garbage collection)."""

    def __init__(self, c: Context, h: VP, kind: str):
        self.c, self.h, self.kind = c, h, kind

    def __del__(self):
        try:
            if self.h:
                self.c.lib.tnad_tape_free(self.h)
        except Exception:
            pass


def farr(x, shape=None) -> np.ndarray:
    a = np.asfortranarray(np.asarray(x, dtype=np.float64))
    if shape is not None and a.shape != tuple(shape):
        raise DimensionMismatch(f"expected shape {tuple(shape)}, got {a.shape}")
    return a


def ptr(a) -> DP:
    if a is None:
        return C.cast(None, DP)
    if isinstance(a, int):  # raw device address
        return C.cast(C.c_void_p(a), DP)
    assert a.flags["F_CONTIGUOUS"] and a.dtype == np.float64
    return a.ctypes.data_as(DP)


def fptr(a) -> FP:
    """float32 column-major host array, raw device address (int) or None."""
    if a is None:
        return C.cast(None, FP)
    if isinstance(a, int):
        return C.cast(C.c_void_p(a), FP)
    assert a.flags["F_CONTIGUOUS"] and a.dtype == np.float32
    return a.ctypes.data_as(FP)


def zarr(x) -> np.ndarray:
    """complex128 column-major array (interleaved re/im, Julia's ComplexF64 layout)."""
    return np.asfortranarray(np.asarray(x, dtype=np.complex128))


def zptr(a) -> DP:
    if a is None:
        return C.cast(None, DP)
    assert a.flags["F_CONTIGUOUS"] and a.dtype == np.complex128
    return a.ctypes.data_as(DP)


def fzeros(shape) -> np.ndarray:
    return np.zeros(shape, dtype=np.float64, order="F")
