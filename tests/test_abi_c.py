"""The C ABI from C: include/tnad.h compiles as C99, libtnad.so links, and the
entry points that need no GPU behave (host arithmetic of model_tensor(::Ising, β),
src/exampletensors.jl:30-35; the default options; a context on a machine without
a CUDA device fails with an error code instead of aborting)."""
import shutil
import subprocess

import numpy as np
import pytest

C_SRC = r"""
#include <stdio.h>
#include "tnad.h"

int main(void) {
  double a[16], da[16];
  tnad_opts o;
  tnad_ctx* ctx = 0;
  int rc;
  printf("version %d\n", tnad_version());
  tnad_opts_default(&o);
  printf("opts %d %d %d %d %.3g %.3g\n", o.prec, o.solver, o.adjoint, o.fp_maxit, o.fp_tol, o.ladder_tol);
  rc = tnad_model_tensor_ising(0.5, a, da);
  printf("ising %d", rc);
  for (int i = 0; i < 16; ++i) printf(" %.17g", a[i]);
  printf("\n");
  rc = tnad_ctx_create(&ctx, 0);
  printf("ctx %d %d\n", rc, ctx == 0);
  if (rc == TNAD_OK) tnad_ctx_destroy(ctx);
  return 0;
}
"""


def test_header_compiles_as_c_and_library_links(tn, orc, tmp_path):
    if shutil.which("gcc") is None:
        pytest.skip("no C compiler")
    lib = tn._lib.LIB_PATH
    root = lib.parent.parent
    src = tmp_path / "abi.c"
    src.write_text(C_SRC)
    exe = tmp_path / "abi"
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", f"-I{root / 'include'}", str(src), "-o", str(exe),
                        f"-L{lib.parent}", "-ltnad", f"-Wl,-rpath,{lib.parent}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    out = dict(line.split(" ", 1) for line in r.stdout.strip().splitlines())
    assert int(out["version"]) > 0
    prec, solver, adjoint, fp_maxit, fp_tol, ladder_tol = out["opts"].split()
    assert (int(prec), int(solver), int(adjoint)) == (0, 0, 0)  # FP64, full SVD, unrolled: the reference
    vals = out["ising"].split()
    assert int(vals[0]) == 0
    a = np.array([float(v) for v in vals[1:]]).reshape((2, 2, 2, 2), order="F")
    assert np.allclose(a, orc.model_tensor_ising(0.5).numpy(), rtol=1e-14, atol=1e-15)
    rc, null = out["ctx"].split()
    import torch

    if not torch.cuda.is_available():
        assert int(rc) < 0 and int(null) == 1  # a negative TNAD_ERR_*, no context, no abort
