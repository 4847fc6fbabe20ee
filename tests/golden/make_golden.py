"""Generate the converged-energy fixtures (E*) of the benchmark workloads with the CPU oracle.

    python tests/golden/make_golden.py [--chi100]

Writes tests/golden/estar.json: for each workload the seeded input recipe, the
oracle energy after every CTMRG step (reference stop rule, tol = 1e-12) and the
converged energy E*.  The benchmark's |ΔE| ≤ 1e-8 target is measured against E*.
Inputs are NumPy default_rng(seed) draws, reproducible on any machine.
"""
from __future__ import annotations

import json
import sys
import time
from pathlib import Path

import numpy as np
import torch

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
from oracle import tnad_oracle as orc  # noqa: E402

OUT = Path(__file__).resolve().parent / "estar.json"

WORKLOADS = {
    "heisenberg_D2_chi20": dict(D=2, chi=20, recipe="uniform", seed=0, tol=1e-12, maxit=400),
    "heisenberg_D3_chi36": dict(D=3, chi=36, recipe="uniform", seed=0, tol=1e-12, maxit=400),
    "heisenberg_D4_chi64": dict(D=4, chi=64, recipe="normal_maxabs", seed=0, tol=1e-12, maxit=400),
    "heisenberg_D4_chi100": dict(D=4, chi=100, recipe="normal_maxabs", seed=0, tol=1e-12, maxit=400),
}


def make_input(w):
    if w["recipe"] == "uniform":
        return orc.ipeps_uniform(w["D"], 2, w["seed"])
    return orc.ipeps_normal_maxabs(w["D"], 2, w["seed"])


def trajectory(w, log=print):
    torch.set_num_threads(max(1, torch.get_num_threads()))
    h = torch.as_tensor(orc.hamiltonian_heisenberg())
    A = torch.as_tensor(make_input(w))
    with torch.no_grad():
        As = orc.indexperm_symmetrize(A)
        ap, a = orc.double_layer(As)
        C, T = orc.init_raw(a, w["chi"])
        n = w["chi"] * a.shape[0]
        old = torch.full((n,), float("inf"), dtype=torch.float64)
        energies, diffs = [], []
        t0 = time.time()
        for k in range(1, w["maxit"] + 2):
            C, T, vals = orc.ctmrgstep(a, C, T)
            e = float(orc.expectationvalue(h, ap, C, T))
            diff = float(torch.linalg.vector_norm(vals - old))
            energies.append(e)
            diffs.append(diff)
            log(f"  step {k:4d}  E={e:.15f}  diff={diff:.3e}  t={time.time() - t0:.1f}s")
            if k > w["maxit"] or diff <= w["tol"]:
                break
            old = vals
    return energies, diffs


def main():
    names = [k for k in WORKLOADS if "--chi100" in sys.argv or "chi100" not in k]
    data = json.loads(OUT.read_text()) if OUT.exists() else {}
    for name in names:
        w = WORKLOADS[name]
        print(name, w, flush=True)
        es, ds = trajectory(w, log=lambda s: print(s, flush=True))
        data[name] = dict(w, steps=len(es), E_star=es[-1], energies=es, diffs=ds,
                          generator="tests/golden/make_golden.py (CPU oracle, FP64)")
        OUT.write_text(json.dumps(data, indent=1))
    print("wrote", OUT)


if __name__ == "__main__":
    main()
