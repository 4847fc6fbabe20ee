"""bench.py's reference arm on the CPU: one JSON line with the contract's keys
(the GPU arm's line is checked by running bench.py on the GPU)."""
import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def test_reference_arm_prints_one_contract_line():
    """Full oracle solves of the small D=2, chi=20 workload (the headline D=4
    workload runs the same code, only longer)."""
    sys.path.insert(0, str(ROOT))
    import bench

    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "2", "--warmup", "1",
                        "--workload", "heisenberg_D2_chi20"],
                       capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.strip().startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["higher_is_better"] is False and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1 and d["cpu_baseline"]["sample"]
    assert d["e2e"]["value"] == d["value"] and d["e2e"]["h2d_bytes_per_step"] == 0
    assert d["config"]["workload"] == "heisenberg_D2_chi20"
    # the GPU arm prints the same metric string for the same workload
    assert d["metric"] == bench.metric_for(bench.ESTAR["heisenberg_D2_chi20"])
    # every timed step is a full solve that reaches the target
    assert d["delta_E"] <= bench.TARGET and d["steps"] == 2 and d["warmup"] == 1


def test_gradient_check_compares_both_gradients_with_a_central_difference():
    """bench.gradient_check on a quadratic energy (exact central difference),
    with a stand-in for the package: the mixed gradient exact, the plain one off."""
    import numpy as np

    sys.path.insert(0, str(ROOT))
    import bench

    Q = np.diag(np.arange(1.0, 9.0))

    class FakeTn:
        @staticmethod
        def default_opts():
            return None

        @staticmethod
        def SquareIPEPS(A):
            return A

        @staticmethod
        def energy(h, A, chi, tol, maxit, opts):
            x = np.asarray(A).ravel()
            return 0.5 * float(x @ Q @ x)

    class FakeSol:
        A = np.linspace(0.1, 0.8, 8).reshape(2, 2, 2)
        h, chi, maxit = None, 4, 10

    g_exact = (Q @ FakeSol.A.ravel()).reshape(2, 2, 2)
    r = bench.gradient_check(FakeTn, FakeSol, g_exact, 1.01 * g_exact)
    assert r["mixed_rel_err"] < 1e-9
    assert abs(r["plain_unrolled_rel_err"] - 0.01) < 1e-8
    assert abs(r["mixed_vs_plain_rel_l2"] - 0.01 / 1.01) < 1e-12
