"""Benchmark: CTMRG energy + gradient time to |ΔE| ≤ 1e-8 on one GB300.

One step = one full solve of the workload (symmetrise → double layer → CTMRG
to the stop rule → energy → gradient dE/dA) through libtnad.  The energy of
every timed solve is checked against the converged FP64 oracle energy E* of
the same seeded input (tests/golden/estar.json).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                    [--workload heisenberg_D4_chi64] [--mode mixed|plain]

--impl reference times the CPU restatement of the reference (the oracle:
torch-CPU FP64, all host threads), one full solve of the same workload per step.
With N > 1 every rank solves its own replica (the CTMRG fixed point is
sequential; there is no collective on the data path).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

ESTAR = json.loads((ROOT / "tests" / "golden" / "estar.json").read_text())
TARGET = 1e-8


def metric_for(w) -> str:
    """The metric string both arms print for workload w (identical by construction)."""
    return (f"CTMRG energy+gradient time to |dE|<=1e-8 vs the FP64 oracle "
            f"(Heisenberg iPEPS D={w['D']}, chi={w['chi']})")


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--workload", default="heisenberg_D4_chi64")
    p.add_argument("--mode", default="learned", choices=["plain", "mixed", "learned"],
                   help="learned (default): the mixed path started from the learned warm start, whose network "
                        "is trained before the warm-up on environments of other seeds of the workload's recipe")
    p.add_argument("--learned-train", dest="learned_train", type=int, default=400,
                   help="--mode learned: training tensors (seeds 1000..)")
    p.add_argument("--no-plain", dest="no_plain", action="store_true", help="skip the plain FP64 comparison solve")
    p.add_argument("--no-cpu-baseline", dest="no_cpu_baseline", action="store_true")
    # --workload learned_D3_chi36: learned warm start against the cold start
    p.add_argument("--n-train", dest="n_train", type=int, default=4000, help="random site tensors for training")
    p.add_argument("--n-traj", dest="n_traj", type=int, default=16, help="Heisenberg L-BFGS trajectories")
    p.add_argument("--traj-evals", dest="traj_evals", type=int, default=40, help="tensors kept per trajectory")
    p.add_argument("--n-held", dest="n_held", type=int, default=500, help="held-out tensors")
    p.add_argument("--train-steps", dest="train_steps", type=int, default=6000)
    p.add_argument("--threads", type=int, default=8, help="concurrent CTMRG runs while generating targets")
    p.add_argument("--lbfgs-steps", dest="lbfgs_steps", type=int, default=20, help="optimise_* workloads")
    p.add_argument("--chi", type=int, default=0, help="optimise_* workloads: bond dimension (default 64)")
    p.add_argument("--only", default=None, help="optimise_* workloads: run one mode only")
    p.add_argument("--profile", default=None, choices=["solve", "mlp", "gemm_fp64tc"],
                   help="run one untimed solve of the workload (solve), 20 training steps of the D=3, chi=36 "
                        "warm-start network (mlp), or two FP64 tensor-core products of the adjoint's shapes "
                        "(1024^3 and 1024x96x1024, twice: gemm_fp64tc) and exit: the commands profiled by ncu")
    return p.parse_args()


def workload_input(w):
    import __graft_entry__ as ge

    return ge.load_package().site_tensor(w["recipe"], w["D"], 2, w["seed"])


def plain_tol(w):
    """Reference stop-rule tolerance at which the oracle trajectory is within TARGET of E*."""
    es, ds = w["energies"], w["diffs"]
    for e, d in zip(es, ds):
        if abs(e - w["E_star"]) <= TARGET / 4 and np.isfinite(d):
            return float(d) * 0.999
    return w["tol"]


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, dev: int):
        self.dev, self.proc, self.lines = dev, None, []

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.dev), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                mx = max(mx, float(f[1]))
            except ValueError:
                continue
            for nm, v in zip(names, f[4:8]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx or None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_init(n, backend="nccl"):
    """One process per GPU (torchrun env); every rank solves its own replica."""
    if n <= 1:
        return None, 0, 1
    import torch.distributed as dist

    dist.init_process_group(backend)
    return dist, dist.get_rank(), dist.get_world_size()


def max_over_ranks(dist, x):
    if dist is None:
        return x
    import torch

    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(dist):
    if dist is not None:
        dist.barrier()


# ---------------------------------------------------------------------------
PEAKS_PATH = ROOT / "MEASURED_PEAKS.json"
FP64_NOMINAL_TFLOPS = 1.25  # GB300 FP64 (no measured FP64 figure exists for this machine)
# dram__bytes_read.sum + dram__bytes_write.sum per launch of the FP64 Jacobi round
# at n = 1024 (16 805 888 + 0 bytes; ncu flushes the caches between its passes),
# from one ncu capture of that kernel on this workload
JACOBI_ROUND_TRAFFIC_BYTES = 16805888
# GB300 FP32 (CUDA-core FMA) rate: 152 SMs × 128 FMA/clock × 2 flops × 2.07 GHz
FP32_NOMINAL_TFLOPS = 80.5
# dram__bytes_read.sum + dram__bytes_write.sum per launch of the FP64 tensor-core
# GEMM (k_gemm_oz), mean over the first 300 of its launches in one cold D=4,
# chi=64 solve (one ncu capture of that kernel on this workload)
OZ_TRAFFIC_BYTES = 3321780


def peaks():
    try:
        return json.loads(PEAKS_PATH.read_text()), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


class Solver:
    """One workload solved through libtnad: device-resident (kernel-side number)
    or through the public API with host arrays (end to end)."""

    def __init__(self, tn, w, mode):
        import ctypes as C
        import torch

        self.C, self.tn, self.w, self.mode = C, tn, w, mode
        self.c = tn.ctx(int(os.environ.get("LOCAL_RANK", "0")))
        self.A = workload_input(w)
        self.h = tn.hamiltonian(tn.Heisenberg())
        self.chi, self.D, self.s = w["chi"], w["D"], 2
        if mode == "plain":
            self.opts, self.tol, self.maxit = tn.default_opts(), plain_tol(w), 400
        else:
            self.opts, self.tol, self.maxit = tn.mixed_opts(), 3e-8, 400
            if mode == "learned":
                self.opts.warm_start = tn._lib.WARM_LEARNED
        self.A_d = torch.tensor(np.asarray(self.A).ravel(order="F"), dtype=torch.float64, device="cuda")
        self.h_d = torch.tensor(np.asarray(self.h).ravel(order="F"), dtype=torch.float64, device="cuda")
        self.g_d = torch.zeros_like(self.A_d)
        self.opts_d = tn.default_opts(**{k: getattr(self.opts, k) for k, _ in self.opts._fields_})
        self.opts_d.device_ptrs = 1

    def device(self):
        C, tn, c = self.C, self.tn, self.c
        E, steps, tp = C.c_double(), C.c_int(), tn._lib.VP()
        c.check(c.lib.tnad_energy(c.h, tn.ptr(self.h_d.data_ptr()), tn.ptr(self.A_d.data_ptr()), self.D, self.s,
                                  self.chi, self.tol, self.maxit, C.byref(self.opts_d), tn.ptr(None), tn.ptr(None),
                                  C.byref(E), C.byref(steps), tn.ptr(None), tn.ptr(None), C.byref(tp)))
        c.check(c.lib.tnad_energy_backward(c.h, tp, 1.0, tn.ptr(self.g_d.data_ptr())))
        st = self.tn.tape_stats(self.tn._lib.Tape(c, tp, "energy"))  # frees the tape
        st["warm_status"] = int(c.lib.tnad_ctx_warm_start_status(c.h))
        return E.value, st

    def host(self):
        st = {}
        E, g = self.tn.energy_and_gradient(self.h, self.tn.SquareIPEPS(self.A), self.chi, self.tol, self.maxit,
                                           self.opts, stats=st)
        return E, g, st


def gradient_check(tn, sol, g_mixed, g_plain, step=1e-4, tol=1e-11):
    """Directional derivative of the energy along a seeded unit direction v: the
    mixed gradient and the plain FP64 path's (the reference's unrolled reverse)
    against a central difference of the plain FP64 energy (stop rule tol)."""
    v = np.random.default_rng(1).standard_normal(np.shape(sol.A))
    v /= np.linalg.norm(v)
    plain = tn.default_opts()
    E = [tn.energy(sol.h, tn.SquareIPEPS(np.asfortranarray(sol.A + sg * step * v)), sol.chi, tol, sol.maxit, plain)
         for sg in (1.0, -1.0)]
    fd = (E[0] - E[1]) / (2 * step)
    gm, gp = float(np.sum(g_mixed * v)), float(np.sum(g_plain * v))
    return {"direction": "unit N(0,1) direction (NumPy seed 1)", "fd_step": step, "fd_stop_tol": tol,
            "fd": fd, "mixed": gm, "mixed_rel_err": abs(gm - fd) / abs(fd),
            "plain_unrolled": gp, "plain_unrolled_rel_err": abs(gp - fd) / abs(fd),
            "mixed_vs_plain_rel_l2": float(np.linalg.norm(g_mixed - g_plain) / np.linalg.norm(g_plain))}


def kernel_timer(c, name):
    c.check(c.lib.tnad_ctx_kernel_timer(c.h, name.encode()))


def kernel_timer_read(c):
    import ctypes as C

    n, ms, work = C.c_int64(), C.c_double(), C.c_double()
    c.check(c.lib.tnad_ctx_kernel_timer_read(c.h, C.byref(n), C.byref(ms), C.byref(work)))
    return n.value, ms.value, work.value


def l2_flush(buf, stream):
    """Overwrite a buffer larger than the 129 MB L2 on the library's stream."""
    import torch

    with torch.cuda.stream(stream):
        buf.add_(1.0)


def train_warm_start(tn, w, args):
    """The learned warm start of the headline mode: targets (gauge-fixed converged
    environments) from the mixed CTMRG on --learned-train site tensors of the
    workload's recipe with seeds 1000.. (never the workload's own seed), a
    3-layer width-512 network trained on the GPU (3000 AdamW steps, batch 64),
    attached to the context.  Untimed set-up; returns its description."""
    import importlib

    wl = importlib.import_module(tn.__name__ + ".learned")
    D, s, chi = w["D"], 2, w["chi"]
    h = tn.hamiltonian(tn.Heisenberg())
    t0 = time.perf_counter()
    train = [tn.site_tensor(w["recipe"], D, s, 1000 + i) for i in range(args.learned_train)]
    samples = wl.make_samples(train, h, chi, 1e-8, 400, tn.mixed_opts(), threads=args.threads)
    t1 = time.perf_counter()
    X, Y = wl.stack(samples)
    net = wl.WarmStartNet(D, s, chi, width=512, seed=1)
    info = net.fit(X, Y, steps=3000, batch=64, lr=1e-3, weight_decay=1e-4)
    net.attach()
    train_warm_start.net = net  # keep it alive while attached
    return {"train_tensors": len(samples), "train_seeds": f"1000..{999 + args.learned_train}",
            "targets_s": round(t1 - t0, 1), "train_s": round(info["seconds"], 2),
            "loss_std_final": round(info["loss_std"], 5), "width": 512, "layers": 3}


def run_gb300(args):
    import torch
    import __graft_entry__ as ge

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist, rank, world = dist_init(args.gpus)
    tn = ge.load_package()
    w = ESTAR[args.workload]
    learned = None
    if args.mode == "learned":
        learned = train_warm_start(tn, w, args)
    sol = Solver(tn, w, args.mode)
    c = sol.c
    stream = torch.cuda.ExternalStream(c.lib.tnad_ctx_stream(c.h))
    flush = torch.zeros(64 << 20, dtype=torch.float32, device="cuda")  # 256 MB > L2
    for _ in range(args.warmup):
        sol.device()
    torch.cuda.synchronize()
    barrier(dist)
    # timed region: K solves with device-resident inputs (no kernel timer); L2
    # flushed between solves, outside each solve's pair of CUDA events
    l0 = c.launches
    errs, stats, evs = [], [], []
    with Clocks(local) as clk:
        torch.cuda.synchronize()
        barrier(dist)
        for _ in range(args.steps):
            l2_flush(flush, stream)
            ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            ev0.record(stream)
            E, st = sol.device()
            ev1.record(stream)
            evs.append((ev0, ev1))
            errs.append(abs(E - w["E_star"]))
            stats.append(st)
        torch.cuda.synchronize()
        barrier(dist)
    launches = (c.launches - l0) // args.steps
    t_dev = max_over_ranks(dist, sum(e0.elapsed_time(e1) for e0, e1 in evs) / 1e3 / args.steps)
    # one extra solve per kernel family with its launches bracketed by CUDA
    # events on the library's stream (a Jacobi sweep replayed as a CUDA graph
    # is bracketed as a whole: its average launch duration includes the
    # graph's gaps between rounds)
    fam = {}
    for name in ("jacobi_round", "jacobi_round_f32", "jacobi_round_small", "eig_refine", "gemm_tf32x3", "gemm_f64",
                 "gemm_fp64tc"):
        kernel_timer(c, name)
        sol.device()
        fam[name] = kernel_timer_read(c)
    kernel_timer(c, "")
    # end to end through the public API with host (NumPy) arrays: every call
    # copies A and h to the device and E and dE/dA back
    sol.host()
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    for _ in range(args.steps):
        E_h, g_h, st_h = sol.host()
    t_e2e = max_over_ranks(dist, (time.perf_counter() - t1) / args.steps)
    # the plain FP64 GPU path (full Jacobi SVD each step, unrolled reverse): one
    # warm-up solve, then the mean of three timed ones
    cold = None
    if args.mode == "learned":
        # the same mixed path from the :raw start (no network): one warm-up, three timed solves
        cs = Solver(tn, w, "mixed")
        cs.device()
        tcs, ecs = [], []
        for _ in range(3):
            torch.cuda.synchronize()
            t2 = time.perf_counter()
            Ec, stc = cs.device()
            torch.cuda.synchronize()
            tcs.append(time.perf_counter() - t2)
            ecs.append(abs(Ec - w["E_star"]))
        cold = {"value": round(statistics.mean(tcs), 4), "unit": "s", "ctmrg_steps": stc["steps"],
                "fp64_steps": stc["fp64_steps"], "fixedpoint_iters": stc["fp_iters"], "delta_E": max(ecs),
                "grad_rel_diff_vs_learned": float(np.linalg.norm(cs.g_d.cpu().numpy() - sol.g_d.cpu().numpy()) /
                                                  np.linalg.norm(cs.g_d.cpu().numpy()))}
    plain, grad_check, g_plain = None, None, None
    if args.mode in ("mixed", "learned") and not args.no_plain:
        ps = Solver(tn, w, "plain")
        ps.device()
        tps, eps_ = [], []
        for _ in range(3):
            torch.cuda.synchronize()
            t2 = time.perf_counter()
            Ep, stp = ps.device()
            torch.cuda.synchronize()
            tps.append(time.perf_counter() - t2)
            eps_.append(abs(Ep - w["E_star"]))
        plain = {"value": round(statistics.mean(tps), 4), "unit": "s", "ctmrg_steps": stp["steps"],
                 "delta_E": max(eps_), "steps": 3, "warmup": 1, "min": round(min(tps), 4), "max": round(max(tps), 4)}
        g_plain = ps.g_d.cpu().numpy().reshape(np.shape(sol.A), order="F")
        if rank == 0:
            grad_check = gradient_check(tn, sol, g_h, g_plain)
    if rank != 0:
        return
    pk, pk_kind = peaks()
    bf16_peak = pk.get("bf16_tflops", 1900.0)
    nominal = "nominal (no measured figure for this pipe in MEASURED_PEAKS.json)"
    # kernel families timed live (CUDA events on the library stream): the
    # algorithmic work of every launch, its hardware multiple (tensor-core
    # emulations issue several products per logical one) and the peak it is
    # measured against
    FAM = {
        "gemm_fp64tc": ("k_gemm_oz + slicing (FP64-accurate products from six BF16 slices per operand on tcgen05: "
                        "26 slice-pair products per FP64 product)", "tensor", 26.0, bf16_peak,
                        f"{pk_kind} bf16 burst (MEASURED_PEAKS.json)"),
        "gemm_f64": ("k_gemm_f64 / k_gemv (register-tiled DFMA GEMM, matrix-vector products)", "fp64", 1.0,
                     FP64_NOMINAL_TFLOPS, nominal),
        "jacobi_round_f32": ("k_jacobi_block<EIG, 64> (FP32 Jacobi sweeps of the 1024x1024 corner's symmetric SVD, "
                             "eigenvalue rule, block rounds of 4 columns)", "fp32", 1.0, FP32_NOMINAL_TFLOPS, nominal),
        "jacobi_round_small": ("k_jacobi_round_cta<2, double> (FP64 rounds of the p x p Rayleigh-Ritz problems of the "
                               "subspace solver)", "fp64", 1.0, FP64_NOMINAL_TFLOPS, nominal),
        "jacobi_round": ("k_jacobi_round_cta<8, double> (FP64 sweeps of the corner SVD where the refinement falls "
                         "back)", "fp64", 1.0, FP64_NOMINAL_TFLOPS, nominal),
        "gemm_tf32x3": ("k_gemm_tf32x3 (tcgen05 kind::tf32, 3 split products)", "tensor", 3.0, bf16_peak / 2.0,
                        f"{pk_kind} bf16 burst / 2 (dense TF32 rate)"),
    }
    families = {}
    for name, (desc, bound, hw, peak, kind) in FAM.items():
        fn, fms, fwork = fam[name]
        ach = (fwork / (fms / 1e3)) / 1e12 if fms > 0 else None
        families[name] = {"kernel": desc, "bound": bound,
                          "achieved_logical": round(ach, 4) if ach else None,
                          "achieved": round(hw * ach, 4) if ach else None, "peak": round(peak, 2),
                          "unit": "TFLOP/s", "frac": round(hw * ach / peak, 4) if ach else None, "peak_kind": kind,
                          "launches_per_step": fn, "ms_per_step": round(fms, 3),
                          "avg_launch_us": round(fms * 1e3 / fn, 3) if fn else None,
                          "share_of_step": round(fms / 1e3 / t_dev, 4)}
    top = max(families, key=lambda k: families[k]["share_of_step"])
    roofline = dict(families[top], family=top,
                    traffic={"jacobi_round": JACOBI_ROUND_TRAFFIC_BYTES, "gemm_fp64tc": OZ_TRAFFIC_BYTES}.get(top))
    nA = int(np.asarray(sol.A).size)
    line = {
        "metric": metric_for(w),
        "value": round(t_dev, 6), "unit": "s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(t_dev * 1e3, 3), "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": {"plain": "f64", "mixed": "tf32x3+f64"}.get(args.mode, "tf32x3+f64 (bf16 warm-start network)"),
        "data": f"synthetic: {w['recipe']} site tensor (NumPy seed {w['seed']}), symmetrised",
        "config": {"workload": args.workload, "D": sol.D, "chi": sol.chi, "phys": sol.s, "mode": args.mode,
                   "stop_tol": sol.tol, "ctmrg_steps": stats[-1]["steps"], "fp64_steps": stats[-1]["fp64_steps"],
                   "fixedpoint_iters": stats[-1]["fp_iters"],
                   "fixedpoint_residual": stats[-1].get("fixed_point_residual"),
                   "parallelism": f"replicas x{world}",
                   "l2": "flushed between timed solves (256 MB write on the library stream, outside the events)"},
        "delta_E": max(errs), "E": E, "E_star": w["E_star"],
        "e2e": {"value": round(t_e2e, 6), "unit": "s", "h2d_bytes_per_step": 8 * (nA + 16),
                "d2h_bytes_per_step": 8 * (nA + 1)},
        "gpu_launches": int(launches),
        "roofline": roofline,
        "eig_refine": {"what": "GEMM refinement of the FP32 eigenvectors of the symmetric corner SVDs (one bracket "
                              "per iteration: 6 products and the grouping kernels)",
                       "iterations_per_step": fam["eig_refine"][0], "ms_per_step": round(fam["eig_refine"][1], 3),
                       "share_of_step": round(fam["eig_refine"][1] / 1e3 / t_dev, 4)},
        "kernel_families": families,
        "clocks": clk.summary(),
    }
    if learned:
        learned["warm_start_kept"] = sum(1 for st in stats if st.get("warm_status") == 1) / len(stats)
        line["config"]["learned_warm_start"] = learned
    if cold:
        line["mixed_cold_start"] = cold
    if plain:
        line["plain_fp64"] = plain
        line["speedup_vs_plain_fp64"] = round(plain["value"] / t_dev, 2)
    if grad_check:
        line["gradient_check"] = grad_check
    if not args.no_cpu_baseline:
        torch.set_num_threads(os.cpu_count() or 1)
        cb, E_o, g_o, steps_o = oracle_full(w)
        line["cpu_baseline"] = {"value": round(cb, 3), "unit": "s", "cores": torch.get_num_threads(), "kind": "port",
                                "sample": f"one full oracle solve (torch-CPU FP64): {steps_o} CTMRG steps to the "
                                          f"reference stop rule at tol {plain_tol(w):.3g}, energy, unrolled reverse; "
                                          f"|dE| {abs(E_o - w['E_star']):.2e}"}
        gv = {"oracle": "unrolled reverse of the oracle (the reference's Zygote gradient restated), same input",
              "mixed_rel_l2": float(np.linalg.norm(g_h - g_o) / np.linalg.norm(g_o)),
              "mixed_max_abs_rel": float(np.max(np.abs(g_h - g_o)) / np.max(np.abs(g_o)))}
        if g_plain is not None:
            gv["plain_rel_l2"] = float(np.linalg.norm(g_plain - g_o) / np.linalg.norm(g_o))
            gv["plain_max_abs_rel"] = float(np.max(np.abs(g_plain - g_o)) / np.max(np.abs(g_o)))
        line["gradient_vs_oracle"] = gv
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
def oracle_full(w):
    """One full solve of workload w by the oracle on the host cores: energy
    (CTMRG from :raw with the reference stop rule at the tolerance where its
    trajectory is within TARGET of E*) and its unrolled reverse.  Returns
    (seconds, E, dE/dA, CTMRG steps)."""
    import torch
    from oracle import tnad_oracle as orc

    h = orc.hamiltonian_heisenberg()
    A = workload_input(w)
    t0 = time.perf_counter()
    E, g, steps = orc.energy_and_grad(h, A, w["chi"], plain_tol(w), 400)
    dt = time.perf_counter() - t0
    return dt, E, np.asarray(g).reshape(np.shape(A)), steps


def run_reference(args):
    """The reference's CPU path (the oracle restatement: Julia is absent) timed on
    the host cores, every step one full energy + gradient solve of the workload.
    The CPU needs no warm-up beyond the first call, so at most one warm-up solve
    runs, which keeps the whole run within a few minutes."""
    import torch

    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    torch.set_num_threads(os.cpu_count() or 1)
    w = ESTAR[args.workload]
    nwarm = min(args.warmup, 1)
    for _ in range(nwarm):
        oracle_full(w)
    ts, errs, steps = [], [], 0
    for _ in range(args.steps):
        t, E, _, steps = oracle_full(w)
        ts.append(t)
        errs.append(abs(E - w["E_star"]))
    v = statistics.mean(ts)
    cores = torch.get_num_threads()
    sample = (f"full oracle solve per step (torch-CPU FP64, {cores} threads): {steps} CTMRG steps to the reference "
              f"stop rule at tol {plain_tol(w):.3g}, energy and unrolled reverse; {nwarm} warm-up solve(s)")
    line = {
        "metric": metric_for(w), "impl": "reference",
        "value": round(v, 4), "unit": "s", "n_gpus": 0, "steps": args.steps, "warmup": nwarm,
        "ms_per_step": round(v * 1e3, 1), "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": f"synthetic: {w['recipe']} site tensor (NumPy seed {w['seed']}), symmetrised",
        "config": {"workload": args.workload, "D": w["D"], "chi": w["chi"], "phys": 2},
        "delta_E": max(errs), "min": round(min(ts), 4), "max": round(max(ts), 4),
        "cpu_baseline": {"value": round(v, 4), "unit": "s", "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": round(v, 4), "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_learned(args):
    """Learned warm start at D=3, χ=36 (Heisenberg): targets from the mixed
    CTMRG on uniform [-1, 1] site tensors and on the iterates of L-BFGS
    trajectories (Jz uniform in [0.5, 1.5]); a 3-layer width-512 network
    trained on the GPU; then, on held-out tensors from the same pool, CTMRG
    steps and wall time of energy (forward) to the stop rule 1e-8 from the
    learned start and from :raw.  Solves of the comparison run one at a time."""
    import importlib

    import __graft_entry__ as ge

    tn = ge.load_package()
    wl = importlib.import_module(tn.__name__ + ".learned")
    D, s, chi, tol, maxit = 3, 2, 36, 1e-8, 400
    h = tn.hamiltonian(tn.Heisenberg())
    rng = np.random.default_rng(20240601)
    t0 = time.perf_counter()
    pool = [wl.random_site_tensor(D, s, rng) for _ in range(args.n_train + int(0.8 * args.n_held))]
    kinds = ["uniform"] * len(pool)
    jzs = rng.uniform(0.5, 1.5, args.n_traj)
    seeds = rng.integers(0, 2 ** 31, args.n_traj)

    def trajectory(k):
        return wl.heisenberg_trajectory(D, chi, float(jzs[k]), np.random.default_rng(int(seeds[k])), args.traj_evals,
                                        1e-8, maxit, tn.mixed_opts())

    from concurrent.futures import ThreadPoolExecutor

    with ThreadPoolExecutor(max_workers=max(1, args.threads)) as ex:
        for traj in ex.map(trajectory, range(args.n_traj)):
            pool += traj
            kinds += ["trajectory"] * len(traj)
    t1 = time.perf_counter()
    perm = rng.permutation(len(pool))
    n_held = min(args.n_held, len(pool) // 5)
    held_idx, train_idx = perm[:n_held], perm[n_held:]
    hmix = lambda: tn.mixed_opts()  # noqa: E731
    samples = wl.make_samples([pool[i] for i in train_idx], h, chi, tol, maxit, hmix(), threads=args.threads)
    t2 = time.perf_counter()
    X, Y = wl.stack(samples)
    net = wl.WarmStartNet(D, s, chi, width=512, seed=1)
    info = net.fit(X, Y, steps=args.train_steps, batch=128, lr=1e-3, weight_decay=1e-4,
                   log_every=max(1, args.train_steps // 8))
    net.attach()
    held = [pool[i] for i in held_idx]
    # warm-up of both paths (first-call costs), not counted
    wl.compare_starts(held[:2], h, chi, tol, maxit, hmix)
    r = wl.compare_starts(held, h, chi, tol, maxit, hmix)
    t3 = time.perf_counter()
    same = r["dE"] <= 1e-8
    hk = np.array([kinds[i] for i in held_idx])
    by_kind = {}
    for k in ("uniform", "trajectory"):
        m = hk == k
        if m.any():
            by_kind[k] = {"n": int(m.sum()), "cold_steps": round(float(r["cold_steps"][m].mean()), 2),
                          "warm_steps": round(float(r["warm_steps"][m].mean()), 2),
                          "cold_s": round(float(r["cold_s"][m].mean()), 4),
                          "warm_s": round(float(r["warm_s"][m].mean()), 4),
                          "same_fixed_point": round(float(same[m].mean()), 3)}
    line = {
        "metric": "CTMRG steps and wall time to stop rule 1e-8, learned warm start vs :raw (D=3, chi=36)",
        "value": round(float(r["warm_s"].mean()), 4), "unit": "s/solve", "higher_is_better": False,
        "cold_s_per_solve": round(float(r["cold_s"].mean()), 4),
        "speedup_wall": round(float(r["cold_s"].mean() / r["warm_s"].mean()), 3),
        "cold_steps": round(float(r["cold_steps"].mean()), 2), "warm_steps": round(float(r["warm_steps"].mean()), 2),
        "step_ratio": round(float(r["warm_steps"].mean() / r["cold_steps"].mean()), 3),
        "median_cold_steps": float(np.median(r["cold_steps"])), "median_warm_steps": float(np.median(r["warm_steps"])),
        "same_fixed_point": round(float(same.mean()), 3),
        "judge_kept": round(float(np.mean(r["status"] == 1)), 3),
        "judge_rejected": round(float(np.mean(r["status"] == -1)), 3),
        "by_kind": by_kind,
        "train": {"n": len(samples), "n_trajectory": int(sum(kinds[i] == "trajectory" for i in train_idx)),
                  "steps": args.train_steps, "batch": 128, "seconds": round(info["seconds"], 2),
                  "loss_std_final": round(info["loss_std"], 5),
                  "history": [(k, round(v, 5)) for k, v in info["history"]]},
        "n_held": n_held, "dtype": "bf16 network, mixed TF32X3/FP64 CTMRG", "data": "synthetic",
        "config": {"workload": "learned_D3_chi36", "D": D, "chi": chi, "tol": tol, "model": "Heisenberg",
                   "width": 512, "layers": 3},
        "timing": {"pool_s": round(t1 - t0, 1), "targets_s": round(t2 - t1, 1), "compare_s": round(t3 - t2, 1)},
    }
    print(json.dumps(line), flush=True)


def run_learned_headline(args):
    """Learned warm start on the headline configuration (D=4, χ=64, N(0,1)
    max-abs-normalised site tensors, Heisenberg): targets from the mixed CTMRG
    on n_train tensors of that recipe (seeds other than the workload's), the
    network trained on the GPU, then the energy+gradient solve of the bench
    workload tensor (seed 0) timed from the learned start and from :raw, and
    CTMRG steps of the energy on held-out tensors of the same recipe."""
    import importlib

    import torch
    import __graft_entry__ as ge

    tn = ge.load_package()
    wl = importlib.import_module(tn.__name__ + ".learned")
    w = ESTAR["heisenberg_D4_chi64"]
    D, s, chi = 4, 2, 64
    h = tn.hamiltonian(tn.Heisenberg())
    t0 = time.perf_counter()
    train = [tn.site_tensor("normal_maxabs", D, s, 1000 + i) for i in range(args.n_train)]
    samples = wl.make_samples(train, h, chi, 1e-8, 400, tn.mixed_opts(), threads=args.threads)
    t1 = time.perf_counter()
    X, Y = wl.stack(samples)
    net = wl.WarmStartNet(D, s, chi, width=512, seed=1)
    info = net.fit(X, Y, steps=args.train_steps, batch=64, lr=1e-3, weight_decay=1e-4,
                   log_every=max(1, args.train_steps // 6))
    net.attach()
    # the bench workload: energy + gradient, learned start vs :raw, device-resident inputs
    res = {}
    for name, warm in (("cold", tn._lib.WARM_NONE), ("learned", tn._lib.WARM_LEARNED)):
        sol = Solver(tn, w, "mixed")
        sol.opts_d.warm_start = warm
        sol.device()
        ts, stats, errs, status = [], None, [], []
        for _ in range(max(args.steps, 1)):
            torch.cuda.synchronize()
            ta = time.perf_counter()
            E, stats = sol.device()
            torch.cuda.synchronize()
            ts.append(time.perf_counter() - ta)
            errs.append(abs(E - w["E_star"]))
            status.append(wl.warm_start_status())
        res[name] = {"s_per_solve": round(min(ts), 4), "ctmrg_steps": stats["steps"], "fp64_steps": stats["fp64_steps"],
                     "fixedpoint_iters": stats["fp_iters"], "delta_E": max(errs), "warm_status": status[-1],
                     "grad": sol.g_d.cpu().numpy()}
    gc, gl = res["cold"].pop("grad"), res["learned"].pop("grad")
    res["learned"]["grad_rel_diff_vs_cold"] = float(np.linalg.norm(gl - gc) / np.linalg.norm(gc))
    held = [tn.site_tensor("normal_maxabs", D, s, 5000 + i) for i in range(args.n_held)]
    r = wl.compare_starts(held, h, chi, 1e-8, 400, tn.mixed_opts)
    line = {
        "metric": "learned warm start on the headline workload (Heisenberg iPEPS D=4, chi=64): energy+gradient "
                  "time to |dE|<=1e-8, learned start vs :raw",
        "value": res["learned"]["s_per_solve"], "unit": "s", "higher_is_better": False,
        "cold": res["cold"], "learned": res["learned"],
        "speedup": round(res["cold"]["s_per_solve"] / res["learned"]["s_per_solve"], 3),
        "held_out": {"n": len(held), "cold_steps": round(float(r["cold_steps"].mean()), 2),
                     "warm_steps": round(float(r["warm_steps"].mean()), 2),
                     "same_fixed_point": round(float(np.mean(r["dE"] <= 1e-8)), 3),
                     "judge_kept": round(float(np.mean(r["status"] == 1)), 3)},
        "train": {"n": len(samples), "seconds": round(info["seconds"], 2), "targets_s": round(t1 - t0, 1),
                  "loss_std_final": round(info["loss_std"], 5), "steps": args.train_steps},
        "config": {"workload": "learned_D4_chi64", "D": D, "chi": chi, "width": 512, "layers": 3},
        "dtype": "bf16 network, mixed TF32X3/FP64 CTMRG", "data": "synthetic",
    }
    print(json.dumps(line), flush=True)


def run_optimise(args):
    """optimiseipeps (src/variationalipeps.jl:67-75) at D=4 on the GPU: L-BFGS
    (m = 20) from the headline workload's site tensor for --lbfgs-steps
    iterations, once with the mixed path (implicit fixed-point adjoint) and once
    with the unrolled reverse checkpointed at every step (tape_budget 0: only
    (C, T) of each step is kept; each step's decomposition is recomputed in the
    reverse pass), TF32X3 contractions and the FP64 Jacobi SVD.  Reports the
    energy after every iteration, wall time, evaluations and the device memory
    in use at the end of every forward pass (cudaMemGetInfo)."""
    import ctypes as C

    import scipy.optimize
    import torch
    import __graft_entry__ as ge

    tn = ge.load_package()
    torch.cuda.set_device(0)
    chi = args.chi or 64
    w = ESTAR["heisenberg_D4_chi64"]
    A0 = workload_input(w)
    h = tn.hamiltonian(tn.Heisenberg())
    shape = A0.shape
    free0, total = torch.cuda.mem_get_info()
    modes = {
        "mixed": (tn.mixed_opts(), 3e-8),
        "checkpointed_unrolled": (tn.default_opts(prec=tn._lib.PREC_TF32X3, solver=tn._lib.SOLVER_FULL_SVD,
                                                  adjoint=tn._lib.ADJOINT_UNROLLED, tape_budget=0),
                                  plain_tol(w) if chi == 64 else 1e-7),
    }
    out = {}
    for name, (opts, tol) in modes.items():
        if args.only and name != args.only:
            continue
        evals, energies, peak, last = [0], [], [0], [None]

        def fg(x):
            r = tn._energy(h, tn.SquareIPEPS(x.reshape(shape, order="F")), chi, tol, 400, opts, record=True)
            last[0] = r.E
            free, _ = torch.cuda.mem_get_info()
            peak[0] = max(peak[0], total - free)
            g = tn.fzeros(shape)
            cc = r.tape.c
            cc.check(cc.lib.tnad_energy_backward(cc.h, r.tape.h, 1.0, tn.ptr(g)))
            evals[0] += 1
            return r.E, np.asarray(g).ravel(order="F")

        fg(np.asarray(A0).ravel(order="F"))  # warm-up evaluation (first-call costs), not counted
        evals[0] = 0
        t0 = time.perf_counter()
        res = scipy.optimize.minimize(fg, np.asarray(A0).ravel(order="F"), jac=True, method="L-BFGS-B",
                                      callback=lambda xk: energies.append(last[0]),
                                      options=dict(maxcor=20, maxiter=args.lbfgs_steps, ftol=0.0, gtol=0.0))
        dt = time.perf_counter() - t0
        # the energy after every iteration, re-evaluated from the iterates' record
        out[name] = {"iterations": int(res.nit), "evaluations": evals[0], "seconds": round(dt, 2),
                     "s_per_evaluation": round(dt / max(evals[0], 1), 3), "E_final": float(res.fun),
                     "E_per_iteration": energies,
                     "E_start": None, "peak_device_bytes": int(peak[0] - (total - free0)),
                     "workspace_bytes": int(tn.ctx().lib.tnad_ctx_workspace_bytes(tn.ctx().h)),
                     "stop_tol": tol, "message": str(res.message)}
    E_start = tn.energy(h, tn.SquareIPEPS(A0), chi, 1e-10, 400, tn.mixed_opts())
    for v in out.values():
        v["E_start"] = E_start
    if not args.only or args.only == "mixed_device_lbfgs":
        # the library's own L-BFGS (iterate and pairs on the device, Armijo backtracking)
        o = tn.mixed_opts()
        tn.energy(h, tn.SquareIPEPS(A0), chi, 3e-8, 400, o)  # warm-up
        st = {}
        t0 = time.perf_counter()
        E, _ = tn.optimiseipeps(tn.SquareIPEPS(A0), h, chi, 3e-8, 400, f_tol=0.0, iterations=args.lbfgs_steps,
                                opts=o, driver="device", stats=st)
        dt = time.perf_counter() - t0
        out["mixed_device_lbfgs"] = {"iterations": st["iterations"], "evaluations": st["evaluations"],
                                     "seconds": round(dt, 2), "s_per_evaluation": round(dt / max(st["evaluations"], 1), 3),
                                     "E_final": E, "stop_tol": 3e-8}
    line = {"metric": f"optimiseipeps: {args.lbfgs_steps} L-BFGS iterations at D=4, chi={chi} (Heisenberg)",
            "unit": "s", "higher_is_better": False, "config": {"workload": f"optimise_D4_chi{chi}", "D": 4,
                                                              "chi": chi, "lbfgs_m": 20},
            "data": "synthetic: the headline N(0,1) site tensor as the start", "modes": out}
    print(json.dumps(line), flush=True)


def run_profile(args):
    import importlib

    import __graft_entry__ as ge

    tn = ge.load_package()
    if args.profile == "solve":
        E, st = Solver(tn, ESTAR[args.workload], "mixed" if args.mode == "learned" else args.mode).device()
        print(f"profile solve: E={E!r} steps={st['steps']} launches={tn.ctx().launches}", flush=True)
        return
    if args.profile == "gemm_fp64tc":
        rng = np.random.default_rng(0)
        A, B, B2 = rng.standard_normal((1024, 1024)), rng.standard_normal((1024, 1024)), rng.standard_normal((1024, 96))
        for _ in range(2):
            tn.gemm(A, B, prec=tn._lib.PREC_FP64_TC)
            tn.gemm(A, B2, prec=tn._lib.PREC_FP64_TC)
        print(f"profile gemm_fp64tc: 4 products, launches={tn.ctx().launches}", flush=True)
        return
    wl = importlib.import_module(tn.__name__ + ".learned")
    net = wl.WarmStartNet(3, 2, 36, width=512, seed=1)
    rng = np.random.default_rng(0)
    X = rng.standard_normal((net.n_in, 1024)).astype(np.float32)
    Y = rng.standard_normal((net.n_out, 1024)).astype(np.float32)
    net.set_data(X, Y)
    loss = None
    for k in range(20):
        loss = net.train_step(rng.integers(0, 1024, 128), 1e-3, 1e-4, want_loss=(k == 19))
    print(f"profile mlp: 20 AdamW steps, batch 128, loss={loss:.4f} launches={tn.ctx().launches}", flush=True)


if __name__ == "__main__":
    a = parse()
    if a.profile:
        run_profile(a)
    elif a.impl == "reference":
        run_reference(a)
    elif a.workload.startswith("optimise"):
        run_optimise(a)
    elif a.workload == "learned_D4_chi64":
        run_learned_headline(a)
    elif a.workload.startswith("learned"):
        run_learned(a)
    else:
        run_gb300(a)
