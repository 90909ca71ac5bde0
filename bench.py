"""Benchmark of the GB300 hot path of Mat (mixed LU + FP64 refinement solve).

Headline (metric "n=16384 LU-solve time at FP64 backward error, mixed+IR vs
FP64; DGEMM TFLOP/s"):
  one step = one mixed-precision LU solve with FP64 iterative refinement,
  n = 16384, 4 right-hand sides, A = Q1 diag(sigma) Q2 (Q = 64 seeded
  Householder reflectors each side, sigma geometric 1 -> 1e-6, cond 1e6),
  b iid N(0,1), to normwise backward error <= 1e-14, inputs resident in HBM
  (A is 2 GiB, larger than L2, so no flush is needed between steps).
value = mean seconds per solve (lower is better).  Beside it on the same
line: the plain FP64 GPU solve of the same system (the "vs FP64" half of the
metric), the FP64 DGEMM rate at M=N=K=1024 (the "DGEMM TFLOP/s" half), an
end-to-end leg through the C ABI with host buffers, the roofline of the
dominant kernel (timed live with CUDA events on the library's stream), the
oracle restatement timed on the host cores, and sampled GPU clocks.

--impl reference: times the CPU implementation of the reference on the same
system (the oracle restatement of Mat's Solve_direct, bit-identical to Mat's
own results; the reference itself is x86 AVX-512 header code absent from the
GPU host) on all host cores: each step one whole n = 16384, 4-RHS solve of
the same A and B, regenerated on the host by the oracle from the same seeded
streams (bit-identical to the GPU generator).  It loads no part of this
library.  Warm-up steps solve an n = 2048 system of the same recipe.
Multi-GPU: replicas only (independent solves, no collective on the path).
"""
from __future__ import annotations

import argparse
import gc
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "n=16384 LU-solve time at FP64 backward error, mixed+IR vs FP64; DGEMM TFLOP/s"
WORKLOAD = ("LU solve of A X = B to FP64 normwise backward error <= 1e-14, n=16384, 4 RHS, "
            "A=Q1*diag(sigma)*Q2 with 64 Householder reflectors per side (seed 3), "
            "sigma geometric 1..1e-6 (cond 1e6), B iid N(0,1) (seed 11)")
METHOD = ("mixed LU (fp32 panels + split-BF16x3 tcgen05 trailing updates) + FP64 iterative refinement "
          "on one GB300")
REF_METHOD = ("Mat Solve_direct (narrow path: blocked PLU, BS=60, then scalar substitutions) in FP64, the "
              "oracle restatement (bit-identical to Mat-8.3.1), all host threads")


def bench_config(n: int, nrhs: int, world: int) -> dict:
    """The workload both arms run (identical dicts: the same system, seeds and target)."""
    return {"workload": WORKLOAD, "n": n, "nrhs": nrhs, "seed_A": 3, "seed_B": 11,
            "parallelism": f"replicas x{world}", "l2": "inputs larger than L2 (A is 2 GiB), no flush"}


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--n", type=int, default=16384)
    p.add_argument("--nrhs", type=int, default=4)
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--no-configs", action="store_true", help="skip the other configurations' rates")
    return p.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def peaks():
    f = ROOT / "MEASURED_PEAKS.json"
    if f.exists():
        d = json.loads(f.read_text())
        return float(d.get("hbm_gbs", 6800.0)), float(d.get("bf16_tflops", 1900.0)), \
            float(d.get("bf16_tflops_sustained", 1700.0)), "measured"
    return 6800.0, 1900.0, 1700.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms during the timed region."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def host_system(n: int, nrhs: int, seed_a: int = 3, seed_b: int = 11):
    """The benchmark system regenerated on the host by the oracle (same seeded
    streams and operation order as the GPU generator: bit-identical)."""
    from oracle.api import gen_svd_matrix, host_fill_normal
    return gen_svd_matrix(n, seed_a, 64, 1e-6), host_fill_normal(n, nrhs, seed_b)


def cpu_solve(A, B):
    """One FP64 Solve_direct of the oracle restatement on all host cores: (seconds, cores, X)."""
    from oracle.api import restatement
    o = restatement()
    cores = os.cpu_count() or 1
    o.set_threads(cores)
    t = time.perf_counter()
    X = o.solve(A, B)
    return time.perf_counter() - t, cores, X


def backward_error(A, X, B) -> float:
    """max over columns of ||b - A x||_inf / (||A||_inf ||x||_inf + ||b||_inf)."""
    import numpy as np
    R = B - A @ X
    an = float(np.abs(A).sum(axis=1).max())
    return float(max(np.abs(R[:, j]).max() / (an * np.abs(X[:, j]).max() + np.abs(B[:, j]).max())
                     for j in range(B.shape[1])))


def config_rates(h, dmma_tf: float, bf16_tf: float) -> dict:
    """The other configurations, measured after the headline (each timed once
    after a warm-up call, wall clock around a synchronised call): FP64 LU +
    solve, LLT (n = 8192, seed 1) and Householder QR (16384 x 4096: R alone
    and with the full 16384 x 16384 Q), and the mixed QR's fp32 factorization
    of the same matrix; the mixed QR solve of the benchmark recipe at
    n = 8192 beside the mixed and FP64 LU solves; the M=N=K=16384 split-BF16
    GEMM on u*2^e entries (seed 3) with its error against FP64 on 256 sampled
    rows, and the SIMT FP32 GEMM's error on the same inputs; the
    Gaussian-process loss + gradient (Cholesky adjoint) at n = 8192 in FP64 and
    FP32, and the mixed SPD solve of its kernel matrix; GMRES-IR at n = 16384,
    cond 1e10; the mixed solve with tournament panels; the Mat-8.1 EVD_Q
    (tridiagonalisation with Q, and the whole eigendecomposition) at n = 1024
    and 4096."""
    import ctypes as C

    import torch

    from mat_gb300.api import colmajor

    def timed(fn):
        fn()
        torch.cuda.synchronize()
        t = time.perf_counter()
        r = fn()
        torch.cuda.synchronize()
        return time.perf_counter() - t, r

    def rate(flops, t, peak):
        return {"s": t, "gflops": flops / t / 1e9, "frac_of_peak": flops / t / 1e12 / peak}

    out = {"fp64_peak_tflops": dmma_tf, "bf16_peak_tflops": bf16_tf}
    n = 8192
    A0 = colmajor(n, n)
    h.fill_normal(A0, 1)
    b = colmajor(n, 1)
    h.fill_normal(b, 2)
    A = A0.clone()
    pos = torch.empty(n, dtype=torch.int32, device="cuda")

    def lu():
        A.copy_(A0)
        return h.dgetrf(A, pos)

    t_lu, _ = timed(lu)
    t_sv, x = timed(lambda: h.dgetrs(A, pos, b))
    r = b - A0 @ x
    out["lu_8192"] = {"factor": rate(2 / 3 * n ** 3, t_lu, dmma_tf), "solve_s": t_sv,
                      "residual_rel": float(r.norm() / (A0.norm() * x.norm()))}
    S0 = colmajor(n, n)
    h.gen_spd_gram(S0, 1)
    S = S0.clone()

    def llt():
        S.copy_(S0)
        return h.dpotrf(S)

    t_llt, _ = timed(llt)
    out["llt_8192"] = {"factor": rate(n ** 3 / 3, t_llt, dmma_tf)}
    del A0, A, S0, S, b
    m, k = 16384, 4096
    Q0 = colmajor(m, k)
    h.fill_normal(Q0, 1)
    Qa = Q0.clone()
    tau = torch.empty(k, dtype=torch.float64, device="cuda")
    T = torch.empty(((k + 47) // 48) * 48 * 48, dtype=torch.float64, device="cuda")

    def geqrf():
        Qa.copy_(Q0)
        h.check(h.lib.mg_dgeqrf(h.h, m, k, C.c_void_p(Qa.data_ptr()), m, C.c_void_p(tau.data_ptr()),
                                C.c_void_p(T.data_ptr())), "mg_dgeqrf")

    t_r, _ = timed(geqrf)
    Qf, Rf = colmajor(m, m), colmajor(m, k)
    t_q, _ = timed(lambda: h.dqr(Q0, Qf, Rf))
    # flop counts: R 2mk^2 - 2k^3/3; full m x m Q from k reflectors (LAPACK dorgqr) 4m^2k - 4mk^2 + 4k^3/3
    fr, fq = 2 * m * k * k - 2 / 3 * k ** 3, 4 * m * m * k - 4 * m * k * k + 4 / 3 * k ** 3
    out["qr_16384x4096"] = {"r_factor": rate(fr, t_r, dmma_tf), "with_full_q": rate(fr + fq, t_q, dmma_tf)}
    del Qf, Rf, tau, T
    torch.cuda.empty_cache()
    # the mixed QR's fp32 factorization (FP64 norm/beta/tau, split-BF16 trailing
    # updates) of the same 16384 x 4096 matrix, against the FP64 R factor above
    Q32 = Q0.float().t().contiguous().t()
    Qs = Q32.clone()

    def sgeqrf():
        Qs.copy_(Q32)
        return h.sgeqrf(Qs)

    t_s, _ = timed(sgeqrf)
    h.profile(True)
    sgeqrf()
    torch.cuda.synchronize()
    prs = h.profile_records()
    h.profile(False)
    out["sgeqrf_16384x4096"] = {"s": t_s, "useful_tflops": fr / t_s / 1e12, "speedup_vs_fp64_r_factor": t_r / t_s,
                                "phases_ms": {k: round(v["ms"], 3) for k, v in prs.items()}}
    del Q0, Qa, Q32, Qs
    torch.cuda.empty_cache()
    # the mixed QR solve (benchmark recipe, n = 8192) against the mixed LU solve
    # and the FP64 LU solve of the same system
    nq = 8192
    Aq = colmajor(nq, nq)
    h.gen_svd_matrix(Aq, 3, nrefl=64, sigma_min=1e-6)
    Bq = colmajor(nq, 4)
    h.fill_normal(Bq, 11)
    t_qs, (Xq, rq) = timed(lambda: h.dsqrsv_ir(Aq, Bq))
    t_ls, _ = timed(lambda: h.dsgesv_ir(Aq, Bq))
    t_d, _ = timed(lambda: h.dgesv(Aq, Bq))
    out["mixed_qr_solve_8192"] = {"s": t_qs, "mixed_lu_solve_s": t_ls, "fp64_lu_solve_s": t_d,
                                  "iterations": rq["iterations"], "path": rq["path"],
                                  "backward_error": rq["backward_error"], "factor_ms": rq["factor_ms"],
                                  "refine_ms": rq["refine_ms"]}
    del Aq, Bq, Xq
    torch.cuda.empty_cache()
    # split GEMM, entries u * 2^e
    N = 16384
    g = torch.Generator(device="cuda").manual_seed(3)

    def wide():
        u = torch.rand((N, N), generator=g, device="cuda", dtype=torch.float64) * 2 - 1
        e = torch.randint(-8, 9, (N, N), generator=g, device="cuda").to(torch.float64)
        return (u * torch.exp2(e)).float().t().contiguous().t()

    Ga, Gb = wide(), wide()
    Gc = colmajor(N, N, dtype=torch.float32)
    t_sg, _ = timed(lambda: h.sgemm_bf16x(Ga, Gb, Gc))
    rows = torch.randperm(N, generator=g, device="cuda")[:256]
    ref = Ga[rows].double() @ Gb.double()
    d = Gc[rows].double() - ref
    useful = 2 * N ** 3
    out["split_gemm_16384"] = {"s": t_sg, "useful_tflops": useful / t_sg / 1e12,
                               "bf16_pipe_tflops": 6 * useful / t_sg / 1e12,
                               "frac_of_bf16_peak": 6 * useful / t_sg / 1e12 / bf16_tf,
                               "max_rel_err": float(d.abs().max() / ref.abs().max()),
                               "normwise_rel_err": float(d.norm() / ref.norm()),
                               "error_sample": "256 random rows vs FP64 product of the same fp32 inputs"}
    # the ordered variant (lower-order products first): more accurate, a second pass over K
    t_so, _ = timed(lambda: h.sgemm_bf16x(Ga, Gb, Gc, ordered=True))
    d = Gc[rows].double() - ref
    out["split_gemm_16384"]["ordered"] = {"s": t_so, "useful_tflops": useful / t_so / 1e12,
                                          "max_rel_err": float(d.abs().max() / ref.abs().max()),
                                          "normwise_rel_err": float(d.norm() / ref.norm())}
    # the same inputs through the SIMT FP32 GEMM (IEEE fp32 accumulation): the
    # accuracy the split form is compared with
    t_ss, _ = timed(lambda: h.sgemm(Ga, Gb, Gc))
    d = Gc[rows].double() - ref
    out["split_gemm_16384"]["fp32_simt"] = {"s": t_ss, "tflops": useful / t_ss / 1e12,
                                           "max_rel_err": float(d.abs().max() / ref.abs().max()),
                                           "normwise_rel_err": float(d.norm() / ref.norm())}
    del Ga, Gb, Gc, ref, d
    torch.cuda.empty_cache()
    # FP64 tensor-core GEMM rate at 4096^3, for the comparison
    Da, Db = colmajor(4096, 4096), colmajor(4096, 4096)
    h.fill_uniform(Da, 0)
    h.fill_uniform(Db, 1)
    Dc = colmajor(4096, 4096)
    t_dg, _ = timed(lambda: h.dgemm(Da, Db, Dc))
    out["split_gemm_16384"]["fp64_gemm_tflops_4096"] = 2 * 4096 ** 3 / t_dg / 1e12
    out["split_gemm_16384"]["speedup_vs_fp64_gemm"] = (useful / t_sg) / (2 * 4096 ** 3 / t_dg)
    del Da, Db, Dc
    # GP loss + gradient, FP64
    gp = torch.Generator(device="cuda").manual_seed(5)
    Xp = torch.rand((3, n), generator=gp, device="cuda", dtype=torch.float64).t()
    y = torch.randn((1, n), generator=gp, device="cuda", dtype=torch.float64).t()
    t_gp, (loss, dell, _) = timed(lambda: h.gp_loss_grad(Xp, y, 0.2))
    out["gp_adjoint_8192_fp64"] = {"s": t_gp, "gflops": n ** 3 / t_gp / 1e9, "loss": loss, "dloss_dell": dell,
                                   "flops_model": "n^3 (Cholesky n^3/3 + its adjoint 2n^3/3)"}
    X32 = Xp.float().t().contiguous().t()
    y32 = y.float().contiguous()
    t_gp32, (loss32, dell32, _) = timed(lambda: h.sgp_loss_grad(X32, y32, 0.2))
    out["gp_adjoint_8192_fp32"] = {"s": t_gp32, "gflops": n ** 3 / t_gp32 / 1e9, "loss": loss32,
                                   "dloss_dell": dell32, "loss_rel_diff_vs_fp64": abs(loss32 - loss) / abs(loss),
                                   "dell_rel_diff_vs_fp64": abs(dell32 - dell) / abs(dell),
                                   "note": "inputs rounded to fp32; the difference is the fp32 conditioning of K"}
    # the mixed SPD solve on the Gaussian-process kernel (fp32 Cholesky with
    # split-BF16 updates + FP64 refinement) against the FP64 Cholesky solve
    K = h.gen_rbf_kernel(Xp, 0.2, 1.0, 1e-2)
    yk = y.clone()
    t_spd, (Xs, rs) = timed(lambda: h.dsposv_ir(K, yk))

    def chol64():
        L = K.clone()
        h.dpotrf(L)
        return h.dpotrs(L, yk.clone())

    t_c64, Xc = timed(chol64)
    out["mixed_spd_solve_8192"] = {"s": t_spd, "fp64_cholesky_solve_s": t_c64, "speedup": t_c64 / t_spd,
                                   "iterations": rs["iterations"], "backward_error": rs["backward_error"],
                                   "path": rs["path"], "rel_diff_vs_fp64": float((Xs - Xc).norm() / Xc.norm()),
                                   "matrix": "RBF kernel, lengthscale 0.2, unit variance, + 1e-2 I, n = 8192"}
    del K, Xs, Xc
    torch.cuda.empty_cache()
    # GMRES-IR beyond plain refinement: the benchmark recipe at condition 1e10
    nA = 16384
    Ag = colmajor(nA, nA)
    h.gen_svd_matrix(Ag, 7, nrefl=64, sigma_min=1e-10)
    Bg = colmajor(nA, 4)
    h.fill_normal(Bg, 13)
    t_g, (Xg, rg) = timed(lambda: h.dsgesv_ir(Ag, Bg, fallback=False))
    out["gmres_ir_16384_cond1e10"] = {"s": t_g, "status": rg["status"], "path": rg["path"],
                                     "iterations": rg["iterations"], "gmres_iterations": rg["gmres_iterations"],
                                     "backward_error": rg["backward_error"], "history": rg["history"]}
    # the tournament-pivoting panel in the same mixed solve (benchmark system)
    Ab = colmajor(nA, nA)
    h.gen_svd_matrix(Ab, 3, nrefl=64, sigma_min=1e-6)
    t_t, (Xt, rt) = timed(lambda: h.dsgesv_ir(Ab, Bg, panel=2))
    t_p, _ = timed(lambda: h.dsgesv_ir(Ab, Bg, panel=1))
    out["mixed_solve_panel_pivoting"] = {"partial_s": t_p, "tournament_s": t_t, "tournament_iterations": rt["iterations"],
                                         "tournament_backward_error": rt["backward_error"],
                                         "tournament_pivot_growth": rt["pivot_growth"]}
    del Ag, Bg, Ab, Xg, Xt
    torch.cuda.empty_cache()
    # EVD_Q of the Mat-8.1 snapshot (EVD_QR): symmetric G + G^T, G iid N(0,1) (seed 7)
    for ne in (1024, 4096):
        G7 = colmajor(ne, ne)
        h.fill_normal(G7, 7)
        Sy = (G7 + G7.T).t().contiguous().t()
        Wk = Sy.clone()

        def tridiag():
            Wk.copy_(Sy)
            return h.dtridiag81(Wk)

        t_td, _ = timed(tridiag)
        t_ev, (w, _, Qe) = timed(lambda: h.devd_q(Sy, 1e-11))
        res = (Sy @ Qe - Qe * w).abs().max().item()
        orth = (Qe.T @ Qe - torch.eye(ne, dtype=torch.float64, device="cuda")).abs().max().item()
        out[f"evd_q81_{ne}"] = {"tridiag_with_q_s": t_td, "evd_s": t_ev, "eps": 1e-11,
                                "max_abs_residual_AQ_minus_QE": res, "max_abs_QtQ_minus_I": orth,
                                "flops_model": "tridiagonalisation 4n^3/3 + Q 4n^3/3 (+ the QR sweeps)",
                                "tridiag_with_q_gflops": 8 / 3 * ne ** 3 / t_td / 1e9}
        del G7, Sy, Wk, w, Qe
    torch.cuda.empty_cache()
    return out


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    n, nrhs = args.n, args.nrhs
    for _ in range(args.warmup):
        Aw, Bw = host_system(2048, nrhs)
        cpu_solve(Aw, Bw)
    t0 = time.perf_counter()
    A, B = host_system(n, nrhs)
    gen_s = time.perf_counter() - t0
    ts = []
    cores = 1
    X = None
    for _ in range(args.steps):
        t, cores, X = cpu_solve(A, B)
        ts.append(t)
    v = statistics.mean(ts)
    sample = (f"one whole Solve_direct per step (A copied, PLU, substitutions) on the benchmark system, "
              f"n={n}, {nrhs} RHS, {cores} threads; warm-up steps at n=2048")
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": v * 1e3, "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": bench_config(n, nrhs, world), "method": REF_METHOD,
        "backward_error": backward_error(A, X, B), "step_s": [round(x, 3) for x in ts],
        "input_generation_s": gen_s,
        "cpu_baseline": {"value": v, "unit": "s", "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": v, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def e2e_run(h, A, B, n, nrhs, steps, barrier, warmup=3):
    """The solve through the C ABI from pinned host buffers (the library's
    mg_host_malloc_pinned), two ways, after
    `warmup` untimed steps each (wall clock, max over ranks by the barrier):

    serial: per step the H2D copy of A and B, the solve, the D2H copy of X
      and a synchronize, all on the library's stream (the latency of one
      solve from host memory);
    pipelined (the reported value): a stream of solves as a solver service
      runs them: two device input buffers; step i's solve on one handle's
      stream while step i+1's inputs are copied H2D on a second handle's
      stream (ordered by events), then X read back D2H.  Every step's copies
      are inside the timed region; the first step's copy is not overlapped.

    The H2D share is timed once more with events on the library's stream."""
    import ctypes as C

    import torch

    import numpy as np

    from mat_gb300.api import Handle, colmajor
    lib = h.lib
    pinned = []

    def host_buffer(rows, cols):
        # page-locked host memory from the library (mg_host_malloc_pinned), as a CPU tensor
        p = C.c_void_p()
        h.check(lib.mg_host_malloc_pinned(C.byref(p), 8 * rows * cols), "mg_host_malloc_pinned")
        pinned.append(p)
        arr = np.ctypeslib.as_array((C.c_double * (rows * cols)).from_address(p.value))
        return torch.from_numpy(arr).view(rows, cols)

    hA = host_buffer(n, n)
    hA.copy_(A.t())  # column-major bytes of A in a row-major (n x n) pinned host buffer
    hBt = host_buffer(nrhs, n)
    hBt.copy_(B.t())
    hXt = host_buffer(nrhs, n)
    h2d = 8 * n * n + 8 * n * nrhs
    d2h = 8 * n * nrhs

    def timed_steps(step, nsteps):
        barrier()
        gc.collect()
        gc.disable()  # no collector pass inside the timed steps
        w0 = time.perf_counter()
        per_step = []
        for i in range(nsteps):
            t = time.perf_counter()
            step(i)
            per_step.append((time.perf_counter() - t) * 1e3)
        barrier()
        total = time.perf_counter() - w0
        gc.enable()
        return total / nsteps, per_step

    # serial
    dA, dB, dX = colmajor(n, n), colmajor(n, nrhs), colmajor(n, nrhs)
    hh = h.h

    def serial_step(i):
        h.check(lib.mg_memcpy(hh, C.c_void_p(dA.data_ptr()), C.c_void_p(hA.data_ptr()), 8 * n * n, 0))
        h.check(lib.mg_memcpy(hh, C.c_void_p(dB.data_ptr()), C.c_void_p(hBt.data_ptr()), 8 * n * nrhs, 0))
        h.dsgesv_ir(dA, dB, dX)
        h.check(lib.mg_memcpy(hh, C.c_void_p(hXt.data_ptr()), C.c_void_p(dX.data_ptr()), 8 * n * nrhs, 1))
        h.check(lib.mg_synchronize(hh))

    for i in range(max(1, warmup)):
        serial_step(i)
    serial_s, serial_ms = timed_steps(serial_step, steps)
    c0, c1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    c0.record()
    h.check(lib.mg_memcpy(hh, C.c_void_p(dA.data_ptr()), C.c_void_p(hA.data_ptr()), 8 * n * n, 0))
    c1.record()
    torch.cuda.synchronize()
    h2d_ms = c0.elapsed_time(c1)
    del dA, dB, dX

    # pipelined
    sc, ss = torch.cuda.Stream(), torch.cuda.Stream()
    hc, hs = Handle(sc), Handle(ss)
    dAs = [colmajor(n, n), colmajor(n, n)]
    dBs = [colmajor(n, nrhs), colmajor(n, nrhs)]
    dXs = [colmajor(n, nrhs), colmajor(n, nrhs)]
    ev_in = [torch.cuda.Event(), torch.cuda.Event()]
    ev_done = [torch.cuda.Event(), torch.cuda.Event()]
    for e in ev_done:
        e.record(ss)

    def copy_in(i):
        b = i & 1
        sc.wait_event(ev_done[b])  # the buffer's previous solve has finished
        hc.check(lib.mg_memcpy(hc.h, C.c_void_p(dAs[b].data_ptr()), C.c_void_p(hA.data_ptr()), 8 * n * n, 0))
        hc.check(lib.mg_memcpy(hc.h, C.c_void_p(dBs[b].data_ptr()), C.c_void_p(hBt.data_ptr()), 8 * n * nrhs, 0))
        ev_in[b].record(sc)

    def make_step(nsteps):
        def step(i):
            b = i & 1
            if i == 0:
                copy_in(0)
            if i + 1 < nsteps:
                copy_in(i + 1)  # overlaps this step's solve
            ss.wait_event(ev_in[b])
            hs.dsgesv_ir(dAs[b], dBs[b], dXs[b])
            hs.check(lib.mg_memcpy(hs.h, C.c_void_p(hXt.data_ptr()), C.c_void_p(dXs[b].data_ptr()), 8 * n * nrhs, 1))
            hs.check(lib.mg_synchronize(hs.h))
            ev_done[b].record(ss)
        return step

    warm = make_step(max(1, warmup))
    for i in range(max(1, warmup)):
        warm(i)
    torch.cuda.synchronize()
    pipe_s, pipe_ms = timed_steps(make_step(steps), steps)
    torch.cuda.synchronize()
    hs.close()
    hc.close()
    del dAs, dBs, dXs, hA, hBt, hXt
    for p in pinned:
        lib.mg_host_free_pinned(p)
    torch.cuda.empty_cache()
    return {"value": pipe_s, "unit": "s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
            "pipelined": True, "step_ms": [round(x, 2) for x in pipe_ms],
            "median_step_ms": round(_median(pipe_ms), 2),
            "serial": {"value": serial_s, "step_ms": [round(x, 2) for x in serial_ms],
                       "median_step_ms": round(_median(serial_ms), 2),
                       "note": "H2D, solve, D2H back to back per step: the latency of one solve from host memory"},
            "note": "value is the mean over the timed steps, slow host copies included; median_step_ms beside it",
            "h2d_ms": h2d_ms, "h2d_gbs": 8 * n * n / (h2d_ms * 1e6)}


def _median(xs):
    v = sorted(xs)
    m = len(v) // 2
    return v[m] if len(v) % 2 else 0.5 * (v[m - 1] + v[m])


def run_ours(args):
    import torch
    import torch.distributed as dist

    from mat_gb300.api import Handle, colmajor

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl")
    h = Handle()
    n, nrhs = args.n, args.nrhs
    hbm, bf16, bf16s, peak_kind = peaks()

    # inputs resident in HBM (replicas: each rank its own seed)
    A = colmajor(n, n)
    h.gen_svd_matrix(A, 3 + rank, nrefl=64, sigma_min=1e-6)
    B = colmajor(n, nrhs)
    h.fill_normal(B, 11 + rank)
    X = colmajor(n, nrhs)
    torch.cuda.synchronize()

    for _ in range(max(3, args.warmup)):
        h.dsgesv_ir(A, B, X)
    torch.cuda.synchronize()

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    # one profiled step outside the timed region: every phase's share, and
    # the dominant kernel family for the roofline
    h.profile(True)
    h.dsgesv_ir(A, B, X)
    prof_all = h.profile_records()
    h.profile(False)
    dom_name = max(prof_all.items(), key=lambda kv: kv[1]["ms"])[0]
    phases = {k: {"ms_per_step": v["ms"], "launches_per_step": v["launches"]}
              for k, v in sorted(prof_all.items(), key=lambda kv: -kv[1]["ms"])}

    # the timed region, without any per-phase events (they would perturb it)
    gc.collect()
    gc.disable()  # no collector pass inside the timed region
    sampler = ClockSampler(local)
    sampler.start()
    launches0 = h.launch_count()
    reps = []
    barrier()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        Xs, rep = h.dsgesv_ir(A, B, X)
        reps.append(rep)
    e1.record()
    barrier()
    launches = h.launch_count() - launches0
    clocks = sampler.stop()
    gc.enable()
    ms = e0.elapsed_time(e1) / args.steps
    t = torch.tensor([ms], device="cuda", dtype=torch.float64)
    if world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    ms = float(t.item())

    # the same steps again with CUDA events around the dominant family's
    # launches only (on the streams they run on): its live per-launch time
    # for the roofline, and the step time as perturbed by those events
    h.profile(True, only=dom_name)
    p0 = torch.cuda.Event(enable_timing=True)
    p1 = torch.cuda.Event(enable_timing=True)
    p0.record()
    for _ in range(args.steps):
        h.dsgesv_ir(A, B, X)
    p1.record()
    torch.cuda.synchronize()
    prof = h.profile_records()
    h.profile(False)
    ms_profiled = p0.elapsed_time(p1) / args.steps

    # end to end through the C ABI: host buffers, copies inside the timed region
    e2e = None
    if not args.no_e2e:
        e2e = e2e_run(h, A, B, n, nrhs, args.steps, barrier, args.warmup)

    # the FP64 half of the metric: plain FP64 GPU solve of the same system, and accuracy
    torch.cuda.synchronize()
    f0 = time.perf_counter()
    Xd, info = h.dgesv(A, B)
    torch.cuda.synchronize()
    fp64_s = time.perf_counter() - f0
    fwd = float((X - Xd).norm() / Xd.norm())

    # DGEMM TFLOP/s at M=N=K=1024 (row-major uniform [-1,1) seeds 0/1, stored column-major)
    m = 1024
    Ga, Gb = colmajor(m, m), colmajor(m, m)
    h.fill_uniform(Ga, 0)
    h.fill_uniform(Gb, 1)
    Gc = h.dgemm(Ga, Gb)
    for _ in range(5):
        h.dgemm(Ga, Gb, Gc)
    torch.cuda.synchronize()
    g0, g1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    g0.record()
    for _ in range(20):
        h.dgemm(Ga, Gb, Gc)
    g1.record()
    torch.cuda.synchronize()
    dgemm_ms = g0.elapsed_time(g1) / 20
    dgemm_tf = 2 * m ** 3 / dgemm_ms / 1e9
    dfma_tf, dmma_tf = h.measure_fp64_peaks()

    # roofline of the dominant kernel, from its launches inside the timed region
    dom = prof[dom_name]
    tensor = dom["flops"] > 0 and dom_name in ("gemm_bf16x",)
    traffic = None
    tf = ROOT / "profiles" / "traffic_per_launch.txt"
    if tf.exists():
        for ln in tf.read_text().splitlines():
            parts = ln.split()
            if len(parts) == 2 and not ln.startswith("#") and parts[0] == dom_name:
                traffic = float(parts[1])
    if tensor:
        achieved = dom["flops"] / (dom["ms"] * 1e-3) / 1e12
        roof = {"kernel": dom_name, "bound": "tensor", "achieved": achieved, "peak": bf16s, "unit": "TFLOP/s",
                "frac": achieved / bf16s, "peak_kind": f"bf16 sustained ({peak_kind})", "traffic": traffic,
                "launches": dom["launches"], "ms_total": dom["ms"], "ms_per_step_with_events": ms_profiled}
    else:
        achieved = dom["bytes"] / (dom["ms"] * 1e-3) / 1e9
        roof = {"kernel": dom_name, "bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                "frac": achieved / hbm, "peak_kind": f"hbm copy ({peak_kind})", "traffic": traffic,
                "launches": dom["launches"], "ms_total": dom["ms"], "ms_per_step_with_events": ms_profiled}


    # the CPU baseline on the same system: the oracle's host copy of A and B
    # (checked equal to the GPU's bit for bit), one whole FP64 Solve_direct on
    # all host cores, whose solution is also compared with the FP64 GPU solve
    cpu = None
    if rank == 0 and not args.no_cpu:
        import numpy as np
        hA, hB = host_system(n, nrhs, 3 + rank, 11 + rank)
        same_A = bool(torch.equal(torch.from_numpy(hA).to("cuda"), A))
        same_B = bool(torch.equal(torch.from_numpy(hB).to("cuda"), B))
        t_cpu, cores, Xc = cpu_solve(hA, hB)
        cpu = {"value": t_cpu, "unit": "s", "cores": cores, "kind": "port",
               "sample": f"one whole oracle Solve_direct (Mat's FP64 narrow path) of the benchmark system, n={n}, "
                         f"{nrhs} RHS, {cores} threads",
               "input_equals_gpu_input": same_A and same_B,
               "fp64_gpu_solve_equals_oracle": bool(np.array_equal(Xd.cpu().numpy(), Xc)),
               "backward_error": backward_error(hA, Xc, hB)}
        del hA, hB, Xc

    configs = None
    if rank == 0 and not args.no_configs:
        configs = config_rates(h, max(dmma_tf, dfma_tf), bf16)

    if rank == 0:
        last = reps[-1]
        line = {
            "metric": METRIC, "value": ms / 1e3, "unit": "s", "n_gpus": world, "steps": args.steps,
            "warmup": max(3, args.warmup), "ms_per_step": ms, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "fp32/bf16x3 factor + f64 refinement", "data": "synthetic",
            "config": bench_config(n, nrhs, world), "method": METHOD,
            "fp64_solve_s": fp64_s, "mixed_vs_fp64": (ms / 1e3) / fp64_s,
            "backward_error": last["backward_error"], "iterations": last["iterations"], "path": last["path"],
            "forward_error_vs_fp64_solve": fwd, "pivot_growth": last.get("pivot_growth"),
            "dgemm": {"config": "M=N=K=1024 fp64, uniform[-1,1) seeds 0/1", "ms": dgemm_ms, "tflops": dgemm_tf,
                      "fp64_dmma_peak_tflops": dmma_tf, "fp64_dfma_peak_tflops": dfma_tf,
                      "frac_of_fp64_peak": dgemm_tf / max(dmma_tf, dfma_tf)},
            "roofline": roof, "phases": phases, "cpu_baseline": cpu, "e2e": e2e,
            "gpu_launches": launches, "clocks": clocks, "configs": configs,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
