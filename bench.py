#!/usr/bin/env python
"""Benchmark: plain 2D CG-SENSE solves per second on one GB300.

Workload (the reference metric's configuration): cgne, 30 iterations, image
256 x 256 complex64 random-ellipse phantom, 32 ring-of-Gaussian coil maps
with linear phase, variable-density spiral 4 interleaves x 4096 samples at
R = 4, Kaiser-Bessel width 4, oversampling 2 (512 x 512 grid), FP32
operators with FP64 CG scalars.  cgne runs with xChangeThresh = [] and
resThresh = [] so that exactly 30 iterations run (1 adjoint + 32 normal
operators per solve).  Inputs are seeded synthetic data of these shapes.

A step is one full solve.  `value` times solves with the k-space data already
in HBM (device pointers through the C ABI); `e2e` times the same solve
through the C ABI with pinned HOST buffers (the data [16384 x 32] complex64
copied in and the image [256 x 256] copied out inside the timed region).
Between timed steps the L2 is flushed by writing a 512 MiB buffer (outside
the per-step events).  `--impl reference` times the reference algorithm's CPU
restatement on the host cores.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "uwobrainhack2026-matmri_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

N_IMG, N_COIL, N_INT, N_SAMP, ACCEL = 256, 32, 4, 4096, 4.0
NIT = 30
METRIC = "CG-SENSE solves/s (cgne 30 it, 256^2, 32 coils, 4x4096 spiral R=4)"
WORKLOAD = "cg-sense 256x256, 32 coils, 4x4096 spiral R=4, kwidth 4, os 2, 30 cgne iterations"
# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of one launch of the fused gridding kernel
# on this workload, from one ncu capture per (coil chunk, tile, coils per CTA): with 16 coils per
# launch the grids stay L2-resident, with 32 part of them comes from DRAM
GRIDNORM_DRAM_BYTES = {(16, 32, 2): 31.92e6, (32, 32, 2): 87.87e6, (32, 16, 4): 84.75e6}


def normal_op_model_bytes(C, N, G, M):
    """Algorithmic bytes of one 2D normal operator A'A (complex64): maps fwd+adj, two FFT passes x
    (read+write) x 2 directions over the grid, samples in+out per coil; image in/out; trajectory."""
    return C * (2 * N * N * 8 + 8 * G * G * 8 + 2 * M * 8) + 2 * N * N * 8 + 2 * M * 8


# 1 adjoint (half a normal operator) + 31 normal operators per 30-iteration solve
SOLVE_MODEL_BYTES = 31.5 * normal_op_model_bytes(N_COIL, N_IMG, 2 * N_IMG, N_INT * N_SAMP)
NORMALS_PER_SOLVE = NIT + 2          # initial residual + explicit residual at nit=0 + 30 iterations
ADJOINTS_PER_SOLVE = 1


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


# Replicas: every rank solves its own independent case (its own seed), no data-path collective;
# the timed region is bracketed by barriers and the job time is the slowest rank's.
def replica_seed(rank):
    return 2000 + rank


def max_over_ranks(v, ws, device):
    if ws > 1:
        import torch
        import torch.distributed as dist
        t = torch.tensor([v], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())
    return v


def job_rate(ws, steps, t_max):
    """Whole-job solves/s: every rank did `steps` solves in at most t_max seconds."""
    return ws * steps / t_max


def make_case(seed=2000):
    from matmri_gb300 import synth
    c = synth.sense_case(N_IMG, N_COIL, N_INT, N_SAMP, ACCEL, seed=seed)
    return c


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons during the timed region."""

    def __init__(self, index):
        self.index = index
        self.rows = []
        self.proc = None

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "20"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            # the timed region is short: start it only once the sampler is producing rows (at most 3 s)
            t0 = time.perf_counter()
            while not self.rows and time.perf_counter() - t0 < 3.0 and self.proc.poll() is None:
                time.sleep(0.01)
            self.rows.clear()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [s.strip() for s in line.split(",")]
            if len(parts) >= 7:
                self.rows.append(parts)

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if r[3 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def cpu_solver(case, cores):
    """The reference algorithm's CPU path, restated in FP64 (oracle/): cgne (cgne.m:135-340) over
    mrSampFunc with a nufftOp (scipy.sparse interpolation matrix, scipy.fft) and an rcvrOp, the coils
    split over `cores` host threads.  Returns (solve(), close())."""
    import oracle.nufft_ref as nr
    from oracle.sense_ref import CoilParallelSense, cgne_ref
    nr.FFT_WORKERS = 1                                 # the threads split the coils; one FFT worker each
    S = nr.NufftRef([N_IMG, N_IMG], case["kloc"], None, 2.0, 4)
    A = CoilParallelSense(S, case["maps"], cores)
    data = A(case["img"].astype(np.complex128), "notransp")
    opt = {"xChangeThresh": None, "resThresh": None}

    def solve():
        # b = A'y, x0 = b, the initial residual, nit-0 explicit residual and 30 iterations:
        # 1 adjoint + 32 normal operators, the same work the GPU arm's solve does
        x, res_sq, *_ = cgne_ref(A, data, None, NIT, opt)
        assert len(res_sq) == NIT + 1
        return x

    return solve, A.close


def cpu_baseline(case, solves=2):
    """Timed full 30-iteration cgne solves of the FP64 CPU restatement on all host cores (a bounded
    sample: `solves` solves after one untimed warm-up solve)."""
    cores = len(os.sched_getaffinity(0))
    solve, close = cpu_solver(case, cores)
    solve()
    t0 = time.perf_counter()
    for _ in range(solves):
        solve()
    t = (time.perf_counter() - t0) / solves
    close()
    return {"value": 1.0 / t, "unit": "solves/s", "cores": cores, "kind": "port",
            "sample": f"{solves} full cgne solves timed (30 iterations: 1 adjoint + {NORMALS_PER_SOLVE} normal "
                      f"operators each) of the FP64 restatement, coils split over {cores} threads "
                      f"(scipy.sparse gridding, scipy.fft); {t:.2f} s per solve"}


LEARNED_SEED = 5000          # held out: training seeds start at 100000, validation at 200000
NRMSE_TARGET = 1e-3


def learned_pcg_comparison(dev, reps=5):
    """Time to NRMSE <= 1e-3 against the converged image: learned-PCG vs plain CG.

    Workload: 256 x 256, 32 randomised coil maps, 4 x 4096 spiral R = 4, SNR 30, the
    Tikhonov-regularised system the preconditioner was trained for ((A'A + lam) x = A'y, cgne with
    gam = lam, R = 1).  The converged image is plain CG run 300 + 100 iterations (its drift over the
    last 100 is reported).  Iteration counts come from the error histories (opt.gtruth); the times are
    then taken for solves of exactly that many iterations from device-resident data.
    """
    import torch
    import matmri_gb300 as mm
    from matmri_gb300 import synth
    from matmri_gb300.learned import PrecondNet, iterations_to, lpcg
    from matmri_gb300 import train_precond as tp
    if not os.path.exists(tp.WEIGHTS):
        return {"unavailable": "no trained weights at " + os.path.relpath(tp.WEIGHTS, ROOT)}
    meta = np.load(tp.WEIGHTS)
    lam = float(meta["lam"])
    net = PrecondNet.load(tp.WEIGHTS)
    c = synth.sense_case(N_IMG, N_COIL, N_INT, N_SAMP, ACCEL, seed=LEARNED_SEED, randomize_coils=True)
    S = mm.nufftOp([N_IMG, N_IMG], c["kloc"], None, 1, 2.0, 4)
    R = mm.rcvrOp(c["maps"], 0)
    A = mm.mrSampOp(S, R)
    from matmri_gb300.autotune import autotune
    autotune(A, rounds=1, use_cache=False)      # the fastest normal operator for both solvers
    y = np.asarray(A(c["img"].astype(np.complex64), "notransp"), dtype=np.complex128)
    y = synth.add_noise(y, 30.0, LEARNED_SEED + 7).astype(np.complex64)
    yd = torch.from_numpy(np.ascontiguousarray(y.T)).to(dev).T
    xs, _, _, _ = lpcg(A, yd, None, NitMax=300, lam=lam)
    xs2, _, _, _ = lpcg(A, yd, None, x0=xs, NitMax=100, lam=lam)
    drift = float(torch.linalg.norm(xs2 - xs) / torch.linalg.norm(xs2))
    xs = xs2
    gn = float(torch.linalg.norm(xs))
    zeros = torch.zeros_like(xs)
    opt = {"resThresh": None, "xChangeThresh": None}
    _, _, mse, _, _, _, _ = mm.cgne(A, yd, zeros, 150, dict(opt, gtruth=xs), lam, 1.0)
    k_cgne = iterations_to(mse, gn, NRMSE_TARGET)
    _, _, err_p, _ = lpcg(A, yd, None, NitMax=150, lam=lam, gtruth=xs)
    k_plain = iterations_to(err_p, gn, NRMSE_TARGET)
    _, _, err_l, info = lpcg(A, yd, net, NitMax=150, lam=lam, gtruth=xs)
    k_learn = iterations_to(err_l, gn, NRMSE_TARGET)
    if None in (k_cgne, k_plain, k_learn):
        return {"unavailable": f"target not reached within 150 iterations (cgne {k_cgne}, plain {k_plain}, "
                               f"learned {k_learn})"}
    st = torch.cuda.current_stream(dev)

    def timed(fn):
        for _ in range(2):
            fn()
        ts = []
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record(st)
            fn()
            e1.record(st)
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1))
        return statistics.median(ts)

    t_cgne = timed(lambda: mm.cgne(A, yd, zeros, k_cgne, opt, lam, 1.0))
    t_plain = timed(lambda: lpcg(A, yd, None, NitMax=k_plain, lam=lam))
    x_l = None

    def run_learned():
        nonlocal x_l
        x_l, _, _, _ = lpcg(A, yd, net, NitMax=k_learn, lam=lam)

    t_learn = timed(run_learned)
    nrmse_l = float(torch.linalg.norm(x_l - xs)) / gn
    t_plain_best = min(t_cgne, t_plain)
    return {"workload": "cg-sense 256x256, 32 randomised coils, 4x4096 spiral R=4, SNR 30, Tikhonov lam = "
                        f"{float(meta['lam_rel']):g} lambda_max(A'A), x0 = 0, seed {LEARNED_SEED} (held out)",
            "nrmse_target": NRMSE_TARGET, "reference_drift": drift,
            "plain_cgne_iters": k_cgne, "plain_cgne_ms": t_cgne,
            "plain_fcg_iters": k_plain, "plain_fcg_ms": t_plain,
            "learned_iters": k_learn, "learned_ms": t_learn, "learned_nrmse": nrmse_l,
            "learned_fell_back_at": info["fell_back_at"], "learned_true_res_rel": info["true_res_rel"],
            "time_ratio_vs_best_plain": t_learn / t_plain_best, "network": os.path.relpath(tp.WEIGHTS, ROOT)}


def batched_comparison(dev, nit=25, reps=3):
    """64 uneven CG-SENSE slices (N in {96,128,192,256}, C in {8,16,32}, 2-8 interleaves x 2048-4096
    samples, own spiral each), cgne with 25 iterations each: the batch advanced by one CUDA graph per
    iteration (every slice a parallel branch; launch shapes autotuned once per (N, C) class) against
    the same 64 solves issued one after another."""
    import torch
    import matmri_gb300 as mm
    from matmri_gb300 import synth
    from matmri_gb300.autotune import autotune
    cases = synth.batched_cases(64)
    ops, ys, classes = [], [], {}
    t0 = time.perf_counter()
    for c in cases:
        N = c["N"]
        A = mm.mrSampOp(mm.nufftOp([N, N], c["kloc"], None, 1, 2.0, 4), mm.rcvrOp(c["maps"], 0))
        y = np.asarray(A(c["img"].astype(np.complex64), "notransp"))
        ys.append(torch.from_numpy(np.ascontiguousarray(y.T)).to(dev).T)
        key = (N, c["C"])
        if key not in classes:
            classes[key] = autotune(A, rounds=1, use_cache=False)
        else:
            A.set_tuning(**classes[key])
        ops.append(A)
    setup_s = time.perf_counter() - t0
    opt = {"resThresh": None, "xChangeThresh": None}
    st = torch.cuda.current_stream(dev)

    def timed(fn):
        fn()
        ts = []
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record(st)
            fn()
            e1.record(st)
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1))
        return statistics.median(ts)

    t_batch = timed(lambda: mm.cgne_batch(ops, ys, nit, opt))
    t_seq = timed(lambda: [mm.cgne(A, y, None, nit, opt) for A, y in zip(ops, ys)])
    return {"workload": "64 uneven cg-sense slices, N in {96,128,192,256}, C in {8,16,32}, 2-8 interleaves x "
                        f"2048-4096 samples, {nit} cgne iterations each, kwidth 4, os 2",
            "slices": len(ops), "size_classes": len(classes), "batched_ms": t_batch, "sequential_ms": t_seq,
            "slices_per_s": len(ops) / (t_batch / 1e3), "speedup_vs_sequential": t_seq / t_batch,
            "setup_s": setup_s}


def _timed_ms(fn, reps, dev):
    import torch
    st = torch.cuda.current_stream(dev)
    for _ in range(3):
        fn()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(st)
    for _ in range(reps):
        fn()
    e1.record(st)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def _dev_cm(a, dev):
    """Column-major complex64 device tensor of a numpy array."""
    import torch
    a = np.asarray(a, dtype=np.complex64)
    if a.ndim < 2:
        return torch.from_numpy(a).to(dev)
    rev = tuple(range(a.ndim - 1, -1, -1))
    return torch.from_numpy(np.ascontiguousarray(a.transpose(rev))).to(dev).permute(rev)


def regridding_measure(dev, reps=200):
    """128 x 128 single-coil regridding (16 x 2048 spiral, kwidth 4, os 2, |k| density compensation,
    SNR 50): microseconds per adjoint + forward pair on device-resident data, its error against the
    FP64 restatement, and the restatement's own time on the host cores."""
    import matmri_gb300 as mm
    from matmri_gb300 import synth
    import oracle.nufft_ref as nr
    c = synth.regridding_case()
    N = c["N"]
    S = mm.nufftOp([N, N], c["kloc"], c["dcf"], 1, c["os"], c["kwidth"])
    Sr = nr.NufftRef([N, N], c["kloc"], c["dcf"], c["os"], c["kwidth"])
    y = synth.add_noise(Sr.mtimes(c["img"]), c["snr"], c["seed"] + 1)
    yd = _dev_cm(y, dev)
    SH = S.H
    us = 1e3 * _timed_ms(lambda: S * (SH * yd), reps, dev)
    x_gpu = (SH * yd).cpu().numpy()
    t0 = time.perf_counter()
    x_ref = Sr.H.mtimes(y)
    y_ref = Sr.mtimes(x_ref)
    t_cpu = time.perf_counter() - t0
    y_gpu = (S * _dev_cm(x_ref, dev)).cpu().numpy()
    err_adj = float(np.linalg.norm(x_gpu - x_ref) / np.linalg.norm(x_ref))
    err_fwd = float(np.linalg.norm(y_gpu - y_ref) / np.linalg.norm(y_ref))
    return {"workload": "regridding 128x128, 16x2048 spiral, kwidth 4, os 2, |k| dcf, 1 coil, SNR 50",
            "us_per_adjoint_forward": us, "rel_err_adjoint_vs_fp64": err_adj, "rel_err_forward_vs_fp64": err_fwd,
            "cpu_fp64_us_per_pair": t_cpu * 1e6, "cpu_cores": len(os.sched_getaffinity(0))}


def toeplitz_measure(dev, reps=20, cpu_coils=4):
    """Toeplitz normal operator (nufftOp.prepToep, nufftOp.m:410-432 and 348-352) on the 256 x 256,
    32-coil, 4 x 4096 spiral case: microseconds per 32-coil S*x of the Toeplitz copy, beside the
    gridding normal operator S'*(S*x) of the same batch; the Toeplitz transfer function's set-up
    time; its error against the FP64 restatement on `cpu_coils` coils and the restatement's time
    for those coils on the host cores (set-up and application)."""
    import matmri_gb300 as mm
    import oracle.nufft_ref as nr
    case = make_case()
    kloc, img, maps = case["kloc"], case["img"], case["maps"]
    S = mm.nufftOp([N_IMG, N_IMG], kloc, None, 1, 2.0, 4)
    t0 = time.perf_counter()
    T = S.prepToep()
    setup_s = time.perf_counter() - t0
    x = (img[:, :, None] * maps).astype(np.complex64)
    xd = _dev_cm(x, dev)
    SH = S.H
    us_toep = 1e3 * _timed_ms(lambda: T * xd, reps, dev)
    us_grid = 1e3 * _timed_ms(lambda: SH * (S * xd), reps, dev)
    yt = (T * xd).cpu().numpy()
    yg = (SH * (S * xd)).cpu().numpy()
    t0 = time.perf_counter()
    Tr = nr.NufftRef([N_IMG, N_IMG], kloc, None, 2.0, 4).prepToep()
    yr = Tr.mtimes(x[:, :, :cpu_coils])
    t_cpu = time.perf_counter() - t0
    err = float(np.linalg.norm(yt[:, :, :cpu_coils] - yr) / np.linalg.norm(yr))
    gap = float(np.linalg.norm(yt - yg) / np.linalg.norm(yg))
    return {"workload": "Toeplitz normal operator 256x256 (2N = 512 transfer function), 32 coils, "
                        "4x4096 spiral R=4, kwidth 4, os 2 (tos 1.5)",
            "us_toeplitz_32coils": us_toep, "us_gridding_normal_32coils": us_grid,
            "speedup_vs_gridding": us_grid / us_toep, "setup_s": setup_s,
            "rel_err_vs_fp64": err, "rel_diff_toeplitz_vs_gridding": gap,
            "cpu_fp64_s_setup_plus_apply": t_cpu, "cpu_coils": cpu_coils,
            "cpu_cores": len(os.sched_getaffinity(0))}


def highorder_measure(dev, reps=5, nit=30):
    """High-order encoding: 128 x 128, single-shot spiral of 16384 samples, 16 spherical-harmonic
    terms, B0 +-100 Hz, 30 ms readout, 16 coils.  Times the 16-coil S*x and S'*y and a cgne solve of
    `nit` iterations on device-resident data; error of S*x against the exact FP64 sum on 256 samples."""
    import matmri_gb300 as mm
    from matmri_gb300 import synth
    from oracle.sho_ref import ShoRef
    b0, t, spha, conc, grid = synth.highorder_inputs(128, 16384)
    S = mm.sampHighOrder(b0, t, spha, conc, grid)
    maps = synth.coil_maps(128, 16, 3001)
    A = mm.mrSampOp(S, mm.rcvrOp(maps, 0))
    img = synth.ellipse_phantom(128, 10, 3002, complex_phase=True)
    xd = _dev_cm(img, dev)
    yd = A(xd, "notransp")
    ms_fwd = _timed_ms(lambda: A(xd, "notransp"), reps, dev)
    ms_adj = _timed_ms(lambda: A(yd, "transp"), reps, dev)
    opt = {"resThresh": None, "xChangeThresh": None}
    ms_solve = _timed_ms(lambda: mm.cgne(A, yd, None, nit, opt), 2, dev)
    # exact FP64 S*x (one coil image) on a sample subset
    xs = img * maps[:, :, 0]
    ys = (S * _dev_cm(xs, dev)).cpu().numpy()
    ref = ShoRef(b0, t, spha, conc, grid)
    rng = np.random.default_rng(7)
    ms_idx = np.sort(rng.choice(t.size, 256, replace=False))
    xv = xs.reshape(-1, order="F")
    B, P = ref.basis_matrix()
    exact = np.exp(1j * (B @ P[:, ms_idx])).T @ xv / math.sqrt(xv.size)     # sampHighOrder.m:376, 387
    rel = float(np.linalg.norm(ys.reshape(-1)[ms_idx] - exact) / np.linalg.norm(exact))
    V, M, C = img.size, t.size, 16
    # approach 1 (SVD + NUFFT interpolation, reference defaults svdThresh 0.05, subFact 5) on the same inputs
    t0 = time.perf_counter()
    S1 = mm.sampHighOrder(b0, t, spha, conc, grid, None, 1, 0, 1)
    plan_s = time.perf_counter() - t0
    A1 = mm.mrSampOp(S1, mm.rcvrOp(maps, 0))
    ms1_fwd = _timed_ms(lambda: A1(xd, "notransp"), reps, dev)
    ms1_adj = _timed_ms(lambda: A1(yd, "transp"), reps, dev)
    ms1_solve = _timed_ms(lambda: mm.cgne(A1, yd, None, nit, opt), 2, dev)
    ys1 = (S1 * _dev_cm(xs, dev)).cpu().numpy()
    rel1 = float(np.linalg.norm(ys1.reshape(-1)[ms_idx] - exact) / np.linalg.norm(exact))
    return {"workload": "sampHighOrder 128x128, 16384-sample spiral, 16 SH terms, B0 +-100 Hz, 30 ms, 16 coils",
            "ms_forward_16coils": ms_fwd, "ms_adjoint_16coils": ms_adj,
            "tflops_forward": 8.0 * V * M * C / (ms_fwd * 1e-3) / 1e12,
            "ms_cgne_solve": ms_solve, "iterations": nit, "solves_per_s": 1e3 / ms_solve,
            "rel_err_forward_vs_fp64_256_samples": rel,
            "interpolated": {"svd_terms": int(S1.svdTime.shape[1]), "plan_s_host": plan_s,
                             "ms_forward_16coils": ms1_fwd, "ms_adjoint_16coils": ms1_adj,
                             "ms_cgne_solve": ms1_solve, "solves_per_s": 1e3 / ms1_solve,
                             "rel_err_forward_vs_fp64_256_samples": rel1}}


def highorder_profile_case(dev, apps=2):
    """Profiling case for the high-order encoding kernels: the operator of highorder_measure
    (128 x 128, 16384-sample spiral, 16 SH terms) applied `apps` times forward and adjoint to
    16 coil images; prints one line."""
    import matmri_gb300 as mm
    from matmri_gb300 import synth
    import torch
    b0, t, spha, conc, grid = synth.highorder_inputs(128, 16384)
    S = mm.sampHighOrder(b0, t, spha, conc, grid)
    rng = np.random.default_rng(5)
    x = (rng.standard_normal((128, 128, 16)) + 1j * rng.standard_normal((128, 128, 16))).astype(np.complex64)
    xd = _dev_cm(x, dev)
    yd = S * xd
    for _ in range(apps):
        yd = S * xd
        S.H * yd
    torch.cuda.synchronize(dev)
    print("highorder profile case: %d forward + %d adjoint 16-coil applications" % (apps + 1, apps), flush=True)


def dense_profile_case(dev, n_img=64, M=4096, C=8):
    """Profiling case for the dense Gram kernel: mrSampFuncMat at n_img x n_img voxels, M samples,
    C coils, full mask, built twice; prints one line."""
    import torch
    import matmri_gb300 as mm
    from matmri_gb300 import synth
    b0, t, spha, conc, grid = synth.highorder_inputs(n_img, M)
    maps = synth.coil_maps(n_img, C, 3001)
    rng = np.random.default_rng(9)
    y = (rng.standard_normal((M, C)) + 1j * rng.standard_normal((M, C))).astype(np.complex64)
    for _ in range(2):
        AtA, _ = mm.mrSampFuncMat(y, maps, b0, t, spha, conc, grid)
    torch.cuda.synchronize(dev)
    print("dense profile case: %d x %d Gram over %d samples, built twice" % (AtA.shape[0], AtA.shape[1], M),
          flush=True)


def finddel_measure(dev, cpu=True):
    """findDelAuto (delay between a field trajectory and the data): wall time of a whole estimation on
    the GPU at 64 x 64, 8 coils, 4096 samples, maxNit 15 (data simulated by the device encoding at a
    0.37-dwell delay), and on a 32 x 32, 4-coil, 2048-sample case both on the GPU and with the FP64
    restatement on the host cores."""
    import torch
    import matmri_gb300 as mm
    from matmri_gb300 import synth

    def case(N, C, M, delay=0.37):
        c = synth.finddel_inputs(N, C, M, 3.0, 6.0, 7)
        dt = c["datatime"]
        S = mm.sampHighOrder(c["b0"], dt, c["phases"](dt + delay).T, np.zeros((4, M)), c["grid"])
        data = mm.mrSampOp(S, mm.rcvrOp(c["maps"], 0))(c["img"], "notransp")
        return c, np.asarray(data)

    def run(c, data, impl):
        args = (data, c["tdwell"], c["traj"], c["conc"], c["datatime"], c["grid"], c["b0"], c["maps"], 15)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        d, hist = impl(0.0, *args)
        torch.cuda.synchronize()
        return time.perf_counter() - t0, float(d), len(hist)

    out = {"workload": "findDelAuto, maxNit 15, coarse search +-2 dwells, delay 0.37 dwell"}
    c, data = case(64, 8, 4096)
    run(c, data, mm.findDelAuto)                        # warm-up (library load, first plans)
    s, d, n = run(c, data, mm.findDelAuto)
    out["gpu_64x64_8coils_4096"] = {"s": s, "delay": d, "iterations": n - 1}
    c, data = case(32, 4, 2048)
    s, d, n = run(c, data, mm.findDelAuto)
    small = {"gpu_s": s, "delay": d, "iterations": n - 1}
    if cpu:
        from oracle.finddel_ref import find_del_auto
        s, d, n = run(c, data, find_del_auto)
        small.update(cpu_s=s, cpu_delay=d, cpu_iterations=n - 1, cores=len(os.sched_getaffinity(0)),
                     cpu_kind="port (FP64 restatement)")
    out["32x32_4coils_2048"] = small
    return out


def dense_measure(dev, cpu=True):
    """mrSampFuncMat at 128 x 128, 16384 samples, 16 coils (full mask): time to build the dense normal
    matrix (16384^2 complex64; the Gram is 8 V^2 M = 35.2 TFLOP), its error against the iterative normal
    operator on one image, and one Tikhonov direct solve; the host restatement's Gram time is measured on
    a 1024-column slice and scaled to the full matrix."""
    import torch
    import matmri_gb300 as mm
    from matmri_gb300 import synth
    N, M, C = 128, 16384, 16
    b0, t, spha, conc, grid = synth.highorder_inputs(N, M)
    maps = synth.coil_maps(N, C, 3001)
    img = synth.ellipse_phantom(N, 10, 3002, complex_phase=True)
    A = mm.mrSampOp(mm.sampHighOrder(b0, t, spha, conc, grid), mm.rcvrOp(maps, 0))
    y = A(_dev_cm(img, dev), "notransp")
    t_build = []
    for _ in range(2):                                 # the first call also loads the cuBLAS kernels
        AtA = None
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        AtA, Aty = mm.mrSampFuncMat(y, maps, b0, t, spha, conc, grid)
        torch.cuda.synchronize()
        t_build.append(time.perf_counter() - t0)
    t_cold, t_build = t_build
    x = _dev_cm(img, dev)
    ref = A(A(x, "notransp"), "transp").T.reshape(-1)
    got = AtA @ x.T.reshape(-1)
    err = float(torch.linalg.vector_norm(got - ref) / torch.linalg.vector_norm(ref))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    xs, method = mm.dense_solve(AtA, Aty, 1e-2)
    torch.cuda.synchronize()
    t_solve = time.perf_counter() - t0
    V = N * N
    out = {"workload": "mrSampFuncMat 128x128, 16384 samples, 16 coils, full mask; (AtA + 1e-2 I) \\ Aty",
           "s_build": t_build, "s_build_first_call": t_cold, "tflops_gram": 8.0 * V * V * M / t_build / 1e12,
           "rel_err_vs_operator": err,
           "s_solve": t_solve, "solve_method": method}
    del AtA, xs
    torch.cuda.empty_cache()
    if cpu:
        from oracle.sho_ref import ShoRef
        ref = ShoRef(b0, t, spha, conc, grid)
        B, P = ref.basis_matrix()
        t0 = time.perf_counter()
        Ef = np.exp(1j * (B @ P[:, :2048]))            # all voxels x 2048 samples
        t_e = time.perf_counter() - t0
        t0 = time.perf_counter()
        G = Ef[:1024].conj() @ Ef.T                    # 1024 rows of the Gram over 2048 samples
        t_g = time.perf_counter() - t0
        out["cpu"] = {"s_build_extrapolated": t_e * (M / 2048) + t_g * (V / 1024) * (M / 2048),
                      "sample": "FP64 numpy: the phases and exponentials of 2048 samples and a 1024 x 16384 x 2048 "
                                "slice of the Gram, scaled to 16384 x 16384 x 16384",
                      "cores": len(os.sched_getaffinity(0)), "kind": "port"}
        del Ef, G
    return out


def config_dict(ws):
    """The workload description both arms print (the GPU arm's launch shapes go under `tuning`)."""
    return {"workload": WORKLOAD, "image": [N_IMG, N_IMG], "coils": N_COIL, "samples": N_INT * N_SAMP,
            "interleaves": N_INT, "acceleration": ACCEL, "iterations": NIT, "kwidth": 4, "os": 2.0,
            "grid": [2 * N_IMG, 2 * N_IMG],
            "l2": "GPU arm: flushed between timed steps (512 MiB write, outside the per-step events)",
            "parallelism": f"replicas x{ws}"}


# Wall-clock budget of the reference arm (warm-up + timed solves); beyond it fewer timed solves run
# than requested, and the line says how many.
REFERENCE_BUDGET_S = 300.0


def run_reference(args):
    """The reference algorithm's CPU path (FP64 restatement, all host cores), one full 30-iteration
    cgne solve per step."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    t_start = time.perf_counter()
    case = make_case()
    cores = len(os.sched_getaffinity(0))
    solve, close = cpu_solver(case, cores)
    warm = []
    for _ in range(args.warmup):
        t0 = time.perf_counter()
        solve()
        warm.append(time.perf_counter() - t0)
    t_est = min(warm) if warm else None
    times = []
    for i in range(args.steps):
        if t_est is not None and i >= 1 and time.perf_counter() - t_start + t_est > REFERENCE_BUDGET_S:
            break
        t0 = time.perf_counter()
        solve()
        times.append(time.perf_counter() - t0)
        t_est = min(times)
    close()
    steps = len(times)
    tot = sum(times)
    v = steps / tot
    sample = (f"{steps} full cgne solves timed back to back (30 iterations: 1 adjoint + {NORMALS_PER_SOLVE} "
              f"normal operators each) after {len(warm)} warm-up solves; FP64 restatement of the reference "
              f"algorithm, coils split over {cores} threads")
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "solves/s", "n_gpus": args.gpus,
            "steps": steps, "warmup": len(warm), "steps_requested": args.steps,
            "ms_per_step": tot / steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "c128", "data": "synthetic",
            "config": config_dict(ws),
            "cpu_baseline": {"value": v, "unit": "solves/s", "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "wall_s": time.perf_counter() - t_start}
    print(json.dumps(line), flush=True)


def extra_summary(name, obj):
    """The headline figures of an extra configuration, repeated compactly on the headline line."""
    keys = {"learned_pcg": ("time_ratio_vs_best_plain", "learned_ms", "plain_cgne_ms"),
            "batched": ("batched_ms", "sequential_ms"),
            "regridding": ("us_per_adjoint_forward",),
            "toeplitz": ("us_toeplitz_32coils",),
            "highorder": ("ms_forward_16coils", "ms_adjoint_16coils", "ms_cgne_solve"),
            "dense": ("s_build",)}.get(name, ())
    return {f"{name}.{k}": obj[k] for k in keys if k in obj}


def fft_comparison(dev, case, stage_ms, reps, G):
    """The hand-written FFT passes of the normal operator against cuFFT (torch.fft) on the same
    batch: 32 coils, 256^2 images zero-padded to the 512^2 grid (nufftOp.m:384, ifftnc with
    sz = osN) and 512^2 grids transformed and cropped back (nufftOp.m:364-372).  The own figures are
    the per-normal-operator stage times (CUDA events) of the first two passes (coil maps and
    deapodisation fused in) and of the last two (crop, deapodisation and the conj-maps coil sum
    fused in); the cuFFT figures time the bare transforms only.  Comparison only: cuFFT is not on
    any path of the library."""
    import torch
    own_fwd = 1e3 * (stage_ms[0] + stage_ms[1]) / reps
    own_adj = 1e3 * (stage_ms[3] + stage_ms[4]) / reps
    x = torch.from_numpy((case["img"][:, :, None] * case["maps"]).astype(np.complex64).transpose(2, 1, 0).copy())
    x = x.to(dev)                                       # [C, N, N], each coil contiguous
    g = torch.fft.ifft2(x, s=(G, G), norm="ortho")
    us_ifft_pad = 1e3 * _timed_ms(lambda: torch.fft.ifft2(x, s=(G, G), norm="ortho"), 20, dev)
    us_fft_crop = 1e3 * _timed_ms(lambda: torch.fft.fft2(g, norm="ortho")[:, :N_IMG, :N_IMG], 20, dev)
    us_fft_full = 1e3 * _timed_ms(lambda: torch.fft.fft2(g, norm="ortho"), 20, dev)
    return {"workload": f"{N_COIL} coils, {N_IMG}^2 image <-> {G}^2 grid, complex64",
            "own_us": {"img_to_grid_2_passes": own_fwd, "grid_to_img_2_passes_and_coil_sum": own_adj,
                       "total": own_fwd + own_adj},
            "cufft_us": {"ifft2_zero_padded": us_ifft_pad, "fft2_then_crop": us_fft_crop,
                         "fft2_full": us_fft_full, "total": us_ifft_pad + us_fft_crop},
            "note": "own passes include the coil maps, deapodisation, crop and coil sum; cuFFT figures "
                    "are the bare transforms"}


def stage_bytes(cc, N, G, M, W, stencil):
    """Algorithmic bytes per launch of each normal-operator stage (complex64 = 8 B)."""
    img, grid, half = N * N * 8, G * G * 8, G * N * 8
    sten = (2 * W - 1) ** 2 * G * G * 4 if stencil else 0
    return [
        img + cc * img + cc * half,          # 0: image x maps x deapod -> first-axis FFT (writes G x N per coil)
        cc * half + cc * grid,               # 1: second-axis FFT (G x N -> G x G per coil)
        2 * cc * grid + sten,                # 2: gridding normal op (grid in, grid out; + stencil weights once)
        cc * grid + cc * half,               # 3: first-axis FFT + crop (G x G -> N x G per coil)
        cc * half + 3 * cc * img + 2 * img,  # 4: second-axis FFT + crop + deapod per coil (writes N x N per coil),
                                             #    then conj maps x per-coil images summed over coils
    ]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-learned", action="store_true", help="skip the learned-PCG vs plain-CG comparison")
    ap.add_argument("--no-batched", action="store_true", help="skip the 64-slice batched comparison")
    ap.add_argument("--no-extra", action="store_true", help="skip the regridding and high-order encoding lines")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--tuning", default=None,
                    help="fixed knobs coil_chunk,tile,coil_group,item,fft_lines,normal_mode (skips the autotuner)")
    ap.add_argument("--ncu", action="store_true",
                    help="profiling mode: one warm-up solve, then one solve; prints nothing else")
    ap.add_argument("--ncu-highorder", action="store_true",
                    help="profiling mode for the high-order encoding: 3 forward + 2 adjoint applications")
    ap.add_argument("--ncu-dense", action="store_true",
                    help="profiling mode for the dense Gram: a 4096^2 mrSampFuncMat built twice")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.ncu_highorder or args.ncu_dense:
        import torch
        _, _, local = dist_env()
        torch.cuda.set_device(local)
        dev = torch.device("cuda", local)
        return highorder_profile_case(dev) if args.ncu_highorder else dense_profile_case(dev)

    import ctypes as C
    import torch
    import matmri_gb300 as mm
    from matmri_gb300 import _lib
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    lib = _lib.load()

    case = make_case(seed=replica_seed(rank))
    S = mm.nufftOp([N_IMG, N_IMG], case["kloc"], None, 1, 2.0, 4)
    R = mm.rcvrOp(case["maps"], 0)
    A = mm.mrSampOp(S, R)
    tuned = None
    if args.tuning:
        knobs = [int(v) for v in args.tuning.split(",")]
        A.set_tuning(*knobs)
    elif not args.no_autotune:
        from matmri_gb300.autotune import autotune
        tuned = autotune(A, use_cache=False)           # plan-time search, outside the timed region
    data = A(case["img"], "notransp")                 # synthetic k-space [M, C] (set-up, not timed)
    M = data.shape[0]
    dev = torch.device("cuda", local)
    dt = torch.from_numpy(np.asfortranarray(data).T.copy()).to(dev).T   # column-major [M, C] on device
    xt = torch.empty((N_IMG, N_IMG), dtype=torch.complex64, device=dev).T
    dh = torch.from_numpy(np.ascontiguousarray(np.asfortranarray(data).T)).pin_memory()
    xh = torch.empty((N_IMG, N_IMG), dtype=torch.complex64).pin_memory()
    opts = _lib.CgneOpts()
    _lib.check(lib.mmr_cgne_default_opts(C.byref(opts)))
    opts.nit_max = NIT
    opts.res_thresh = float("nan")
    opts.x_change_thresh = float("nan")
    stream = torch.cuda.current_stream(dev)
    sp = stream.cuda_stream
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def solve(dev_ptrs=True):
        if dev_ptrs:
            r = lib.mmr_cgne_solve(A.handle, dt.data_ptr(), None, None, C.byref(opts), xt.data_ptr(), None, sp)
        else:
            r = lib.mmr_cgne_solve(A.handle, dh.data_ptr(), None, None, C.byref(opts), xh.data_ptr(), None, sp)
        _lib.check(r)

    def timed(n, dev_ptrs):
        tot = 0.0
        for _ in range(n):
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record(stream)
            solve(dev_ptrs)
            e1.record(stream)
            torch.cuda.synchronize()
            tot += e0.elapsed_time(e1) / 1e3
        return tot

    if args.ncu:
        solve(True)
        torch.cuda.synchronize()
        solve(True)
        torch.cuda.synchronize()
        print("ncu mode: 2 solves done", flush=True)
        return

    # warm-up (graph capture, scratch sizing, clocks)
    for _ in range(max(args.warmup, 3)):
        solve(True)
        solve(False)
    torch.cuda.synchronize()

    def barrier():
        if ws > 1:
            import torch.distributed as dist
            dist.barrier()
        torch.cuda.synchronize()

    c0 = C.c_uint64()
    _lib.check(lib.mmr_kernel_launches(C.byref(c0)))
    with ClockSampler(local) as clk:
        barrier()
        t_dev = timed(args.steps, True)
        barrier()
    c1 = C.c_uint64()
    _lib.check(lib.mmr_kernel_launches(C.byref(c1)))
    barrier()
    t_e2e = timed(args.steps, False)
    barrier()
    t_dev = max_over_ranks(t_dev, ws, dev)
    t_e2e = max_over_ranks(t_e2e, ws, dev)
    launches = int(c1.value - c0.value)

    # live per-stage timing of the normal operator (CUDA events on the launching stream)
    p = torch.from_numpy(np.asfortranarray(case["img"].astype(np.complex64)).T.copy()).to(dev).T
    q = torch.empty_like(p)
    ms = (C.c_double * 5)()
    cnt = (C.c_int32 * 5)()
    reps = 20
    _lib.check(lib.mmr_sense_profile_normal(A.handle, p.data_ptr(), q.data_ptr(), reps, ms, cnt, sp))
    cc, tile, cgrp, item, flines, nmode = A.get_tuning()
    G = S.osN[0]
    sb = stage_bytes(cc, N_IMG, G, M, 4, nmode == 2)
    total_ms = sum(ms[i] for i in range(5))
    dom = max(range(5), key=lambda i: ms[i])
    per_launch_s = ms[dom] / 1e3 / max(cnt[dom], 1)
    achieved = sb[dom] / per_launch_s / 1e9
    peak, peak_kind = peaks()
    stage_names = ["fft_img_to_grid_axis0", "fft_axis1", "gridnorm_stencil" if nmode == 2 else "gridnorm_interp_spread",
                   "fft_grid_axis0", "fft_axis1_coilsum"]
    # DRAM bytes per launch of the fused gridding kernel (ncu, per coil chunk; null when not captured)
    traffic = GRIDNORM_DRAM_BYTES.get((cc, tile, cgrp)) if (dom == 2 and nmode != 2) else None
    # whole-solve model: 1 adjoint + 31 normal operators of 580.1 MB each (grid passes, maps, samples,
    # image, trajectory; complex64) per 30-iteration solve = 18.27 GB
    solve_bytes = SOLVE_MODEL_BYTES

    if rank == 0:
        value = job_rate(ws, args.steps, t_dev)
        fft_cmp = fft_comparison(dev, case, ms, reps, G)
        line = {
            "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_dev / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "c64 (FP64 CG scalars)", "data": "synthetic",
            "config": config_dict(ws),
            "tuning": {"coil_chunk": cc, "tile": tile, "coil_group": cgrp, "item": item, "fft_lines": flines,
                       "normal_mode": "stencil" if nmode == 2 else "fused", "autotuned": tuned is not None},
            "e2e": {"value": job_rate(ws, args.steps, t_e2e), "unit": "solves/s",
                    "h2d_bytes_per_step": int(M * N_COIL * 8), "d2h_bytes_per_step": int(N_IMG * N_IMG * 8)},
            "gpu_launches": launches,
            "roofline": {"bound": "hbm", "kernel": stage_names[dom], "achieved": achieved, "peak": peak,
                         "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
                         "algorithmic_bytes_per_launch": sb[dom], "avg_launch_us": per_launch_s * 1e6,
                         "stage_share": {stage_names[i]: round(ms[i] / total_ms, 4) for i in range(5)},
                         "solve_model": {"bytes_per_solve": solve_bytes,
                                         "achieved": value * solve_bytes / 1e9,
                                         "frac": value * solve_bytes / 1e9 / peak}},
            "clocks": clk.summary(),
            "fft": {k: fft_cmp[k] for k in ("own_us", "cufft_us")},
        }
        # the other configurations: one JSON line each, printed before the headline line (which stays last)
        extras = {"fft": lambda: fft_cmp}
        if not args.no_learned:
            extras["learned_pcg"] = lambda: learned_pcg_comparison(dev)
        if not args.no_batched:
            extras["batched"] = lambda: batched_comparison(dev)
        if not args.no_extra:
            extras["regridding"] = lambda: regridding_measure(dev)
            extras["toeplitz"] = lambda: toeplitz_measure(dev)
            extras["highorder"] = lambda: highorder_measure(dev)
            extras["finddel"] = lambda: finddel_measure(dev, cpu=not args.no_cpu_baseline)
            extras["dense"] = lambda: dense_measure(dev, cpu=not args.no_cpu_baseline)
        summary = {}
        for name, fn in extras.items():
            obj = fn()
            print(json.dumps({"extra": name, **obj}), flush=True)
            summary.update(extra_summary(name, obj))
        if summary:
            line["extras"] = summary
        if not args.no_cpu_baseline:
            line["cpu_baseline"] = cpu_baseline(case)
        print(json.dumps(line), flush=True)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
