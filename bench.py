"""Benchmark: ms per FLD linear solve (SOLVE_WITH_SOR's system) to relative
residual 1e-10 on one GB300, through libttfld's C ABI.

Workload (shell256): the 100 x 256 x 128 (r x phi x theta) synthetic shell
(3,276,800 cells, dt = 100 s, seed 1) after the set-up BOUNDS/KAPPA; a
"step" is one solve of the SOLVE_WITH_SOR system of its implicit step's
first outer iteration (ppenergy.f:375).  The product path starts from the
learned initial guess (trained before the timed region, on the GPU, on 16
pairs the solver generates from other irradiations and time steps of the
same shell), keeps it only if it beats the zero guess over the first four
sweeps, and runs FP32 red-black sweeps inside FP64 defect correction.  The
same system from zero, and the plain FP64 red-black SOR (exact reference
rounding, and Jacobi-scaled with FMA), are timed in the same run.

Beside the headline line's timed region, the same run reports
  * "step": ms per implicit step (COUPLED_ENERGY_EQS, ppenergy.f:2-791) of
    the shell256 run over the same K steps for the product path (learned
    guess, then the previous step's solution, FP32/FP64) and for the plain
    FP64 SOR (exact rounding and scaled), with the error of each against the
    exact FP64 SOR at EPSMAT = 1e-12 over those steps;
  * "shell512" / "stiff512": the 160 x 512 x 256 shells (dt = 300 s,
    opacity contrast 1e4; dt = 1000 s, contrast 1e6): 30 / 10 implicit
    steps by the product path and by the plain scaled FP64 SOR, their
    per-step ratio, the learned guess's fallback rate, errors after 3 steps
    against the FP64 SOR at 1e-12, and the FP32 sweep's roofline at a size
    beyond L2;
  * "cpu_baseline": complete solves of the bench system by the C oracle (the
    reference loop and stopping rule) on all host cores, and on one core.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
                  [--steps512 S] [--no-shell512] [--no-cpu]

Under torchrun with N > 1 every rank solves its own replica (the path does
not shard across GPUs here), value = max-over-ranks time / (K * N).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "ms per FLD solve to rel. residual 1e-10: learned+FP32/FP64 vs plain FP64 SOR"
SHELL = "shell256"
WORKLOAD = ("shell256: 100x256x128 (r x phi x theta) synthetic spherical shell, 3276800 cells, "
            "dt=100 s, seed 1; the SOLVE_WITH_SOR system of its implicit step's first outer "
            "iteration, solved to ||b-Ax||_1/||b||_1 <= 1e-10")
TRAIN_PAIRS, TRAIN_EPOCHS, TRAIN_LR = 16, 20, 5e-4
# Algorithmic bytes per cell update of one sweep (both colours):
#   FP32 scaled sweep: 6 coefficients + rhat + e read + e write, and the
#                      other colour's e (each of its values read once per
#                      half-sweep)                               = 10 x 4 B
#   FP64 exact sweep : 7 coefficients + b + x read + x write      = 10 x 8 B
# (at 160x512x256, beyond L2, ncu measures 40.5 B of DRAM traffic per FP32
# cell update)
BYTES_FP32_SWEEP = 40
BYTES_FP64_SWEEP = 80


def max_over_ranks(value: float, device: str) -> float:
    """The largest value over the ranks of the process group (the timed
    region's length is the slowest rank's)."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled while the timed region runs."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.lines = []
        if self.proc is not None:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in getattr(self, "lines", []):
            p = [x.strip() for x in l.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                smax = float(p[2])
            except ValueError:
                continue
            for n, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def load_traffic():
    """DRAM bytes (read + write) per sweep of the FP32 sweep kernel of the
    product path (the neighbour-flag kernel), from the committed ncu summary
    (one full sweep is the unit of `achieved`)."""
    p = os.path.join(ROOT, "profiles", "sweeps32_local_shell256.md")
    if os.path.exists(p):
        with open(p) as f:
            for line in f:
                if line.startswith("traffic_bytes_per_sweep:"):
                    return int(line.split(":")[1])
    return None


def first_system(f):
    """Assemble the SOLVE_WITH_SOR system of an implicit step's first outer
    iteration (one outer iteration of COUPLED_ENERGY_EQS leaves it in
    SOR_A..G / RHS_ER) and put back the state the step started from, which
    is what the learned guess reads."""
    from ttcode_gb300 import _ffi
    import ctypes
    keep = {n: f.download(n) for n in ("T", "ER", "DELTA_ER")}
    itmax = f.params["itmax"]
    f.set_params(itmax=1)
    f.set_solver("mixed", tol=1e-10, max_sweeps=64)
    st = _ffi.StepStats()
    f.L.ttfld_coupled_energy_eqs(f.h, 1, ctypes.byref(st))
    for n, a in keep.items():
        f.upload(n, a)
    f.set_params(itmax=itmax)


def build_system(device, train=True):
    """The shell on the device with the learned guess trained (on pairs from
    other irradiations and time steps) and the bench system assembled."""
    from ttcode_gb300 import guess
    from ttcode_gb300.fld import start_run
    from ttcode_gb300.synthetic import shell
    sh = shell(SHELL, seed=1)
    sh.params["epsmat"] = 1e-10
    sh.params["itmax"] = 200000
    f = start_run(sh, device=device)
    info = None
    if train:
        t0 = time.perf_counter()
        guess.init(f, seed=1, capacity=TRAIN_PAIRS)
        npairs = guess.capture_pairs(f, sh, guess.random_cases(TRAIN_PAIRS, seed=10))
        t1 = time.perf_counter()
        losses = [guess.train(f, epochs=1, lr=TRAIN_LR, seed=e) for e in range(TRAIN_EPOCHS)]
        t2 = time.perf_counter()
        info = {"pairs": npairs, "epochs": TRAIN_EPOCHS, "lr": TRAIN_LR, "capture_s": round(t1 - t0, 2),
                "train_s": round(t2 - t1, 2), "loss_first_epoch": losses[0], "loss_last_epoch": losses[-1],
                "pairs_from": "16 seeded irradiations (phi0, T_irr in [1500, 2500] K) and dt in [50, 500] s "
                              "of the same shell; the timed system (T_irr 2048 K, dt 100 s) is not among them"}
        # back to the bench case (start_run's set-up)
        f.load_shell(sh)
        f.set_params(iii=0, delt=sh.params["delt"])
        f.bounds()
        f.kappa()
        f.set_params(iii=sh.params.get("iii", 1))
    first_system(f)
    return sh, f, info


def flush_l2(torch, buf):
    buf.add_(1.0)  # 256 MB written: larger than the 126 MB L2


def run_profile_solve(args):
    """For the ncu summaries under profiles/: after the set-up (training
    included), one product-path solve and one exact FP64 solve of the
    shell256 system inside cudaProfilerStart/Stop, so that
    `ncu --profile-from-start off` lists exactly their launches."""
    import torch
    torch.cuda.set_device(0)
    sh, f, _ = build_system(0)
    torch.cuda.synchronize()
    torch.cuda.cudart().cudaProfilerStart()
    for solver, g in (("mixed", "learned"), ("sor64_exact", "zero")):
        f.set_solver(solver, guess=g, tol=1e-10)
        f.begin_step(new_run=True)
        st = f.solve_system()
        print(json.dumps({"solver": solver, "guess": g, "sweeps": st.sor_iter, "ms": st.solve_ms}), flush=True)
    torch.cuda.synchronize()
    torch.cuda.cudart().cudaProfilerStop()
    f.close()


def run_profile_pcg(args):
    """For the PCG summaries under profiles/: the shell256 system of one
    implicit step, then inside cudaProfilerStart/Stop one PCG solve of
    SOLVE_WITH_SOR's system (zero guess, 1e-10) and one SOLVE_WITH_HYPRE
    with the reference's settings (1e-6, 50 iterations)."""
    import torch
    from ttcode_gb300.fld import start_run
    from ttcode_gb300.synthetic import shell
    torch.cuda.set_device(0)
    sh = shell(SHELL, seed=1)
    f = start_run(sh)
    f.set_solver("mixed", tol=1e-10)
    f.coupled_energy_eqs(True)
    f.fill_sor_matrix()
    f.set_solver("pcg", tol=1e-10)
    f.solve_system()                       # warm: workspace allocated, kernels loaded
    torch.cuda.synchronize()
    torch.cuda.cudart().cudaProfilerStart()
    st = f.solve_system()
    sh_st = f.solve_with_hypre()
    torch.cuda.synchronize()
    torch.cuda.cudart().cudaProfilerStop()
    print(json.dumps({"pcg": {"ms": st.solve_ms, "iterations": st.sor_iter, "anchors": st.corrections},
                      "hypre": {"ms": sh_st.solve_ms, "iterations": sh_st.sor_iter, "status": sh_st.status}}),
          flush=True)
    f.close()


def run_profile_step(args):
    """For the step's launch list: the shell256 shell, two implicit steps
    (mixed solver, previous-step guess), then a third inside
    cudaProfilerStart/Stop."""
    import torch
    from ttcode_gb300.fld import start_run
    from ttcode_gb300.synthetic import shell
    torch.cuda.set_device(0)
    sh = shell(SHELL, seed=1)
    f = start_run(sh)
    f.set_solver("mixed", guess="previous", tol=1e-10)
    for _ in range(2):
        f.coupled_energy_eqs(True)
    torch.cuda.synchronize()
    torch.cuda.cudart().cudaProfilerStart()
    st = f.coupled_energy_eqs(True)
    torch.cuda.synchronize()
    torch.cuda.cudart().cudaProfilerStop()
    print(json.dumps({"step_ms": st.step_ms, "solve_ms": st.solve_ms, "sweeps": st.sor_total}), flush=True)
    f.close()


def run_profile_conv(args):
    """For the convolution summaries under profiles/: the learned guess's
    network (seeded random weights) on the shell256 shell's half-resolution
    grid; after one inference with each form outside the profiled range,
    one inference with the mma.sync convolutions and one with the tcgen05
    ones inside cudaProfilerStart/Stop."""
    import torch
    from ttcode_gb300 import guess
    from ttcode_gb300._ffi import check
    from ttcode_gb300.fld import start_run
    from ttcode_gb300.synthetic import shell
    torch.cuda.set_device(0)
    sh = shell(SHELL, seed=1)
    f = start_run(sh)
    guess.init(f, seed=5)
    n = sh.dims[0] * sh.dims[1] * sh.dims[2]
    feat = np.random.default_rng(1).uniform(-1.0, 1.0, (n, 5)).astype(np.float32)
    pred = np.zeros(n, dtype=np.float32)

    def infer(form):
        check("ttfld_guess_set_conv", f.L.ttfld_guess_set_conv(form))
        check("ttfld_guess_predict", f.L.ttfld_guess_predict(f.h, feat.ctypes.data, pred.ctypes.data))
        return pred.copy()

    infer(0), infer(1)
    torch.cuda.synchronize()
    torch.cuda.cudart().cudaProfilerStart()
    p0, p1 = infer(0), infer(1)
    torch.cuda.synchronize()
    torch.cuda.cudart().cudaProfilerStop()
    check("ttfld_guess_set_conv", f.L.ttfld_guess_set_conv(2))   # the default form
    print(json.dumps({"pred_rel_diff": float(np.linalg.norm(p1 - p0) / np.linalg.norm(p0))}), flush=True)
    f.close()


def run_sweep_forms(args):
    """For the sweep-form comparison under profiles/: on the shell of
    --profile-dims (default 160,512,256), the first system of an implicit
    step, then ttfld_time_sweeps (CUDA events, 48 sweeps in one launch, the
    in-sweep norm every 8th, twice each) for the neighbour-flag kernel (the
    solver's), the grid-barrier kernel, the TMA-staged form, two launches per
    sweep, and the wavefront form with its own window size and with windows
    of 1, 2, 3, 4, 6 and 8 theta planes."""
    import torch
    from ttcode_gb300.fld import start_run
    from ttcode_gb300.synthetic import make_shell
    torch.cuda.set_device(0)
    nx, ny, nz = (int(v) for v in (args.profile_dims or "160,512,256").split(","))
    sh = make_shell(nx, ny, nz, seed=1, delt=100.0)
    sh.params["epsmat"] = 1e-10
    f = start_run(sh)
    first_system(f)
    forms = [("neighbour", "mixed"), ("grid", "mixed_grid"), ("tma", "mixed_tma"), ("split", "mixed_split"),
             ("wave", "mixed_wave")]
    forms += [(f"wave_{p}_planes", 16 + p) for p in (1, 2, 3, 4, 6, 8)]
    out = {"dims": [nx, ny, nz], "unit": "us per sweep"}
    for name, code in forms:
        out[name] = [round(f.time_sweeps(code, 48) * 1e3, 2) for _ in range(2)]
    print(json.dumps(out), flush=True)
    f.close()


def run_profile_sweeps(args):
    """For the ncu capture of the dominant kernel: the shell256 system (or a
    shell of --profile-dims NX,NY,NZ, e.g. 160,256,128 for a working set
    beyond L2), then inside cudaProfilerStart/Stop one launch of 8 FP32
    sweeps (the warm-up of ttfld_time_sweeps) and one of 16 (in-sweep norm
    every 8th)."""
    import torch
    torch.cuda.set_device(0)
    if args.profile_dims:
        from ttcode_gb300.fld import start_run
        from ttcode_gb300.synthetic import make_shell
        nx, ny, nz = (int(v) for v in args.profile_dims.split(","))
        sh = make_shell(nx, ny, nz, seed=1, delt=100.0)
        sh.params["epsmat"] = 1e-10
        f = start_run(sh)
        first_system(f)
    else:
        sh, f, _ = build_system(0, train=False)
    torch.cuda.synchronize()
    torch.cuda.cudart().cudaProfilerStart()
    ms = f.time_sweeps("mixed", 16)
    torch.cuda.synchronize()
    torch.cuda.cudart().cudaProfilerStop()
    print(json.dumps({"ms_per_sweep": ms}), flush=True)
    f.close()


def run_gpu(args):
    import torch
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    from ttcode_gb300 import _ffi
    L = _ffi.lib()
    sh, f, train_info = build_system(local)
    nx, ny, nz = sh.dims
    ncells = nx * ny * nz
    stream = torch.cuda.ExternalStream(f.stream_ptr(), device=torch.device("cuda", local))
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")

    # reference-accuracy solution: exact FP64 SOR (the reference loop, bitwise)
    # converged to 1e-12 on the same system
    f.set_params(epsmat=1e-12)
    f.set_solver("sor64_exact")
    st_ref = f.solve_system()
    x_ref = f.download("DELTA_ER")
    f.set_params(epsmat=1e-10)

    def solve_timed(solver, guess="zero"):
        f.set_solver(solver, guess=guess, tol=1e-10)
        f.begin_step(new_run=True)   # every timed solve is a run's first: no previous solution
        flush_l2(torch, flush)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        st = f.solve_system()
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1), st

    # warm-up
    for _ in range(args.warmup):
        solve_timed("mixed", "learned")
    # timed region: K product-path solves
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    launches0 = L.ttfld_kernel_launches()
    times, stats = [], []
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            ms, st = solve_timed("mixed", "learned")
            times.append(ms)
            stats.append(st)
    torch.cuda.synchronize()
    launches = int(L.ttfld_kernel_launches() - launches0)
    if ws > 1:
        torch.distributed.barrier()
    x_mixed = f.download("DELTA_ER")
    total_ms = float(sum(times))
    if ws > 1:
        total_ms = max_over_ranks(total_ms, "cuda")
    ms_per_solve = total_ms / args.steps / ws
    r_l1, b_l1 = f.true_residual()
    err = float(np.linalg.norm((x_mixed - x_ref).ravel()) / np.linalg.norm(x_ref.ravel()))

    # the same mixed solver from the zero guess
    zl = [solve_timed("mixed", "zero") for _ in range(3)]
    zero_guess = {"ms": min(m for m, _ in zl), "sweeps": zl[-1][1].sor_iter}
    # the same system by FP32 PCG (radial line preconditioner) in FP64 defect
    # correction, same stopping rule, from zero and from the learned guess
    pcg = {}
    for g in ("zero", "learned"):
        pl = [solve_timed("pcg", g) for _ in range(3)]
        xs = f.download("DELTA_ER")
        pcg[g] = {"ms": min(m for m, _ in pl), "iterations": pl[-1][1].sor_iter,
                  "anchors": pl[-1][1].corrections, "fallback": pl[-1][1].fallback,
                  "err_vs_fp64_1e-12": float(np.linalg.norm((xs - x_ref).ravel()) / np.linalg.norm(x_ref.ravel()))}
    # the plain FP64 red-black SOR on the same GPU (same stopping rule as the
    # reference, in-sweep L1 ratio <= 1e-10)
    plain = {}
    for solver in ("sor64_exact", "sor64_fast"):
        ms_list, st = [], None
        for _ in range(2):
            ms, st = solve_timed(solver)
            ms_list.append(ms)
        xs = f.download("DELTA_ER")
        plain[solver] = {"ms": min(ms_list), "sweeps": st.sor_iter,
                         "err_vs_fp64_1e-12": float(np.linalg.norm((xs - x_ref).ravel()) / np.linalg.norm(x_ref.ravel()))}

    # roofline of the dominant kernel: FP32 sweep, timed live on the library stream
    f.set_solver("mixed")
    ms_sweep32 = f.time_sweeps("mixed", 50)
    ms_sweep64 = f.time_sweeps("sor64_exact", 20)
    peak, peak_kind = measured_peaks()
    achieved = BYTES_FP32_SWEEP * ncells / (ms_sweep32 * 1e-3) / 1e9   # GB/s per full sweep (2 launches)
    traffic = load_traffic()

    # e2e: the reference-facing SOLVE_WITH_SOR call with host (pinned) buffers:
    # upload the EVAL arrays, RHS_ER and UPPERBND, fill + solve, download DELTA_ER
    names = ("EVAL1", "EVAL2", "EVAL3", "EVAL4", "EVAL5", "EVAL6", "EVAL7", "EVAL8", "EVAL_1_6", "RHS_ER")
    host = {}
    for n in names:
        a = f.download(n)
        t = torch.empty(a.size, dtype=torch.float64, pin_memory=True)
        t.numpy()[:] = a.ravel(order="F")
        host[n] = t
    ub = f.download("UPPERBND")
    out = torch.empty(f.download("DELTA_ER").size, dtype=torch.float64, pin_memory=True)
    h2d = sum(host[n].numel() * 8 for n in names) + ub.size * 4
    d2h = out.numel() * 8
    f.set_solver("mixed", guess="learned", tol=1e-10)
    e2e = []
    for it in range(args.warmup + args.steps):
        flush_l2(torch, flush)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for n in names:
            _ffi.check(n, L.ttfld_upload(f.h, _ffi.FIELDS[n], host[n].data_ptr()))
        _ffi.check("ub", L.ttfld_upload(f.h, _ffi.FIELDS["UPPERBND"], ub.ctypes.data))
        st = _ffi.SolveStats()
        import ctypes
        _ffi.check("begin", L.ttfld_begin_step(f.h, 1))   # a run's first solve, as in the device-timed loop
        _ffi.check("solve", L.ttfld_solve_with_sor(f.h, 1, ctypes.byref(st)), ok=(0, 1, 2))
        _ffi.check("dl", L.ttfld_download(f.h, _ffi.FIELDS["DELTA_ER"], out.data_ptr()))
        t1 = time.perf_counter()
        if it >= args.warmup:
            e2e.append((t1 - t0) * 1e3)
    e2e_ms = float(sum(e2e) / len(e2e))

    line = {
        "metric": METRIC, "value": ms_per_solve, "unit": "ms", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "fp32 sweeps / fp64 residual",
        "data": "synthetic (seeded analytic shell, no dataset)",
        "config": {"workload": WORKLOAD, "cells": ncells, "solver": "mixed FP32/FP64 defect correction",
                   "guess": "learned (half-resolution 3-D U-Net, BF16); falls back to zero unless it beats zero after four sweeps",
                   "tol": 1e-10, "omega": sh.params["sorparam"],
                   "l2": "flushed between timed solves (256 MB write)", "parallelism": "replicas"},
        "sweeps_per_solve": stats[-1].sor_iter, "corrections_per_solve": stats[-1].corrections,
        # cell updates per second of the product path (sweeps x cells / solve time) and of one
        # FP32 sweep on its own
        "cell_updates_per_s": float(np.mean([s.sor_iter for s in stats])) * ncells / (ms_per_solve * 1e-3),
        "cell_updates_per_s_sweep": ncells / (ms_sweep32 * 1e-3),
        "fallbacks": int(sum(s.fallback for s in stats)), "guess_ms": stats[-1].guess_ms,
        "guess_training": train_info, "zero_guess_mixed": zero_guess, "pcg": pcg,
        "true_rel_residual": r_l1 / b_l1,
        "err_vs_fp64_1e-12": err, "fp64_1e-12_sweeps": st_ref.sor_iter,
        "plain_fp64": plain,
        "speedup_vs_plain_fp64_exact": plain["sor64_exact"]["ms"] / ms_per_solve,
        "speedup_vs_plain_fp64_fast": plain["sor64_fast"]["ms"] / ms_per_solve,
        "e2e": {"value": e2e_ms, "unit": "ms", "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                "call": "ttfld_upload x11 + ttfld_begin_step + ttfld_solve_with_sor + ttfld_download (pinned host)"},
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "kernel": "sweeps32_local (one full sweep)", "achieved": achieved,
                     "peak": peak, "unit": "GB/s", "frac": achieved / peak, "peak_kind": peak_kind,
                     "algorithmic_bytes_per_sweep": BYTES_FP32_SWEEP * ncells, "ms_per_sweep": ms_sweep32,
                     "traffic": traffic},
        "fp64_sweep": {"ms_per_sweep": ms_sweep64,
                       "achieved_gbs": BYTES_FP64_SWEEP * ncells / (ms_sweep64 * 1e-3) / 1e9},
        "clocks": clk.summary(),
    }
    if rank == 0 and ws == 1 and not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline(f, sh)
    from ttcode_gb300 import guess as G
    blob = G.save_weights(f)
    f.close()
    # per implicit step, and the 512 x 256 x 160 configuration (not timed
    # regions of the headline; rank 0 of a single-replica run)
    if rank == 0 and ws == 1:
        line["step"] = step_block(sh, args.steps, blob)
        if not args.no_shell512 and args.steps512 > 0:
            line["shell512"] = big_block("shell512", args.steps512, peak, peak_kind)
        if not args.no_shell512 and args.stiff_steps > 0:
            line["stiff512"] = big_block("stiff512", args.stiff_steps, peak, peak_kind)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()


STEP_KEYS = ("ms_per_step", "solve_ms_per_step", "sweeps_per_solve", "outer_iter_per_step", "solves_per_step",
             "fallbacks", "worst_status")


def _variants(sh, names, nsteps, snap_at, ref_snap, blob):
    from ttcode_gb300 import runs
    out = {}
    for name in names:
        steps, snap = runs.run_variant(sh, name, nsteps, snap_at, blob=blob if "learned" in name else None)
        s = runs.summarize(name, steps, snap, ref_snap, snap_at)
        out[name] = {k: s[k] for k in STEP_KEYS + ("err_vs_fp64_1e-12",) if k in s}
    return out


def step_block(sh, nsteps, blob):
    """ms per implicit step (COUPLED_ENERGY_EQS) of the shell256 run over the
    same nsteps steps: the product path (learned guess for the run's first
    solve, then the previous step's solution; FP32/FP64) against the plain
    FP64 red-black SOR from zero, exact and scaled.  Errors of E_R and T
    after the last step against the exact FP64 SOR at EPSMAT = 1e-12."""
    from ttcode_gb300 import runs
    _, ref_snap = runs.run_variant(sh, "fp64_exact", nsteps, nsteps, epsmat=1e-12)
    v = _variants(sh, ("mixed_learned", "fp64_fast", "fp64_exact"), nsteps, nsteps, ref_snap, blob)
    prod = v["mixed_learned"]["ms_per_step"]
    return {"workload": "shell256, consecutive implicit steps from the set-up state", "steps": nsteps,
            "reference": "exact FP64 SOR (the reference loop) at EPSMAT 1e-12 over the same steps",
            **v, "speedup_vs_fp64_fast": v["fp64_fast"]["ms_per_step"] / prod,
            "speedup_vs_fp64_exact": v["fp64_exact"]["ms_per_step"] / prod}


BIG_SHELLS = {
    "shell512": ("160x512x256 (r x phi x theta), 20971520 cells, dt=300 s, opacity contrast 1e4", (150.0, 600.0)),
    "stiff512": ("160x512x256 (r x phi x theta), 20971520 cells, dt=1000 s, opacity contrast 1e6", (500.0, 2000.0)),
}


def big_block(name, nsteps, peak, peak_kind):
    """A 160 x 512 x 256 shell (shell512: dt 300 s, opacity contrast 1e4;
    stiff512: dt 1000 s, contrast 1e6): nsteps implicit steps by the product
    path (a network trained on 8 first solves of other irradiations and time
    steps of the same shell; its guess kept only if it beats zero, the
    fallbacks counted) and by the plain scaled FP64 SOR from zero, errors
    after 3 steps against the scaled FP64 SOR at EPSMAT = 1e-12, and the
    FP32 sweep's CUDA-event roofline on the shell's first system (a working
    set beyond L2)."""
    import torch
    from ttcode_gb300 import runs
    from ttcode_gb300.fld import start_run
    from ttcode_gb300.synthetic import shell
    desc, dt_range = BIG_SHELLS[name]
    sh = shell(name, seed=1)
    sh.params["epsmat"] = 1e-10
    sh.params["itmax"] = 200000
    t0 = time.perf_counter()
    blob, info = runs.train_guess(sh, 8, 12, 5e-4, dt_range)
    snap_at = min(3, nsteps)
    _, ref_snap = runs.run_variant(sh, "fp64_fast", snap_at, snap_at, epsmat=1e-12)
    v = _variants(sh, ("mixed_learned", "fp64_fast"), nsteps, snap_at, ref_snap, blob)
    f = start_run(sh)
    first_system(f)
    nx, ny, nz = sh.dims
    ms = f.time_sweeps("mixed", 50)
    # SOLVE_WITH_HYPRE on the same EVAL arrays with the reference's settings
    # (tol 1e-6, 50 iterations): the first call chooses the preconditioner's
    # sweep count, the second reuses it
    hyp = []
    for _ in range(2):
        h = f.solve_with_hypre()
        hyp.append({"status": h.status, "iterations": h.sor_iter, "gs_sweeps": h.gs_sweeps, "ms": h.solve_ms,
                    "ratio": h.rnorm / h.rhsnorm if h.rhsnorm > 0 else None})
    f.close()
    torch.cuda.synchronize()
    achieved = BYTES_FP32_SWEEP * nx * ny * nz / (ms * 1e-3) / 1e9
    return {"workload": f"{name}: {desc}, seed 1; consecutive implicit steps from the set-up state, tol 1e-10",
            "steps": nsteps, "training": info,
            "reference": f"scaled FP64 SOR at EPSMAT 1e-12 over the first {snap_at} steps",
            **v, "speedup_per_step_vs_fp64_fast": v["fp64_fast"]["ms_per_step"] / v["mixed_learned"]["ms_per_step"],
            "fallback_rate": v["mixed_learned"]["fallbacks"] / max(1, nsteps),
            "solve_with_hypre": {"first": hyp[0], "second": hyp[1]},
            "roofline": {"kernel": "sweeps32_local (one full sweep)", "ms_per_sweep": ms,
                         "algorithmic_bytes_per_sweep": BYTES_FP32_SWEEP * nx * ny * nz, "achieved": achieved,
                         "peak": peak, "unit": "GB/s", "frac": achieved / peak, "peak_kind": peak_kind},
            "wall_s": round(time.perf_counter() - t0, 1)}


def oracle_system(sh, f=None):
    """The bench system in the CPU oracle: from the device context when given,
    else assembled by the oracle itself (the first outer iteration of
    COUPLED_ENERGY_EQS, its solve cut to one sweep by ITMAX = 1, as the GPU
    side assembles it)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as ormod
    from ttcode_gb300.grid import full_1d
    ormod.build()
    o = ormod.Oracle(*sh.dims)
    for n in sh.grid.m:
        a = full_1d(sh.grid, n)
        o.f(n)[:a.size] = a
    for n, a in sh.fields.items():
        o.f(n)[...] = a
    for k, v in sh.params.items():
        if k != "kappa_model":
            o.set(k, v)
    o.set("epsmat", 1e-10)
    if f is not None:
        for n in ("SOR_A", "SOR_B", "SOR_C", "SOR_D", "SOR_E", "SOR_F", "SOR_G", "RHS_ER"):
            o.f(n)[...] = f.download(n)
    else:
        o.set("iii", 0)
        o.call("bounds")
        o.call("kappa")
        o.set("iii", 1)
        o.set("itmax", 1)
        o.call("coupled_energy_eqs", 1)
    o.set("itmax", 200000)
    return o


def host_threads() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def oracle_solve_ms(o, threads: int):
    """One complete solve of the oracle's current system from zero: the
    reference's red-black loop and stopping rule (ppsor.f:29-177), on
    `threads` theta slabs (one thread each, the reference's rank per slab),
    or the serial loop with threads = 1.  Returns (ms, sweeps)."""
    t0 = time.perf_counter()
    if threads > 1:
        rc = o.call("solve_with_sor_mt", threads)
    else:
        rc = o.call("solve_with_sor", 0, 0)
    ms = (time.perf_counter() - t0) * 1e3
    if rc != 0:
        raise RuntimeError(f"oracle solve status {rc}")
    return ms, int(o.get("sor_iter"))


def cpu_baseline(f, sh):
    o = oracle_system(sh, f)
    th = host_threads()
    runs = [oracle_solve_ms(o, th) for _ in range(2)]
    ms, sweeps = min(runs)
    serial_ms, serial_sweeps = oracle_solve_ms(o, 1)
    return {"value": ms, "unit": "ms", "cores": th, "kind": "port",
            "sample": f"complete solves of the same 100x256x128 system to 1e-10 by the C oracle (gcc -O2; the "
                      f"reference loop and stopping rule; {th} threads on theta slabs, a barrier per colour): "
                      f"best of 2, {sweeps} sweeps",
            "serial_1core_ms": serial_ms, "serial_sweeps": serial_sweeps}


def run_reference(args):
    """The reference's CPU path (the C restatement of ppsor.f) on all the
    host cores, as the reference runs one serial rank per core on a slab of
    the grid: each step is one complete solve of the shell256 system to
    1e-10 from zero (the reference's stopping rule), one thread per theta
    slab.  One serial solve on one core is reported beside it."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    from ttcode_gb300.synthetic import shell
    sh = shell(SHELL, seed=1)
    o = oracle_system(sh, None)
    th = host_threads()
    vals, sweeps = [], 0
    for it in range(args.warmup + args.steps):
        ms, sweeps = oracle_solve_ms(o, th)
        if it >= args.warmup:
            vals.append(ms)
    v = float(sum(vals) / len(vals))
    serial_ms, serial_sweeps = oracle_solve_ms(o, 1)
    line = {"metric": METRIC, "value": v, "unit": "ms", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": v, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "fp64", "data": "synthetic (seeded analytic shell, no dataset)",
            "config": {"workload": WORKLOAD, "cells": int(np.prod(sh.dims)), "solver": "FP64 red-black SOR",
                       "guess": "zero", "tol": 1e-10, "omega": sh.params["sorparam"]},
            "impl": "reference",
            "cpu_baseline": {"value": v, "unit": "ms", "cores": th, "kind": "port",
                             "sample": f"per step: one complete solve of the shell256 system to 1e-10 from zero "
                                       f"by the C oracle (the reference loop and stopping rule, {sweeps} sweeps) "
                                       f"on {th} threads (theta slabs, a barrier per colour)",
                             "serial_1core_ms": serial_ms, "serial_sweeps": serial_sweeps},
            "e2e": {"value": v, "unit": "ms", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the cpu_baseline leg")
    ap.add_argument("--steps512", type=int, default=30, help="implicit steps of the 160x512x256 block")
    ap.add_argument("--stiff-steps", type=int, default=10,
                    help="implicit steps of the 160x512x256 dt=1000 s, contrast 1e6 block")
    ap.add_argument("--no-shell512", action="store_true", help="skip the 160x512x256 blocks")
    ap.add_argument("--profile-solve", action="store_true",
                    help="only build the system and run one mixed and one exact FP64 solve")
    ap.add_argument("--profile-sweeps", action="store_true",
                    help="only build the system and run 8 + 16 FP32 sweeps")
    ap.add_argument("--profile-dims", default="", help="NX,NY,NZ of the --profile-sweeps shell (default shell256)")
    ap.add_argument("--profile-step", action="store_true",
                    help="only run three implicit steps, the third inside cudaProfilerStart/Stop")
    ap.add_argument("--sweep-forms", action="store_true",
                    help="only time the FP32 sweep kernel's forms on the --profile-dims shell")
    ap.add_argument("--profile-conv", action="store_true",
                    help="only run one inference of the guess network with each convolution form")
    ap.add_argument("--profile-pcg", action="store_true",
                    help="only build the system and run one PCG and one SOLVE_WITH_HYPRE solve")
    args = ap.parse_args()
    if args.profile_solve:
        run_profile_solve(args)
        return
    if args.profile_sweeps:
        run_profile_sweeps(args)
        return
    if args.profile_step:
        run_profile_step(args)
        return
    if args.profile_pcg:
        run_profile_pcg(args)
        return
    if args.profile_conv:
        run_profile_conv(args)
        return
    if args.sweep_forms:
        run_sweep_forms(args)
        return
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
