"""Multi-step runs of the benchmark configurations through the C ABI.

    python -m ttcode_gb300.runs CONFIG [--steps N] [--ref-steps M]
                                [--variants a,b,...] [--pairs P --epochs E]

CONFIG is a shell of `synthetic.SHELLS` (shell256, shell512, stiff512, ...).
Every variant starts from the same seeded shell (after the set-up BOUNDS and
KAPPA) and takes N implicit steps (COUPLED_ENERGY_EQS, ppenergy.f:2-791)
with its solver and initial guess:

    fp64_exact      the reference loop in FP64 (bitwise per sweep), zero guess
    fp64_fast       the same iteration on Jacobi-scaled FP64 with FMA
    mixed_zero      FP32 sweeps in FP64 defect correction, zero guess
    mixed_previous  ... each step's first solve from the previous solution
    mixed_learned   ... the run's first solve from the learned guess (with the
                    first-sweep fallback to zero), later ones from the
                    previous solution
    pcg_zero        FP32 conjugate gradients (radial line preconditioner) in
                    FP64 defect correction, zero guess
    pcg_previous    ... each step's first solve from the previous solution
    pcg_learned     ... the run's first solve from the learned guess (kept if
                    its preconditioned residual is below zero's), later ones
                    from the previous solution

One JSON line per variant: mean and total device time per step (CUDA events
inside the library), outer iterations, solves, sweeps and fallbacks per step,
and the relative L2 error of E_R and T after step M against the
reference-accuracy run (the exact FP64 SOR at EPSMAT = 1e-12, M steps).
The learned guess is trained first, on the GPU, on pairs the mixed solver
generates from seeded random irradiations and time steps of the same shell
(the runs themselves use the shell's own irradiation).
"""
from __future__ import annotations

import argparse
import ctypes
import json
import time

import numpy as np

from . import _ffi
from . import guess as G
from .fld import start_run
from .synthetic import SHELLS, shell

VARIANTS = {
    "fp64_exact": dict(solver="sor64_exact", guess="zero"),
    "fp64_fast": dict(solver="sor64_fast", guess="zero"),
    "mixed_zero": dict(solver="mixed", guess="zero"),
    "mixed_previous": dict(solver="mixed", guess="previous"),
    "mixed_learned": dict(solver="mixed", guess="learned"),
    "pcg_zero": dict(solver="pcg", guess="zero"),
    "pcg_previous": dict(solver="pcg", guess="previous"),
    "pcg_learned": dict(solver="pcg", guess="learned"),
}


def rel_l2(a: np.ndarray, b: np.ndarray) -> float:
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


def interior(a: np.ndarray) -> np.ndarray:
    return a[2:-2, 2:-2, 2:-2]


def train_guess(sh, pairs: int, epochs: int, lr: float, dt_range, steps_per_case: int = 1,
                seed: int = 10) -> tuple[bytes, dict]:
    """Train the learned guess on `pairs` first solves of steps: runs of
    `steps_per_case` steps from seeded random irradiations and dt; returns
    the weights blob and a summary."""
    f = start_run(sh)
    t0 = time.perf_counter()
    G.init(f, seed=1, capacity=pairs)
    ncases = (pairs + steps_per_case - 1) // steps_per_case
    cases = G.random_cases(ncases, seed=seed, dt_range=dt_range)
    if steps_per_case == 1:
        n = G.capture_pairs(f, sh, cases, first_solve_only=True)
    else:
        n = G.capture_pairs(f, sh, cases, steps_per_case=steps_per_case)
    t1 = time.perf_counter()
    losses = [G.train(f, epochs=1, lr=lr, seed=e) for e in range(epochs)]
    t2 = time.perf_counter()
    blob = G.save_weights(f)
    f.close()
    return blob, {"pairs": n, "steps_per_case": steps_per_case, "epochs": epochs, "lr": lr, "dt_range": list(dt_range),
                  "capture_s": round(t1 - t0, 2), "train_s": round(t2 - t1, 2),
                  "loss_first": losses[0], "loss_last": losses[-1]}


def run_variant(sh, name: str, nsteps: int, snap_at: int, epsmat: float = 1e-10, blob: bytes | None = None):
    v = VARIANTS[name]
    p = dict(sh.params)
    sh.params["epsmat"] = epsmat
    f = start_run(sh)
    sh.params.update(p)
    if v["guess"] == "learned":
        G.load_weights(f, blob)
    f.set_solver(v["solver"], guess=v["guess"], tol=epsmat)
    steps, snap = [], None
    e0 = f.energy_sums()
    for s in range(nsteps):
        st = _ffi.StepStats()
        rc = f.L.ttfld_coupled_energy_eqs(f.h, 1, ctypes.byref(st))
        st.status = rc
        steps.append(dict(status=st.status, energy_iter=st.energy_iter, solves=st.solves, sweeps=st.sor_total,
                          fallbacks=st.fallbacks, step_ms=st.step_ms, solve_ms=st.solve_ms))
        if st.status < 0:
            break
        if s + 1 == snap_at:
            snap = (interior(f.download("ER")), interior(f.download("T")))
    e1 = f.energy_sums()
    f.close()
    steps[-1]["energy"] = {"start": e0, "end": e1}
    return steps, snap


def summarize(name: str, steps, snap, ref_snap, snap_at: int) -> dict:
    n = len(steps)
    tot = lambda k: float(sum(s[k] for s in steps))
    out = {"variant": name, **VARIANTS[name], "steps": n,
           "ms_per_step": tot("step_ms") / n, "solve_ms_per_step": tot("solve_ms") / n,
           "total_s": tot("step_ms") / 1e3,
           "outer_iter_per_step": tot("energy_iter") / n, "solves_per_step": tot("solves") / n,
           "sweeps_per_step": tot("sweeps") / n, "sweeps_per_solve": tot("sweeps") / max(tot("solves"), 1),
           "fallbacks": int(tot("fallbacks")), "fallback_rate": tot("fallbacks") / max(tot("solves"), 1),
           "worst_status": min(s["status"] for s in steps)}
    if "energy" in steps[-1]:
        e0, e1 = steps[-1]["energy"]["start"], steps[-1]["energy"]["end"]
        out["energy"] = {"e_rad_start": e0["e_rad"], "e_rad_end": e1["e_rad"], "e_gas_start": e0["e_gas"],
                         "e_gas_end": e1["e_gas"], "heating_end": e1["heating"],
                         "flux_bottom_end": e1["flux_bottom"], "flux_top_end": e1["flux_top"]}
    if snap is not None and ref_snap is not None:
        out["err_vs_fp64_1e-12"] = {"after_steps": snap_at, "ER": rel_l2(snap[0], ref_snap[0]),
                                     "T": rel_l2(snap[1], ref_snap[1])}
    return out


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("config", choices=sorted(SHELLS))
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--ref-steps", type=int, default=0,
                    help="steps of the FP64 1e-12 reference run the errors are taken at (0: no errors)")
    ap.add_argument("--variants", default="fp64_exact,mixed_zero,mixed_previous,mixed_learned")
    ap.add_argument("--pairs", type=int, default=16)
    ap.add_argument("--epochs", type=int, default=12)
    ap.add_argument("--lr", type=float, default=5e-4)
    ap.add_argument("--dt-range", default="50,500")
    ap.add_argument("--steps-per-case", type=int, default=1,
                    help="consecutive steps per training case (1: each pair is a run's first solve)")
    ap.add_argument("--delt", type=float, default=0.0, help="override the shell's dt")
    args = ap.parse_args(argv)
    sh = shell(args.config, seed=args.seed)
    if args.delt > 0:
        sh.params["delt"] = args.delt
    names = [v for v in args.variants.split(",") if v]
    ref_snap = None
    if args.ref_steps > 0:
        steps, ref_snap = run_variant(sh, "fp64_exact", args.ref_steps, args.ref_steps, epsmat=1e-12)
        s = summarize("fp64_exact", steps, None, None, 0)
        s["variant"] = "reference_fp64_exact_1e-12"
        print(json.dumps({"config": args.config, **s}), flush=True)
    blob = None
    if "mixed_learned" in names or "pcg_learned" in names:
        lo, hi = (float(x) for x in args.dt_range.split(","))
        blob, info = train_guess(sh, args.pairs, args.epochs, args.lr, (lo, hi), args.steps_per_case)
        print(json.dumps({"config": args.config, "training": info}), flush=True)
    for name in names:
        steps, snap = run_variant(sh, name, args.steps, args.ref_steps, blob=blob)
        print(json.dumps({"config": args.config, "dt": sh.params["delt"],
                          **summarize(name, steps, snap, ref_snap, args.ref_steps)}), flush=True)


if __name__ == "__main__":
    main()
