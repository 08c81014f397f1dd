"""Training and evaluation of the learned initial guess (host side).

Pairs come from the solver itself: for a seeded random irradiation pattern
(substellar longitude phi0 and T_irr) and a time step dt in [50, 500] s the
shell's implicit step is taken with SOLVE_WITH_SOR's answer captured as the
target.  Training runs entirely on the GPU through the C ABI
(`ttfld_guess_train`); evaluation counts the sweeps the solver needs from
the zero, the previous-step and the learned initial guess.
"""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass

import numpy as np

from . import _ffi
from ._ffi import check
from .fld import FLD
from .synthetic import MU_MIN, Shell


def irradiation(shell: Shell, phi0: float, tirr: float):
    """MU_STAR and TINCIDENT planes of CALCMUSTAR / CALC_TINCIDENT (F_INCIDENT=2)
    with the substellar point moved to longitude phi0."""
    g = shell.grid
    ny, nz = g.ny, g.nz
    yb = np.array([g.at("xyb", j) for j in range(-1, ny + 3)])
    zb = np.array([g.at("xzb", k) for k in range(-1, nz + 3)])
    cyz = np.cos(yb - phi0)[:, None] * np.cos(zb)[None, :]
    mu = np.asfortranarray(np.maximum(cyz, MU_MIN))
    tinc = np.where(cyz >= 0, tirr * np.power(np.maximum(cyz, 0.0), 0.25), 0.0)
    return mu, np.asfortranarray(np.maximum(tinc, 0.0))


@dataclass
class Case:
    phi0: float
    tirr: float
    dt: float


def random_cases(n: int, seed: int, dt_range=(50.0, 500.0)):
    rng = np.random.default_rng(seed)
    return [Case(float(rng.uniform(0, 2 * math.pi)), float(rng.uniform(1500.0, 2500.0)),
                 float(math.exp(rng.uniform(math.log(dt_range[0]), math.log(dt_range[1])))))
            for _ in range(n)]


def reset_state(f: FLD, shell: Shell, case: Case):
    """The shell's starting state with one case's irradiation and dt."""
    for n in ("T", "RH", "CV", "ER", "KMUL"):
        f.upload(n, shell.fields[n])
    mu, tinc = irradiation(shell, case.phi0, case.tirr)
    f.upload("MU_STAR", mu)
    f.upload("TINCIDENT", tinc)
    f.set_params(delt=case.dt, iii=0)
    f.bounds()
    f.kappa()
    f.set_params(iii=1)
    f.begin_step(new_run=True)   # no previous solution belongs to this state


def capture_pairs(f: FLD, shell: Shell, cases, solver="mixed", tol=1e-10, first_solve_only=False,
                  steps_per_case=1):
    """For each case, `steps_per_case` consecutive implicit steps from the
    case's starting state; the first solve of every step becomes a pair (its
    starting state and its solution).
    With first_solve_only (one step per case) the step stops after its first
    outer iteration: the pair is the same, the rest of the step is not
    needed for it."""
    L = f.L
    itmax = f.params["itmax"]
    f.set_solver(solver, guess="zero", tol=tol, max_sweeps=itmax if first_solve_only else 0)
    for case in cases:
        reset_state(f, shell, case)
        for _ in range(1 if first_solve_only else steps_per_case):
            check("capture", L.ttfld_guess_capture_next(f.h))
            if first_solve_only:
                f.set_params(itmax=1)   # one outer iteration; the solve keeps its own budget
                st = _ffi.StepStats()
                check("capture step", L.ttfld_coupled_energy_eqs(f.h, 1, ctypes.byref(st)), ok=(0, 1, 2))
                f.set_params(itmax=itmax)
            else:
                f.coupled_energy_eqs(True)
    return L.ttfld_guess_dataset_count(f.h)


def train(f: FLD, epochs: int, lr: float, seed: int = 0) -> float:
    loss = ctypes.c_double()
    check("train", f.L.ttfld_guess_train(f.h, epochs, lr, seed, ctypes.byref(loss)))
    return loss.value


def sweeps_with(f: FLD, shell: Shell, case: Case, guess: str, solver="mixed", tol=1e-10):
    """Sweeps, solves, fallbacks and solve time of one implicit step whose
    first solve starts from the given guess (with the learned guess the
    step's later solves start from the previous solution)."""
    reset_state(f, shell, case)
    f.set_solver(solver, guess=guess, tol=tol)
    st = f.coupled_energy_eqs(True)
    return st.sor_total, st.solves, st.fallbacks, st.solve_ms


def save_weights(f: FLD) -> bytes:
    need = ctypes.c_size_t()
    check("size", f.L.ttfld_guess_save(f.h, None, 0, ctypes.byref(need)))
    buf = (ctypes.c_char * need.value)()
    check("save", f.L.ttfld_guess_save(f.h, buf, need.value, ctypes.byref(need)))
    return bytes(buf)


def load_weights(f: FLD, blob: bytes):
    buf = (ctypes.c_char * len(blob)).from_buffer_copy(blob)
    check("load", f.L.ttfld_guess_load(f.h, buf, len(blob)))


def init(f: FLD, seed: int, capacity: int = 0):
    check("init", f.L.ttfld_guess_init(f.h, seed))
    if capacity:
        check("dataset", f.L.ttfld_guess_dataset(f.h, capacity))


def num_params() -> int:
    return int(_ffi.lib().ttfld_guess_num_params())
