"""Host-side mirror of the reference's FLD subroutine interface.

``FLD`` owns one libttfld context: the module arrays of the step live on the
GPU and the methods are named after the Fortran subroutines they replace
(SOLVE_WITH_SOR, FILL_EVALUES, DIFF, COUPLED_ENERGY_EQS, DIFFUSION, ...).
Every call goes through the C ABI in include/ttfld.h; there is no CPU path.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _ffi
from ._ffi import FIELDS, GUESS, SOLVER, check, lib
from .grid import Grid

HALO = ("T", "RH", "CV", "ER", "ER_OLD", "DELTA_ER", "XKAPR", "XKAPP", "XKAPA", "DXKAPP_DT",
        "DXKAPA_DT", "KMUL", "Q", "SCALAR")
CELL = ("EVAL1", "EVAL2", "EVAL3", "EVAL4", "EVAL5", "EVAL6", "EVAL7", "EVAL8", "EVAL_1_6",
        "JACOB_ETA", "RHS_ER", "SOR_A", "SOR_B", "SOR_C", "SOR_D", "SOR_E", "SOR_F", "SOR_G",
        "FQ", "FR", "DIVF", "DELTA_Q")


def field_shape(name: str, nx: int, ny: int, nz: int):
    if name in HALO:
        return (nx + 4, ny + 4, nz + 4)
    if name in CELL:
        return (nx, ny, nz)
    if name in ("FLIMX", "DIFRX", "FLUX_X"):
        return (nx + 1, ny, nz)
    if name in ("FLIMY", "DIFRY", "FLUX_Y"):
        return (nx, ny + 1, nz)
    if name in ("FLIMZ", "DIFRZ", "FLUX_Z"):
        return (nx, ny, nz + 1)
    if name in ("UPPERBND", "MU_STAR", "TINCIDENT"):
        return (ny + 4, nz + 4)
    if name == "STELLARINPUT":
        return (nx, ny + 4, nz + 4)
    if name in ("STELLARTAU", "DTAUS"):
        return (nx + 1, ny + 4, nz + 4)
    raise KeyError(name)


def make_params(p: dict) -> _ffi.Params:
    out = _ffi.Params()
    for k, _ in _ffi.Params._fields_:
        setattr(out, k, p[k])
    return out


class FLD:
    """One device-resident FLD step (one rank's module arrays)."""

    def __init__(self, grid: Grid, params: dict, device: int = 0):
        self.L = lib()
        self.grid = grid
        self.nx, self.ny, self.nz = grid.nx, grid.ny, grid.nz
        self.params = dict(params)
        dims = _ffi.Dims(self.nx, self.ny, self.nz, int(self.params.get("poles", 0)))
        self._metric_keep = {}
        m = _ffi.Metrics()
        for n in _ffi.METRIC_NAMES:
            a = np.ascontiguousarray(grid.m[n], dtype=np.float64)
            self._metric_keep[n] = a
            setattr(m, n, a.ctypes.data_as(_ffi.P_double))
        h = ctypes.c_void_p()
        check("ttfld_create", self.L.ttfld_create(ctypes.byref(h), ctypes.byref(dims), ctypes.byref(m),
                                                  ctypes.byref(make_params(self.params)), device))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.L.ttfld_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # ---- parameters -----------------------------------------------------
    def set_params(self, **kw):
        self.params.update(kw)
        check("ttfld_set_params", self.L.ttfld_set_params(self.h, ctypes.byref(make_params(self.params))))

    def set_solver(self, solver: str = "sor64_exact", guess: str = "zero", tol: float = 1e-10,
                   inner_digits: int = 0, max_sweeps: int = 0,
                   fallback: str = "four_sweeps", sweep_form: str = "neighbour"):
        """ttfld_set_solver: the solver of SOLVE_WITH_SOR's system (a key of
        SOLVER: sor64_exact, the reference loop; sor64_fast; mixed, FP32
        sweeps in FP64 defect correction; pcg), the initial guess (zero,
        previous, learned), the tolerance on ||b - Ax||_1 / ||b||_1, the
        mixed solver's inner target (0: its default of four digits) and sweep
        budget (0: ITMAX), the guess's fallback rule (a key of FALLBACK) and
        the mixed solver's FP32 sweep kernel (a key of SWEEP_FORM: neighbour,
        the default; grid; split; tma; wave -- all the same iterate)."""
        o = _ffi.SolveOpts(SOLVER[solver], GUESS[guess], tol, inner_digits, 0, max_sweeps,
                           _ffi.FALLBACK[fallback], _ffi.SWEEP_FORM[sweep_form])
        check("ttfld_set_solver", self.L.ttfld_set_solver(self.h, ctypes.byref(o)))

    # ---- module arrays ----------------------------------------------------
    def upload(self, name: str, arr):
        shp = field_shape(name, self.nx, self.ny, self.nz)
        dt = np.int32 if name == "UPPERBND" else np.float64
        a = np.asfortranarray(np.asarray(arr, dtype=dt))
        if a.shape != shp:
            raise ValueError(f"{name}: shape {a.shape} != {shp}")
        check(f"upload {name}", self.L.ttfld_upload(self.h, FIELDS[name], a.ctypes.data_as(ctypes.c_void_p)))

    def download(self, name: str) -> np.ndarray:
        shp = field_shape(name, self.nx, self.ny, self.nz)
        dt = np.int32 if name == "UPPERBND" else np.float64
        a = np.empty(shp, dtype=dt, order="F")
        check(f"download {name}", self.L.ttfld_download(self.h, FIELDS[name], a.ctypes.data_as(ctypes.c_void_p)))
        return a

    def load_shell(self, shell):
        for n, a in shell.fields.items():
            self.upload(n, a)

    # ---- the reference subroutines ---------------------------------------
    def bounds(self):
        check("BOUNDS", self.L.ttfld_bounds(self.h))

    def kappa(self):
        check("KAPPA", self.L.ttfld_kappa(self.h))

    def stellarinput_heating(self):
        check("STELLARINPUT_HEATING", self.L.ttfld_stellarinput_heating(self.h))

    def diff(self, energy_iter: int = 0):
        check("DIFF", self.L.ttfld_diff(self.h, energy_iter))

    def calculateflux(self, energy_iter: int = 0):
        check("CALCULATEFLUX", self.L.ttfld_calculateflux(self.h, energy_iter))

    def fill_evalues(self, theta: float = 1.0):
        check("FILL_EVALUES", self.L.ttfld_fill_evalues(self.h, theta))

    def fill_sor_matrix(self):
        check("FILL_SOR_MATRIX", self.L.ttfld_fill_sor_matrix(self.h))

    def solve_with_sor(self, print_max_values: bool = True) -> _ffi.SolveStats:
        st = _ffi.SolveStats()
        check("SOLVE_WITH_SOR", self.L.ttfld_solve_with_sor(self.h, int(print_max_values), ctypes.byref(st)),
              ok=(0, 1, 2))
        return st

    def solve_system(self) -> _ffi.SolveStats:
        st = _ffi.SolveStats()
        check("solve_system", self.L.ttfld_solve_system(self.h, ctypes.byref(st)), ok=(0, 1, 2))
        return st

    def solve_with_hypre(self, tol: float = 0.0, maxit: int = 0) -> _ffi.SolveStats:
        """SOLVE_WITH_HYPRE (IRAD=2): PCG on the FILLHYPREMATRIX system; tol
        and maxit 0 select the reference's 1e-6 and 50."""
        st = _ffi.SolveStats()
        check("SOLVE_WITH_HYPRE", self.L.ttfld_solve_with_hypre(self.h, tol, maxit, ctypes.byref(st)), ok=(0, 1))
        return st

    def raddif(self, d_t: float = 0.0, tinit_bottom: float = 0.0, modver: int = 1,
               energy_iter: int = 0) -> _ffi.SolveStats:
        """RADDIF (IRAD=1): ER from T, DIFFEL, SOLVMAT with RADIATIVEBOUND,
        T from ER (ttfld_raddif)."""
        from .grid import volumes
        vx, vy, vz = (np.ascontiguousarray(v, dtype=np.float64) for v in volumes(self.grid))
        p = _ffi.RaddifParams(d_t, tinit_bottom, modver, energy_iter, vx.ctypes.data, vy.ctypes.data,
                              vz.ctypes.data)
        st = _ffi.SolveStats()
        check("RADDIF", self.L.ttfld_raddif(self.h, ctypes.byref(p), ctypes.byref(st)), ok=(0, 1))
        return st

    def set_opacity_table(self, log_t, log_rho, log_ross, log_plnk, log_abs):
        """The (T, rho) opacity table kappa_model 2 interpolates (BurrowsOPC):
        log10 nodes and log10 means, shape (len(log_t), len(log_rho))."""
        keep = [np.ascontiguousarray(log_t, dtype=np.float64), np.ascontiguousarray(log_rho, dtype=np.float64)]
        keep += [np.asfortranarray(a, dtype=np.float64) for a in (log_ross, log_plnk, log_abs)]
        nt, nrh = keep[0].size, keep[1].size
        if any(a.shape != (nt, nrh) for a in keep[2:]):
            raise ValueError("opacity arrays must be (len(log_t), len(log_rho))")
        t = _ffi.OpacityTable(nt, nrh, *[a.ctypes.data for a in keep])
        check("ttfld_set_opacity_table", self.L.ttfld_set_opacity_table(self.h, ctypes.byref(t)))

    def set_wave_table(self, log_waveopac, bstar_bin, rstar: float, semi: float):
        """The per-bin part of the kappa_model 2 table for IKAPTYP 20-24 (KAPPA's
        per-bin opacities and the binned STELLARINPUT_HEATING): log10
        BurrowsXKAP_waveopac, shape (nt, nrh, nbins); BSTAR_BIN (nbins); RSTAR
        (solar radii) and the semi-major axis (cm).  nbins = 0 (an empty
        bstar_bin) goes back to the grey heating."""
        bs = np.ascontiguousarray(bstar_bin, dtype=np.float64)
        w = np.asfortranarray(log_waveopac, dtype=np.float64)
        if bs.size and w.shape[2] != bs.size:
            raise ValueError("log_waveopac must be (nt, nrh, nbins) with nbins = len(bstar_bin)")
        self._wave_keep = (w, bs)
        t = _ffi.WaveTable(bs.size, w.ctypes.data, bs.ctypes.data, float(rstar), float(semi))
        check("ttfld_set_wave_table", self.L.ttfld_set_wave_table(self.h, ctypes.byref(t)))

    def set_freedman_table(self, log_ross, log_plnk, log_abs, mu_gas: float):
        """FreedmanOPC's table for kappa_model 3 (the IKAPTYP 4:5 branch):
        log10 means on the 42 x 18 (T, P) nodes, and mu_gas."""
        keep = [np.asfortranarray(a, dtype=np.float64) for a in (log_ross, log_plnk, log_abs)]
        if any(a.shape != (42, 18) for a in keep):
            raise ValueError("Freedman means must be (42, 18): FreedmanTVAL x FreedmanPVAL")
        t = _ffi.FreedmanTableC(*[a.ctypes.data for a in keep], float(mu_gas))
        check("ttfld_set_freedman_table", self.L.ttfld_set_freedman_table(self.h, ctypes.byref(t)))

    def set_burrows_table(self, table):
        """A table of ``opacity.read_burrows_table`` for KAPPA's IKAPTYP 20:25
        branch (pprphy.f:321-351; ``kappa_model`` 2): its nodes and its
        Rosseland, Planck and absorption means."""
        if table.ikaptyp not in (20, 21, 22, 23, 24, 25):
            raise ValueError(f"IKAPTYP {table.ikaptyp}: the device implements KAPPA's 20:25 branch")
        self.set_opacity_table(table.log_t, table.log_rho, table.ross, table.plnk, table.absk)

    def sor_sweeps(self, n: int):
        r, b = ctypes.c_double(), ctypes.c_double()
        check("sor_sweeps", self.L.ttfld_sor_sweeps(self.h, n, ctypes.byref(r), ctypes.byref(b)))
        return r.value, b.value

    def true_residual(self):
        r, b = ctypes.c_double(), ctypes.c_double()
        check("true_residual", self.L.ttfld_true_residual(self.h, ctypes.byref(r), ctypes.byref(b)))
        return r.value, b.value

    def adjust_sor_param(self) -> float:
        w = ctypes.c_double()
        check("ADJUST_SOR_PARAM", self.L.ttfld_adjust_sor_param(self.h, ctypes.byref(w)))
        self.params["sorparam"] = w.value
        return w.value

    def begin_step(self, new_run: bool = False):
        """The next solve is an implicit step's first (ttfld_begin_step)."""
        check("begin_step", self.L.ttfld_begin_step(self.h, int(new_run)))

    def coupled_energy_eqs(self, do_bounds: bool = True) -> _ffi.StepStats:
        st = _ffi.StepStats()
        check("COUPLED_ENERGY_EQS", self.L.ttfld_coupled_energy_eqs(self.h, int(do_bounds), ctypes.byref(st)),
              ok=(0, 1, 2))
        return st

    def diffusion(self) -> _ffi.SolveStats:
        st = _ffi.SolveStats()
        check("DIFFUSION", self.L.ttfld_diffusion(self.h, ctypes.byref(st)), ok=(0, 1))
        return st

    def energy_sums(self) -> dict:
        """FP64 energy sums of the current state (ttfld_energy_sums)."""
        e = _ffi.Energy()
        check("energy_sums", self.L.ttfld_energy_sums(self.h, ctypes.byref(e)))
        return {n: getattr(e, n) for n, _ in _ffi.Energy._fields_}

    def stream_ptr(self) -> int:
        """The cudaStream_t the library issues this context's work on."""
        return int(self.L.ttfld_stream(self.h))

    def time_sweeps(self, solver, n: int) -> float:
        """Mean device time of one sweep: solver is a key of TIMED_SWEEPS or
        the ABI's code (16 + P: the wavefront form with P-plane windows)."""
        code = solver if isinstance(solver, int) else _ffi.TIMED_SWEEPS[solver]
        ms = ctypes.c_double()
        check("time_sweeps", self.L.ttfld_time_sweeps(self.h, code, n, ctypes.byref(ms)))
        return ms.value

    def synchronize(self):
        check("synchronize", self.L.ttfld_synchronize(self.h))


def start_run(shell, device: int = 0, opacity_table=None) -> FLD:
    """Context loaded with a synthetic shell and the initial BOUNDS/KAPPA of
    the main program's set-up (pp.f:419-463): BOUNDS at III=0, then KAPPA.
    ``opacity_table`` (an ``opacity.BurrowsTable``) is set before them, as
    READBURROWSOPCTABLE runs before the set-up; kappa_model 2 needs it."""
    f = FLD(shell.grid, shell.params, device)
    if opacity_table is not None:
        f.set_burrows_table(opacity_table)
        t = opacity_table
        if t.ikaptyp in (20, 21, 22, 23, 24) and t.bstar_bin is not None and t.semi:
            f.set_wave_table(t.waveopac, t.bstar_bin, t.rstar, t.semi)
    f.load_shell(shell)
    f.set_params(iii=0)
    f.bounds()
    f.kappa()
    f.set_params(iii=shell.params.get("iii", 1))
    return f
