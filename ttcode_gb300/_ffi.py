"""ctypes binding of libttfld (include/ttfld.h).

This is the same binding a Python caller of the reference-facing C ABI would
write; the structures mirror the header field for field.  Importing it never
falls back to a CPU path: if the library is missing or cannot be loaded the
error propagates.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libttfld.so")

c_int32 = ctypes.c_int32
c_double = ctypes.c_double
P_double = ctypes.POINTER(ctypes.c_double)


class Dims(ctypes.Structure):
    _fields_ = [("nx", c_int32), ("ny", c_int32), ("nz", c_int32), ("poles", c_int32)]


METRIC_NAMES = ("xxa", "xxb", "dxa", "dxb", "xya", "xyb", "dya", "dyb", "xza", "xzb", "dza", "dzb",
                "ddx0", "ddx1", "ddy0", "ddy1", "ddz0", "ddz1", "surxa", "surxb", "surza", "surzb",
                "geoxg", "geoxh", "geoxga", "geoxha", "geozg", "geozga")


class Metrics(ctypes.Structure):
    _fields_ = [(n, P_double) for n in METRIC_NAMES]


class Params(ctypes.Structure):
    _fields_ = [("delt", c_double), ("sorparam", c_double), ("epsmat", c_double),
                ("fbottom", c_double), ("tirr", c_double), ("xnue", c_double),
                ("pr_num", c_double), ("kap0", c_double), ("itmax", c_int32),
                ("bcxmin", c_int32), ("ibdrad", c_int32), ("iflimtyp", c_int32),
                ("f_incident", c_int32), ("ieta", c_int32), ("isigtyp", c_int32),
                ("iii", c_int32), ("adjust_sor", c_int32), ("kappa_model", c_int32)]


class SolveOpts(ctypes.Structure):
    _fields_ = [("solver", c_int32), ("guess", c_int32), ("tol", c_double),
                ("inner_digits", c_int32), ("reserved", c_int32), ("max_sweeps", c_int32),
                ("fallback_rule", c_int32), ("sweep_form", c_int32)]


FALLBACK = {"first_sweep": 0, "never": 1, "residual": 2, "four_sweeps": 3}
SWEEP_FORM = {"neighbour": 0, "tma": 1, "split": 2, "wave": 3, "grid": 4}


class SolveStats(ctypes.Structure):
    _fields_ = [("sor_iter", c_int32), ("corrections", c_int32), ("fallback", c_int32),
                ("status", c_int32), ("rnorm", c_double), ("rhsnorm", c_double),
                ("true_resid_l1", c_double), ("guess_resid_l1", c_double), ("solve_ms", c_double),
                ("guess_ms", c_double), ("stalls", c_int32), ("gs_sweeps", c_int32)]


class RaddifParams(ctypes.Structure):
    _fields_ = [("d_t", ctypes.c_double), ("tinit_bottom", ctypes.c_double), ("modver", ctypes.c_int32),
                ("energy_iter", ctypes.c_int32), ("volxb", ctypes.c_void_p), ("volyb", ctypes.c_void_p),
                ("volzb", ctypes.c_void_p)]


class OpacityTable(ctypes.Structure):
    _fields_ = [("nt", ctypes.c_int32), ("nrh", ctypes.c_int32), ("log_t", ctypes.c_void_p),
                ("log_rho", ctypes.c_void_p), ("log_ross", ctypes.c_void_p), ("log_plnk", ctypes.c_void_p),
                ("log_abs", ctypes.c_void_p)]


class WaveTable(ctypes.Structure):
    _fields_ = [("nbins", ctypes.c_int32), ("log_waveopac", ctypes.c_void_p), ("bstar_bin", ctypes.c_void_p),
                ("rstar", ctypes.c_double), ("semi", ctypes.c_double)]


class FreedmanTableC(ctypes.Structure):
    _fields_ = [("log_ross", ctypes.c_void_p), ("log_plnk", ctypes.c_void_p), ("log_abs", ctypes.c_void_p),
                ("mu_gas", ctypes.c_double)]


class Energy(ctypes.Structure):
    _fields_ = [(n, c_double) for n in ("volume", "e_rad", "e_gas", "heating", "flux_bottom", "flux_top",
                                        "flux_theta")]


class StepStats(ctypes.Structure):
    _fields_ = [("energy_iter", c_int32), ("sor_total", c_int32), ("solves", c_int32),
                ("fallbacks", c_int32), ("status", c_int32), ("stalls", c_int32),
                ("global_deltaq", c_double), ("global_deltaer", c_double),
                ("solve_ms", c_double), ("step_ms", c_double)]


# enum ttfld_field
FIELDS = {
    "T": 0, "RH": 1, "CV": 2, "ER": 3, "ER_OLD": 4, "DELTA_ER": 5, "XKAPR": 6, "XKAPP": 7,
    "XKAPA": 8, "DXKAPP_DT": 9, "DXKAPA_DT": 10, "KMUL": 11, "Q": 12, "SCALAR": 13,
    "EVAL1": 32, "EVAL2": 33, "EVAL3": 34, "EVAL4": 35, "EVAL5": 36, "EVAL6": 37, "EVAL7": 38,
    "EVAL8": 39, "EVAL_1_6": 40, "JACOB_ETA": 41, "RHS_ER": 42, "SOR_A": 43, "SOR_B": 44,
    "SOR_C": 45, "SOR_D": 46, "SOR_E": 47, "SOR_F": 48, "SOR_G": 49, "FQ": 50, "FR": 51,
    "DIVF": 52, "DELTA_Q": 53,
    "FLIMX": 64, "FLIMY": 65, "FLIMZ": 66, "DIFRX": 67, "DIFRY": 68, "DIFRZ": 69,
    "FLUX_X": 70, "FLUX_Y": 71, "FLUX_Z": 72,
    "UPPERBND": 96, "MU_STAR": 97, "TINCIDENT": 98,
    "STELLARINPUT": 112, "STELLARTAU": 113, "DTAUS": 114,
}

SOLVER = {"sor64_exact": 0, "sor64_fast": 1, "mixed": 2, "pcg": 3}
# ttfld_time_sweeps also times the per-colour launches, the TMA-staged and the
# wavefront forms (an int 16 + P: the wavefront with windows of P theta planes)
TIMED_SWEEPS = dict(SOLVER, mixed_split=3, mixed_tma=4, mixed_wave=5, mixed_grid=6)
GUESS = {"zero": 0, "previous": 1, "learned": 2}

STATUS = {0: "ok", 1: "iteration limit reached", 2: "learned guess rejected",
          -1: "bad argument", -2: "CUDA error", -3: "configuration not implemented",
          -7: "non-positive Q (CLEAN_STOP)", -8: "non-finite norm", -9: "no learned-guess model",
          -10: "opacity table: T <= 0 or outside the table", -11: "internal invariant broken (library bug)"}

EXPORTS = ("ttfld_abi_version", "ttfld_status_string", "ttfld_create", "ttfld_destroy",
           "ttfld_set_params", "ttfld_get_params", "ttfld_set_solver", "ttfld_upload",
           "ttfld_download", "ttfld_field_size", "ttfld_device_ptr", "ttfld_copy_field",
           "ttfld_synchronize", "ttfld_stream", "ttfld_bounds", "ttfld_kappa", "ttfld_stellarinput_heating",
           "ttfld_diff", "ttfld_calculateflux", "ttfld_fill_evalues", "ttfld_fill_sor_matrix",
           "ttfld_solve_with_sor", "ttfld_solve_system", "ttfld_sor_sweeps",
           "ttfld_true_residual", "ttfld_adjust_sor_param", "ttfld_coupled_energy_eqs",
           "ttfld_diffusion", "ttfld_guess_load", "ttfld_guess_save", "ttfld_time_sweeps",
           "ttfld_kernel_launches", "ttfld_sor_solve_noalloc", "ttfld_guess_init",
           "ttfld_guess_dataset", "ttfld_guess_capture_next", "ttfld_guess_dataset_count",
           "ttfld_guess_train", "ttfld_guess_gradients", "ttfld_guess_predict",
           "ttfld_guess_num_params", "ttfld_begin_step", "ttfld_guess_set_conv", "ttfld_energy_sums",
           "ttfld_solve_with_hypre", "ttfld_raddif", "ttfld_set_opacity_table", "ttfld_set_wave_table",
           "ttfld_set_freedman_table")

_lib = None


class TTFLDError(RuntimeError):
    def __init__(self, where: str, status: int):
        super().__init__(f"{where}: status {status} ({STATUS.get(status, 'unknown')})")
        self.status = status


def lib():
    """Load libttfld.so (building it first if this checkout has no build)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        from . import build as _build
        _build.build()
    L = ctypes.CDLL(LIB_PATH)
    vp = ctypes.c_void_p
    L.ttfld_abi_version.restype = ctypes.c_int
    L.ttfld_status_string.restype = ctypes.c_char_p
    L.ttfld_status_string.argtypes = [ctypes.c_int]
    L.ttfld_create.argtypes = [ctypes.POINTER(vp), ctypes.POINTER(Dims), ctypes.POINTER(Metrics),
                               ctypes.POINTER(Params), ctypes.c_int]
    L.ttfld_destroy.argtypes = [vp]
    L.ttfld_set_params.argtypes = [vp, ctypes.POINTER(Params)]
    L.ttfld_get_params.argtypes = [vp, ctypes.POINTER(Params)]
    L.ttfld_set_solver.argtypes = [vp, ctypes.POINTER(SolveOpts)]
    L.ttfld_upload.argtypes = [vp, ctypes.c_int, vp]
    L.ttfld_download.argtypes = [vp, ctypes.c_int, vp]
    L.ttfld_field_size.restype = ctypes.c_size_t
    L.ttfld_field_size.argtypes = [vp, ctypes.c_int]
    L.ttfld_device_ptr.restype = vp
    L.ttfld_device_ptr.argtypes = [vp, ctypes.c_int]
    L.ttfld_copy_field.argtypes = [vp, ctypes.c_int, ctypes.c_int]
    L.ttfld_synchronize.argtypes = [vp]
    L.ttfld_stream.restype = vp
    L.ttfld_stream.argtypes = [vp]
    for n in ("ttfld_bounds", "ttfld_kappa", "ttfld_stellarinput_heating", "ttfld_fill_sor_matrix"):
        getattr(L, n).argtypes = [vp]
    L.ttfld_diff.argtypes = [vp, ctypes.c_int]
    L.ttfld_calculateflux.argtypes = [vp, ctypes.c_int]
    L.ttfld_fill_evalues.argtypes = [vp, ctypes.c_double]
    L.ttfld_solve_with_sor.argtypes = [vp, ctypes.c_int, ctypes.POINTER(SolveStats)]
    L.ttfld_solve_system.argtypes = [vp, ctypes.POINTER(SolveStats)]
    L.ttfld_solve_with_hypre.argtypes = [vp, ctypes.c_double, ctypes.c_int, ctypes.POINTER(SolveStats)]
    L.ttfld_raddif.argtypes = [vp, ctypes.POINTER(RaddifParams), ctypes.POINTER(SolveStats)]
    L.ttfld_set_opacity_table.argtypes = [vp, ctypes.POINTER(OpacityTable)]
    L.ttfld_set_wave_table.argtypes = [vp, ctypes.POINTER(WaveTable)]
    L.ttfld_set_freedman_table.argtypes = [vp, ctypes.POINTER(FreedmanTableC)]
    L.ttfld_sor_sweeps.argtypes = [vp, ctypes.c_int, P_double, P_double]
    L.ttfld_true_residual.argtypes = [vp, P_double, P_double]
    L.ttfld_adjust_sor_param.argtypes = [vp, P_double]
    L.ttfld_coupled_energy_eqs.argtypes = [vp, ctypes.c_int, ctypes.POINTER(StepStats)]
    L.ttfld_diffusion.argtypes = [vp, ctypes.POINTER(SolveStats)]
    L.ttfld_time_sweeps.argtypes = [vp, ctypes.c_int, ctypes.c_int, P_double]
    L.ttfld_kernel_launches.restype = ctypes.c_uint64
    L.ttfld_kernel_launches.argtypes = []
    L.ttfld_sor_solve_noalloc.argtypes = [vp] * 9 + [ctypes.c_int] * 3 + [ctypes.c_double] * 2 + \
        [ctypes.c_int] * 2 + [vp, ctypes.POINTER(ctypes.c_int), P_double, P_double]
    L.ttfld_guess_init.argtypes = [vp, ctypes.c_uint64]
    L.ttfld_guess_dataset.argtypes = [vp, ctypes.c_int]
    L.ttfld_guess_capture_next.argtypes = [vp]
    L.ttfld_guess_dataset_count.argtypes = [vp]
    L.ttfld_guess_train.argtypes = [vp, ctypes.c_int, ctypes.c_double, ctypes.c_uint64, P_double]
    L.ttfld_guess_gradients.argtypes = [vp, vp, vp, vp, P_double, vp]
    L.ttfld_guess_predict.argtypes = [vp, vp, vp]
    L.ttfld_begin_step.argtypes = [vp, ctypes.c_int]
    L.ttfld_guess_set_conv.argtypes = [ctypes.c_int]
    L.ttfld_energy_sums.argtypes = [vp, ctypes.POINTER(Energy)]
    L.ttfld_guess_num_params.restype = ctypes.c_size_t
    L.ttfld_guess_num_params.argtypes = []
    L.ttfld_guess_load.argtypes = [vp, vp, ctypes.c_size_t]
    L.ttfld_guess_save.argtypes = [vp, vp, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)]
    _lib = L
    return L


def check(where: str, rc: int, ok=(0,)) -> int:
    if rc not in ok:
        raise TTFLDError(where, rc)
    return rc
