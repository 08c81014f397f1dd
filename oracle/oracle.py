"""ctypes wrapper around the CPU oracle (test infrastructure only).

The oracle (``ttfld_oracle.c``) restates ttcode's implicit FLD energy step in
plain C; this wrapper exposes its arrays as numpy views in Fortran order with
the reference's shapes.  Only tests, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` leg of ``bench.py`` import this module.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libttfld_oracle.so")
_lib = None

HALO = ("T", "RH", "CV", "ER", "ER_OLD", "Q", "Q_OLD", "DELTA_ER", "XKAPR", "XKAPP",
        "XKAPA", "DXKAPP_DT", "DXKAPA_DT", "KMUL", "RHQX", "RHQY", "RHQZ",
        "STELLARTAU", "DTAUS", "STELLARINPUT", "SCALAR")
CELL = ("EVAL1", "EVAL2", "EVAL3", "EVAL4", "EVAL5", "EVAL6", "EVAL7", "EVAL8",
        "EVAL_1_6", "JACOB_ETA", "FQ", "FR", "RHS_ER", "SOR_A", "SOR_B", "SOR_C",
        "SOR_D", "SOR_E", "SOR_F", "SOR_G", "DIVF", "DIVF_OLD", "DFQ_DQ", "DFR_DQ",
        "DELTA_Q", "RHS_DIF", "HYP_A", "HYP_B", "HYP_C", "HYP_D", "HYP_E", "HYP_F",
        "HYP_G", "HYP_RHS", "RAD_AX", "RAD_CX", "RAD_AY", "RAD_CY", "RAD_AZ", "RAD_CZ", "RAD_B",
        "RAD_RHS")
FACE = ("FLIMX", "FLIMY", "FLIMZ", "DIFRX", "DIFRY", "DIFRZ", "FLUX_X", "FLUX_Y", "FLUX_Z")
PLANE = ("MU_STAR", "TINCIDENT")


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile; returns the library path."""
    if force or not os.path.exists(_LIB_PATH) or \
            os.path.getmtime(_LIB_PATH) < os.path.getmtime(os.path.join(_HERE, "ttfld_oracle.c")):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def _load():
    global _lib
    if _lib is None:
        build()
        lib = ctypes.CDLL(_LIB_PATH)
        vp = ctypes.c_void_p
        lib.ttor_create.restype = vp
        lib.ttor_create.argtypes = [ctypes.c_int] * 3
        lib.ttor_destroy.argtypes = [vp]
        lib.ttor_field.restype = ctypes.POINTER(ctypes.c_double)
        lib.ttor_field.argtypes = [vp, ctypes.c_char_p, ctypes.POINTER(ctypes.c_size_t)]
        lib.ttor_ifield.restype = ctypes.POINTER(ctypes.c_int)
        lib.ttor_ifield.argtypes = [vp, ctypes.c_char_p, ctypes.POINTER(ctypes.c_size_t)]
        lib.ttor_set.argtypes = [vp, ctypes.c_char_p, ctypes.c_double]
        lib.ttor_get.restype = ctypes.c_double
        lib.ttor_get.argtypes = [vp, ctypes.c_char_p]
        for name in ("gitter", "calcmustar", "bounds", "kappa", "qdens", "flim", "diff",
                     "calculateflux", "flux_bc", "stellarinput_heating", "fill_sor_matrix", "fill_hypre_system",
                     "b_vector_boundaries", "adjust_sor_param", "diffusion"):
            f = getattr(lib, "ttor_" + name)
            f.restype = ctypes.c_int
            f.argtypes = [vp]
        lib.ttor_planetshift.argtypes = [vp, ctypes.c_char_p]
        lib.ttor_fill_evalues.argtypes = [vp, ctypes.c_double]
        lib.ttor_calculatedivf_withf.argtypes = [vp, ctypes.c_int, ctypes.c_double]
        lib.ttor_solve_with_sor.argtypes = [vp, ctypes.c_int, ctypes.c_int]
        lib.ttor_sor_sweeps.argtypes = [vp, ctypes.c_int]
        lib.ttor_sor_sweeps_mt.argtypes = [vp, ctypes.c_int, ctypes.c_int]
        lib.ttor_solve_with_sor_mt.argtypes = [vp, ctypes.c_int]
        lib.ttor_set_freedman_table.argtypes = [vp, vp, vp, vp, ctypes.c_double]
        lib.ttor_set_wave_table.argtypes = [vp, ctypes.c_int, vp, vp, ctypes.c_double, ctypes.c_double]
        lib.ttor_coupled_energy_eqs.argtypes = [vp, ctypes.c_int]
        lib.ttor_raddif.argtypes = [vp, ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_int]
        lib.ttor_set_opacity_table.argtypes = [vp, ctypes.c_int, ctypes.c_int] + [vp] * 5
        lib.ttor_true_residual_l1.restype = ctypes.c_double
        lib.ttor_true_residual_l1.argtypes = [vp]
        _lib = lib
    return _lib


class Oracle:
    """One oracle state (the reference's module variables) of size nx, ny, nz."""

    def __init__(self, nx: int, ny: int, nz: int):
        self.lib = _load()
        self.nx, self.ny, self.nz = nx, ny, nz
        self.h = self.lib.ttor_create(nx, ny, nz)
        if not self.h:
            raise ValueError("oracle: bad dimensions")

    def close(self):
        if self.h:
            self.lib.ttor_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- arrays -------------------------------------------------------
    def shape_of(self, name: str):
        nx, ny, nz = self.nx, self.ny, self.nz
        if name in HALO:
            return (nx + 4, ny + 4, nz + 4)
        if name in CELL:
            return (nx, ny, nz)
        if name in FACE:
            return (nx + 1, ny + 1, nz + 1)
        if name in PLANE or name == "UPPERBND":
            return (ny + 4, nz + 4)
        return None

    def f(self, name: str) -> np.ndarray:
        """A writable Fortran-ordered view of oracle array ``name``."""
        n = ctypes.c_size_t()
        if name == "UPPERBND":
            p = self.lib.ttor_ifield(self.h, name.encode(), ctypes.byref(n))
            flat = np.ctypeslib.as_array(p, shape=(n.value,))
        else:
            p = self.lib.ttor_field(self.h, name.encode(), ctypes.byref(n))
            if not p:
                raise KeyError(name)
            flat = np.ctypeslib.as_array(p, shape=(n.value,))
        shp = self.shape_of(name)
        if shp is None:
            return flat
        return flat.reshape(shp, order="F")

    def set(self, name: str, value):
        if self.lib.ttor_set(self.h, name.encode(), float(value)) != 0:
            raise KeyError(name)

    def get(self, name: str) -> float:
        return self.lib.ttor_get(self.h, name.encode())

    # ---- routines -----------------------------------------------------
    def call(self, name: str, *args) -> int:
        fn = getattr(self.lib, "ttor_" + name)
        if name == "planetshift":
            return fn(self.h, args[0].encode())
        return fn(self.h, *args)
