"""The run's input file ``ipp`` as readinitfile reads it (ppmod.f:42-78), and
what the FLD step takes from it.

``read_ipp`` makes the same list-directed reads, record for record: every
input_init variable the file sets, by its Fortran name in lower case
(``int_tmp1``, ``dbl_tmp3``, ... for the scratch record), and ``poles``
from inc_poles (ppmod.f:73-77).  A value the file leaves null is None.

``params_of_ipp`` gives the parameters of an ``fld.FLD`` context (after
MISC_CHECKS, ``misc_checks``), ``grid_of_ipp`` the grid GITTER builds from
XMIN..ZMAX, and ``initial_bottom`` / ``bottom_gradients`` the bottom values
LOCALINIT sets (TinitBottom, RHinitbottom, D_RH, D_T; the IRAD=1 step's
boundary), so that a ttcode run directory (ipp plus its AKTTD) drives the
library:

    ipp = read_ipp("ipp")
    f = start_run(akttd.shell_of_restart(akttd.read_restart("AKTTD"), grid_of_ipp(ipp),
                                         params_of_ipp(ipp, delt=...)))
"""
from __future__ import annotations

import os

import numpy as np

from .fortio import ListDirected, integer, real
from .grid import Grid, gitter

I, D = integer, real
# one entry per READ(15,*) of readinitfile, ppmod.f:44-71; () = a READ with no items
RECORDS = (
    (("istepmax", I), ("irea", I), ("fdelt", D), ("dtmax", D)),
    (("iprstep", I), ("filestart", I)),
    (("ietot", I), ("isoth", I), ("isoden", I)),
    (("iadv", I), ("ifor", I), ("igrav", I), ("ivis", I), ("irad", I), ("inuc", I), ("iscal", I), ("idif", I)),
    (("irho", I), ("rhmin", D)),
    (("itemp", I), ("tempmax", D), ("tempmin", D)),
    (("ivel", I), ("velmax", D), ("veldamp", D), ("damp_steps", I)),
    (("ivistyp", I), ("xnue", D), ("idiss", I), ("alpha", D), ("ieta", I), ("iartvis", I), ("pr_num", D)),
    (("igastyp", I), ("gamma", D), ("mu_gas", D), ("icstyp", I), ("aspect", D)),
    (("ikaptyp", I), ("isigtyp", I), ("zkapmult", D), ("gamma_opc", D)),
    (("irotate", I), ("prot", D), ("ramp_start", D), ("ramp_full", D), ("windamp", D)),
    (("ibdrad", I), ("iflimtyp", I), ("f_incident", I), ("bcxmin", I), ("fbot", D)),
    (("sorparam", D), ("itmax", I), ("epsmat", D)),
    (),
    (("iperturb", I), ("perturb_typ", I), ("perturb_iter", I)),
    (("porb", D), ("ecc", D), ("ecc_start", D)),
    (("ifbotramp", I), ("framp_steps", I), ("fbot_final", D)),
    (("int_tmp1", I), ("dbl_tmp3", D), ("dbl_tmp2", D), ("dbl_tmp1", D)),
    (),
    (("ncosys", I), ("inc_poles", I)),
    (("modtyp", I), ("modver", I), ("planet_num", I)),
    (("startyp", D), ("rstar", D), ("tstar", D), ("mstar1", D), ("tirr", D), ("rh0", D)),
    (("rstar2", D), ("mstar2", D), ("rp", D), ("phip", D), ("psoft", D)),
    (("numdim", I),),
    (("global_nx", I), ("xmin", D), ("xmax", D), ("dxmin", D)),
    (("global_ny", I), ("ymin", D), ("ymax", D), ("dymin", D)),
    (("global_nz", I), ("zmin", D), ("zmax", D), ("dzmin", D)),
)


class IppError(ValueError):
    """An ipp file readinitfile would stop on, or a setting the library
    does not implement."""


def read_ipp(source) -> dict:
    """readinitfile (ppmod.f:42-78).  ``source`` is a path or the lines."""
    if isinstance(source, (str, os.PathLike)):
        with open(source) as fh:
            lines, name = fh.readlines(), os.fspath(source)
    else:
        lines, name = list(source), "<ipp>"
    rd = ListDirected(lines, name, IppError)
    out = {"nparticles": 3}                       # the one initialised variable, ppmod.f:13
    for rec in RECORDS:
        if not rec:
            rd.skip()
            continue
        vals = rd.read(len(rec), tuple(conv for _, conv in rec))
        out.update({n: v for (n, _), v in zip(rec, vals)})
    out["poles"] = out["inc_poles"] is not None and out["inc_poles"] >= 1
    return out


def misc_checks(ipp: dict) -> None:
    """MISC_CHECKS (ppsub.f:816-881) on the settings: IETOT was removed,
    IKAPTYP 15-19 needs MODTYP 2, and IBDRAD 10 stops whatever IKAPTYP is
    (the reference's test, IKAPTYP.ne.20 .or. IKAPTYP.ne.21, always holds).
    Its first test, open y boundaries, cannot fail for one rank with a
    periodic phi axis."""
    if ipp.get("ietot") is not None and ipp["ietot"] >= 1:
        raise IppError("removed from ttadv (IETOT >= 1)")
    kt = ipp.get("ikaptyp")
    if kt is not None and 15 <= kt <= 19 and ipp.get("modtyp") != 2:
        raise IppError("Elizas opacities only available for modtyp=2")
    if ipp.get("ibdrad") == 10 and (kt != 20 or kt != 21):
        raise IppError("wavelength dependent source term only available for ikaptyp=20")


def _need(ipp: dict, *names):
    missing = [n for n in names if ipp.get(n) is None]
    if missing:
        raise IppError(f"ipp leaves {', '.join(missing)} undefined")


def grid_of_ipp(ipp: dict) -> Grid:
    """GITTER's grid from the ipp extents: NCOSYS = 2, linear spacing
    (DXMIN = DYMIN = DZMIN = 0), the only grids the library implements."""
    _need(ipp, "ncosys", "global_nx", "global_ny", "global_nz", "xmin", "xmax", "ymin", "ymax", "zmin", "zmax",
          "dxmin", "dymin", "dzmin")
    if ipp["ncosys"] != 2:
        raise IppError(f"NCOSYS={ipp['ncosys']}: only the spherical grid (2) is implemented")
    if any(ipp[n] != 0.0 for n in ("dxmin", "dymin", "dzmin")):
        raise IppError("DXMIN/DYMIN/DZMIN != 0: only linear grids are implemented")
    return gitter(ipp["global_nx"], ipp["global_ny"], ipp["global_nz"], ipp["xmin"], ipp["xmax"], ipp["ymin"],
                  ipp["ymax"], ipp["zmin"], ipp["zmax"])


def params_of_ipp(ipp: dict, delt: float, poles_off: bool = False, **overrides) -> dict:
    """The FLD parameters a run with this ipp uses: SORPARAM, EPSMAT, ITMAX,
    FBOT, TIRR, XNUE, PR_NUM, IBDRAD, IFLIMTYP, F_INCIDENT, BCXMIN, IETA,
    ISIGTYP as read; ADJUST_SOR_PARAM where the IRAD=3 step calls it
    (ppenergy.f:372-374); the opacity source from IKAPTYP (20-25: the table
    of ``set_burrows_table``; 4-5 and 9-12, 14: prescribed, the arrays of
    ``opacity.freedman_kappa`` / ``opacity.burrows_kappa`` uploaded before
    each step; any other IKAPTYP needs ``kappa_model`` among the
    overrides).  DELT is the run's (the restart file's) time step.
    inc_poles >= 1 gives ``poles`` = 1 (the one-rank pole shifts; the IRAD=3
    step with the exact or FP32/FP64 SOR), unless ``poles_off``."""
    _need(ipp, "sorparam", "epsmat", "itmax", "fbot", "tirr", "xnue", "pr_num", "ibdrad", "iflimtyp",
          "f_incident", "bcxmin", "ieta", "isigtyp", "ikaptyp", "irad")
    misc_checks(ipp)
    p = dict(delt=float(delt), sorparam=ipp["sorparam"], epsmat=ipp["epsmat"], fbottom=ipp["fbot"],
             tirr=ipp["tirr"], xnue=ipp["xnue"], pr_num=ipp["pr_num"], kap0=1.0e-2, itmax=ipp["itmax"],
             bcxmin=ipp["bcxmin"], ibdrad=ipp["ibdrad"], iflimtyp=ipp["iflimtyp"], f_incident=ipp["f_incident"],
             ieta=ipp["ieta"], isigtyp=ipp["isigtyp"], iii=1, adjust_sor=int(ipp["irad"] == 3),
             poles=int(bool(ipp["poles"]) and not poles_off))
    if 20 <= ipp["ikaptyp"] <= 25:
        p["kappa_model"] = 2
    elif ipp["ikaptyp"] in (4, 5, 9, 10, 11, 12, 14):
        p["kappa_model"] = 1
    elif "kappa_model" not in overrides:
        raise IppError(f"IKAPTYP={ipp['ikaptyp']}: give kappa_model (0 analytic, 1 prescribed) among the overrides")
    unknown = set(overrides) - set(p) - {"kappa_model"}
    if unknown:
        raise IppError(f"not FLD parameters: {sorted(unknown)}")
    p.update(overrides)
    return p


# ---- LOCALINIT's bottom boundary values (ppinit.f:113-245) -------------------
def _f32(x: float) -> float:
    import numpy as np
    return float(np.float32(x))


def _f32_neg_product(a: float, e: float) -> float:
    """-a*(10.**e) with default-REAL operands: the power folded to the
    single-precision value of 10**e, the product rounded to single."""
    import numpy as np
    return -float(np.float32(np.float32(a) * np.float32(10.0 ** e)))


def initial_bottom(ipp: dict, restart=None, t=None, rh=None) -> tuple[float, float]:
    """TinitBottom and RHinitbottom: a restarted run (IREA mod 10 = 1) takes
    them from the restart file's scalars (READRESTART); a new run from the
    state's first cell, T(1,1,1) and RH(1,1,1) (ppinit.f:113-118), with
    ``t`` and ``rh`` given as (NX, NY, NZ) interior arrays."""
    _need(ipp, "irea")
    if ipp["irea"] % 10 == 1:
        if restart is None:
            raise IppError("a restarted run (IREA mod 10 = 1) takes TinitBottom from its AKTTD")
        return restart.scalars["TinitBottom"], restart.scalars["rhinitbottom"]
    if t is None or rh is None:
        raise IppError("a new run takes TinitBottom and RHinitbottom from T(1,1,1) and RH(1,1,1)")
    return float(t[0, 0, 0]), float(rh[0, 0, 0])


def bottom_gradients(ipp: dict, tinit_bottom: float, rhinit_bottom: float, table=None):
    """D_RH and D_T as LOCALINIT sets them for MODTYP = 2 (ppinit.f:149-245):
    the constants of MODVER 0-2, 4, 5 (default-REAL expressions evaluated in
    single precision, MODVER 4 / planet 1 in double), and for MODVER 3 the
    radiative gradient -3 Fbot kappa_R rho / (4 a c T^3) at the bottom with
    kappa_R from BurrowsOPC (``table``, an ``opacity.BurrowsTable``).  Where
    the reference leaves them unset (a MODVER/NX/planet without values,
    MODVER >= 6) the result is None."""
    from .opacity import burrows_opc
    from .synthetic import ARAD
    _need(ipp, "modtyp", "modver", "planet_num", "global_nx", "fbot")
    if ipp["modtyp"] != 2:
        raise IppError(f"MODTYP={ipp['modtyp']}: only the planet models (MODTYP 2) are implemented")
    mv, nx, planet = ipp["modver"], ipp["global_nx"], ipp["planet_num"]
    if mv == 0:
        return _f32_neg_product(2.1870361, -12.0), _f32_neg_product(1.3611882, -6.0)
    if mv == 1:
        return _f32_neg_product(2.7934540, -9.0), _f32(-0.00097568917)
    if mv == 2:
        return _f32_neg_product(2.3748328, -11.0), _f32_neg_product(4.0182995, -6.0)
    if mv == 3:
        if table is None:
            raise IppError("MODVER 3 takes kappa_R at the bottom from the Burrows table")
        kr = burrows_opc(table, tinit_bottom, rhinit_bottom).kap_r
        fd = _f32(2.99792458e10)
        t3 = (tinit_bottom * tinit_bottom) * tinit_bottom
        return 0.0, -(3.0 * ipp["fbot"] * kr * rhinit_bottom / (4.0 * ARAD * fd * t3))
    if mv == 4:
        if planet == 1:
            return ((-(_f32(2.1976300) * 10.0 ** -10.0), -(_f32(5.0305445) * 10.0 ** -6.0)) if nx == 100
                    else (None, None))
        if planet == 2:
            return ((_f32_neg_product(4.1081340, -10.0), _f32_neg_product(4.6779189, -5.0)) if nx == 100
                    else (None, None))
        if planet == 5:
            return (_f32(-5.5412161e-12), _f32(-4.1841993e-06)) if nx == 100 else (None, None)
        raise IppError(f"No initiliation file defined for planet_num {planet}")
    if mv == 5:
        if nx == 60:
            return _f32_neg_product(1.9417530, -10.0), _f32_neg_product(6.2500764, -6.0)
        if nx == 100:
            return _f32_neg_product(1.9756314, -10.0), _f32_neg_product(5.9942251, -6.0)
        return None, None
    return None, None


def semi_major_axis(ipp: dict) -> float:
    """The orbit's semi-major axis in cm, pp.f:205-206:
    (GRAV*MSOL*(mstar1+mstar2)*((Porb*DAY)**2)/(4*PI*PI))**(1/3), with
    the single-precision constants of ppmod.f:1074-1092."""
    import math
    grav, msol, day = float(np.float32(6.672e-8)), float(np.float32(1.989e33)), float(np.float32(8.64e4))
    pd = ipp["porb"] * day
    x = grav * msol * (ipp["mstar1"] + ipp["mstar2"]) * (pd * pd) / (4.0 * math.pi * math.pi)
    return math.pow(x, 1.0 / 3.0)


def open_run_directory(directory: str, poles_off: bool = False, **overrides):
    """A ttcode run directory as the set-up reads it: ``ipp`` (readinitfile),
    the restart file ``AKTTD`` (or ``AKTTD_ASCII``, READRESTART) on GITTER's
    grid, and for IKAPTYP 20-25 the Burrows tables (READBURROWSOPCTABLE;
    for 20-24 with the BSTAR bins, RSTAR and the semi-major axis the binned
    stellar heating needs).
    Returns (shell, table, ipp, restart): ``fld.start_run(shell,
    opacity_table=table)`` starts a context from them (for IKAPTYP 4-5 and
    9-14 the caller uploads ``opacity.freedman_kappa`` /
    ``opacity.burrows_kappa`` arrays as prescribed opacities).  DELT is the
    restart file's; ``overrides`` go to ``params_of_ipp``."""
    from . import akttd, opacity
    ipp = read_ipp(os.path.join(directory, "ipp"))
    binary = os.path.join(directory, "AKTTD")
    if os.path.exists(binary):
        rst = akttd.read_restart(binary)
    else:
        rst = akttd.read_restart_ascii(os.path.join(directory, "AKTTD_ASCII"))
    params = params_of_ipp(ipp, rst.delt, poles_off=poles_off, **overrides)
    table = None
    if params["kappa_model"] == 2:
        table = opacity.read_opacity_tables(directory, ipp["planet_num"], ipp["ikaptyp"], ipp["gamma_opc"],
                                            ipp["mu_gas"])
        table.rstar, table.semi = ipp["rstar"], semi_major_axis(ipp)
    shell = akttd.shell_of_restart(rst, grid_of_ipp(ipp), params)
    return shell, table, ipp, rst
