"""The run's input file ``ipp`` as readinitfile reads it (ppmod.f:42-78), and
what the FLD step takes from it.

``read_ipp`` makes the same list-directed reads, record for record: every
input_init variable the file sets, by its Fortran name in lower case
(``int_tmp1``, ``dbl_tmp3``, ... for the scratch record), and ``poles``
from inc_poles (ppmod.f:73-77).  A value the file leaves null is None.

``params_of_ipp`` gives the parameters of an ``fld.FLD`` context (after
MISC_CHECKS, ``misc_checks``) and ``grid_of_ipp`` the grid GITTER builds from
XMIN..ZMAX, so that a ttcode run directory (ipp plus its AKTTD) drives the
library:

    ipp = read_ipp("ipp")
    f = start_run(akttd.shell_of_restart(akttd.read_restart("AKTTD"), grid_of_ipp(ipp),
                                         params_of_ipp(ipp, delt=...)))
"""
from __future__ import annotations

import os

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
    of ``set_burrows_table``; any other IKAPTYP needs ``kappa_model`` among
    the overrides).  DELT is the run's (the restart file's) time step.  The
    library has no poles: inc_poles >= 1 is refused unless ``poles_off``."""
    _need(ipp, "sorparam", "epsmat", "itmax", "fbot", "tirr", "xnue", "pr_num", "ibdrad", "iflimtyp",
          "f_incident", "bcxmin", "ieta", "isigtyp", "ikaptyp", "irad")
    misc_checks(ipp)
    if ipp["poles"] and not poles_off:
        raise IppError("inc_poles >= 1: the library implements poles = .false. only (pass poles_off=True "
                       "to run without them)")
    p = dict(delt=float(delt), sorparam=ipp["sorparam"], epsmat=ipp["epsmat"], fbottom=ipp["fbot"],
             tirr=ipp["tirr"], xnue=ipp["xnue"], pr_num=ipp["pr_num"], kap0=1.0e-2, itmax=ipp["itmax"],
             bcxmin=ipp["bcxmin"], ibdrad=ipp["ibdrad"], iflimtyp=ipp["iflimtyp"], f_incident=ipp["f_incident"],
             ieta=ipp["ieta"], isigtyp=ipp["isigtyp"], iii=1, adjust_sor=int(ipp["irad"] == 3))
    if 20 <= ipp["ikaptyp"] <= 25:
        p["kappa_model"] = 2
    elif "kappa_model" not in overrides:
        raise IppError(f"IKAPTYP={ipp['ikaptyp']}: give kappa_model (0 analytic, 1 prescribed) among the overrides")
    unknown = set(overrides) - set(p) - {"kappa_model"}
    if unknown:
        raise IppError(f"not FLD parameters: {sorted(unknown)}")
    p.update(overrides)
    return p
