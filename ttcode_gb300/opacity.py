"""Burrows (T, rho) opacity tables on the host: BurrowsOPC's node grid and the
table files KAPPA's Burrows branches read.

* ``BURROWS_LOG_T``, ``BURROWS_LOG_RHO``: the 50 + 50 interpolation nodes
  (log10 K and log10 g/cm^3) of the module arrays BurrowsT / BurrowsRH
  (ppmod.f:660, set by DATA statements at ppmod.f:735-757).  The DATA
  constants are default REAL, so each node is the single-precision value of
  its literal widened to double, as here.
* ``read_burrows_table``: READBURROWSOPCTABLE (pprphy.f:1231-1505): ten
  header records, the stellar temperature the absorption means were made
  for, then one list-directed record per (T, rho) node, T outer, of 5
  (IKAPTYP 9-14), 35 (20, 21) or 95 (22-25) values: T, rho, log10 of the
  Planck, Rosseland and absorption means, then 30 stellar-wavelength bins,
  30 local-wavelength bins and 30 local black-body weights.  Every array
  starts at -7 (a missing value); the IKAPTYP 11, 12, 14, 20, 24, 25
  adjustments follow the reads as in the reference.
* ``read_bstar_bins``: the BSTAR_WAVEBINS file of the wavelength types
  (pprphy.f:1507-1540).
* ``burrows_file_name``, ``bstar_file_name``: the file a planet and IKAPTYP
  open (OPENOPACITYFILE_WOTIOVO / OPENOPACITYFILE_WITH_TIOVO,
  ppplanets.f:90-213; pprphy.f:1510-1527).
* ``planet_kap_extra``: SETPLANETKAPEXTRA (ppplanets.f:36-59).
* ``burrows_opc``: BurrowsOPC's interpolation at one (T, rho) on the host,
  the wavelength bins included (the device interpolates the three means);
  ``burrows_kappa``: KAPPA's IKAPTYP 9:12 and 14 branches on the host, for
  prescribed opacities (``kappa_model`` 1).
* Freedman (T, P) tables of IKAPTYP 4-7: ``read_freedman_table``
  (READFREEDMANOPCTABLE, pprphy.f:944-1002), ``freedman_opc`` (FreedmanOPC,
  pprphy.f:800-942) and ``freedman_kappa`` (KAPPA's 4:5 branch with the
  ideal-gas pressure) on the host; the opacities reach the device as
  prescribed arrays (``kappa_model`` 1).

``FLD.set_burrows_table`` hands a table of the IKAPTYP 20:25 types to the
device (``kappa_model`` 2).  The table files are not part of the reference
tree; the tests write files in this layout.
"""
from __future__ import annotations

import math
import os
from dataclasses import dataclass, field

import numpy as np

from .fortio import ListDirected, ListDirectedError, integer
from .synthetic import RGAS

WAVE_BINS = 30          # nwave_bins, ppmod.f:489
NODES = 50              # BurrowsT(50), BurrowsRH(50), ppmod.f:660
MISSING = -7.0          # pprphy.f:1285-1288

# DATA BurrowsT / BurrowsRH, ppmod.f:735-757 (default-REAL constants)
BURROWS_LOG_T = np.array([
    1.69896, 1.73978, 1.78061, 1.82143, 1.86225, 1.90308, 1.94390, 1.98473, 2.02555, 2.06637,
    2.10720, 2.14802, 2.18884, 2.22967, 2.27049, 2.31132, 2.35214, 2.39296, 2.43379, 2.47461,
    2.51543, 2.55626, 2.59708, 2.63790, 2.67873, 2.71955, 2.76038, 2.80120, 2.84202, 2.88285,
    2.92367, 2.96406, 3.00488, 3.04571, 3.08653, 3.12735, 3.16818, 3.20900, 3.24983, 3.29065,
    3.33147, 3.37230, 3.41312, 3.45394, 3.49477, 3.53559, 3.57642, 3.61724, 3.65806, 3.69889,
], dtype=np.float32).astype(np.float64)
BURROWS_LOG_RHO = np.array([
    -11.9996, -11.7954, -11.5913, -11.3872, -11.1831, -10.9790, -10.7748, -10.5707, -10.3666, -10.1625,
    -9.95837, -9.75425, -9.55014, -9.34602, -9.14190, -8.93778, -8.73366, -8.52954, -8.32543, -8.12131,
    -7.91719, -7.71307, -7.50895, -7.30483, -7.10071, -6.89660, -6.69248, -6.48836, -6.28424, -6.08012,
    -5.87600, -5.67189, -5.46777, -5.26365, -5.05953, -4.85541, -4.65129, -4.44718, -4.24479, -4.04068,
    -3.83656, -3.63244, -3.42875, -3.22464, -3.02052, -2.81640, -2.61228, -2.40816, -2.20404, -1.99993,
], dtype=np.float32).astype(np.float64)

WITH_TIOVO = (9, 20)                               # pprphy.f:1273
WITHOUT_TIOVO = (10, 11, 12, 14, 21, 23, 24, 25)   # pprphy.f:1275-1277
WAVELENGTH_TYPES = (20, 21, 22, 23, 24, 25)        # pprphy.f:1299-1301, 1508-1509
LOCAL_WAVE_TYPES = (22, 23, 24, 25)                # pprphy.f:1363-1364


def _f32(x: float) -> float:
    return float(np.float32(x))


class OpacityFileError(ListDirectedError):
    """A table the reference's reader would stop on (clean_stop or a Fortran
    runtime error)."""


# ---- file selection ----------------------------------------------------------
def planet_kap_extra(planet_num: int) -> float:
    """SETPLANETKAPEXTRA (ppplanets.f:36-59): the extra absorber in cm^2/g
    (default-REAL constants)."""
    table = {1: 0.1, 2: 0.035, 3: 0.0, 4: 0.0, 5: 0.0}
    if planet_num not in table:
        raise OpacityFileError(f"planet_num notavail:readbur,extra {planet_num}")
    return _f32(table[planet_num])


def burrows_file_name(planet_num: int, ikaptyp: int) -> str:
    """The table file READBURROWSOPCTABLE opens (pprphy.f:1273-1282 with
    ppplanets.f:90-213)."""
    if ikaptyp in WITH_TIOVO:
        if planet_num == 1:
            return "BURROWS6070_wTiVO_wavelth.dat" if ikaptyp == 20 else "BURROWS6117_wTiVO.dat"
        if planet_num == 2:
            return "BURROWS5040_wTiVO.dat"
        if 3 <= planet_num <= 8:
            raise OpacityFileError(f"no w/TiVO opacity file created for this planet {planet_num}")
        raise OpacityFileError(f"planet_num not avail {planet_num}")
    if ikaptyp not in WITHOUT_TIOVO:
        raise OpacityFileError(f"ikaptyp= {ikaptyp} not avail in readburrowsopctable")
    if planet_num == 1:
        if ikaptyp == 21:
            return "BURROWS6070_woTiVO_wavelth.dat"
        if ikaptyp in (23, 24):
            return "BURROWS6070_woTiVO_radtransfer.dat"
        return "BURROWS6117_woutTiVO.dat"
    if planet_num == 2:
        if ikaptyp == 21:
            return "BURROWS5040_woTiVO_wavelth.dat"
        if ikaptyp in (23, 24):
            return "BURROWS5040_woTiVO_radtransfer.dat"
        if ikaptyp == 25:
            return "BURROWS5040_Ray_woTiVO_radtransfer.dat"
        return "BURROWS5040_woutTiVO.dat"
    if planet_num == 5:
        if ikaptyp == 21:
            return "BURROWS6300_woTiVO_wavelth.dat"
        if ikaptyp in (23, 24):
            return "BURROWS6300_woTiVO_radtransfer.dat"
        raise OpacityFileError("check opacity file for WASP-12b")
    fixed = {3: "BURROWS5226_woutTiVO.dat", 4: "BURROWS6147_woutTiVO.dat", 6: "BURROWS6079_woutTiVO.dat",
             7: "BURROWS6290_woutTiVO.dat", 8: "BURROWS6350_woutTiVO.dat"}
    if planet_num in fixed:
        return fixed[planet_num]
    raise OpacityFileError(f"planet_num not avail {planet_num}")


def bstar_file_name(planet_num: int) -> str:
    """The stellar wavelength-bin file of the wavelength types
    (pprphy.f:1510-1527)."""
    names = {1: "BSTAR_WAVEBINS_TS6070.dat", 2: "BSTAR_WAVEBINS_TS5040.dat", 5: "BSTAR_WAVEBINS_TS6300.dat"}
    if planet_num not in names:
        raise OpacityFileError("Need to create a BSTAR_WAVEBIN file for this Tstar")
    return names[planet_num]


# ---- the table -----------------------------------------------------------------
def _values_per_record(ikaptyp: int) -> int:
    if ikaptyp in (20, 21):
        return 5 + WAVE_BINS
    if ikaptyp in LOCAL_WAVE_TYPES:
        return 5 + 3 * WAVE_BINS
    return 5


@dataclass
class BurrowsTable:
    """The arrays READBURROWSOPCTABLE fills (ppmod.f:660-666): log10 means in
    cm^2/g, index [T node, rho node] (and [..., bin])."""
    ikaptyp: int
    t_absorption: float
    plnk: np.ndarray
    ross: np.ndarray
    absk: np.ndarray
    waveopac: np.ndarray
    localwave: np.ndarray
    local_bb: np.ndarray
    bin_tstar: float | None = None
    bstar_bin: np.ndarray | None = None
    rstar: float | None = None      # RSTAR (solar radii) and the orbit's semi-major axis (cm) of the
    semi: float | None = None       # run, for the binned stellar heating of IKAPTYP 20-24
    log_t: np.ndarray = field(default_factory=lambda: BURROWS_LOG_T.copy())
    log_rho: np.ndarray = field(default_factory=lambda: BURROWS_LOG_RHO.copy())


def _add_absorber(v: float, kap_ext: float) -> float:
    # LOG10(10.d0**v + kap_ext), pprphy.f:1451-1454, 1467-1470, 1482-1489
    return math.log10(math.pow(10.0, v) + kap_ext)


def read_burrows_table(source, ikaptyp: int, planet_num: int = 1, gamma_opc: float = 1.0,
                       mu_gas: float = 2.3) -> BurrowsTable:
    """READBURROWSOPCTABLE's table part (pprphy.f:1283-1505).  ``source`` is
    a path or the file's lines; ``gamma_opc`` and ``mu_gas`` are the input
    file's gamma_OPC and mu_gas (ppmod.f:52-53)."""
    if ikaptyp not in WITH_TIOVO + WITHOUT_TIOVO:
        raise OpacityFileError(f"ikaptyp= {ikaptyp} not avail in readburrowsopctable")
    if isinstance(source, (str, os.PathLike)):
        with open(source) as fh:
            lines, name = fh.readlines(), os.fspath(source)
    else:
        lines, name = list(source), "<table>"
    rd = ListDirected(lines, name, OpacityFileError)
    shape = (NODES, NODES)
    plnk, ross, absk = (np.full(shape, MISSING) for _ in range(3))
    wave, lwave, lbb = (np.full(shape + (WAVE_BINS,), MISSING) for _ in range(3))
    for _ in range(10):
        rd.read_text()
    t_abs = rd.read(1)[0]
    if t_abs is None:
        raise OpacityFileError(f"{name}: no value for T_star")
    nval = _values_per_record(ikaptyp)
    held = [None] * nval          # a null value keeps the variable's last value
    kap_ext = planet_kap_extra(planet_num) if ikaptyp in (11, 20, 24, 25) else 0.0
    gamma_term = 4.0 * math.log10(gamma_opc) if ikaptyp in (12, 14) else 0.0
    for it in range(NODES):
        for ir in range(NODES):
            vals = rd.read(nval)
            for m, v in enumerate(vals):
                if v is not None:
                    held[m] = v
            if any(v is None for v in held):
                raise OpacityFileError(f"{name}: undefined value in the record of node ({it + 1}, {ir + 1})")
            t_read, rh_read, kp, kr, ka = held[:5]
            plnk[it, ir], ross[it, ir], absk[it, ir] = kp, kr, ka
            if ikaptyp in WAVELENGTH_TYPES:
                wave[it, ir, :] = held[5:5 + WAVE_BINS]
                if ikaptyp in LOCAL_WAVE_TYPES:
                    lwave[it, ir, :] = held[5 + WAVE_BINS:5 + 2 * WAVE_BINS]
                    lbb[it, ir, :] = held[5 + 2 * WAVE_BINS:5 + 3 * WAVE_BINS]
            if ikaptyp in (12, 14):                     # pprphy.f:1434-1437
                absk[it, ir] = kp + gamma_term
            if ikaptyp == 14:                           # pprphy.f:1438-1440
                ross[it, ir] = kp
            if ikaptyp == 11:                           # pprphy.f:1442-1456
                pg_test = (RGAS * t_read * rh_read / mu_gas) * 1e-6
                if pg_test <= _f32(0.03):
                    absk[it, ir] = _add_absorber(absk[it, ir], kap_ext)
            if ikaptyp in (20, 24, 25):                 # pprphy.f:1458-1490
                wave[it, ir, :] = [_add_absorber(v, kap_ext) for v in wave[it, ir, :]]
            if ikaptyp == 25:
                lwave[it, ir, :] = [_add_absorber(v, kap_ext) for v in lwave[it, ir, :]]
    return BurrowsTable(ikaptyp, t_abs, plnk, ross, absk, wave, lwave, lbb)


def read_bstar_bins(source, nwave_bins: int = WAVE_BINS):
    """The BSTAR_WAVEBINS file (pprphy.f:1528-1539): three header records,
    the stellar temperature, the bin count (which must equal nwave_bins),
    then one record per bin whose second value is kept."""
    if isinstance(source, (str, os.PathLike)):
        with open(source) as fh:
            lines, name = fh.readlines(), os.fspath(source)
    else:
        lines, name = list(source), "<bins>"
    rd = ListDirected(lines, name, OpacityFileError)
    for _ in range(3):
        rd.read_text()
    tstar = rd.read(1)[0]
    nbin = rd.read(1, conv=integer)[0]
    if nbin != nwave_bins:
        raise OpacityFileError("Some problem with the number of bins in file")
    bins = np.empty(nwave_bins)
    held = [None, None]
    for i in range(nwave_bins):
        for m, v in enumerate(rd.read(2)):
            if v is not None:
                held[m] = v
        if held[1] is None:
            raise OpacityFileError(f"{name}: undefined value in bin {i + 1}")
        bins[i] = held[1]
    return tstar, bins


@dataclass
class OpacityPoint:
    """What BurrowsOPC returns for one (T, rho): the three means in cm^2/g,
    the dkappa/dT stand-ins, and per wavelength bin the stellar and local
    opacities and the local black-body weights (-7 where the type has none)."""
    kap_p: float
    kap_r: float
    kap_a: float
    dkap_p_dt: float
    dkap_a_dt: float
    wave: np.ndarray
    localwave: np.ndarray
    local_bb: np.ndarray


def _log10_or_limit(x: float) -> float:
    if x > 0.0:
        return math.log10(x)
    return -math.inf if x == 0.0 else math.nan


def _bracket(nodes: np.ndarray, v: float, what: str) -> tuple[int, int]:
    # DO K = 1,50: the first node above v (pprphy.f:1050-1052, 1087-1089)
    for k in range(nodes.size):
        if nodes[k] > v:
            if k == 0:
                raise OpacityFileError(f"underflow in opacity {what} array")
            return k, k - 1
    raise OpacityFileError(f"Overflow in opacity {what} array")


def burrows_opc(table: BurrowsTable, t_in: float, rh_in: float) -> OpacityPoint:
    """BurrowsOPC (pprphy.f:1005-1229) on the host, operation for operation:
    log10 T and log10 rho clamped inside the nodes (default-REAL limits),
    the bracketing nodes, bilinear weights in log10, 10** of the
    interpolated log means; the dkappa/dT stand-ins from the bracketing T
    nodes at the upper rho node.  The reference's stops (T <= 0, a search
    off the table, a non-positive mean) raise OpacityFileError."""
    if not t_in > 0.0:
        raise OpacityFileError(f"NEG. T. IN BURROWS OPC= {t_in}")
    rh1, tm1 = _log10_or_limit(rh_in), math.log10(t_in)
    if tm1 < _f32(1.69896):
        tm1 = _f32(1.69897)
    if tm1 > _f32(3.69889):
        tm1 = _f32(3.69888)
    if rh1 < _f32(-11.9996):
        rh1 = _f32(-11.9995)
    if rh1 > _f32(-1.99993):
        rh1 = _f32(-1.99994)
    bt, br = table.log_t, table.log_rho
    it, it1 = _bracket(bt, tm1, "temperature")
    iw, iw1 = _bracket(br, rh1, "pressure")
    ws1 = bt[it1] - tm1
    ws = bt[it1] - bt[it]
    ws1 = ws1 / ws
    ws = 1.0 - ws1
    ws2 = rh1 - br[iw1]
    ws3 = br[iw] - br[iw1]
    ws2 = ws2 / ws3
    ws3 = 1.0 - ws2

    def interp(a):      # a[IT,IW], a[IT,IW1], a[IT1,IW1], a[IT1,IW] -> log value
        v00, v10, v11, v01 = a[it, iw], a[it, iw1], a[it1, iw1], a[it1, iw]
        return ws2 * (ws1 * v00 + ws * v01) + ws3 * (ws1 * v10 + ws * v11)

    kr = math.pow(10.0, interp(table.ross))
    kp = math.pow(10.0, interp(table.plnk))
    ka = math.pow(10.0, interp(table.absk))
    nb = table.waveopac.shape[2]
    kt = table.ikaptyp
    wave = (np.array([math.pow(10.0, interp(table.waveopac[:, :, m])) for m in range(nb)])
            if kt in WAVELENGTH_TYPES else np.full(nb, MISSING))
    if kt in LOCAL_WAVE_TYPES:
        lwave = np.array([math.pow(10.0, interp(table.localwave[:, :, m])) for m in range(nb)])
        lbb = np.array([interp(table.local_bb[:, :, m]) for m in range(nb)])
    else:
        lwave, lbb = np.full(nb, MISSING), np.full(nb, MISSING)
    dT = math.pow(10.0, bt[it]) - math.pow(10.0, bt[it1])
    dkp = (math.pow(10.0, table.plnk[it, iw]) - math.pow(10.0, table.plnk[it1, iw])) / dT
    dka = (math.pow(10.0, table.absk[it, iw]) - math.pow(10.0, table.absk[it1, iw])) / dT
    if kr <= 0.0 or kp <= 0.0 or ka <= 0.0:
        raise OpacityFileError("neg/zero BKAP_R,BKAP_P,BKAP_A")
    return OpacityPoint(kp, kr, ka, dkp, dka, wave, lwave, lbb)


def burrows_kappa(table: BurrowsTable, T: np.ndarray, RH: np.ndarray, upperbnd: np.ndarray) -> dict:
    """KAPPA's IKAPTYP 9:12 and 14 branches for MODTYP 2 (pprphy.f:199-275)
    on the host: BurrowsOPC at i = -1..UPPERBND(j,k) and the values of
    UPPERBND(j,k) above it (the 20:25 branch, which the device runs, copies
    from UPPERBND-1 instead).  Arguments and result as ``freedman_kappa``;
    vectorised with numpy's log10 and power (last-bit differences from the
    C library's)."""
    if table.ikaptyp not in (9, 10, 11, 12, 14):
        raise OpacityFileError(f"IKAPTYP {table.ikaptyp}: burrows_kappa is KAPPA's 9:12 and 14 branches")
    T = np.asarray(T, dtype=np.float64)
    RH = np.asarray(RH, dtype=np.float64)
    nxh = T.shape[0]
    q = np.arange(nxh)[:, None, None]
    top = np.minimum(np.asarray(upperbnd, dtype=np.int64) + 1, nxh - 1)[None, :, :]
    src = np.broadcast_to(np.minimum(q, top), T.shape)
    Ts = np.take_along_axis(T, src, axis=0)
    Rs = np.take_along_axis(RH, src, axis=0)
    if not np.all(Ts > 0.0):
        raise OpacityFileError("NEG. T. IN BURROWS OPC")
    with np.errstate(divide="ignore", invalid="ignore"):
        rh1 = np.log10(Rs)
    tm1 = np.log10(Ts)
    tm1 = np.where(tm1 < _f32(1.69896), _f32(1.69897), tm1)
    tm1 = np.where(tm1 > _f32(3.69889), _f32(3.69888), tm1)
    rh1 = np.where(rh1 < _f32(-11.9996), _f32(-11.9995), rh1)
    rh1 = np.where(rh1 > _f32(-1.99993), _f32(-1.99994), rh1)
    bt, br = table.log_t, table.log_rho
    it = np.searchsorted(bt, tm1, side="right")
    iw = np.searchsorted(br, rh1, side="right")
    if np.any(it == 0) or np.any(iw == 0) or np.any(it == bt.size) or np.any(iw == br.size):
        raise OpacityFileError("(T, rho) outside the opacity table")
    it1, iw1 = it - 1, iw - 1
    ws1 = bt[it1] - tm1
    ws = bt[it1] - bt[it]
    ws1 = ws1 / ws
    ws = 1.0 - ws1
    ws2 = rh1 - br[iw1]
    ws3 = br[iw] - br[iw1]
    ws2 = ws2 / ws3
    ws3 = 1.0 - ws2

    def interp(a):
        v00, v10, v11, v01 = a[it, iw], a[it, iw1], a[it1, iw1], a[it1, iw]
        return ws2 * (ws1 * v00 + ws * v01) + ws3 * (ws1 * v10 + ws * v11)

    out = {"XKAPR": np.power(10.0, interp(table.ross)), "XKAPP": np.power(10.0, interp(table.plnk)),
           "XKAPA": np.power(10.0, interp(table.absk))}
    dT = np.power(10.0, bt[it]) - np.power(10.0, bt[it1])
    out["DXKAPP_DT"] = (np.power(10.0, table.plnk[it, iw]) - np.power(10.0, table.plnk[it1, iw])) / dT
    out["DXKAPA_DT"] = (np.power(10.0, table.absk[it, iw]) - np.power(10.0, table.absk[it1, iw])) / dT
    if not (np.all(out["XKAPR"] > 0) and np.all(out["XKAPP"] > 0) and np.all(out["XKAPA"] > 0)):
        raise OpacityFileError("neg/zero BKAP_R,BKAP_P,BKAP_A")
    return {n: np.asfortranarray(a) for n, a in out.items()}


# ---- Freedman (T, P) tables (IKAPTYP 4-7) -------------------------------------
# DATA FreedmanTVAL (K) and FreedmanPVAL (mbar), ppmod.f:686-697 (double constants)
FREEDMAN_T = np.array([
    75.0, 100.0, 110.0, 120.0, 130.0, 140.0, 150.0, 160.0, 170.0, 180.0, 190.0, 200.0, 210.0, 220.0,
    230.0, 240.0, 250.0, 275.0, 300.0, 400.0, 500.0, 575.0, 650.0, 725.0, 800.0, 900.0, 1000.0, 1100.0,
    1200.0, 1300.0, 1400.0, 1500.0, 1600.0, 1700.0, 1800.0, 1900.0, 2000.0, 2300.0, 2600.0, 3000.0,
    3500.0, 4000.0])
FREEDMAN_P = np.array([
    0.001, 0.003, 0.01, 0.03, 0.1, 0.3, 1.0, 3.0, 10.0, 30.0, 100.0, 300.0, 1000.0, 3000.0, 10000.0,
    30000.0, 100000.0, 300000.0])
FREEDMAN_ENTRIES = 736          # N_entries, pprphy.f:974


def freedman_file_name(ikaptyp: int) -> str:
    """The table READFREEDMANOPCTABLE opens (pprphy.f:961-970)."""
    if ikaptyp in (4, 6):
        return "Freedman6117.dat"
    if ikaptyp in (5, 7):
        return "Freedman6117_noTIVO.dat"
    raise OpacityFileError(f"ikaptyp= {ikaptyp} not avail in readfreedmanopctable")


@dataclass
class FreedmanTable:
    """FreedmanXKAP_plnk/_ross/_abs (ppmod.f:653-655): log10 means,
    index [T node, P node], -7 where the file gives no entry."""
    ikaptyp: int
    t_absorption: float
    plnk: np.ndarray
    ross: np.ndarray
    absk: np.ndarray


def read_freedman_table(source, ikaptyp: int, entries: int = FREEDMAN_ENTRIES) -> FreedmanTable:
    """READFREEDMANOPCTABLE (pprphy.f:944-1002): ten header records, the
    stellar temperature, then ``entries`` records T, P, log kappa_P,
    log kappa_R, log kappa_abs, each placed at the node its T and P equal
    exactly.  A T or P that is no node (the reference would then store
    outside the arrays) raises OpacityFileError."""
    freedman_file_name(ikaptyp)
    if isinstance(source, (str, os.PathLike)):
        with open(source) as fh:
            lines, name = fh.readlines(), os.fspath(source)
    else:
        lines, name = list(source), "<table>"
    rd = ListDirected(lines, name, OpacityFileError)
    shape = (FREEDMAN_T.size, FREEDMAN_P.size)
    plnk, ross, absk = (np.full(shape, MISSING) for _ in range(3))
    for _ in range(10):
        rd.read_text()
    t_abs = rd.read(1)[0]
    held = [None] * 5
    for q in range(entries):
        for m, v in enumerate(rd.read(5)):
            if v is not None:
                held[m] = v
        if any(v is None for v in held):
            raise OpacityFileError(f"{name}: undefined value in entry {q + 1}")
        t, p, kp, kr, ka = held
        it = np.flatnonzero(FREEDMAN_T == t)
        ip = np.flatnonzero(FREEDMAN_P == p)
        if it.size == 0 or ip.size == 0:
            raise OpacityFileError(f"{name}: entry {q + 1} (T={t}, P={p}) is not a node of the table")
        plnk[it[0], ip[0]], ross[it[0], ip[0]], absk[it[0], ip[0]] = kp, kr, ka
    return FreedmanTable(ikaptyp, t_abs, plnk, ross, absk)


def freedman_opc(table: FreedmanTable, t_in: float, pg_in: float):
    """FreedmanOPC (pprphy.f:800-942) at one (T, P_gas in dyn/cm^2),
    operation for operation: P in mbar, T and P clamped inside the nodes,
    bilinear in T and P (linear nodes) of the log means, 10** of the
    result; the dkappa/dT stand-ins from the bracketing T nodes.  Returns
    (kap_p, kap_r, kap_a, dkap_p_dt, dkap_a_dt); the reference's stops
    raise OpacityFileError."""
    if not t_in > 0.0:
        raise OpacityFileError(f"NEG. T. IN FREEDMAN OPC= {t_in}")
    pg1 = pg_in * 0.001
    tm1 = t_in
    if tm1 < 75.0:
        tm1 = 75.001
    if tm1 > 4000.0:
        tm1 = 3999.9
    if pg1 < 0.001:
        pg1 = 0.001001
    if pg1 > 300000.0:
        pg1 = 299999.9
    it, it1 = _bracket(FREEDMAN_T, tm1, "temperature")
    iw, iw1 = _bracket(FREEDMAN_P, pg1, "pressure")
    bt, bp = FREEDMAN_T, FREEDMAN_P
    ws1 = bt[it1] - tm1
    ws = bt[it1] - bt[it]
    ws1 = ws1 / ws
    ws = 1.0 - ws1
    ws2 = pg1 - bp[iw1]
    ws3 = bp[iw] - bp[iw1]
    ws2 = ws2 / ws3
    ws3 = 1.0 - ws2

    def interp(a):
        v00, v10, v11, v01 = a[it, iw], a[it, iw1], a[it1, iw1], a[it1, iw]
        return ws2 * (ws1 * v00 + ws * v01) + ws3 * (ws1 * v10 + ws * v11)

    kr = math.pow(10.0, interp(table.ross))
    kp = math.pow(10.0, interp(table.plnk))
    ka = math.pow(10.0, interp(table.absk))
    dT = bt[it] - bt[it1]
    dkp = (math.pow(10.0, table.plnk[it, iw]) - math.pow(10.0, table.plnk[it1, iw])) / dT
    dka = (math.pow(10.0, table.absk[it, iw]) - math.pow(10.0, table.absk[it1, iw])) / dT
    if kr <= 0.0 or kp <= 0.0 or ka <= 0.0:
        raise OpacityFileError("neg/zero BKAP_R,BKAP_P,BKAP_A")
    return kp, kr, ka, dkp, dka


def freedman_kappa(table: FreedmanTable, T: np.ndarray, RH: np.ndarray, upperbnd: np.ndarray,
                   mu_gas: float) -> dict:
    """KAPPA's IKAPTYP 4:5 branch for MODTYP 2 (pprphy.f:88-110) on the
    host: PRESSG's ideal-gas pressure PG = Rgas T RH / mu_gas
    (ppphy.f:17-20), FreedmanOPC at i = -1..UPPERBND(j,k), the values of
    UPPERBND(j,k) above it.  T and RH are halo arrays (-1:NX+2,...),
    UPPERBND the plane (-1:NY+2,-1:NZ+2) after BOUNDS; the result holds
    XKAPR, XKAPP, XKAPA, DXKAPP_DT, DXKAPA_DT for ``FLD.upload`` with
    kappa_model 1 (KAPPA freezes the opacities after an implicit step's
    first outer iteration, so opacities formed at the step's start are the
    ones the reference uses).  Vectorised: the operations of
    ``freedman_opc`` in its order, with numpy's power (which may differ
    from the C library's in the last bit)."""
    T = np.asarray(T, dtype=np.float64)
    RH = np.asarray(RH, dtype=np.float64)
    nxh = T.shape[0]
    q = np.arange(nxh)[:, None, None]
    top = np.minimum(np.asarray(upperbnd, dtype=np.int64) + 1, nxh - 1)[None, :, :]   # index of i = UPPERBND
    src = np.minimum(q, top)                       # cells above UPPERBND take its values
    Ts = np.take_along_axis(T, np.broadcast_to(src, T.shape), axis=0)
    Rs = np.take_along_axis(RH, np.broadcast_to(src, T.shape), axis=0)
    if not np.all(Ts > 0.0):
        raise OpacityFileError("NEG. T. IN FREEDMAN OPC")
    pg1 = (RGAS * Ts * Rs / mu_gas) * 0.001
    tm1 = np.where(Ts < 75.0, 75.001, Ts)
    tm1 = np.where(tm1 > 4000.0, 3999.9, tm1)
    pg1 = np.where(pg1 < 0.001, 0.001001, pg1)
    pg1 = np.where(pg1 > 300000.0, 299999.9, pg1)
    bt, bp = FREEDMAN_T, FREEDMAN_P
    it = np.searchsorted(bt, tm1, side="right")      # the first node above, as the DO loops find it
    iw = np.searchsorted(bp, pg1, side="right")
    if np.any(it == 0) or np.any(iw == 0):
        raise OpacityFileError("underflow in opacity temperature/pressure array")
    if np.any(it == bt.size) or np.any(iw == bp.size):
        raise OpacityFileError("Overflow in opacity temperature/pressure array")
    it1, iw1 = it - 1, iw - 1
    ws1 = bt[it1] - tm1
    ws = bt[it1] - bt[it]
    ws1 = ws1 / ws
    ws = 1.0 - ws1
    ws2 = pg1 - bp[iw1]
    ws3 = bp[iw] - bp[iw1]
    ws2 = ws2 / ws3
    ws3 = 1.0 - ws2

    def interp(a):
        v00, v10, v11, v01 = a[it, iw], a[it, iw1], a[it1, iw1], a[it1, iw]
        return ws2 * (ws1 * v00 + ws * v01) + ws3 * (ws1 * v10 + ws * v11)

    out = {"XKAPR": np.power(10.0, interp(table.ross)), "XKAPP": np.power(10.0, interp(table.plnk)),
           "XKAPA": np.power(10.0, interp(table.absk))}
    dT = bt[it] - bt[it1]
    out["DXKAPP_DT"] = (np.power(10.0, table.plnk[it, iw]) - np.power(10.0, table.plnk[it1, iw])) / dT
    out["DXKAPA_DT"] = (np.power(10.0, table.absk[it, iw]) - np.power(10.0, table.absk[it1, iw])) / dT
    if not (np.all(out["XKAPR"] > 0) and np.all(out["XKAPP"] > 0) and np.all(out["XKAPA"] > 0)):
        raise OpacityFileError("neg/zero BKAP_R,BKAP_P,BKAP_A")
    return {n: np.asfortranarray(a) for n, a in out.items()}


def read_opacity_tables(directory, planet_num: int, ikaptyp: int, gamma_opc: float = 1.0,
                        mu_gas: float = 2.3) -> BurrowsTable:
    """READBURROWSOPCTABLE as a whole: the planet's table file from
    ``directory`` and, for the wavelength types, its BSTAR bins."""
    t = read_burrows_table(os.path.join(directory, burrows_file_name(planet_num, ikaptyp)), ikaptyp,
                           planet_num, gamma_opc, mu_gas)
    if ikaptyp in WAVELENGTH_TYPES:
        t.bin_tstar, t.bstar_bin = read_bstar_bins(os.path.join(directory, bstar_file_name(planet_num)))
    return t


def write_burrows_table(path, ikaptyp: int, t_absorption: float, plnk, ross, absk, waveopac=None,
                        localwave=None, local_bb=None, header=None):
    """A table file in the layout read_burrows_table reads: node values
    written as T and rho in cgs (10**node), means as given (log10), every
    value with 17 significant digits."""
    nval = _values_per_record(ikaptyp)
    hdr = list(header or [f"table{i + 1}" for i in range(10)])
    if len(hdr) != 10:
        raise ValueError("the header is ten records")
    with open(path, "w") as fh:
        for h in hdr:
            fh.write(f"{h}\n")
        fh.write(f"{t_absorption!r}\n")
        for it in range(NODES):
            for ir in range(NODES):
                row = [10.0 ** BURROWS_LOG_T[it], 10.0 ** BURROWS_LOG_RHO[ir], plnk[it, ir], ross[it, ir],
                       absk[it, ir]]
                if nval > 5:
                    row += list(waveopac[it, ir, :])
                if nval > 5 + WAVE_BINS:
                    row += list(localwave[it, ir, :]) + list(local_bb[it, ir, :])
                fh.write(" ".join(f"{float(v):.17g}" for v in row) + "\n")


def analytic_freedman_table(kap0: float = 1e-2, mu_gas: float = 2.3, dplnk: float = 0.1,
                            dabs: float = -0.1) -> FreedmanTable:
    """A table in FreedmanOPC's layout for tests (the reference's table files
    are not in its tree): on the FreedmanTVAL x FreedmanPVAL nodes, log10 of
    the analytic kappa = kap0 sqrt(rho) (T/1000)^1.5 with the ideal-gas
    density rho = P mu_gas / (Rgas T) (P in dyn/cm^2) as the Rosseland
    mean, offset by dplnk and dabs decades for the Planck and absorption
    means."""
    T, P = np.meshgrid(FREEDMAN_T, FREEDMAN_P * 1000.0, indexing="ij")
    rho = P * mu_gas / (RGAS * T)
    lk = math.log10(kap0) + 0.5 * np.log10(rho) + 1.5 * np.log10(T / 1000.0)
    return FreedmanTable(4, 6117.0, np.asfortranarray(lk + dplnk), np.asfortranarray(lk),
                         np.asfortranarray(lk + dabs))
