"""Seeded synthetic spherical shells standing in for a ttcode restart.

The reference's own runs start from model files and opacity tables that are
not part of it; the benchmark shells are defined analytically instead:

* grid: NCOSYS=2, linear, r in [1.0, 1.1] R_J (RJUP, ppmod.f:1078), phi in
  [0, 1] * 2 pi (periodic), theta in [-0.95, 0.95] * pi/2 (ipp:25-27),
  poles off unless asked for (``poles=True``: the one-rank pole shifts);
* rho = 1e-2 exp(-(r - r0)/H) with H = (r1 - r0)/8 (8 scale heights);
* T = 2500 - 1300 (r - r0)/(r1 - r0) K;
* E_R = a T^4 (optically thick start);
* c_v = R/(mu (gamma - 1)) with gamma = 1.4, mu = 2.3 (ipp:9, GASINIT
  ppinit.f:1408-1417);
* kappa_R = 1e-2 rho^0.5 (T/1000)^1.5 * KMUL, where KMUL holds seeded 5 %
  lognormal noise and, for the high-contrast shells, a radial factor that
  stretches the bottom/top opacity ratio to the requested contrast;
* day-side irradiation through the grey STELLARINPUT_HEATING with
  T_irr = 2048 K (ipp:22) and the cos(phi)cos(theta) pattern of
  CALC_TINCIDENT (pprad.f:321-330) and CALCMUSTAR (ppsub.f:163-169).

Each array is returned in the reference's Fortran layout and bounds.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from .grid import RJUP, Grid, gitter

ARAD = float(np.float32(7.56596e-15))
RGAS = float(np.float32(8.315e7))
MU_MIN = float(np.float32(1.0e-7))

# Benchmark configurations (phi x theta x r -> NX=r, NY=phi, NZ=theta).
SHELLS = {
    "shell64": dict(nx=40, ny=64, nz=32, delt=100.0, contrast=None),
    "shell256": dict(nx=100, ny=256, nz=128, delt=100.0, contrast=None),
    "shell512": dict(nx=160, ny=512, nz=256, delt=300.0, contrast=1e4),
    "stiff512": dict(nx=160, ny=512, nz=256, delt=1000.0, contrast=1e6),
}


def default_params(delt: float = 100.0) -> dict:
    """input_init values of the shipped ipp (ipp:1-27) with the benchmark's
    omega=1.7 and a solve tolerance of 1e-10."""
    return dict(delt=delt, sorparam=1.7, epsmat=1e-10, fbottom=15844.23, tirr=2048.0,
                xnue=1.0e9, pr_num=1.0, kap0=1.0e-2, itmax=200000, bcxmin=9, ibdrad=9,
                iflimtyp=2, f_incident=2, ieta=4, isigtyp=0, iii=1, adjust_sor=0,
                kappa_model=0, poles=0)


@dataclass
class Shell:
    grid: Grid
    fields: dict      # name -> Fortran-ordered array (reference bounds)
    params: dict
    seed: int

    @property
    def dims(self):
        return self.grid.nx, self.grid.ny, self.grid.nz


def mu_star_tincident(g: Grid, tirr: float, f_incident: int = 2):
    """CALCMUSTAR (ppsub.f:156-179) and CALC_TINCIDENT (pprad.f:296-405)
    on (-1:NY+2, -1:NZ+2)."""
    ny, nz = g.ny, g.nz
    mu = np.ones((ny + 4, nz + 4), order="F")
    tinc = np.zeros((ny + 4, nz + 4), order="F")
    for k in range(-1, nz + 3):
        ck = math.cos(g.at("xzb", k))
        for j in range(-1, ny + 3):
            cyz = math.cos(g.at("xyb", j)) * ck
            if f_incident in (2, 3, 8):
                mu[j + 1, k + 1] = max(cyz, MU_MIN)
            t = 0.0
            if f_incident in (2, 3):
                if cyz >= 0:
                    t = max(tirr * math.pow(cyz, 0.25), 0.0)
            elif f_incident in (4, 5):
                t = tirr
            tinc[j + 1, k + 1] = t
    return mu, tinc


def make_shell(nx: int, ny: int, nz: int, seed: int = 0, delt: float = 100.0,
               contrast: float | None = None, noise: float = 0.05, poles: bool = False) -> Shell:
    r0 = 1.0 * RJUP
    r1 = 1.1 * RJUP
    g = gitter(nx, ny, nz, r0, r1)
    r = g.m["xxb"]                       # (-1:NX+2)
    frac = (r - r0) / (r1 - r0)
    H = (r1 - r0) / 8.0
    rho1 = 1e-2 * np.exp(-(r - r0) / H)
    t1 = 2500.0 - 1300.0 * frac
    shape = (nx + 4, ny + 4, nz + 4)
    RH = np.asfortranarray(np.broadcast_to(rho1[:, None, None], shape).copy())
    T = np.asfortranarray(np.broadcast_to(t1[:, None, None], shape).copy())
    t2 = T * T
    ER = np.asfortranarray(ARAD * (t2 * t2))
    cv = RGAS / (2.3 * (1.4 - 1.0))
    CV = np.full(shape, cv, order="F")
    rng = np.random.default_rng(seed)
    KMUL = np.exp(noise * rng.standard_normal(shape))
    if contrast is not None:
        # kappa_0 at the bottom and top of the noise-free profile
        def k0(rho, t):
            th = t / 1000.0
            return math.sqrt(rho) * th * math.sqrt(th)
        base = k0(1e-2, 2500.0) / k0(1e-2 * math.exp(-8.0), 1200.0)
        s = math.log(contrast / base)
        KMUL = KMUL * np.exp(-s * frac)[:, None, None]
    KMUL = np.asfortranarray(KMUL)
    params = default_params(delt)
    params["poles"] = int(poles)
    mu, tinc = mu_star_tincident(g, params["tirr"], params["f_incident"])
    fields = dict(T=T, RH=RH, CV=CV, ER=ER, KMUL=KMUL, MU_STAR=mu, TINCIDENT=tinc)
    return Shell(g, fields, params, seed)


def analytic_opacity_table(kap0: float = 1e-2, nt: int = 50, nrh: int = 50):
    """A table in BurrowsOPC's layout (log10 T, log10 rho nodes spanning the
    range its clamps allow, pprphy.f:1045-1049; log10 means, T index
    fastest) holding the analytic model kappa = kap0 sqrt(rho) (T/1000)^1.5
    for all three means.  log10 kappa is linear in log10 T and log10 rho, so
    the bilinear interpolation reproduces the model up to rounding."""
    lt = np.linspace(1.69896, 3.69889, nt)
    lr = np.linspace(-11.9996, -1.99993, nrh)
    k = math.log10(kap0) + 0.5 * lr[None, :] + 1.5 * (lt[:, None] - 3.0)
    k = np.asfortranarray(k)
    return lt, lr, k, k.copy(order="F"), k.copy(order="F")


def shell(name: str, seed: int = 0) -> Shell:
    cfg = SHELLS[name]
    return make_shell(cfg["nx"], cfg["ny"], cfg["nz"], seed=seed, delt=cfg["delt"],
                      contrast=cfg["contrast"])
