"""Spherical grid metrics of GITTER (ppinit.f:1028-1406) for NCOSYS=2 with
linear grids (DXMIN=DYMIN=DZMIN=0) and one rank.

Each metric is returned with the reference's own bounds, as a numpy array
starting at the Fortran lower bound (``Grid.lo[name]``), which is exactly
what a Fortran caller passes through the C ABI.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

# The reference's REAL*4 literals (ppmod.f:1078).
RJUP = float(np.float32(7.1492e9))

BOUNDS = {  # name -> (lo, hi-offset relative to N)   (ppmod.f:615-641)
    "xxa": (0, 2), "xxb": (-1, 2), "dxa": (1, 2), "dxb": (0, 2),
    "xya": (0, 2), "xyb": (-1, 2), "dya": (1, 2), "dyb": (0, 2),
    "xza": (0, 2), "xzb": (-1, 2), "dza": (1, 2), "dzb": (0, 2),
    "ddx0": (0, 2), "ddx1": (0, 2), "ddy0": (0, 2), "ddy1": (0, 2), "ddz0": (0, 2), "ddz1": (0, 2),
    "surxa": (0, 2), "surxb": (0, 2), "surza": (0, 2), "surzb": (0, 2),
    "geoxg": (-1, 2), "geoxh": (-1, 2), "geoxga": (0, 2), "geoxha": (0, 2),
    "geozg": (-1, 2), "geozga": (0, 2),
}
AXIS = {}
for _n in ("xxa", "xxb", "dxa", "dxb", "ddx0", "ddx1", "surxa", "surxb", "geoxg", "geoxh",
           "geoxga", "geoxha"):
    AXIS[_n] = "x"
for _n in ("xya", "xyb", "dya", "dyb", "ddy0", "ddy1"):
    AXIS[_n] = "y"
for _n in ("xza", "xzb", "dza", "dzb", "ddz0", "ddz1", "surza", "surzb", "geozg", "geozga"):
    AXIS[_n] = "z"


@dataclass
class Grid:
    nx: int
    ny: int
    nz: int
    xmin: float
    xmax: float
    ymin: float = 0.0
    ymax: float = 1.0
    zmin: float = -0.95
    zmax: float = 0.95
    m: dict = field(default_factory=dict)   # name -> array over [lo, hi]
    lo: dict = field(default_factory=dict)

    def at(self, name: str, i):
        """The metric at Fortran index i."""
        return self.m[name][np.asarray(i) - self.lo[name]]


def gitter(nx: int, ny: int, nz: int, xmin: float, xmax: float, ymin: float = 0.0,
           ymax: float = 1.0, zmin: float = -0.95, zmax: float = 0.95) -> Grid:
    """GITTER for NCOSYS=2: y in units of 2*pi (ppinit.f:1064-1065), z the
    latitude in units of pi/2 (:1066-1067), linear spacing everywhere."""
    g = Grid(nx, ny, nz, xmin, xmax, ymin, ymax, zmin, zmax)
    pi = math.pi
    ymax1, ymin1 = ymax * 2.0 * pi, ymin * 2.0 * pi
    zmax1, zmin1 = (zmax / 2.0) * pi, (zmin / 2.0) * pi

    def axis(n, lo, hi):
        # arrays stored on -1..n+2 (offset +1)
        d = (hi - lo) / n
        a = np.zeros(n + 4)   # xa on 0..n+2 at a[i+1]
        b = np.zeros(n + 4)   # xb on -1..n+2
        da = np.zeros(n + 4)  # da on 1..n+2
        da[2:] = d
        a[2] = lo + (0 * (hi - lo) / 1)
        a[1] = a[2] - da[2]
        for i in range(2, n + 3):
            a[i + 1] = a[i] + da[i + 1]
        for i in range(0, n + 2):
            b[i + 1] = (a[i + 1] + a[i + 2]) / 2.0
        d3 = da[n + 3] * 1.0
        an3 = a[n + 3] + d3
        b[n + 3] = (a[n + 3] + an3) / 2.0
        d3 = da[2] / 1.0
        an3 = a[1] - d3
        b[0] = (a[1] + an3) / 2.0
        db = np.zeros(n + 4)
        for i in range(0, n + 3):
            db[i + 1] = b[i + 1] - b[i]
        return a, b, da, db

    xa, xb, dxa, dxb = axis(nx, xmin, xmax)
    ya, yb, dya, dyb = axis(ny, ymin1, ymax1)
    za, zb, dza, dzb = axis(nz, zmin1, zmax1)
    full = {"xxa": xa, "xxb": xb, "dxa": dxa, "dxb": dxb, "xya": ya, "xyb": yb, "dya": dya,
            "dyb": dyb, "xza": za, "xzb": zb, "dza": dza, "dzb": dzb}
    for n in ("ddx0", "ddx1"):
        full[n] = np.full(nx + 4, 0.5)
    for n in ("ddy0", "ddy1"):
        full[n] = np.full(ny + 4, 0.5)
    for n in ("ddz0", "ddz1"):
        full[n] = np.full(nz + 4, 0.5)
    xxa1 = xa[2] if xa[2] != 0.0 else float(np.float32(1.e-20))
    full["surxa"] = xa * xa
    full["surxb"] = xb * xb
    full["geoxga"] = xa.copy()
    full["geoxha"] = xa.copy()
    full["geoxga"][2] = xxa1
    full["geoxha"][2] = xxa1
    full["geoxg"] = xb.copy()
    full["geoxh"] = xb.copy()
    full["surza"] = np.array([math.cos(v) for v in za])
    full["surzb"] = np.array([math.cos(v) for v in zb])
    full["geozga"] = np.array([math.cos(v) for v in za])
    full["geozg"] = np.array([math.cos(v) for v in zb])
    if full["geozga"][nz + 2] == 0.0:
        full["geozga"][nz + 2] = float(np.float32(1.e-10))
    if full["geozga"][2] == 0.0:
        full["geozga"][2] = float(np.float32(1.e-10))
    n_of = {"x": nx, "y": ny, "z": nz}
    for name, (lo, hioff) in BOUNDS.items():
        n = n_of[AXIS[name]]
        hi = n + hioff
        g.m[name] = np.ascontiguousarray(full[name][lo + 1:hi + 2])
        g.lo[name] = lo
    return g


def volumes(g: Grid):
    """VOLXB(1:NX), VOLYB(1:NY), VOLZB(1:NZ) of GITTER for NCOSYS=2
    (ppinit.f:1346, 1364, 1375): (r_a(i+1)^3 - r_a(i)^3)/3, the phi width,
    sin(theta_a(k+1)) - sin(theta_a(k))."""
    xa = lambda i: float(g.at("xxa", i))
    vx = np.array([(xa(i + 1) * xa(i + 1) * xa(i + 1) - xa(i) * xa(i) * xa(i)) / 3.0 for i in range(1, g.nx + 1)])
    vy = np.array([float(g.at("xya", j + 1)) - float(g.at("xya", j)) for j in range(1, g.ny + 1)])
    vz = np.array([math.sin(float(g.at("xza", k + 1))) - math.sin(float(g.at("xza", k))) for k in range(1, g.nz + 1)])
    return vx, vy, vz


def full_1d(g: Grid, name: str) -> np.ndarray:
    """The metric on (-1:N+2) with zeros outside its reference bounds (the
    storage the oracle uses)."""
    n = {"x": g.nx, "y": g.ny, "z": g.nz}[AXIS[name]]
    out = np.zeros(n + 4)
    lo = g.lo[name]
    out[lo + 1:lo + 1 + g.m[name].size] = g.m[name]
    return out
