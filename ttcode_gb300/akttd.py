"""ttcode's restart and snapshot files read into, and written from, the
arrays this library works on.

Two layouts.  Each rank writes its own file with PRINTOUT(1): SNAP_r.nnn and
RSRT_r.nnn during a run (pp.f:565-582), AKTTD_r at its end (pp.f:827-831).
ppcombine joins the ranks' files into one global file, GLOB.nnn or AKTTD
(PRINTGLOBAL, ppcombine.f:603-657), and a restart reads that global AKTTD
(READRESTART, ppinit.f:1544-1646, or its list-directed AKTTD_ASCII form).

PRINTOUT(1) (ppprt.f:13-124) writes, on unit 12, one Fortran unformatted
sequential file per rank; each WRITE is one record framed by its byte
length (a 4-byte marker before and after).  As gfortran writes them,
records longer than 2**31-9 bytes are split into sub-records: a sub-record's
leading marker is negative when another one follows, its trailing marker is
negative on every sub-record after the first.  The records, in order:

     1  global_NX, global_NY, global_NZ                      INTEGER
     2  locNX, locNY, locNZ, numprocs                        INTEGER
     3  myid, proc_coords(1:3)                               INTEGER
     4  proc_dims(1:3)                                       INTEGER
     5  ZEIT, DELT (DOUBLE PRECISION), NUM_ITER (INTEGER)
  6-14  XXA(0:NX+2) XXB(-1:NX+2) DXA(1:NX+2), the same for Y and Z
 15-17  V(0:NX+2,-1:NY+2,-1:NZ+2), G(-1:NX+2,0:NY+2,-1:NZ+2),
        H(-1:NX+2,-1:NY+2,0:NZ+2)
 18-21  RH, T, ER, PG on (-1:NX+2,-1:NY+2,-1:NZ+2)
    22  CS(0:NX+1,0:NY+1,0:NZ+1)
    23  UPPERBND(1:NY,1:NZ)                                  INTEGER
    24  TinitBottom, Tinittop, rhinittop, rhinitbottom, hydrotime, Maccreated
    25  NCOSYS                                               INTEGER
 26-34  on (1:NX,1:NY,1:NZ): xkapR, flimx(1:NX,...), conv_flux(1), conv_flux(2),
        conv_flux(3), xkapA, STELLARINPUT, disfn, xkapP

(records 25-34 are "not read back into a restart", ppprt.f:44).  Arrays are
column-major, first index fastest.  `read` returns a `Snapshot`; `stitch`
joins the files of a (phi, theta) decomposition by proc_coords; `grid_of`
rebuilds GITTER's NCOSYS=2 metrics (ppinit.f:1028-1406) from the coordinate
records; `shell_of` makes the state a `synthetic.Shell` that
`fld.start_run` accepts, so that a ttcode state drives the solver;
`snapshot_of_fld` writes a device state back as a record.

The global file holds interior cells only: the three global extents (one
record each), the local extents and rank count, ZEIT/DELT/NUM_ITER, XXB,
XYB, XZB on 1..N, V G H RH T ER PG CS on (1:NX,1:NY,1:NZ), UPPERBND, the six
boundary scalars, then NCOSYS and nine interior extras that a restart does
not read.  `read_restart` / `read_restart_ascii` / `write_restart` handle it,
`combine` is ppcombine's FILLGLOBAL over the ranks' files, and
`shell_of_restart` starts a run from it as READRESTART and LOCALINIT do.
"""
from __future__ import annotations

import math
import struct
from dataclasses import dataclass, field

import numpy as np

from .grid import BOUNDS, AXIS, Grid

COORDS = ("xxa", "xxb", "dxa", "xya", "xyb", "dya", "xza", "xzb", "dza")
COORD_LO = {"xxa": 0, "xxb": -1, "dxa": 1, "xya": 0, "xyb": -1, "dya": 1, "xza": 0, "xzb": -1, "dza": 1}
FIELDS3 = ("V", "G", "H", "RH", "T", "ER", "PG", "CS")
EXTRAS = ("xkapR", "flimx", "conv_flux1", "conv_flux2", "conv_flux3", "xkapA", "STELLARINPUT", "disfn",
          "xkapP")
SCALARS = ("TinitBottom", "Tinittop", "rhinittop", "rhinitbottom", "hydrotime", "Maccreated")


def field_bounds(name: str, nx: int, ny: int, nz: int):
    """((lo_i, hi_i), (lo_j, hi_j), (lo_k, hi_k)) of a 3-D record."""
    h = lambda n: (-1, n + 2)
    if name == "V":
        return (0, nx + 2), h(ny), h(nz)
    if name == "G":
        return h(nx), (0, ny + 2), h(nz)
    if name == "H":
        return h(nx), h(ny), (0, nz + 2)
    if name == "CS":
        return (0, nx + 1), (0, ny + 1), (0, nz + 1)
    if name in EXTRAS:
        return (1, nx), (1, ny), (1, nz)
    return h(nx), h(ny), h(nz)


def _shape(b):
    return tuple(hi - lo + 1 for lo, hi in b)


@dataclass
class Snapshot:
    nx: int
    ny: int
    nz: int
    global_dims: tuple
    numprocs: int
    myid: int
    proc_coords: tuple
    proc_dims: tuple
    zeit: float
    delt: float
    num_iter: int
    coords: dict = field(default_factory=dict)   # name -> 1-D array from its lower bound
    arrays: dict = field(default_factory=dict)   # V G H RH T ER PG CS, extras; Fortran order
    upperbnd: np.ndarray | None = None           # (1:NY, 1:NZ) int32
    scalars: dict = field(default_factory=dict)
    ncosys: int | None = None


class _Records:
    def __init__(self, data: bytes, endian: str):
        self.b = data
        self.p = 0
        self.e = endian

    def next(self) -> bytes:
        out = bytearray()
        while True:
            if self.p + 4 > len(self.b):
                raise EOFError("truncated record marker")
            (n,) = struct.unpack_from(self.e + "i", self.b, self.p)
            more = n < 0
            n = abs(n)
            start = self.p + 4
            if start + n + 4 > len(self.b):
                raise EOFError("truncated record")
            out += self.b[start:start + n]
            (m,) = struct.unpack_from(self.e + "i", self.b, start + n)
            if abs(m) != n:
                raise ValueError(f"record markers disagree at byte {self.p}: {n} vs {m}")
            self.p = start + n + 4
            if not more:
                return bytes(out)

    def done(self) -> bool:
        return self.p >= len(self.b)


def _ints(rec: bytes, n: int, e: str):
    if len(rec) != 4 * n:
        raise ValueError(f"expected {n} INTEGERs, record has {len(rec)} bytes")
    return struct.unpack(e + f"{n}i", rec)


def _doubles(rec: bytes, shape, e: str) -> np.ndarray:
    n = int(np.prod(shape))
    if len(rec) != 8 * n:
        raise ValueError(f"expected {n} DOUBLE PRECISION values, record has {len(rec)} bytes")
    return np.frombuffer(rec, dtype=np.dtype(e + "f8")).astype(np.float64).reshape(shape, order="F")


def read(path: str, endian: str = "<") -> Snapshot:
    """One rank's file (SNAP_r.nnn, RSRT_r.nnn, AKTTD_r)."""
    with open(path, "rb") as f:
        r = _Records(f.read(), endian)
    e = endian
    gx, gy, gz = _ints(r.next(), 3, e)
    nx, ny, nz, nprocs = _ints(r.next(), 4, e)
    rec = _ints(r.next(), 4, e)
    myid, pc = rec[0], tuple(rec[1:])
    pd = tuple(_ints(r.next(), 3, e))
    rec = r.next()
    if len(rec) != 20:
        raise ValueError("ZEIT, DELT, NUM_ITER record is not 8+8+4 bytes")
    zeit, delt = struct.unpack_from(e + "2d", rec, 0)
    (num_iter,) = struct.unpack_from(e + "i", rec, 16)
    s = Snapshot(nx, ny, nz, (gx, gy, gz), nprocs, myid, pc, pd, zeit, delt, num_iter)
    n_of = {"x": nx, "y": ny, "z": nz}
    for name in COORDS:
        n = n_of[name[1]]
        s.coords[name] = _doubles(r.next(), (n + 2 - COORD_LO[name] + 1,), e)
    for name in FIELDS3:
        s.arrays[name] = _doubles(r.next(), _shape(field_bounds(name, nx, ny, nz)), e)
    rec = r.next()
    if len(rec) != 4 * ny * nz:
        raise ValueError("UPPERBND record size")
    s.upperbnd = np.frombuffer(rec, dtype=np.dtype(e + "i4")).astype(np.int32).reshape((ny, nz), order="F")
    rec = r.next()
    vals = struct.unpack(e + "6d", rec)
    s.scalars = dict(zip(SCALARS, vals))
    if r.done():
        return s
    (s.ncosys,) = _ints(r.next(), 1, e)
    for name in EXTRAS:
        if r.done():
            break
        s.arrays[name] = _doubles(r.next(), (nx, ny, nz), e)
    return s


MAX_SUBRECORD = 2**31 - 9   # gfortran's largest sub-record with 4-byte markers


def _record(payload: bytes, endian: str, max_sub: int = MAX_SUBRECORD) -> bytes:
    """One Fortran unformatted sequential record in gfortran's sub-record
    layout: head marker -len if another sub-record follows, else +len; tail
    marker -len on every sub-record after the first, else +len."""
    out = bytearray()
    chunks = [payload[i:i + max_sub] for i in range(0, len(payload), max_sub)] or [b""]
    for q, c in enumerate(chunks):
        head = -len(c) if q + 1 < len(chunks) else len(c)
        tail = -len(c) if q > 0 else len(c)
        out += struct.pack(endian + "i", head) + c + struct.pack(endian + "i", tail)
    return bytes(out)


def write(path: str, s: Snapshot, endian: str = "<", max_sub: int = MAX_SUBRECORD):
    """The same record sequence (restart files made from this library's
    state, and the round-trip tests)."""
    e = endian
    F = lambda a: np.asarray(a, dtype=np.float64).astype(np.dtype(e + "f8")).tobytes(order="F")
    recs = [struct.pack(e + "3i", *s.global_dims), struct.pack(e + "4i", s.nx, s.ny, s.nz, s.numprocs),
            struct.pack(e + "4i", s.myid, *s.proc_coords), struct.pack(e + "3i", *s.proc_dims),
            struct.pack(e + "2di", s.zeit, s.delt, s.num_iter)]
    recs += [F(s.coords[n]) for n in COORDS]
    recs += [F(s.arrays[n]) for n in FIELDS3]
    recs.append(np.asarray(s.upperbnd, dtype=np.dtype(e + "i4")).tobytes(order="F"))
    recs.append(struct.pack(e + "6d", *[s.scalars.get(n, 0.0) for n in SCALARS]))
    if s.ncosys is not None:
        recs.append(struct.pack(e + "i", s.ncosys))
        # the records are positional: the ones before the last present are
        # written as zeros when absent
        last = max((q for q, n in enumerate(EXTRAS) if n in s.arrays), default=-1)
        recs += [F(s.arrays[n]) if n in s.arrays else F(np.zeros((s.nx, s.ny, s.nz))) for n in EXTRAS[:last + 1]]
    with open(path, "wb") as f:
        for r in recs:
            f.write(_record(r, e, max_sub))


def stitch(parts: list[Snapshot]) -> Snapshot:
    """One snapshot from the per-rank files of a decomposition in phi and
    theta (proc_coords(2), proc_coords(3)); the radial direction must not be
    split.  Ghost layers come from the rank that owns them."""
    if not parts:
        raise ValueError("no files")
    p0 = parts[0]
    if any(p.proc_dims[0] != 1 for p in parts):
        raise ValueError("a radial decomposition cannot be stitched")
    py, pz = p0.proc_dims[1], p0.proc_dims[2]
    if len(parts) != py * pz:
        raise ValueError(f"{len(parts)} files for a {py} x {pz} decomposition")
    by = {(p.proc_coords[1], p.proc_coords[2]): p for p in parts}
    nx, ny, nz = p0.nx, p0.ny * py, p0.nz * pz
    out = Snapshot(nx, ny, nz, p0.global_dims, 1, 0, (0, 0, 0), (1, 1, 1), p0.zeit, p0.delt, p0.num_iter)
    out.scalars = dict(p0.scalars)
    out.ncosys = p0.ncosys
    out.coords["xxa"], out.coords["xxb"], out.coords["dxa"] = (p0.coords[n] for n in ("xxa", "xxb", "dxa"))
    for ax, (names, nloc, idx) in {"y": (("xya", "xyb", "dya"), p0.ny, 1), "z": (("xza", "xzb", "dza"), p0.nz, 2)}.items():
        nb = py if ax == "y" else pz
        for name in names:
            lo = COORD_LO[name]
            full = np.zeros((ny if ax == "y" else nz) + 2 - lo + 1)
            for b in range(nb):
                p = by[(b, 0)] if ax == "y" else by[(0, b)]
                a = p.coords[name]
                # local index l (lo..nloc+2) -> global b*nloc + l
                for l in range(lo, nloc + 3):
                    g = b * nloc + l
                    if (l >= 1 and l <= nloc) or (b == 0 and l < 1) or (b == nb - 1 and l > nloc):
                        full[g - lo] = a[l - lo]
            out.coords[name] = full
    for name in list(p0.arrays):
        (li, hi), (lj, hj), (lk, hk) = field_bounds(name, p0.nx, p0.ny, p0.nz)
        gb = field_bounds(name, nx, ny, nz)
        full = np.zeros(_shape(gb), order="F")
        for (cy, cz), p in by.items():
            a = p.arrays[name]
            for l in range(lj, hj + 1):
                if not ((1 <= l <= p0.ny) or (cy == 0 and l < 1) or (cy == py - 1 and l > p0.ny)):
                    continue
                gj = cy * p0.ny + l
                for m in range(lk, hk + 1):
                    if not ((1 <= m <= p0.nz) or (cz == 0 and m < 1) or (cz == pz - 1 and m > p0.nz)):
                        continue
                    gk = cz * p0.nz + m
                    full[:, gj - gb[1][0], gk - gb[2][0]] = a[:, l - lj, m - lk]
        out.arrays[name] = full
    ub = np.zeros((ny, nz), dtype=np.int32, order="F")
    for (cy, cz), p in by.items():
        ub[cy * p0.ny:(cy + 1) * p0.ny, cz * p0.nz:(cz + 1) * p0.nz] = p.upperbnd
    out.upperbnd = ub
    return out


def grid_of(s: Snapshot, dxmin: float = 0.0, dymin: float = 0.0, dzmin: float = 0.0) -> Grid:
    """GITTER's NCOSYS=2 metrics (ppinit.f:1180-1406) from the coordinate
    records.  DXMIN = 0 (linear grids) sets DDX0 = DDX1 = 1/2
    (ppinit.f:1198-1202); otherwise they are formed from XXA, XXB, DXB."""
    if s.ncosys not in (None, 2):
        raise ValueError(f"NCOSYS={s.ncosys}: only the spherical grid (2) is implemented")
    nx, ny, nz = s.nx, s.ny, s.nz
    c = s.coords
    full = {}

    def on_halo(name, n):   # -> array over -1..n+2 (index +1)
        a = np.zeros(n + 4)
        lo = COORD_LO[name]
        a[lo + 1:lo + 1 + c[name].size] = c[name]
        return a

    n_of = {"x": nx, "y": ny, "z": nz}
    for ax, (a_, b_, da_, db_) in {"x": ("xxa", "xxb", "dxa", "dxb"), "y": ("xya", "xyb", "dya", "dyb"),
                                   "z": ("xza", "xzb", "dza", "dzb")}.items():
        n = n_of[ax]
        full[a_], full[b_], full[da_] = on_halo(a_, n), on_halo(b_, n), on_halo(da_, n)
        db = np.zeros(n + 4)
        for i in range(0, n + 3):
            db[i + 1] = full[b_][i + 1] - full[b_][i]
        full[db_] = db
        dmin = {"x": dxmin, "y": dymin, "z": dzmin}[ax]
        d0, d1 = np.zeros(n + 4), np.zeros(n + 4)
        for i in range(0, n + 3):
            if dmin == 0.0:
                d0[i + 1] = d1[i + 1] = 0.5
            else:
                d0[i + 1] = (full[b_][i + 1] - full[a_][i + 1]) / db[i + 1]
                d1[i + 1] = (full[a_][i + 1] - full[b_][i]) / db[i + 1]
        full["dd" + ax + "0"], full["dd" + ax + "1"] = d0, d1
    xa, xb, za, zb = full["xxa"], full["xxb"], full["xza"], full["xzb"]
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
    g = Grid(nx, ny, nz, float(xa[2]), float(xa[nx + 2]), float(c["xya"][1] / (2 * math.pi)),
             float(c["xya"][ny + 1] / (2 * math.pi)), float(c["xza"][1] / (math.pi / 2)),
             float(c["xza"][nz + 1] / (math.pi / 2)))
    for name, (lo, hioff) in BOUNDS.items():
        n = n_of[AXIS[name]]
        g.m[name] = np.ascontiguousarray(full[name][lo + 1:n + hioff + 2])
        g.lo[name] = lo
    return g


def shell_of(s: Snapshot, params: dict | None = None, dxmin: float = 0.0):
    """The snapshot as a `synthetic.Shell`: grid from the coordinates, T, RH
    and ER as written, c_v of GASINIT (ppinit.f:1408-1417) for the params'
    gamma and mu, the stellar geometry of the grid.  With the snapshot's
    xkapR/xkapA/xkapP records the opacities are prescribed there
    (kappa_model 1 uploads them; they hold the interior only, so the halo
    takes the nearest interior value); otherwise the analytic model runs."""
    from . import synthetic as S
    g = grid_of(s, dxmin)
    p = dict(S.default_params(s.delt))
    if params:
        p.update(params)
    shape = (s.nx + 4, s.ny + 4, s.nz + 4)
    gamma, mu = p.pop("gamma", 1.4), p.pop("mu", 2.3)
    fields = {"T": np.asfortranarray(s.arrays["T"]), "RH": np.asfortranarray(s.arrays["RH"]),
              "ER": np.asfortranarray(s.arrays["ER"]),
              "CV": np.full(shape, S.RGAS / (mu * (gamma - 1.0)), order="F"),
              "KMUL": np.ones(shape, order="F")}
    mu_s, tinc = S.mu_star_tincident(g, p["tirr"], p["f_incident"])
    fields["MU_STAR"], fields["TINCIDENT"] = mu_s, tinc
    if all(n in s.arrays for n in ("xkapR", "xkapA", "xkapP")) and p.get("kappa_model", 0) == 1:
        for src, dst in (("xkapR", "XKAPR"), ("xkapA", "XKAPA"), ("xkapP", "XKAPP")):
            fields[dst] = np.asfortranarray(np.pad(s.arrays[src], 2, mode="edge"))
    return S.Shell(g, fields, p, seed=-1)


def snapshot_of(sh, zeit: float = 0.0, num_iter: int = 0, upperbnd=None) -> Snapshot:
    """A one-rank snapshot of a `synthetic.Shell` (or of any state with the
    same fields): the arrays PRINTOUT writes that this library holds, zero
    velocities, pressure and sound speed."""
    g = sh.grid
    nx, ny, nz = g.nx, g.ny, g.nz
    s = Snapshot(nx, ny, nz, (nx, ny, nz), 1, 0, (0, 0, 0), (1, 1, 1), zeit, sh.params["delt"], num_iter)
    for name in COORDS:
        lo = COORD_LO[name]
        n = {"x": nx, "y": ny, "z": nz}[name[1]]
        s.coords[name] = np.array([g.at(name, i) for i in range(lo, n + 3)])
    for name in FIELDS3:
        src = {"RH": "RH", "T": "T", "ER": "ER"}.get(name)
        shp = _shape(field_bounds(name, nx, ny, nz))
        s.arrays[name] = np.asfortranarray(sh.fields[src]) if src else np.zeros(shp, order="F")
    s.upperbnd = (np.full((ny, nz), nx - 1, dtype=np.int32) if upperbnd is None
                  else np.asarray(upperbnd, dtype=np.int32))
    s.scalars = {n: 0.0 for n in SCALARS}
    s.ncosys = 2
    return s


def snapshot_of_fld(f, zeit: float = 0.0, num_iter: int = 0) -> Snapshot:
    """A one-rank snapshot of a device state (an `fld.FLD`, or anything with
    its `grid`, `params` and `download`): T, RH, ER and UPPERBND as PRINTOUT
    writes them, and the interior records xkapR, xkapA, STELLARINPUT, xkapP
    (ppprt.f:46-117; the records it has no counterpart for are zero)."""
    g = f.grid
    nx, ny, nz = g.nx, g.ny, g.nz
    s = Snapshot(nx, ny, nz, (nx, ny, nz), 1, 0, (0, 0, 0), (1, 1, 1), zeit, f.params["delt"], num_iter)
    for name in COORDS:
        lo = COORD_LO[name]
        n = {"x": nx, "y": ny, "z": nz}[name[1]]
        s.coords[name] = np.array([g.at(name, i) for i in range(lo, n + 3)])
    for name in FIELDS3:
        if name in ("RH", "T", "ER"):
            s.arrays[name] = np.asfortranarray(f.download(name))
        else:
            s.arrays[name] = np.zeros(_shape(field_bounds(name, nx, ny, nz)), order="F")
    s.upperbnd = np.asfortranarray(f.download("UPPERBND")[2:ny + 2, 2:nz + 2].astype(np.int32))
    s.scalars = {n: 0.0 for n in SCALARS}
    s.ncosys = 2
    inner = lambda a: np.asfortranarray(a[2:nx + 2, 2:ny + 2, 2:nz + 2])
    for rec, src in (("xkapR", "XKAPR"), ("xkapA", "XKAPA"), ("xkapP", "XKAPP")):
        s.arrays[rec] = inner(f.download(src))
    si = f.download("STELLARINPUT")                 # (1:NX, -1:NY+2, -1:NZ+2)
    s.arrays["STELLARINPUT"] = np.asfortranarray(si[:, 2:ny + 2, 2:nz + 2])
    return s



def _i33(n: int) -> str:
    if not 0 <= n <= 999:
        raise ValueError(f"{n} does not fit the I3.3 of the file names")
    return f"{n:03d}"


def rank_file_name(kind: str, rank: int, num: int | None = None) -> str:
    """The names a rank's files get: SNAP_rrr.nnn (every IREA/10 steps) and
    RSRT_rrr.nnn (the first of a restarted run), pp.f:565-575; AKTTD_rrr at
    the end of a run, pp.f:827; CRSH_rrr from CLEAN_STOP, ppsub.f:718-719.
    rrr and nnn are written with I3.3."""
    if kind in ("SNAP", "RSRT"):
        if num is None:
            raise ValueError(f"{kind} files carry a print number")
        return f"{kind}_{_i33(rank)}.{_i33(num)}"
    if kind in ("AKTTD", "CRSH"):
        return f"{kind}_{_i33(rank)}"
    raise ValueError(f"unknown file kind {kind!r}")


def write_crash_dump(f, directory: str = ".", rank: int = 0, zeit: float = 0.0, num_iter: int = 0) -> str:
    """CLEAN_STOP's dump (ppsub.f:707-735): the rank's state as PRINTOUT(1)
    records in CRSH_rrr.  The library returns a CLEAN_STOP status (-7)
    instead of stopping; the caller writes the dump from the context."""
    import os
    path = os.path.join(directory, rank_file_name("CRSH", rank))
    s = snapshot_of_fld(f, zeit, num_iter)
    s.myid = rank
    write(path, s)
    return path

# ---- the global restart file: AKTTD as READRESTART reads it ------------------
GLOBAL3 = ("V", "G", "H", "RH", "T", "ER", "PG", "CS")
GLOBAL_EXTRAS = ("xkapR", "flimx", "EdepFor", "EdepAdv", "EdepRad", "xkapA", "stellarinput", "delta_ER",
                 "xkapP")
# the per-rank record each global extra is filled from (ppcombine.f:695-707
# reads PRINTOUT's records in this order; xkapP is set to zero there)
EXTRA_SOURCE = dict(zip(GLOBAL_EXTRAS, EXTRAS[:8] + (None,)))


@dataclass
class Restart:
    """The global file PRINTGLOBAL writes (ppcombine.f:603-657: GLOB.xxx, and
    AKTTD when ppcombine joins the ranks' AKTTD_xxx files) and READRESTART
    reads (ppinit.f:1544-1646).  Interior cells only, (1:NX,1:NY,1:NZ),
    column-major; NX, NY, NZ are the global extents."""
    nx: int
    ny: int
    nz: int
    loc_dims: tuple
    numprocs: int
    zeit: float
    delt: float
    num_iter: int
    xb: dict = field(default_factory=dict)        # xxb, xyb, xzb on 1..N
    arrays: dict = field(default_factory=dict)    # GLOBAL3 and extras, (NX, NY, NZ)
    upperbnd: np.ndarray | None = None            # (NY, NZ) int32
    scalars: dict = field(default_factory=dict)
    ncosys: int | None = None


def read_restart(path: str, endian: str = "<") -> Restart:
    """READRESTART's binary branch (ppinit.f:1563-1598): the global extents
    (one record each), the local extents and rank count, ZEIT/DELT/NUM_ITER,
    XXB, XYB, XZB, V, G, H, RH, T, ER, PG, CS, UPPERBND and the six boundary
    scalars; then, when present, the records PRINTGLOBAL appends that a
    restart does not read (NCOSYS and the extras)."""
    with open(path, "rb") as f:
        r = _Records(f.read(), endian)
    e = endian
    (nx,), (ny,), (nz,) = (_ints(r.next(), 1, e) for _ in range(3))
    lx, ly, lz, nprocs = _ints(r.next(), 4, e)
    rec = r.next()
    if len(rec) != 20:
        raise ValueError("ZEIT, DELT, NUM_ITER record is not 8+8+4 bytes")
    zeit, delt = struct.unpack_from(e + "2d", rec, 0)
    (num_iter,) = struct.unpack_from(e + "i", rec, 16)
    out = Restart(nx, ny, nz, (lx, ly, lz), nprocs, zeit, delt, num_iter)
    for name, n in (("xxb", nx), ("xyb", ny), ("xzb", nz)):
        out.xb[name] = _doubles(r.next(), (n,), e)
    for name in GLOBAL3:
        out.arrays[name] = _doubles(r.next(), (nx, ny, nz), e)
    rec = r.next()
    if len(rec) != 4 * ny * nz:
        raise ValueError("UPPERBND record size")
    out.upperbnd = np.frombuffer(rec, dtype=np.dtype(e + "i4")).astype(np.int32).reshape((ny, nz), order="F")
    out.scalars = dict(zip(SCALARS, struct.unpack(e + "6d", r.next())))
    if r.done():
        return out
    (out.ncosys,) = _ints(r.next(), 1, e)
    for name in GLOBAL_EXTRAS:
        if r.done():
            break
        out.arrays[name] = _doubles(r.next(), (nx, ny, nz), e)
    return out


def read_restart_ascii(path: str) -> Restart:
    """READRESTART's AKTTD_ASCII branch (ppinit.f:1599-1632): the same items
    as list-directed reads, one READ per binary record."""
    from .fortio import ListDirected, integer, real
    with open(path) as fh:
        rd = ListDirected(fh.readlines(), path, ValueError)

    def one(conv):
        v = rd.read(1, conv)[0]
        if v is None:
            raise ValueError(f"{path}: null value at record {rd.pos}")
        return v

    def many(n, conv=real):
        v = rd.read(n, conv)
        if any(x is None for x in v):
            raise ValueError(f"{path}: null value before record {rd.pos}")
        return v

    nx, ny, nz = one(integer), one(integer), one(integer)
    lx, ly, lz, nprocs = many(4, integer)
    zeit, delt, num_iter = many(3, (real, real, integer))
    out = Restart(nx, ny, nz, (lx, ly, lz), nprocs, zeit, delt, num_iter)
    for name, n in (("xxb", nx), ("xyb", ny), ("xzb", nz)):
        out.xb[name] = np.array(many(n))
    for name in GLOBAL3:
        out.arrays[name] = np.array(many(nx * ny * nz)).reshape((nx, ny, nz), order="F")
    out.upperbnd = np.array(many(ny * nz, integer), dtype=np.int32).reshape((ny, nz), order="F")
    out.scalars = dict(zip(SCALARS, many(6)))
    return out


def write_restart(path: str, g: Restart, endian: str = "<", max_sub: int = MAX_SUBRECORD):
    """PRINTGLOBAL's record sequence (ppcombine.f:603-657); the extras
    follow NCOSYS when ``ncosys`` is set, missing ones before the last present
    written as zeros."""
    e = endian
    F = lambda a: np.asarray(a, dtype=np.float64).astype(np.dtype(e + "f8")).tobytes(order="F")
    recs = [struct.pack(e + "i", g.nx), struct.pack(e + "i", g.ny), struct.pack(e + "i", g.nz),
            struct.pack(e + "4i", *g.loc_dims, g.numprocs), struct.pack(e + "2di", g.zeit, g.delt, g.num_iter)]
    recs += [F(g.xb[n]) for n in ("xxb", "xyb", "xzb")]
    recs += [F(g.arrays[n]) for n in GLOBAL3]
    recs.append(np.asarray(g.upperbnd, dtype=np.dtype(e + "i4")).tobytes(order="F"))
    recs.append(struct.pack(e + "6d", *[g.scalars.get(n, 0.0) for n in SCALARS]))
    if g.ncosys is not None:
        recs.append(struct.pack(e + "i", g.ncosys))
        last = max((q for q, n in enumerate(GLOBAL_EXTRAS) if n in g.arrays), default=-1)
        zero = np.zeros((g.nx, g.ny, g.nz))
        recs += [F(g.arrays.get(n, zero)) for n in GLOBAL_EXTRAS[:last + 1]]
    with open(path, "wb") as f:
        for rec in recs:
            f.write(_record(rec, e, max_sub))


def combine(parts: list[Snapshot]) -> Restart:
    """ppcombine's FILLGLOBAL (ppcombine.f:370-457, EXCLUDEREGION off) over
    the ranks' files: every rank's interior at its offset locN*proc_coords
    (a radial split included), the coordinate of each axis from the ranks on
    that axis, the per-rank extras by position with xkapP zero (ppcombine.f
    :706-707 does not read it)."""
    if not parts:
        raise ValueError("no files")
    p0 = parts[0]
    nx, ny, nz = p0.global_dims
    lx, ly, lz = p0.nx, p0.ny, p0.nz
    if len(parts) != p0.numprocs:
        raise ValueError(f"{len(parts)} files for {p0.numprocs} ranks")
    g = Restart(nx, ny, nz, (lx, ly, lz), p0.numprocs, p0.zeit, p0.delt, p0.num_iter)
    g.xb = {n: np.zeros(m) for n, m in (("xxb", nx), ("xyb", ny), ("xzb", nz))}
    g.arrays = {n: np.zeros((nx, ny, nz), order="F") for n in GLOBAL3 + GLOBAL_EXTRAS}
    g.upperbnd = np.zeros((ny, nz), dtype=np.int32, order="F")
    seen = np.zeros((nx, ny, nz), dtype=bool)
    for p in parts:
        if (p.nx, p.ny, p.nz) != (lx, ly, lz) or tuple(p.global_dims) != (nx, ny, nz):
            raise ValueError("the ranks' files disagree on the extents")
        cx, cy, cz = p.proc_coords
        ox, oy, oz = lx * cx, ly * cy, lz * cz
        if ox + lx > nx or oy + ly > ny or oz + lz > nz or min(ox, oy, oz) < 0:
            raise ValueError(f"rank {p.myid}: proc_coords {p.proc_coords} outside the global grid")
        if cy == 0 and cz == 0:
            g.xb["xxb"][ox:ox + lx] = p.coords["xxb"][2:lx + 2]
        if cx == 0 and cz == 0:
            g.xb["xyb"][oy:oy + ly] = p.coords["xyb"][2:ly + 2]
        if cx == 0 and cy == 0:
            g.xb["xzb"][oz:oz + lz] = p.coords["xzb"][2:lz + 2]
        sl = np.s_[ox:ox + lx, oy:oy + ly, oz:oz + lz]
        for name in GLOBAL3:
            (li, _), (lj, _), (lk, _) = field_bounds(name, lx, ly, lz)
            a = p.arrays[name]
            g.arrays[name][sl] = a[1 - li:1 - li + lx, 1 - lj:1 - lj + ly, 1 - lk:1 - lk + lz]
        for name in GLOBAL_EXTRAS:
            src = EXTRA_SOURCE[name]
            if src is not None and src in p.arrays:
                g.arrays[name][sl] = p.arrays[src]
        g.upperbnd[oy:oy + ly, oz:oz + lz] = p.upperbnd
        seen[sl] = True
    if not seen.all():
        raise ValueError("the ranks' files do not cover the global grid")
    g.scalars = dict(p0.scalars)
    g.ncosys = p0.ncosys if p0.ncosys is not None else 2
    return g


def _halo_of_interior(a: np.ndarray) -> np.ndarray:
    """(NX,NY,NZ) -> (-1:NX+2,-1:NY+2,-1:NZ+2): the one-rank PLANETSHIFT copy
    in phi (j = -1, 0 from NY-1, NY; NY+1, NY+2 from 1, 2), the nearest
    interior value in r and theta."""
    b = np.concatenate([a[:, -2:, :], a, a[:, :2, :]], axis=1)
    return np.asfortranarray(np.pad(b, ((2, 2), (0, 0), (2, 2)), mode="edge"))


def shell_of_restart(g: Restart, grid: Grid, params: dict | None = None, check_grid: bool = True):
    """A restart file as a `synthetic.Shell` for `fld.start_run`, following
    READRESTART + LOCALINIT (ppinit.f:1544-1646, 1-69): T, ER, RH of the
    interior from the file, the grid from GITTER and the run's parameters
    (READRESTART reads the coordinates into dummies), c_v of GASINIT.  The
    ghost layers take the periodic copy in phi and the nearest interior
    value in r and theta; BOUNDS (run by `start_run`) then sets those of T
    and RH, and the step sets those of ER.  RH below the bottom (i = 0, -1),
    which BOUNDXMIN(9) leaves alone (ppinit.f:62-69), keeps RH(1).  With
    ``check_grid`` the grid's cell centres must agree with the file's
    XXB/XYB/XZB to 1e-12."""
    from . import synthetic as S
    if (grid.nx, grid.ny, grid.nz) != (g.nx, g.ny, g.nz):
        raise ValueError(f"grid {(grid.nx, grid.ny, grid.nz)} vs file {(g.nx, g.ny, g.nz)}")
    if check_grid:
        for name, n in (("xxb", g.nx), ("xyb", g.ny), ("xzb", g.nz)):
            mine = np.array([grid.at(name, i) for i in range(1, n + 1)])
            scale = max(np.max(np.abs(mine)), 1e-300)
            if np.max(np.abs(mine - g.xb[name])) > 1e-12 * scale:
                raise ValueError(f"{name}: the grid's cell centres differ from the file's")
    p = dict(S.default_params(g.delt))
    if params:
        p.update(params)
    shape = (g.nx + 4, g.ny + 4, g.nz + 4)
    gamma, mu = p.pop("gamma", 1.4), p.pop("mu", 2.3)
    fields = {n: _halo_of_interior(g.arrays[n]) for n in ("T", "RH", "ER")}
    fields["CV"] = np.full(shape, S.RGAS / (mu * (gamma - 1.0)), order="F")
    fields["KMUL"] = np.ones(shape, order="F")
    fields["MU_STAR"], fields["TINCIDENT"] = S.mu_star_tincident(grid, p["tirr"], p["f_incident"])
    return S.Shell(grid, fields, p, seed=-1)
