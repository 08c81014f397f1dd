"""The restart-record reader/writer (ttcode_gb300.akttd) against the record
layout of PRINTOUT(1), ppprt.f:13-124, and a state driven from a record."""
import struct

import numpy as np
import pytest

from ttcode_gb300 import akttd as A
from ttcode_gb300.synthetic import make_shell


@pytest.fixture(scope="module")
def sh():
    return make_shell(12, 16, 8, seed=4, delt=100.0)


def _raw_records(path):
    b = open(path, "rb").read()
    p, out = 0, []
    while p < len(b):
        (n,) = struct.unpack_from("<i", b, p)
        out.append(b[p + 4:p + 4 + n])
        assert struct.unpack_from("<i", b, p + 4 + n)[0] == n
        p += n + 8
    return out


def test_record_layout_follows_printout(sh, tmp_path):
    s = A.snapshot_of(sh, zeit=12.5, num_iter=7)
    s.arrays["xkapR"] = np.random.default_rng(1).random((12, 16, 8))
    f = tmp_path / "AKTTD"
    A.write(str(f), s)
    r = _raw_records(str(f))
    nx, ny, nz = 12, 16, 8
    assert struct.unpack("<3i", r[0]) == (nx, ny, nz)                       # ppprt.f:15
    assert struct.unpack("<4i", r[1]) == (nx, ny, nz, 1)                    # :16
    assert struct.unpack("<4i", r[2]) == (0, 0, 0, 0)                       # :17
    assert struct.unpack("<3i", r[3]) == (1, 1, 1)                          # :18
    assert struct.unpack("<2di", r[4]) == (12.5, 100.0, 7)                  # :19
    assert len(r[5]) == 8 * (nx + 3) and len(r[6]) == 8 * (nx + 4) and len(r[7]) == 8 * (nx + 2)  # :20-22
    assert len(r[14]) == 8 * (nx + 3) * (ny + 4) * (nz + 4)                 # V, :29
    assert len(r[15]) == 8 * (nx + 4) * (ny + 3) * (nz + 4)                 # G
    assert len(r[16]) == 8 * (nx + 4) * (ny + 4) * (nz + 3)                 # H
    T = np.frombuffer(r[18], "<f8").reshape((nx + 4, ny + 4, nz + 4), order="F")
    assert np.array_equal(T, sh.fields["T"])                                # :34-35
    assert len(r[21]) == 8 * (nx + 2) * (ny + 2) * (nz + 2)                 # CS, :40
    assert len(r[22]) == 4 * ny * nz                                        # UPPERBND, :41
    assert len(r[23]) == 6 * 8                                              # :42-43
    assert struct.unpack("<i", r[24]) == (2,)                               # NCOSYS, :45
    assert np.array_equal(np.frombuffer(r[25], "<f8").reshape((nx, ny, nz), order="F"), s.arrays["xkapR"])


@pytest.mark.parametrize("max_sub", [A.MAX_SUBRECORD, 1000])
def test_round_trip(sh, tmp_path, max_sub):
    s = A.snapshot_of(sh, zeit=3.0, num_iter=2)
    s.arrays["V"][...] = np.random.default_rng(2).random(s.arrays["V"].shape)
    for n in A.EXTRAS:
        s.arrays[n] = np.random.default_rng(hash(n) % 1000).random((12, 16, 8))
    f = tmp_path / "SNAP.000"
    A.write(str(f), s, max_sub=max_sub)
    t = A.read(str(f))
    assert (t.nx, t.ny, t.nz, t.zeit, t.delt, t.num_iter, t.ncosys) == (12, 16, 8, 3.0, 100.0, 2, 2)
    for n in A.COORDS:
        assert np.array_equal(t.coords[n], s.coords[n]), n
    for n in list(A.FIELDS3) + list(A.EXTRAS):
        assert np.array_equal(t.arrays[n], s.arrays[n]), n
    assert np.array_equal(t.upperbnd, s.upperbnd)


def test_subrecord_markers_are_gfortrans():
    """A record split into three sub-records: head markers negative while
    another sub-record follows, tail markers negative after the first (the
    layout gfortran writes for records over 2**31-9 bytes)."""
    import struct
    payload = bytes(range(10))
    b = A._record(payload, "<", max_sub=4)
    marks, data, p = [], b"", 0
    for n in (4, 4, 2):
        marks.append(struct.unpack_from("<i", b, p)[0])
        data += b[p + 4:p + 4 + n]
        marks.append(struct.unpack_from("<i", b, p + 4 + n)[0])
        p += 8 + n
    assert p == len(b) and data == payload
    assert marks == [-4, 4, -4, -4, 2, -2]
    assert A._record(payload, "<", max_sub=16) == struct.pack("<i", 10) + payload + struct.pack("<i", 10)
    assert A.MAX_SUBRECORD == 2**31 - 9
    assert A._Records(b, "<").next() == payload


def test_truncated_file_is_an_error(sh, tmp_path):
    f = tmp_path / "AKTTD"
    A.write(str(f), A.snapshot_of(sh))
    b = open(f, "rb").read()
    open(f, "wb").write(b[:len(b) // 2])
    with pytest.raises(EOFError):
        A.read(str(f))


def test_grid_rebuilt_from_coordinates(sh):
    g = A.grid_of(A.snapshot_of(sh))
    for name in sh.grid.m:
        assert np.array_equal(g.m[name], sh.grid.m[name]), name
        assert g.lo[name] == sh.grid.lo[name]


def _split(s, py, pz):
    """The per-rank snapshots a py x pz (phi, theta) decomposition writes."""
    out = []
    ny, nz = s.ny // py, s.nz // pz
    for cy in range(py):
        for cz in range(pz):
            p = A.Snapshot(s.nx, ny, nz, s.global_dims, py * pz, cy * pz + cz, (0, cy, cz), (1, py, pz),
                           s.zeit, s.delt, s.num_iter)
            p.scalars, p.ncosys = dict(s.scalars), s.ncosys
            for name in A.COORDS:
                lo = A.COORD_LO[name]
                a = s.coords[name]
                if name[1] == "x":
                    p.coords[name] = a.copy()
                else:
                    c, n = (cy, ny) if name[1] == "y" else (cz, nz)
                    p.coords[name] = np.array([a[c * n + l - lo] for l in range(lo, n + 3)])
            for name, a in s.arrays.items():
                (li, _), (lj, hj), (lk, hk) = A.field_bounds(name, s.nx, ny, nz)
                gb = A.field_bounds(name, s.nx, s.ny, s.nz)
                J = [cy * ny + l - gb[1][0] for l in range(lj, hj + 1)]
                K = [cz * nz + m - gb[2][0] for m in range(lk, hk + 1)]
                p.arrays[name] = np.asfortranarray(a[:, J][:, :, K])
            p.upperbnd = np.asfortranarray(s.upperbnd[cy * ny:(cy + 1) * ny, cz * nz:(cz + 1) * nz])
            out.append(p)
    return out


def test_stitch_phi_theta_decomposition(sh, tmp_path):
    s = A.snapshot_of(sh, zeit=1.0)
    s.arrays["xkapP"] = np.random.default_rng(3).random((12, 16, 8))
    s.upperbnd = np.asfortranarray(np.arange(16 * 8, dtype=np.int32).reshape(16, 8) % 11 + 1)
    parts = []
    for q, p in enumerate(_split(s, 2, 2)):
        f = tmp_path / f"SNAP.{q:03d}"
        A.write(str(f), p)
        parts.append(A.read(str(f)))
    t = A.stitch(parts)
    for n in A.COORDS:
        assert np.array_equal(t.coords[n], s.coords[n]), n
    for n, a in s.arrays.items():
        assert np.array_equal(t.arrays[n], a), n
    assert np.array_equal(t.upperbnd, s.upperbnd)


def test_shell_of_snapshot(sh):
    t = A.shell_of(A.snapshot_of(sh))
    for n in ("T", "RH", "ER", "CV", "MU_STAR", "TINCIDENT"):
        assert np.array_equal(t.fields[n], sh.fields[n]), n
    assert t.params["delt"] == sh.params["delt"]


@pytest.mark.gpu
def test_step_driven_from_a_record(tmp_path):
    """The implicit step started from a record of a state gives the step
    started from the state itself, bit for bit."""
    from ttcode_gb300.fld import start_run
    s0 = make_shell(24, 32, 16, seed=6, delt=100.0)
    s0.fields["KMUL"] = np.ones_like(s0.fields["KMUL"])   # the record carries no opacity multiplier
    f = tmp_path / "AKTTD"
    A.write(str(f), A.snapshot_of(s0))
    s1 = A.shell_of(A.read(str(f)))
    out = []
    for s in (s0, s1):
        ctx = start_run(s)
        ctx.set_solver("sor64_exact")
        st = ctx.coupled_energy_eqs(True)
        out.append((st.sor_total, ctx.download("ER"), ctx.download("T")))
        ctx.close()
    assert out[0][0] == out[1][0]
    assert np.array_equal(out[0][1], out[1][1]) and np.array_equal(out[0][2], out[1][2])


def test_snapshot_of_a_device_state(sh, tmp_path):
    """snapshot_of_fld takes what a context holds (through download) into the
    records; with a stand-in for the context, checked on the CPU."""
    nx, ny, nz = sh.dims
    rng = np.random.default_rng(9)
    arrays = {"T": sh.fields["T"], "RH": sh.fields["RH"], "ER": sh.fields["ER"],
              "UPPERBND": np.full((ny + 4, nz + 4), nx - 1, dtype=np.int32),
              "XKAPR": rng.random((nx + 4, ny + 4, nz + 4)), "XKAPA": rng.random((nx + 4, ny + 4, nz + 4)),
              "XKAPP": rng.random((nx + 4, ny + 4, nz + 4)), "STELLARINPUT": rng.random((nx, ny + 4, nz + 4))}

    class Ctx:
        grid, params = sh.grid, sh.params

        def download(self, name):
            return np.asfortranarray(arrays[name])

    s = A.snapshot_of_fld(Ctx(), zeit=5.0, num_iter=3)
    f = tmp_path / "AKTTD"
    A.write(str(f), s)
    t = A.read(str(f))
    assert (t.zeit, t.num_iter) == (5.0, 3)
    assert np.array_equal(t.arrays["T"], sh.fields["T"])
    assert np.array_equal(t.upperbnd, np.full((ny, nz), nx - 1))
    assert np.array_equal(t.arrays["xkapP"], arrays["XKAPP"][2:nx + 2, 2:ny + 2, 2:nz + 2])
    assert np.array_equal(t.arrays["STELLARINPUT"], arrays["STELLARINPUT"][:, 2:ny + 2, 2:nz + 2])
    for n in ("flimx", "conv_flux1", "disfn"):
        assert not t.arrays[n].any()


# ---- the global restart file (PRINTGLOBAL / READRESTART) ---------------------
def _full_snapshot(sh):
    s = A.snapshot_of(sh, zeit=2.5, num_iter=11)
    rng = np.random.default_rng(12)
    for n in ("V", "G", "H", "PG", "CS"):
        s.arrays[n] = np.asfortranarray(rng.random(s.arrays[n].shape))
    for n in A.EXTRAS:
        s.arrays[n] = np.asfortranarray(rng.random((s.nx, s.ny, s.nz)))
    s.upperbnd = np.asfortranarray(rng.integers(2, s.nx, (s.ny, s.nz)).astype(np.int32))
    s.scalars = {n: float(q + 1) for q, n in enumerate(A.SCALARS)}
    return s


def _inner(s, name):
    (li, _), (lj, _), (lk, _) = A.field_bounds(name, s.nx, s.ny, s.nz)
    return s.arrays[name][1 - li:1 - li + s.nx, 1 - lj:1 - lj + s.ny, 1 - lk:1 - lk + s.nz]


def test_restart_record_layout(sh, tmp_path):
    """PRINTGLOBAL's records (ppcombine.f:607-657), the first twenty of which
    READRESTART reads (ppinit.f:1566-1598)."""
    s = _full_snapshot(sh)
    g = A.combine([s])
    f = tmp_path / "AKTTD"
    A.write_restart(str(f), g)
    r = _raw_records(str(f))
    nx, ny, nz = 12, 16, 8
    n3 = 8 * nx * ny * nz
    assert [struct.unpack("<i", r[q])[0] for q in range(3)] == [nx, ny, nz]
    assert struct.unpack("<4i", r[3]) == (nx, ny, nz, 1)
    assert struct.unpack("<2di", r[4]) == (2.5, 100.0, 11)
    assert [len(r[q]) for q in (5, 6, 7)] == [8 * nx, 8 * ny, 8 * nz]
    assert np.array_equal(np.frombuffer(r[5], "<f8"), s.coords["xxb"][2:nx + 2])
    assert all(len(r[q]) == n3 for q in range(8, 16))
    T = np.frombuffer(r[12], "<f8").reshape((nx, ny, nz), order="F")
    assert np.array_equal(T, sh.fields["T"][2:-2, 2:-2, 2:-2])
    assert np.array_equal(np.frombuffer(r[15], "<f8").reshape((nx, ny, nz), order="F"), _inner(s, "CS"))
    assert np.array_equal(np.frombuffer(r[16], "<i4").reshape((ny, nz), order="F"), s.upperbnd)
    assert struct.unpack("<6d", r[17]) == (1.0, 2.0, 3.0, 4.0, 5.0, 6.0)
    assert struct.unpack("<i", r[18]) == (2,)
    assert len(r) == 19 + 9 and all(len(x) == n3 for x in r[19:])
    # the extras by position; xkapP is written as zero (ppcombine.f:706-707)
    assert np.array_equal(np.frombuffer(r[21], "<f8").reshape((nx, ny, nz), order="F"), s.arrays["conv_flux1"])
    assert np.array_equal(np.frombuffer(r[26], "<f8").reshape((nx, ny, nz), order="F"), s.arrays["disfn"])
    assert not np.frombuffer(r[27], "<f8").any()


@pytest.mark.parametrize("max_sub", [A.MAX_SUBRECORD, 999])
def test_restart_round_trip(sh, tmp_path, max_sub):
    g = A.combine([_full_snapshot(sh)])
    f = tmp_path / "AKTTD"
    A.write_restart(str(f), g, max_sub=max_sub)
    t = A.read_restart(str(f))
    assert (t.nx, t.ny, t.nz, t.loc_dims, t.numprocs, t.zeit, t.delt, t.num_iter, t.ncosys) == \
        (12, 16, 8, (12, 16, 8), 1, 2.5, 100.0, 11, 2)
    for n in ("xxb", "xyb", "xzb"):
        assert np.array_equal(t.xb[n], g.xb[n]), n
    for n in A.GLOBAL3 + A.GLOBAL_EXTRAS:
        assert np.array_equal(t.arrays[n], g.arrays[n]), n
    assert np.array_equal(t.upperbnd, g.upperbnd) and t.scalars == g.scalars
    # the twenty records a restart reads are a complete file too
    g.ncosys = None
    A.write_restart(str(f), g)
    t = A.read_restart(str(f))
    assert t.ncosys is None and set(t.arrays) == set(A.GLOBAL3)


def test_ascii_restart(sh, tmp_path):
    """AKTTD_ASCII (ppinit.f:1599-1632): the same items, list-directed; a
    READ spans as many lines as its items need."""
    g = A.combine([_full_snapshot(sh)])
    f = tmp_path / "AKTTD_ASCII"

    def vals(a, fmt="{!r}"):
        flat = np.ravel(a, order="F")
        return "\n".join(" ".join(fmt.format(v.item()) for v in flat[q:q + 5]) for q in range(0, flat.size, 5))

    with open(f, "w") as fh:
        fh.write(f"{g.nx}\n{g.ny}\n{g.nz}\n")
        fh.write(" ".join(str(v) for v in (*g.loc_dims, g.numprocs)) + "\n")
        fh.write(f"{g.zeit!r}, {g.delt!r} {g.num_iter}\n")
        for n in ("xxb", "xyb", "xzb"):
            fh.write(vals(g.xb[n], "{:.17E}").replace("E", "D") + "\n")
        for n in A.GLOBAL3:
            fh.write(vals(g.arrays[n]) + "\n")
        fh.write(vals(g.upperbnd, "{}") + "\n")
        fh.write(" ".join(repr(g.scalars[n]) for n in A.SCALARS) + "\n")
    t = A.read_restart_ascii(str(f))
    assert (t.nx, t.ny, t.nz, t.zeit, t.delt, t.num_iter) == (12, 16, 8, 2.5, 100.0, 11)
    for n in ("xxb", "xyb", "xzb"):
        assert np.array_equal(t.xb[n], g.xb[n]), n
    for n in A.GLOBAL3:
        assert np.array_equal(t.arrays[n], g.arrays[n]), n
    assert np.array_equal(t.upperbnd, g.upperbnd) and t.scalars == g.scalars


def _split_radial(s, px):
    """Per-rank snapshots of a radial split into px ranks (interior and
    coordinates; ppcombine joins interiors only)."""
    out = []
    lx = s.nx // px
    for cx in range(px):
        p = A.Snapshot(lx, s.ny, s.nz, s.global_dims, px, cx, (cx, 0, 0), (px, 1, 1), s.zeit, s.delt,
                       s.num_iter)
        p.scalars, p.ncosys = dict(s.scalars), s.ncosys
        for name in A.COORDS:
            lo = A.COORD_LO[name]
            a = s.coords[name]
            p.coords[name] = (np.array([a[cx * lx + l - lo] for l in range(lo, lx + 3)]) if name[1] == "x"
                              else a.copy())
        for name, a in s.arrays.items():
            if name in A.EXTRAS:
                p.arrays[name] = np.asfortranarray(a[cx * lx:(cx + 1) * lx])
                continue
            b = A.field_bounds(name, lx, s.ny, s.nz)
            (li, _), (lj, _), (lk, _) = b
            sub = np.zeros(A._shape(b), order="F")
            sub[1 - li:1 - li + lx, 1 - lj:1 - lj + s.ny, 1 - lk:1 - lk + s.nz] = \
                _inner(s, name)[cx * lx:(cx + 1) * lx]
            p.arrays[name] = sub
        p.upperbnd = s.upperbnd.copy(order="F")
        out.append(p)
    return out


@pytest.mark.parametrize("split", ["phi_theta", "radial"])
def test_combine_joins_the_ranks(sh, tmp_path, split):
    """ppcombine's FILLGLOBAL over the ranks' files equals the one-rank
    combine (a radial split included, which ppcombine allows)."""
    s = _full_snapshot(sh)
    whole = A.combine([s])
    parts = _split(s, 2, 2) if split == "phi_theta" else _split_radial(s, 3)
    read_back = []
    for q, p in enumerate(parts):
        f = tmp_path / f"AKTTD_{q:03d}"
        A.write(str(f), p)
        read_back.append(A.read(str(f)))
    g = A.combine(read_back[::-1])
    for n in ("xxb", "xyb", "xzb"):
        assert np.array_equal(g.xb[n], whole.xb[n]), n
    for n in A.GLOBAL3 + A.GLOBAL_EXTRAS:
        assert np.array_equal(g.arrays[n], whole.arrays[n]), n
    assert np.array_equal(g.upperbnd, whole.upperbnd)
    with pytest.raises(ValueError):
        A.combine(read_back[1:])


def test_restart_drives_the_step(tmp_path):
    """A state written as AKTTD and restarted (READRESTART, LOCALINIT's copy,
    BOUNDS) takes the same implicit step as the state itself, bit for bit,
    in the oracle; the ghost values the file does not hold are rebuilt or
    never read.  The state's RH below the bottom holds RH(1), the value the
    restart gives it."""
    from conftest import oracle_from_shell
    s0 = make_shell(16, 24, 12, seed=3, delt=100.0)
    s0.fields["KMUL"][...] = 1.0
    rh = s0.fields["RH"]
    rh[0], rh[1] = rh[2], rh[2]
    f = tmp_path / "AKTTD"
    A.write_restart(str(f), A.combine([A.snapshot_of(s0)]))
    s1 = A.shell_of_restart(A.read_restart(str(f)), s0.grid)
    for n in ("T", "RH", "ER"):
        assert np.array_equal(s1.fields[n][2:-2, 2:-2, 2:-2], s0.fields[n][2:-2, 2:-2, 2:-2])
    assert not np.array_equal(s1.fields["ER"], s0.fields["ER"])       # the ghosts differ
    o0, o1 = oracle_from_shell(s0, eps=1e-12), oracle_from_shell(s1, eps=1e-12)
    assert o0.call("coupled_energy_eqs", 1) == 0 and o1.call("coupled_energy_eqs", 1) == 0
    assert o0.get("energy_iter") == o1.get("energy_iter")
    for n in ("T", "ER"):
        assert np.array_equal(o0.f(n)[2:-2, 2:-2, 2:-2], o1.f(n)[2:-2, 2:-2, 2:-2]), n
    # the grid comes from the run's parameters; a different one is refused
    from ttcode_gb300.grid import gitter
    with pytest.raises(ValueError):
        A.shell_of_restart(A.read_restart(str(f)), gitter(16, 24, 12, 1.0e9, 1.2e9))


def test_file_names_and_crash_dump(sh, tmp_path):
    assert A.rank_file_name("SNAP", 3, 17) == "SNAP_003.017"
    assert A.rank_file_name("RSRT", 0, 0) == "RSRT_000.000"
    assert A.rank_file_name("AKTTD", 12) == "AKTTD_012"
    assert A.rank_file_name("CRSH", 0) == "CRSH_000"
    for bad in (("SNAP", 1, None), ("SNAP", 1000, 1), ("GLOB", 0, 1)):
        with pytest.raises(ValueError):
            A.rank_file_name(*bad)
    nx, ny, nz = sh.dims

    class Ctx:                                  # a context after a CLEAN_STOP status
        grid, params = sh.grid, sh.params

        def download(self, name):
            if name == "UPPERBND":
                return np.full((ny + 4, nz + 4), nx - 1, dtype=np.int32)
            if name == "STELLARINPUT":
                return np.zeros((nx, ny + 4, nz + 4))
            return np.asfortranarray(sh.fields.get(name, np.zeros((nx + 4, ny + 4, nz + 4))))

    path = A.write_crash_dump(Ctx(), str(tmp_path), rank=2, zeit=7.5, num_iter=9)
    assert path.endswith("CRSH_002")
    t = A.read(path)
    assert (t.myid, t.zeit, t.num_iter) == (2, 7.5, 9)
    assert np.array_equal(t.arrays["T"], sh.fields["T"])
