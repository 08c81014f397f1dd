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


@pytest.mark.parametrize("max_sub", [2**31 - 1, 1000])
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
