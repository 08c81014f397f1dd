"""The Burrows table reader (ttcode_gb300.opacity) against READBURROWSOPCTABLE
(pprphy.f:1231-1541), the file selection of ppplanets.f:36-213 and the node
grid of ppmod.f:735-757; a table file driving the oracle's KAPPA."""
import math

import numpy as np
import pytest

from conftest import oracle_from_shell, rel_l2
from ttcode_gb300 import fortio
from ttcode_gb300 import opacity as O
from ttcode_gb300.synthetic import RGAS, make_shell


def _random_table(rng, ikaptyp):
    s = (O.NODES, O.NODES)
    a = {n: rng.uniform(-4.0, 2.0, s) for n in ("plnk", "ross", "absk")}
    for n in ("waveopac", "localwave", "local_bb"):
        a[n] = rng.uniform(-4.0, 2.0, s + (O.WAVE_BINS,))
    return a


def test_nodes_are_the_single_precision_literals():
    assert O.BURROWS_LOG_T.size == O.NODES and O.BURROWS_LOG_RHO.size == O.NODES
    assert O.BURROWS_LOG_T[0] == float(np.float32(1.69896)) != 1.69896
    assert O.BURROWS_LOG_RHO[-1] == float(np.float32(-1.99993))
    assert np.all(np.diff(O.BURROWS_LOG_T) > 0) and np.all(np.diff(O.BURROWS_LOG_RHO) > 0)
    # BurrowsOPC's clamps (pprphy.f:1045-1049) keep log T and log rho strictly
    # inside the nodes, so the bracketing search never runs off either end
    f = lambda x: float(np.float32(x))
    assert O.BURROWS_LOG_T[0] < f(1.69897) and f(3.69888) < O.BURROWS_LOG_T[-1]
    assert O.BURROWS_LOG_RHO[0] < f(-11.9995) and f(-1.99994) < O.BURROWS_LOG_RHO[-1]
    # the nodes are the logs of the commented-out linear table (ppmod.f:714-733)
    assert abs(10 ** O.BURROWS_LOG_T[-1] / 4999.04 - 1) < 1e-4
    assert abs(10 ** O.BURROWS_LOG_RHO[0] / 1.00102e-12 - 1) < 1e-4


def test_list_directed_reads():
    rd = fortio.ListDirected([
        "  header, with a comma\n",
        "1.5 2.5d0\n",                 # a read of 4 continues on the next record
        "3.0E+1, 4 9 9 9\n",           # ... and drops the rest of it
        "2*7.0 ,, 1.0-3\n",            # repeat count, a null value, a signed exponent
        "8.0 / 5.0\n",                 # a slash ends the read
        "\n",                          # a blank record gives no value
        "'quoted text' rest\n",
    ])
    assert rd.read_text() == "header"
    assert rd.read(4) == [1.5, 2.5, 30.0, 4.0]
    assert rd.read(4) == [7.0, 7.0, None, 1.0e-3]
    assert rd.read(3) == [8.0, None, None]
    assert rd.read_text() == "quoted text"
    with pytest.raises(fortio.ListDirectedError):
        rd.read(1)
    # a READ of mixed types (ZEIT, DELT, NUM_ITER) and a bad item
    rd = fortio.ListDirected(["1.5d3, 2.0 17\n", "x\n"])
    v = rd.read(3, conv=(fortio.real, fortio.real, fortio.integer))
    assert v == [1500.0, 2.0, 17] and isinstance(v[2], int)
    with pytest.raises(fortio.ListDirectedError):
        rd.read(1)


@pytest.mark.parametrize("ikaptyp", [10, 21, 23])
def test_table_round_trip(tmp_path, ikaptyp):
    a = _random_table(np.random.default_rng(ikaptyp), ikaptyp)
    p = tmp_path / "t.dat"
    O.write_burrows_table(p, ikaptyp, 5040.0, **a)
    t = O.read_burrows_table(p, ikaptyp)
    assert t.t_absorption == 5040.0 and t.ikaptyp == ikaptyp
    for n in ("plnk", "ross", "absk"):
        assert np.array_equal(getattr(t, n), a[n]), n
    wave = ikaptyp in O.WAVELENGTH_TYPES
    local = ikaptyp in O.LOCAL_WAVE_TYPES
    assert np.array_equal(t.waveopac, a["waveopac"]) if wave else np.all(t.waveopac == O.MISSING)
    for n in ("localwave", "local_bb"):
        assert np.array_equal(getattr(t, n), a[n]) if local else np.all(getattr(t, n) == O.MISSING)
    assert np.array_equal(t.log_t, O.BURROWS_LOG_T) and np.array_equal(t.log_rho, O.BURROWS_LOG_RHO)


def test_records_may_span_lines_and_hold_null_values(tmp_path):
    """List-directed records: a node's values split over two lines, and a
    null value keeping the value of the record before it."""
    a = _random_table(np.random.default_rng(7), 10)
    p = tmp_path / "t.dat"
    O.write_burrows_table(p, 10, 6070.0, **a)
    lines = open(p).read().splitlines()
    v = lines[11].split()
    lines[11] = " ".join(v[:2])
    lines.insert(12, " ".join(v[2:]) + " 123.0")
    w = lines[13].split()
    lines[13] = ", ".join(w[:3]) + ", , " + w[4]          # node (1, 2): the Rosseland mean is null
    t = O.read_burrows_table(lines, 10)
    assert np.array_equal(t.plnk, a["plnk"])
    assert t.ross[0, 1] == a["ross"][0, 0]
    ross = a["ross"].copy()
    ross[0, 1] = a["ross"][0, 0]
    assert np.array_equal(t.ross, ross)
    with pytest.raises(O.OpacityFileError):
        O.read_burrows_table(lines[:-1], 10)                 # a node short


def test_type_adjustments(tmp_path):
    rng = np.random.default_rng(3)
    a = _random_table(rng, 25)
    gamma, mu = 0.7, 2.3
    p = tmp_path / "t.dat"
    # 12: the absorption mean from the Planck mean and gamma; 14: Rosseland too
    O.write_burrows_table(p, 12, 6000.0, **a)
    t12 = O.read_burrows_table(p, 12, gamma_opc=gamma)
    assert np.array_equal(t12.absk, a["plnk"] + 4.0 * math.log10(gamma))
    assert np.array_equal(t12.ross, a["ross"])
    O.write_burrows_table(p, 14, 6000.0, **a)
    t14 = O.read_burrows_table(p, 14, gamma_opc=gamma)
    assert np.array_equal(t14.ross, a["plnk"]) and np.array_equal(t14.absk, t12.absk)
    # 11: the planet's extra absorber where the gas pressure is <= 0.03 bar
    O.write_burrows_table(p, 11, 6000.0, **a)
    t11 = O.read_burrows_table(p, 11, planet_num=2, mu_gas=mu)
    T = 10.0 ** O.BURROWS_LOG_T[:, None]
    R = 10.0 ** O.BURROWS_LOG_RHO[None, :]
    low = (RGAS * T * R / mu) * 1e-6 <= float(np.float32(0.03))
    assert 0 < low.sum() < low.size
    kext = float(np.float32(0.035))
    np.testing.assert_allclose(t11.absk[low], np.log10(10.0 ** a["absk"][low] + kext), rtol=0, atol=1e-14)
    assert np.array_equal(t11.absk[~low], a["absk"][~low])
    # 24: the extra absorber in the stellar bins only; 25: in the local bins too
    O.write_burrows_table(p, 24, 6070.0, **a)
    t24 = O.read_burrows_table(p, 24, planet_num=1)
    kext = float(np.float32(0.1))
    np.testing.assert_allclose(t24.waveopac, np.log10(10.0 ** a["waveopac"] + kext), rtol=0, atol=1e-14)
    assert np.array_equal(t24.localwave, a["localwave"]) and np.array_equal(t24.absk, a["absk"])
    O.write_burrows_table(p, 25, 5040.0, **a)
    t25 = O.read_burrows_table(p, 25, planet_num=2)
    kext = float(np.float32(0.035))
    np.testing.assert_allclose(t25.localwave, np.log10(10.0 ** a["localwave"] + kext), rtol=0, atol=1e-14)
    assert np.array_equal(t25.local_bb, a["local_bb"])
    # SETPLANETKAPEXTRA stops for planets without a value
    with pytest.raises(O.OpacityFileError):
        O.read_burrows_table(p, 25, planet_num=6)


def test_file_selection():
    assert O.burrows_file_name(1, 21) == "BURROWS6070_woTiVO_wavelth.dat"
    assert O.burrows_file_name(1, 24) == "BURROWS6070_woTiVO_radtransfer.dat"
    assert O.burrows_file_name(1, 10) == "BURROWS6117_woutTiVO.dat"
    assert O.burrows_file_name(1, 20) == "BURROWS6070_wTiVO_wavelth.dat"
    assert O.burrows_file_name(1, 9) == "BURROWS6117_wTiVO.dat"
    assert O.burrows_file_name(2, 25) == "BURROWS5040_Ray_woTiVO_radtransfer.dat"
    assert O.burrows_file_name(2, 9) == "BURROWS5040_wTiVO.dat"
    assert O.burrows_file_name(3, 21) == "BURROWS5226_woutTiVO.dat"
    assert O.burrows_file_name(5, 23) == "BURROWS6300_woTiVO_radtransfer.dat"
    assert O.burrows_file_name(8, 10) == "BURROWS6350_woutTiVO.dat"
    for planet, kt in ((1, 22), (1, 13), (3, 9), (5, 10), (9, 10), (9, 20)):
        with pytest.raises(O.OpacityFileError):
            O.burrows_file_name(planet, kt)
    assert O.bstar_file_name(2) == "BSTAR_WAVEBINS_TS5040.dat"
    with pytest.raises(O.OpacityFileError):
        O.bstar_file_name(3)
    assert O.planet_kap_extra(1) == float(np.float32(0.1))


def _write_bins(path, n, tstar=5040.0):
    with open(path, "w") as fh:
        fh.write("bins\nof the star\nin the wavelength bins\n")
        fh.write(f"{tstar}\n{n}\n")
        for i in range(n):
            fh.write(f"{1.0 + i} {float(i) * 0.5 + 0.25!r}\n")


def test_bstar_bins(tmp_path):
    p = tmp_path / "b.dat"
    _write_bins(p, O.WAVE_BINS)
    tstar, bins = O.read_bstar_bins(p)
    assert tstar == 5040.0 and np.array_equal(bins, np.arange(O.WAVE_BINS) * 0.5 + 0.25)
    _write_bins(p, O.WAVE_BINS - 1)
    with pytest.raises(O.OpacityFileError):
        O.read_bstar_bins(p)


def test_table_file_drives_kappa(tmp_path):
    """The analytic opacity written as an IKAPTYP 21 file on the reference's
    nodes, read back, set into the oracle's BurrowsOPC: KAPPA reproduces the
    analytic model inside the table's range; FLD.set_burrows_table passes the
    same arrays."""
    sh = make_shell(20, 16, 8, seed=2, delt=100.0)
    o = oracle_from_shell(sh, start=False)
    o.f("KMUL")[...] = 1.0
    o.set("iii", 0)
    assert o.call("bounds") == 0 and o.call("kappa") == 0
    ref = {n: o.f(n).copy() for n in ("XKAPR", "XKAPP", "XKAPA")}
    lt, lr = O.BURROWS_LOG_T, O.BURROWS_LOG_RHO
    k = math.log10(1e-2) + 0.5 * lr[None, :] + 1.5 * (lt[:, None] - 3.0)
    wave = np.zeros(k.shape + (O.WAVE_BINS,))
    O.write_burrows_table(tmp_path / O.burrows_file_name(1, 21), 21, 6070.0, k, k, k, waveopac=wave)
    _write_bins(tmp_path / O.bstar_file_name(1), O.WAVE_BINS, 6070.0)
    t = O.read_opacity_tables(tmp_path, 1, 21)
    assert t.bin_tstar == 6070.0 and t.bstar_bin.size == O.WAVE_BINS
    keep = [np.ascontiguousarray(t.log_t), np.ascontiguousarray(t.log_rho)]
    keep += [np.asfortranarray(x) for x in (t.ross, t.plnk, t.absk)]
    lib = __import__("oracle")._load()
    assert lib.ttor_set_opacity_table(o.h, O.NODES, O.NODES, *[x.ctypes.data for x in keep]) == 0
    assert o.call("kappa") == 0
    lrho, ltem = np.log10(o.f("RH")), np.log10(o.f("T"))
    inside = (lrho < -1.99994) & (lrho > -11.9995) & (ltem > 1.69897) & (ltem < 3.69888)
    assert inside.sum() > 0.5 * inside.size
    for n, x in ref.items():
        assert rel_l2(o.f(n)[inside], x[inside]) <= 1e-12, n

    class Stand:                              # FLD without a device
        def set_opacity_table(self, *arrays):
            self.arrays = arrays
    from ttcode_gb300.fld import FLD
    s = Stand()
    FLD.set_burrows_table(s, t)
    assert [x is y for x, y in zip(s.arrays, (t.log_t, t.log_rho, t.ross, t.plnk, t.absk))] == [True] * 5
    t.ikaptyp = 10
    with pytest.raises(ValueError):
        FLD.set_burrows_table(s, t)


def test_host_burrows_opc_equals_the_oracle():
    """opacity.burrows_opc, the host restatement, gives the oracle's KAPPA
    output bit for bit at every cell KAPPA interpolates (i < UPPERBND),
    ghosts outside the table's range (clamped) included; its stops raise."""
    sh = make_shell(20, 16, 8, seed=4, delt=100.0)
    o = oracle_from_shell(sh, start=False)
    lt, lr = O.BURROWS_LOG_T, O.BURROWS_LOG_RHO
    rng = np.random.default_rng(8)
    base = math.log10(1e-2) + 0.5 * lr[None, :] + 1.5 * (lt[:, None] - 3.0)
    a = {n: base + 0.05 * rng.standard_normal(base.shape) for n in ("plnk", "ross", "absk")}
    t = O.BurrowsTable(21, 6070.0, a["plnk"], a["ross"], a["absk"],
                       rng.uniform(-3, 1, base.shape + (O.WAVE_BINS,)), np.full(base.shape + (O.WAVE_BINS,), -7.0),
                       np.full(base.shape + (O.WAVE_BINS,), -7.0))
    keep = [np.ascontiguousarray(t.log_t), np.ascontiguousarray(t.log_rho)]
    keep += [np.asfortranarray(x) for x in (t.ross, t.plnk, t.absk)]
    lib = __import__("oracle")._load()
    assert lib.ttor_set_opacity_table(o.h, O.NODES, O.NODES, *[x.ctypes.data for x in keep]) == 0
    o.set("iii", 0)
    assert o.call("bounds") == 0 and o.call("kappa") == 0
    T, RH, ub = o.f("T"), o.f("RH"), o.f("UPPERBND")
    nx, ny, nz = sh.dims
    checked = 0
    for k in range(nz + 4):
        for j in range(ny + 4):
            for i in range(0, ub[j, k] + 1):          # i = -1 .. upperbnd(j,k) - 1
                p = O.burrows_opc(t, T[i, j, k], RH[i, j, k])
                got = (p.kap_r, p.kap_p, p.kap_a, p.dkap_p_dt, p.dkap_a_dt)
                want = tuple(o.f(n)[i, j, k] for n in ("XKAPR", "XKAPP", "XKAPA", "DXKAPP_DT", "DXKAPA_DT"))
                assert got == want, (i, j, k, got, want)
                checked += 1
    assert checked == int((ub.astype(np.int64) + 1).sum()) > (nx - 2) * (ny + 4) * (nz + 4)
    p = O.burrows_opc(t, 1500.0, 1e-6)
    assert p.wave.shape == (O.WAVE_BINS,) and np.all(p.wave > 0) and np.all(p.localwave == -7.0)
    with pytest.raises(O.OpacityFileError):
        O.burrows_opc(t, 0.0, 1e-6)


# ---- Freedman (T, P) tables -------------------------------------------------
def _freedman_file(path, logk, skip=()):
    with open(path, "w") as fh:
        for q in range(10):
            fh.write(f"header{q}\n")
        fh.write("6117.0\n")
        n = 0
        for ip in range(O.FREEDMAN_P.size)[::-1]:           # any order: entries are placed by value
            for it in range(O.FREEDMAN_T.size):
                if (it, ip) in skip:
                    continue
                row = (O.FREEDMAN_T[it], O.FREEDMAN_P[ip], logk[0][it, ip], logk[1][it, ip], logk[2][it, ip])
                fh.write(" ".join(repr(float(v)) for v in row) + "\n")
                n += 1
    return n


def test_freedman_table_reader(tmp_path):
    rng = np.random.default_rng(5)
    shape = (O.FREEDMAN_T.size, O.FREEDMAN_P.size)
    logk = [rng.uniform(-4, 1, shape) for _ in range(3)]
    skip = {(q, q % 18) for q in range(20)}
    p = tmp_path / O.freedman_file_name(5)
    n = _freedman_file(p, logk, skip)
    assert n == O.FREEDMAN_ENTRIES
    t = O.read_freedman_table(p, 5)
    assert t.t_absorption == 6117.0
    for got, want in zip((t.plnk, t.ross, t.absk), logk):
        mask = np.ones(shape, bool)
        for s in skip:
            mask[s] = False
        assert np.array_equal(got[mask], want[mask]) and np.all(got[~mask] == O.MISSING)
    lines = open(p).read().splitlines()
    lines[11] = "76.0 " + " ".join(lines[11].split()[1:])       # a T that is no node
    with pytest.raises(O.OpacityFileError):
        O.read_freedman_table(lines, 5)
    with pytest.raises(O.OpacityFileError):
        O.read_freedman_table(p, 9)
    assert O.freedman_file_name(4) == "Freedman6117.dat"


def test_freedman_interpolation_and_kappa_branch():
    """FreedmanOPC is bilinear in T and P: a table linear in both is
    reproduced to rounding; the clamps, the derivative stand-ins, the stops;
    KAPPA's 4:5 branch on a shell (ideal-gas pressure, values above
    UPPERBND from UPPERBND)."""
    T_, P_ = np.meshgrid(O.FREEDMAN_T, O.FREEDMAN_P, indexing="ij")
    lin = -2.0 + 3e-4 * T_ + 2e-6 * P_
    t = O.FreedmanTable(4, 6117.0, lin + 0.1, lin, lin - 0.2)
    for tq, pq in ((320.0, 4.5e3), (1234.5, 2.0e5), (3999.0, 2.9e5)):
        kp, kr, ka, dkp, dka = O.freedman_opc(t, tq, pq * 1000.0)
        assert abs(math.log10(kr) - (-2.0 + 3e-4 * tq + 2e-6 * pq)) < 1e-12
        assert abs(math.log10(kp) - math.log10(kr) - 0.1) < 1e-12
    # clamps (pprphy.f:830-833): below 75 K as 75.001 K, above 3e5 mbar as 299999.9 mbar
    assert O.freedman_opc(t, 50.0, 1e6) == O.freedman_opc(t, 75.001, 1e6)
    assert O.freedman_opc(t, 500.0, 1e12) == O.freedman_opc(t, 500.0, 299999.9 * 1000.0)
    kp, kr, ka, dkp, dka = O.freedman_opc(t, 450.0, 5e4)       # T nodes 400, 500; P node above 50 mbar: 100
    it, it1, iw = 20, 19, 10
    assert dkp == (10.0 ** t.plnk[it, iw] - 10.0 ** t.plnk[it1, iw]) / (O.FREEDMAN_T[it] - O.FREEDMAN_T[it1])
    with pytest.raises(O.OpacityFileError):
        O.freedman_opc(t, -1.0, 1e6)

    sh = make_shell(10, 8, 6, seed=1, delt=100.0)
    T, RH = sh.fields["T"], sh.fields["RH"]
    ub = np.full((8 + 4, 6 + 4), 9, dtype=np.int32)
    ub[3, 4] = 6
    out = O.freedman_kappa(t, T, RH, ub, 2.3)
    from ttcode_gb300.synthetic import RGAS
    for (q, j, k) in ((0, 0, 0), (5, 3, 4), (7, 3, 4), (10, 2, 2)):
        got = np.array([out[n][q, j, k] for n in ("XKAPP", "XKAPR", "XKAPA", "DXKAPP_DT", "DXKAPA_DT")])
        want = np.array(O.freedman_opc(t, T[q, j, k], RGAS * T[q, j, k] * RH[q, j, k] / 2.3))
        np.testing.assert_allclose(got, want, rtol=1e-14, atol=0, err_msg=str((q, j, k)))
    assert np.all(out["XKAPR"][8:, 3, 4] == out["XKAPR"][7, 3, 4])     # above i = UPPERBND = 6
    assert abs(out["XKAPR"][8, 3, 4] / O.freedman_opc(t, T[8, 3, 4], RGAS * T[8, 3, 4] * RH[8, 3, 4] / 2.3)[1]
               - 1.0) > 1e-6
    assert np.all(out["XKAPR"][11:, 2, 2] == out["XKAPR"][10, 2, 2])   # above i = 9
    # every cell against the scalar restatement (numpy's power: last-bit differences)
    for j in range(12):
        for k in range(10):
            top = min(int(ub[j, k]) + 1, 13)
            for q in range(14):
                c = min(q, top)
                want = O.freedman_opc(t, T[c, j, k], RGAS * T[c, j, k] * RH[c, j, k] / 2.3)
                got = [out[n][q, j, k] for n in ("XKAPP", "XKAPR", "XKAPA", "DXKAPP_DT", "DXKAPA_DT")]
                np.testing.assert_allclose(got, want, rtol=1e-14, atol=0)


@pytest.mark.gpu
def test_table_file_reaches_the_device(tmp_path):
    """A Burrows table file read on the host and handed over by
    start_run(opacity_table=...), the path a run directory takes: the
    device's BOUNDS and KAPPA equal the oracle's on the same table."""
    from ttcode_gb300.fld import start_run
    sh = make_shell(24, 32, 16, seed=6, delt=100.0)
    lt, lr = O.BURROWS_LOG_T, O.BURROWS_LOG_RHO
    k = math.log10(1e-2) + 0.5 * lr[None, :] + 1.5 * (lt[:, None] - 3.0)
    O.write_burrows_table(tmp_path / O.burrows_file_name(1, 21), 21, 6070.0, k + 0.01, k, k - 0.02,
                          waveopac=np.zeros(k.shape + (O.WAVE_BINS,)))
    _write_bins(tmp_path / O.bstar_file_name(1), O.WAVE_BINS, 6070.0)
    t = O.read_opacity_tables(tmp_path, 1, 21)
    o = oracle_from_shell(sh, start=False)
    keep = [np.ascontiguousarray(t.log_t), np.ascontiguousarray(t.log_rho)]
    keep += [np.asfortranarray(x) for x in (t.ross, t.plnk, t.absk)]
    assert __import__("oracle")._load().ttor_set_opacity_table(o.h, O.NODES, O.NODES,
                                                               *[x.ctypes.data for x in keep]) == 0
    o.set("iii", 0)
    assert o.call("bounds") == 0 and o.call("kappa") == 0
    sh.params = dict(sh.params, kappa_model=2)
    f = start_run(sh, opacity_table=t)
    for n in ("XKAPR", "XKAPP", "XKAPA", "DXKAPP_DT", "DXKAPA_DT", "T"):
        assert rel_l2(f.download(n), o.f(n)) <= 1e-13, n
    f.close()


def test_burrows_kappa_branch_9_14():
    """KAPPA's IKAPTYP 9:12/14 branch on the host: BurrowsOPC up to
    UPPERBND, the UPPERBND values above it; every cell against the scalar
    restatement (numpy's log10/power: last-bit differences)."""
    lt, lr = O.BURROWS_LOG_T, O.BURROWS_LOG_RHO
    rng = np.random.default_rng(2)
    base = math.log10(1e-2) + 0.5 * lr[None, :] + 1.5 * (lt[:, None] - 3.0)
    rest = np.full(base.shape + (O.WAVE_BINS,), -7.0)
    t = O.BurrowsTable(10, 6117.0, base + 0.05 * rng.standard_normal(base.shape), base.copy(), base - 0.3, rest,
                       rest, rest)
    sh = make_shell(10, 8, 6, seed=1, delt=100.0)
    T, RH = sh.fields["T"], sh.fields["RH"]
    ub = np.full((12, 10), 9, dtype=np.int32)
    ub[5, 5] = 4
    out = O.burrows_kappa(t, T, RH, ub)
    for j in range(12):
        for k in range(10):
            top = min(int(ub[j, k]) + 1, 13)
            for q in range(14):
                c = min(q, top)
                p = O.burrows_opc(t, T[c, j, k], RH[c, j, k])
                want = [p.kap_p, p.kap_r, p.kap_a, p.dkap_p_dt, p.dkap_a_dt]
                got = [out[n][q, j, k] for n in ("XKAPP", "XKAPR", "XKAPA", "DXKAPP_DT", "DXKAPA_DT")]
                np.testing.assert_allclose(got, want, rtol=1e-14, atol=0)
    assert np.all(out["XKAPR"][6:, 5, 5] == out["XKAPR"][5, 5, 5])
    t.ikaptyp = 21
    with pytest.raises(O.OpacityFileError):
        O.burrows_kappa(t, T, RH, ub)


# ---- FreedmanOPC and the binned stellar heating in the oracle --------------
def _oracle_freedman(sh, tab, mu=2.3):
    o = oracle_from_shell(sh, start=False)
    keep = [np.asfortranarray(a) for a in (tab.ross, tab.plnk, tab.absk)]
    assert __import__("oracle")._load().ttor_set_freedman_table(o.h, *[a.ctypes.data for a in keep], mu) == 0
    o.set("iii", 0)
    assert o.call("bounds") == 0 and o.call("kappa") == 0
    o.set("iii", 1)
    return o


def test_oracle_freedman_kappa_matches_host():
    """The oracle's KAPPA IKAPTYP 4:5 branch (C FreedmanOPC, PRESSG's ideal-gas
    pressure) against the host restatement on the same shell and table."""
    sh = make_shell(16, 12, 10, seed=3, delt=100.0)
    tab = O.analytic_freedman_table()
    o = _oracle_freedman(sh, tab)
    want = O.freedman_kappa(tab, o.f("T"), o.f("RH"), o.f("UPPERBND"), 2.3)
    for n in ("XKAPR", "XKAPP", "XKAPA", "DXKAPP_DT", "DXKAPA_DT"):
        assert rel_l2(o.f(n), want[n]) <= 1e-14, n


def _oracle_table(sh, f_incident, bins=None, bstar=None, rstar=1.0, semi=7.0e11):
    """The oracle on a kappa_model 2 table of the analytic model, with an
    optional per-bin part (log opacities (nt, nrh, nb) and BSTAR)."""
    from ttcode_gb300.synthetic import analytic_opacity_table
    lt, lr, kr, kp, ka = analytic_opacity_table(1e-2)
    L = __import__("oracle")._load()
    o = oracle_from_shell(sh, start=False)
    o.set("f_incident", f_incident)
    keep = [np.ascontiguousarray(lt), np.ascontiguousarray(lr)] + [np.asfortranarray(a) for a in (kr, kp, ka)]
    assert L.ttor_set_opacity_table(o.h, lt.size, lr.size, *[a.ctypes.data for a in keep]) == 0
    if bins is not None:
        w = np.asfortranarray(bins)
        b = np.ascontiguousarray(bstar, dtype=np.float64)
        assert L.ttor_set_wave_table(o.h, b.size, w.ctypes.data, b.ctypes.data, rstar, semi) == 0
    o.set("iii", 0)
    assert o.call("bounds") == 0 and o.call("kappa") == 0
    o.set("iii", 1)
    assert o.call("stellarinput_heating") == 0
    return o, ka


def test_binned_heating_reduces_to_grey():
    """With one bin whose opacity is the absorption mean, constant incident
    temperature and mu = 1 (F_INCIDENT 4), the binned STELLARINPUT is the
    grey one times BSTAR (RSTAR RSOL / semi)^2 / (SBCONST T_irr^4); three
    bins of that opacity add their BSTAR (linearity in the bins)."""
    sh = make_shell(20, 12, 10, seed=4, delt=100.0)
    from ttcode_gb300.synthetic import mu_star_tincident
    mu, tinc = mu_star_tincident(sh.grid, sh.params["tirr"], 4)
    sh.fields["MU_STAR"], sh.fields["TINCIDENT"] = mu, tinc
    og, ka = _oracle_table(sh, 4)
    grey = og.f("STELLARINPUT")[2:22].copy()
    rstar, semi, b = 1.155, 6.8e11, 3.0e9
    ob, _ = _oracle_table(sh, 4, ka[:, :, None], [b], rstar, semi)
    f = rstar * float(np.float32(6.9598e10)) / semi
    ratio = b * (f * f) / (float(np.float32(5.6705e-5)) * sh.params["tirr"] ** 4)
    assert rel_l2(ob.f("STELLARINPUT")[2:22], grey * ratio) <= 1e-14
    o3, _ = _oracle_table(sh, 4, np.repeat(ka[:, :, None], 3, axis=2), [b, 2 * b, 0.5 * b], rstar, semi)
    assert rel_l2(o3.f("STELLARINPUT")[2:22], 3.5 * ob.f("STELLARINPUT")[2:22]) <= 1e-14
