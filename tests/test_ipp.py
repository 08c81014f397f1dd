"""The ipp reader (ttcode_gb300.ipp) against readinitfile (ppmod.f:42-78), the
parameters and grid a run takes from it, and a run directory (ipp + AKTTD)
driving the oracle's step."""
import numpy as np
import pytest

from conftest import oracle_from_shell
from ttcode_gb300 import akttd as A
from ttcode_gb300.ipp import (IppError, bottom_gradients, grid_of_ipp, initial_bottom, misc_checks,
                              open_run_directory, params_of_ipp, read_ipp)
from ttcode_gb300.grid import RJUP, gitter
from ttcode_gb300.synthetic import default_params, make_shell

# the benchmark run's settings, one line per READ(15,*), with trailing notes
# (a list-directed read ignores the rest of a record once its items are read)
SHIPPED = """\
1000000 10001 0.98 1.d12      run length, restart flag, CFL factor, max dt
1000, 0                       print interval, first file
0 0 0                         ietot isoth isoden
1 1 1 1 3 0 0 0               IADV IFOR IGRAV IVIS IRAD INUC ISCAL IDIF
1 1.e-11                      IRHO RHMIN
0 1.e+4 1.e1                  ITEMP TEMPMAX TEMPMIN
0 6.e5 0.0 100000             IVEL VELMAX VELDAMP DAMP_STEPS
1 1.e9 1 1.0e-4 4 1 0.0       IVISTYP XNUE IDISS ALPHA IETA IARTVIS PR_NUM
1 1.4 2.3 0 0.04              IGASTYP GAMMA MU_GAS ICSTYP ASPECT
21 0 1.0 0.1                  IKAPTYP ISIGTYP ZKAPMULT GAMMA_OPC
1 3.52 0.0 0.0 1.0e+0         IROTATE PROT RAMP_START RAMP_FULL WINDAMP
9 2 2 9 15844.230             IBDRAD IFLIMTYP F_INCIDENT BCXMIN FBOT
1.71 500 1.0e-7               SORPARAM ITMAX EPSMAT
----- switches -----
0 0 100                       iperturb perturb_typ perturb_iter
3.52 0.0 0.0                  Porb ecc ecc_start
0 3000 2000.0                 iFbotramp Framp_steps Fbot_final
-1 -1.0 -1.0 -1.0             scratch
----- model -----
2 1                           NCOSYS inc_poles
2 3 1                         MODTYP MODVER PLANET_NUM
0. 1.155 6070.0 1.119 2048.0 0.   STARTYP RSTAR TSTAR MSTAR1 TIRR RH0
0.e0 0.000654 0.0 1.0 1.0     RSTAR2 MSTAR2 RP PHIP PSOFT
3                             NUMDIM
200 8.50e9 1.03e10 0.0        NX XMIN XMAX DXMIN
160 0.00e0 1.0 0.0            NY YMIN YMAX DYMIN
64 -0.95 0.95 0.0             NZ ZMIN ZMAX DZMIN
"""


def _ipp(**repl):
    lines = SHIPPED.splitlines()
    for q, text in repl.items():
        lines[int(q[1:])] = text
    return lines


def test_reads_the_record_layout():
    d = read_ipp(SHIPPED.splitlines())
    assert (d["istepmax"], d["irea"], d["fdelt"], d["dtmax"]) == (1000000, 10001, 0.98, 1e12)
    assert d["irad"] == 3 and d["ieta"] == 4 and d["pr_num"] == 0.0 and d["xnue"] == 1e9
    assert (d["ikaptyp"], d["isigtyp"], d["gamma_opc"]) == (21, 0, 0.1)
    assert (d["ibdrad"], d["iflimtyp"], d["f_incident"], d["bcxmin"], d["fbot"]) == (9, 2, 2, 9, 15844.23)
    assert (d["sorparam"], d["itmax"], d["epsmat"]) == (1.71, 500, 1e-7)      # doubles, exact decimals
    assert (d["int_tmp1"], d["dbl_tmp3"], d["dbl_tmp1"]) == (-1, -1.0, -1.0)
    assert (d["ncosys"], d["inc_poles"], d["poles"]) == (2, 1, True)
    assert (d["modtyp"], d["modver"], d["planet_num"], d["tirr"]) == (2, 3, 1, 2048.0)
    assert (d["global_nx"], d["xmin"], d["xmax"]) == (200, 8.5e9, 1.03e10)
    assert (d["global_ny"], d["global_nz"], d["zmin"], d["zmax"]) == (160, 64, -0.95, 0.95)
    assert d["nparticles"] == 3
    assert isinstance(d["itmax"], int) and isinstance(d["sorparam"], float)


def test_null_values_and_bad_items():
    d = read_ipp(_ipp(l12="1.71,,1.0e-7"))
    assert d["itmax"] is None
    with pytest.raises(IppError):
        params_of_ipp(d, 100.0, poles_off=True)
    with pytest.raises(IppError):
        read_ipp(_ipp(l12="1.71 5.e2 1.0e-7"))           # a real where an INTEGER is read
    with pytest.raises(IppError):
        read_ipp(SHIPPED.splitlines()[:-1])              # a record short


def test_params_and_grid():
    d = read_ipp(SHIPPED.splitlines())
    assert params_of_ipp(d, 100.0)["poles"] == 1         # inc_poles = 1
    p = params_of_ipp(d, 250.0, poles_off=True)
    assert p["poles"] == 0
    assert (p["delt"], p["sorparam"], p["epsmat"], p["itmax"], p["fbottom"]) == (250.0, 1.71, 1e-7, 500, 15844.23)
    assert p["adjust_sor"] == 1 and p["kappa_model"] == 2      # IRAD = 3; IKAPTYP 21: the Burrows table
    d3 = read_ipp(_ipp(l9="3 0 1.0 0.1"))
    with pytest.raises(IppError):
        params_of_ipp(d3, 100.0, poles_off=True)
    assert params_of_ipp(d3, 100.0, poles_off=True, kappa_model=0)["kappa_model"] == 0
    assert params_of_ipp(read_ipp(_ipp(l9="5 0 1.0 0.1")), 100.0, poles_off=True)["kappa_model"] == 1
    with pytest.raises(IppError):
        params_of_ipp(d, 100.0, poles_off=True, omega=1.7)
    g = grid_of_ipp(d)
    ref = gitter(200, 160, 64, 8.5e9, 1.03e10, 0.0, 1.0, -0.95, 0.95)
    for n in ref.m:
        assert np.array_equal(g.m[n], ref.m[n]), n
    with pytest.raises(IppError):
        grid_of_ipp(read_ipp(_ipp(l24="200 8.50e9 1.03e10 0.1")))
    with pytest.raises(IppError):
        grid_of_ipp(read_ipp(_ipp(l19="1 0")))


def test_misc_checks():
    """MISC_CHECKS (ppsub.f:863-880), run by params_of_ipp."""
    misc_checks(read_ipp(SHIPPED.splitlines()))
    for repl in ({"l2": "1 0 0"}, {"l9": "16 0 1.0 0.1", "l20": "1 3 1"}, {"l11": "10 2 2 9 15844.230"},
                 {"l11": "10 2 2 9 15844.230", "l9": "20 0 1.0 0.1"}):
        with pytest.raises(IppError):
            params_of_ipp(read_ipp(_ipp(**repl)), 100.0, poles_off=True, kappa_model=0)
    misc_checks(read_ipp(_ipp(l9="16 0 1.0 0.1")))              # Eliza's tables with MODTYP 2


def test_synthetic_defaults_are_the_shipped_run():
    """default_params is the shipped run with the benchmark's settings: omega
    1.7 fixed, tolerance 1e-10, ITMAX raised, the analytic opacity, and
    PR_NUM 1 (read only with IETA = 5)."""
    d = read_ipp(SHIPPED.splitlines())
    p = params_of_ipp(d, 100.0, poles_off=True, sorparam=1.7, epsmat=1e-10, itmax=200000, adjust_sor=0,
                      kappa_model=0, pr_num=1.0)
    assert p == default_params(100.0)


def test_run_directory_drives_the_step(tmp_path):
    """ipp + AKTTD of a small run: the grid from the ipp, the state from the
    restart file; the oracle's step from them equals the step from the
    state itself, bit for bit."""
    ipp = _ipp(l19="2 0", l24=f"16 {RJUP!r} {1.1 * RJUP!r} 0.0", l25="24 0.0 1.0 0.0", l26="12 -0.95 0.95 0.0")
    (tmp_path / "ipp").write_text("\n".join(ipp) + "\n")
    s0 = make_shell(16, 24, 12, seed=5, delt=100.0)
    s0.fields["KMUL"][...] = 1.0
    rh = s0.fields["RH"]
    rh[0], rh[1] = rh[2], rh[2]
    A.write_restart(str(tmp_path / "AKTTD"), A.combine([A.snapshot_of(s0, zeit=10.0, num_iter=4)]))

    d = read_ipp(tmp_path / "ipp")
    r = A.read_restart(str(tmp_path / "AKTTD"))
    params = params_of_ipp(d, r.delt, kappa_model=0, adjust_sor=0)
    s1 = A.shell_of_restart(r, grid_of_ipp(d), params)
    assert s1.params["epsmat"] == 1e-7 and s1.params["sorparam"] == 1.71
    s0.params = dict(s1.params)
    o0, o1 = oracle_from_shell(s0, eps=1e-7), oracle_from_shell(s1, eps=1e-7)
    assert o0.call("coupled_energy_eqs", 1) == 0 and o1.call("coupled_energy_eqs", 1) == 0
    assert o0.get("energy_iter") == o1.get("energy_iter")
    for n in ("T", "ER"):
        assert np.array_equal(o0.f(n)[2:-2, 2:-2, 2:-2], o1.f(n)[2:-2, 2:-2, 2:-2]), n


def test_bottom_gradients():
    """LOCALINIT's D_RH and D_T (ppinit.f:149-245): default-REAL expressions
    rounded to single precision, MODVER 4 / planet 1 in double, unset cases
    None; MODVER 3 from the Burrows table, pinned bit for bit to the oracle's
    BOUNDXMIN(9) at III = 0 (the same gradient sets T below the bottom)."""
    from ttcode_gb300 import opacity as O
    f32 = lambda x: float(np.float32(x))
    d = read_ipp(SHIPPED.splitlines())
    mv = lambda m, nx=200, planet=1: dict(d, modver=m, global_nx=nx, planet_num=planet)
    d_rh, d_t = bottom_gradients(mv(0), 0.0, 0.0)
    assert d_t == -float(np.float32(1.3611882) * np.float32(1e-6)) and d_t != -1.3611882e-6
    assert d_rh == -float(np.float32(2.1870361) * np.float32(1e-12))
    assert bottom_gradients(mv(1), 0.0, 0.0)[1] == f32(-0.00097568917)
    assert bottom_gradients(mv(4, 100, 1), 0.0, 0.0) == (-(f32(2.1976300) * 1e-10), -(f32(5.0305445) * 1e-6))
    assert bottom_gradients(mv(4, 200, 1), 0.0, 0.0) == (None, None)
    assert bottom_gradients(mv(5, 60), 0.0, 0.0)[1] == -float(np.float32(6.2500764) * np.float32(1e-6))
    assert bottom_gradients(mv(6), 0.0, 0.0) == (None, None)
    with pytest.raises(IppError):
        bottom_gradients(mv(4, 100, 3), 0.0, 0.0)
    with pytest.raises(IppError):
        bottom_gradients(mv(3), 2000.0, 1e-3)                  # no table

    sh = make_shell(12, 16, 8, seed=2, delt=100.0)
    o = oracle_from_shell(sh, start=False)
    lt, lr = O.BURROWS_LOG_T, O.BURROWS_LOG_RHO
    k = np.log10(1e-2) + 0.5 * lr[None, :] + 1.5 * (lt[:, None] - 3.0)
    rest = np.full(k.shape + (O.WAVE_BINS,), -7.0)
    t = O.BurrowsTable(21, 6070.0, k.copy(), k + 0.01, k - 0.02, rest, rest, rest)
    keep = [np.ascontiguousarray(lt), np.ascontiguousarray(lr)] + [np.asfortranarray(x) for x in (t.ross, t.plnk, t.absk)]
    assert __import__("oracle")._load().ttor_set_opacity_table(o.h, 50, 50, *[x.ctypes.data for x in keep]) == 0
    o.set("iii", 0)
    assert o.call("bounds") == 0
    T, RH = o.f("T"), o.f("RH")
    tb, rb = initial_bottom(dict(d, irea=10000), t=T[2:-2, 2:-2, 2:-2], rh=RH[2:-2, 2:-2, 2:-2])
    assert (tb, rb) == (T[2, 2, 2], RH[2, 2, 2])
    d_rh, d_t = bottom_gradients(dict(d, modver=3, fbot=sh.params["fbottom"]), tb, rb, t)
    assert d_rh == 0.0 and d_t < 0.0
    g = sh.grid
    for j in range(16 + 4):
        assert T[1, j, 5] == T[2, j, 5] - d_t * (g.at("xxb", 1) - g.at("xxb", 0))
        assert T[0, j, 5] == T[2, j, 5] - d_t * (g.at("xxb", 1) - g.at("xxb", -1))
    # a restarted run takes them from its AKTTD
    r = A.combine([A.snapshot_of(sh)])
    r.scalars.update(TinitBottom=1234.5, rhinitbottom=6.5e-3)
    assert initial_bottom(dict(d, irea=10001), restart=r) == (1234.5, 6.5e-3)
    with pytest.raises(IppError):
        initial_bottom(dict(d, irea=10001))


def test_open_run_directory(tmp_path):
    """ipp + AKTTD + the Burrows tables of a run directory (IKAPTYP 21):
    the shell, the table, the parameters, as the set-up reads them."""
    from ttcode_gb300 import opacity as O
    ipp = _ipp(l19="2 0", l24=f"16 {RJUP!r} {1.1 * RJUP!r} 0.0", l25="24 0.0 1.0 0.0", l26="12 -0.95 0.95 0.0")
    (tmp_path / "ipp").write_text("\n".join(ipp) + "\n")
    s0 = make_shell(16, 24, 12, seed=5, delt=250.0)
    A.write_restart(str(tmp_path / "AKTTD"), A.combine([A.snapshot_of(s0, zeit=10.0, num_iter=4)]))
    lt, lr = O.BURROWS_LOG_T, O.BURROWS_LOG_RHO
    k = np.log10(1e-2) + 0.5 * lr[None, :] + 1.5 * (lt[:, None] - 3.0)
    O.write_burrows_table(tmp_path / O.burrows_file_name(1, 21), 21, 6070.0, k, k, k,
                          waveopac=np.zeros(k.shape + (O.WAVE_BINS,)))
    with open(tmp_path / O.bstar_file_name(1), "w") as fh:
        fh.write("a\nb\nc\n6070.0\n30\n" + "".join(f"{i} 1.0\n" for i in range(30)))
    sh, table, d, r = open_run_directory(str(tmp_path))
    assert table is not None and table.ikaptyp == 21 and r.num_iter == 4
    assert sh.params["delt"] == 250.0 and sh.params["kappa_model"] == 2 and sh.params["adjust_sor"] == 1
    assert np.array_equal(sh.fields["T"][2:-2, 2:-2, 2:-2], s0.fields["T"][2:-2, 2:-2, 2:-2])
    # the ASCII restart file when there is no binary one; IKAPTYP 3 needs kappa_model
    (tmp_path / "AKTTD").unlink()
    with pytest.raises(FileNotFoundError):
        open_run_directory(str(tmp_path))
    A.write_restart(str(tmp_path / "AKTTD"), A.combine([A.snapshot_of(s0)]))
    ipp3 = list(ipp)
    ipp3[9] = "3 0 1.0 0.1"
    (tmp_path / "ipp").write_text("\n".join(ipp3) + "\n")
    with pytest.raises(IppError):
        open_run_directory(str(tmp_path))
    sh, table, _, _ = open_run_directory(str(tmp_path), kappa_model=0)
    assert table is None and sh.params["kappa_model"] == 0
