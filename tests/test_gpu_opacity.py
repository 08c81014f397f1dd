"""GPU against the oracle for the table opacities of KAPPA beyond BurrowsOPC:
FreedmanOPC (the IKAPTYP 4:5 branch, kappa_model 3, pprphy.f:88-110 and
800-942) and the wavelength-binned stellar heating of IKAPTYP 20-24
(pprad.f:433-448, 519-568) with its per-bin opacities (pprphy.f:1138-1151).

Bars: opacities and the heating within 1e-13 / 1e-12 (the device's pow and
exp may differ from libm's in the last bit), a full implicit step within
1e-9 with the oracle's outer-iteration count.
"""
import numpy as np
import pytest

from conftest import oracle_from_shell, rel_l2

pytestmark = pytest.mark.gpu

TOL = 1e-9


def _freedman_pair(sh, tab, mu=2.3):
    import oracle as orc
    from ttcode_gb300.fld import FLD
    o = oracle_from_shell(sh, eps=1e-12, start=False)
    keep = [np.asfortranarray(a) for a in (tab.ross, tab.plnk, tab.absk)]
    assert orc._load().ttor_set_freedman_table(o.h, *[a.ctypes.data for a in keep], mu) == 0
    o.set("iii", 0)
    assert o.call("bounds") == 0 and o.call("kappa") == 0
    o.set("iii", sh.params.get("iii", 1))
    p = dict(sh.params, kappa_model=3, epsmat=1e-10, itmax=200000)
    f = FLD(sh.grid, p)
    f.set_freedman_table(tab.ross, tab.plnk, tab.absk, mu)
    f.load_shell(sh)
    f.set_params(iii=0)
    f.bounds()
    f.kappa()
    f.set_params(iii=sh.params.get("iii", 1))
    return o, f


@pytest.mark.parametrize("poles", [False, True])
def test_freedman_kappa_and_step_match_oracle(poles):
    from ttcode_gb300 import opacity as O
    from ttcode_gb300.synthetic import make_shell
    sh = make_shell(40, 64, 32, seed=8, delt=100.0, poles=poles)
    o, f = _freedman_pair(sh, O.analytic_freedman_table())
    for n in ("XKAPR", "XKAPP", "XKAPA", "DXKAPP_DT", "DXKAPA_DT", "T"):
        assert rel_l2(f.download(n), o.f(n)) <= 1e-13, n
    f.set_solver("mixed", tol=1e-10)
    assert o.call("coupled_energy_eqs", 1) == 0
    st = f.coupled_energy_eqs(True)
    assert st.status == 0 and st.energy_iter == int(o.get("energy_iter"))
    for n in ("ER", "T"):
        assert rel_l2(f.download(n), o.f(n)) <= TOL, n
    f.close()


def _wave_pair(sh, nbins=30, rstar=1.155, semi=6.8e11, seed=2):
    import oracle as orc
    from ttcode_gb300.fld import FLD
    from ttcode_gb300.synthetic import analytic_opacity_table
    lt, lr, kr, kp, ka = analytic_opacity_table(1e-2)
    rng = np.random.default_rng(seed)
    waveopac = np.asfortranarray(ka[:, :, None] + rng.uniform(-1.0, 1.0, nbins)[None, None, :])
    bstar = rng.uniform(0.5, 1.5, nbins) * 7.3e10 / nbins
    L = orc._load()
    o = oracle_from_shell(sh, eps=1e-12, start=False)
    keep = [np.ascontiguousarray(lt), np.ascontiguousarray(lr)] + [np.asfortranarray(a) for a in (kr, kp, ka)]
    assert L.ttor_set_opacity_table(o.h, lt.size, lr.size, *[a.ctypes.data for a in keep]) == 0
    assert L.ttor_set_wave_table(o.h, nbins, waveopac.ctypes.data, bstar.ctypes.data, rstar, semi) == 0
    o.set("iii", 0)
    assert o.call("bounds") == 0 and o.call("kappa") == 0
    o.set("iii", sh.params.get("iii", 1))
    p = dict(sh.params, kappa_model=2, epsmat=1e-10, itmax=200000)
    f = FLD(sh.grid, p)
    f.set_opacity_table(lt, lr, kr, kp, ka)
    f.set_wave_table(waveopac, bstar, rstar, semi)
    f.load_shell(sh)
    f.set_params(iii=0)
    f.bounds()
    f.kappa()
    f.set_params(iii=sh.params.get("iii", 1))
    return o, f


@pytest.mark.parametrize("poles", [False, True])
def test_binned_heating_matches_oracle(poles):
    from ttcode_gb300.synthetic import make_shell
    sh = make_shell(40, 64, 32, seed=9, delt=100.0, poles=poles)
    o, f = _wave_pair(sh)
    assert o.call("stellarinput_heating") == 0
    f.stellarinput_heating()
    nx = sh.dims[0]
    got, want = f.download("STELLARINPUT"), o.f("STELLARINPUT")[2:nx + 2]
    assert np.all(np.isfinite(got)) and np.abs(want).max() > 0
    assert rel_l2(got, want) <= 1e-12
    f.set_solver("mixed", tol=1e-10)
    assert o.call("coupled_energy_eqs", 1) == 0
    st = f.coupled_energy_eqs(True)
    assert st.status == 0 and st.energy_iter == int(o.get("energy_iter"))
    for n in ("ER", "T"):
        assert rel_l2(f.download(n), o.f(n)) <= TOL, n
    # nbins = 0 goes back to the grey heating
    f.set_wave_table(np.zeros((1, 1, 0)), [], 1.0, 1.0)
    f.stellarinput_heating()
    assert not np.allclose(f.download("STELLARINPUT"), got)
    f.close()
