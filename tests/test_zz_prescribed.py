"""Prescribed opacities (kappa_model 1), through the C ABI: KAPPA is the
caller's, so the context takes XKAPR/XKAPP/XKAPA and their T-derivatives as
uploaded (the path of the host-side FreedmanOPC and of KAPPA's IKAPTYP 9:12
and 14 branches).  Uploading the oracle's own opacities after its BOUNDS
and KAPPA (which are idempotent there: a second BOUNDS + KAPPA returns the
same bits) must give the oracle's implicit step, since the reference
evaluates KAPPA only at a step's start and in its first outer iteration, on
the same T.  Collected at the end, after the tests of the other paths.
"""
import numpy as np
import pytest

from conftest import oracle_from_shell, rel_l2

pytestmark = pytest.mark.gpu

OPAC = ("XKAPR", "XKAPP", "XKAPA", "DXKAPP_DT", "DXKAPA_DT")


def test_prescribed_opacities_step_matches_oracle():
    from ttcode_gb300.fld import FLD
    from ttcode_gb300.synthetic import make_shell
    sh = make_shell(40, 64, 32, seed=3, delt=100.0)
    o = oracle_from_shell(sh, eps=1e-12)
    assert o.call("bounds") == 0 and o.call("kappa") == 0
    p = dict(sh.params, kappa_model=1, epsmat=1e-10, itmax=200000)
    f = FLD(sh.grid, p)
    f.load_shell(sh)
    for n in ("T", "RH", "UPPERBND") + OPAC:
        f.upload(n, o.f(n))
    f.kappa()                                         # no-op: the uploaded opacities stay
    for n in OPAC:
        assert np.array_equal(f.download(n), o.f(n)), n
    f.set_solver("mixed", tol=1e-10)
    assert o.call("coupled_energy_eqs", 1) == 0
    st = f.coupled_energy_eqs(True)
    assert st.energy_iter == int(o.get("energy_iter"))
    for n in ("ER", "T"):
        assert rel_l2(f.download(n), o.f(n)) <= 1e-9, n
    f.close()
