"""GPU parity of ttfld_raddif (RADDIF / DIFFEL / SOLVMAT / RADIATIVEBOUND,
the IRAD=1 path) against the oracle's restatement, through the C ABI.

Bars: the same SOLVMAT iteration count; E_R bitwise where no pow() enters
(IBDRAD = 4, 7: fixed and zero-gradient tops), relative L2 <= 1e-12 where
it does (IBDRAD = 9 reads the stellar heating, whose exp() may differ from
libm in the last bit); T = (E_R/arad)^(1/4) within 1e-15.
"""
import numpy as np
import pytest

from conftest import fld_from_shell, rel_l2
from test_oracle import rad_oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sh():
    from ttcode_gb300.synthetic import make_shell
    return make_shell(24, 16, 12, seed=11, delt=100.0)


@pytest.mark.parametrize("ibdrad,eps,itmax", [(7, 1e-6, 3000), (7, 1e-10, 60), (4, 1e-10, 40), (9, 1e-10, 40)])
def test_raddif_matches_oracle(sh, ibdrad, eps, itmax):
    o = rad_oracle(sh, ibdrad, eps, itmax)
    rc_o = o.call("raddif", 0.0, 0.0, 1, 0)
    f = fld_from_shell(sh, eps=eps, itmax=itmax)
    f.set_params(ibdrad=ibdrad, iii=2)
    f.stellarinput_heating()
    st = f.raddif(0.0, 0.0, 1, 0)
    assert st.status == rc_o
    assert st.sor_iter == int(o.get("sor_iter"))
    er, t = f.download("ER"), f.download("T")
    if ibdrad in (4, 7):
        assert np.array_equal(er, o.f("ER"))
    else:
        assert rel_l2(er, o.f("ER")) <= 1e-12
    assert rel_l2(t, o.f("T")) <= 1e-15 if ibdrad in (4, 7) else rel_l2(t, o.f("T")) <= 1e-12
    assert abs(st.rnorm / st.rhsnorm - o.get("global_rnorm") / o.get("global_rhsnorm")) <= 1e-12 * (
        o.get("global_rnorm") / o.get("global_rhsnorm"))


def test_raddif_rejects_unimplemented_bottom(sh):
    """RADIATIVEBOUND's bottom for MODVER > 5 is not implemented: status -3,
    as the oracle returns."""
    f = fld_from_shell(sh, eps=1e-6, itmax=10)
    f.set_params(ibdrad=9, iii=2)
    from ttcode_gb300._ffi import TTFLDError
    with pytest.raises(TTFLDError) as e:
        f.raddif(0.0, 0.0, 6, 0)
    assert e.value.status == -3
