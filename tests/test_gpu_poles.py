"""GPU against the CPU oracle with inc_poles on one rank.

The partner across each pole is the rank itself (ppshift.f:820-833): every
phi exchange is followed by the pole shifts that mirror planes NZ-1..NZ-3 onto
NZ..NZ+2 and planes 1, 2 onto 0, -1 (NORTH/SOUTH_POLE_SHIFT,
ppshift.f:2217-2453), the theta edges are ordinary rows of the SOR system
(ppsor.f:228-272) and SOLVE_WITH_SOR stops at NZ-1 (ppsor.f:39-43).

Bars as for the shells without poles: bitwise for BOUNDS, KAPPA, the exact
FP64 sweeps and solve, DIFFUSION and RADDIF (where no exp() enters); the
exact step's counts identical and its fields within 1e-9; the FP32/FP64
solver's, the scaled FP64 SOR's and PCG's steps within 1e-9 of the oracle
converged to 1e-12.  SOLVE_WITH_HYPRE, whose pole graph is hypre's,
refuses the context.
"""
import numpy as np
import pytest

from conftest import fld_from_shell, oracle_from_shell, rel_l2

pytestmark = pytest.mark.gpu

TOL = 1e-9


@pytest.fixture(scope="module")
def polar():
    from ttcode_gb300.synthetic import make_shell
    return make_shell(40, 64, 32, seed=11, delt=100.0, poles=True)


def _same_system(f, o):
    for n in ("SOR_A", "SOR_B", "SOR_C", "SOR_D", "SOR_E", "SOR_F", "SOR_G", "RHS_ER"):
        f.upload(n, o.f(n))


def test_poles_bounds_and_kappa_bitwise(polar):
    o = oracle_from_shell(polar)
    f = fld_from_shell(polar)
    for n in ("T", "RH", "XKAPR", "XKAPP", "XKAPA"):
        assert np.array_equal(f.download(n), o.f(n)), n
    f.close()


def test_poles_exact_step(polar):
    o = oracle_from_shell(polar)
    f = fld_from_shell(polar)
    f.set_solver("sor64_exact")
    assert o.call("coupled_energy_eqs", 1) == 0
    st = f.coupled_energy_eqs(True)
    assert st.energy_iter == int(o.get("energy_iter"))
    assert st.sor_total == int(o.get("sor_total"))
    for n in ("ER", "T", "DELTA_ER"):
        assert rel_l2(f.download(n), o.f(n)) <= TOL, n
    f.close()


@pytest.mark.parametrize("nsweeps", [1, 4])
def test_poles_exact_sweeps_and_solve_bitwise(polar, nsweeps):
    o = oracle_from_shell(polar)
    assert o.call("coupled_energy_eqs", 1) == 0
    f = fld_from_shell(polar)
    _same_system(f, o)
    f.upload("DELTA_ER", np.zeros_like(o.f("DELTA_ER")))
    o.f("DELTA_ER")[...] = 0.0
    f.sor_sweeps(nsweeps)
    assert o.call("sor_sweeps", nsweeps) == 0
    assert np.array_equal(f.download("DELTA_ER"), o.f("DELTA_ER"))
    # the whole solve from zero: same sweep count, same bits
    o.f("DELTA_ER")[...] = 0.0
    assert o.call("solve_with_sor", 0, 0) == 0
    f.set_solver("sor64_exact")
    f.begin_step(new_run=True)
    st = f.solve_system()
    assert st.sor_iter == int(o.get("sor_iter"))
    assert np.array_equal(f.download("DELTA_ER"), o.f("DELTA_ER"))
    f.close()


def test_poles_mixed_steps(polar):
    """Five consecutive steps of the FP32/FP64 solver, each from the previous
    solution, against the oracle at 1e-12."""
    o = oracle_from_shell(polar, eps=1e-12)
    f = fld_from_shell(polar)
    f.set_solver("mixed", guess="previous", tol=1e-10)
    for step in (1, 2, 3, 4, 5):
        o.set("iii", step)
        f.set_params(iii=step)
        assert o.call("coupled_energy_eqs", 1) == 0
        st = f.coupled_energy_eqs(True)
        assert st.status == 0
        assert st.energy_iter == int(o.get("energy_iter")), step
        for n in ("ER", "T"):
            assert rel_l2(f.download(n), o.f(n)) <= TOL, (step, n)
    f.close()


def test_poles_diffusion_bitwise(polar):
    """DIFFUSION with poles: every theta row swept, the scalar pole-shifted
    after each colour (ppdif.f:45-135); as in the reference the overwritten
    row NZ keeps the residual above EPSMAT and the loop runs to SORITMAX.
    The same count and the same scalar, bit for bit."""
    o = oracle_from_shell(polar)
    f = fld_from_shell(polar)
    nx, ny, nz = polar.dims
    rng = np.random.default_rng(7)
    o.f("SCALAR")[...] = 1.0 + rng.random((nx + 4, ny + 4, nz + 4))
    assert o.call("planetshift", "SCALAR") == 0      # callers pass an exchanged halo
    o.set("pr_num", 1.0)
    o.set("xnue", 1.0e15)
    f.set_params(pr_num=1.0, xnue=1.0e15)
    f.upload("SCALAR", o.f("SCALAR").copy())
    rc = o.call("diffusion")
    st = f.diffusion()
    assert st.status == rc and st.sor_iter == int(o.get("sor_iter"))
    assert np.array_equal(f.download("SCALAR"), o.f("SCALAR"))
    f.close()


@pytest.mark.parametrize("ibdrad,eps,itmax", [(7, 1e-6, 3000), (4, 1e-10, 60), (9, 1e-10, 40)])
def test_poles_raddif(ibdrad, eps, itmax):
    """RADDIF with poles (SOLVMAT over k = 1..NZ, the pole shifts after every
    PLANETSHIFT(6), RADIATIVEBOUND without its theta copies): the oracle's
    iteration count, E_R bitwise for the tops without exp() (IBDRAD 4, 7),
    within 1e-12 for IBDRAD 9."""
    from test_oracle import rad_oracle
    from ttcode_gb300.synthetic import make_shell
    sh = make_shell(24, 16, 12, seed=11, delt=100.0, poles=True)
    o = rad_oracle(sh, ibdrad, eps, itmax)
    rc_o = o.call("raddif", 0.0, 0.0, 1, 0)
    f = fld_from_shell(sh, eps=eps, itmax=itmax)
    f.set_params(ibdrad=ibdrad, iii=2)
    f.stellarinput_heating()
    st = f.raddif(0.0, 0.0, 1, 0)
    assert st.status == rc_o
    assert st.sor_iter == int(o.get("sor_iter"))
    if ibdrad in (4, 7):
        assert np.array_equal(f.download("ER"), o.f("ER"))
    else:
        assert rel_l2(f.download("ER"), o.f("ER")) <= 1e-12
    assert rel_l2(f.download("T"), o.f("T")) <= 1e-12
    f.close()


def test_poles_fast64_solve_and_step(polar):
    """The scaled FP64 SOR with poles (FMA on Jacobi-scaled coefficients, the
    same iteration as the reference loop): the step's system solved from zero
    takes the oracle's sweep count up to a last-bit tie and meets the
    oracle's 1e-12 solution to 1e-9; a full step matches the oracle's."""
    o = oracle_from_shell(polar)
    assert o.call("coupled_energy_eqs", 1) == 0
    f = fld_from_shell(polar)
    _same_system(f, o)
    o.f("DELTA_ER")[...] = 0.0
    assert o.call("solve_with_sor", 0, 0) == 0
    n64 = int(o.get("sor_iter"))
    o.set("epsmat", 1e-12)
    o.f("DELTA_ER")[...] = 0.0
    assert o.call("solve_with_sor", 0, 0) == 0
    f.set_solver("sor64_fast", tol=1e-10)
    f.begin_step(new_run=True)
    st = f.solve_system()
    assert abs(st.sor_iter - n64) <= 1
    assert rel_l2(f.download("DELTA_ER"), o.f("DELTA_ER")) <= TOL
    f.close()
    o = oracle_from_shell(polar, eps=1e-12)
    f = fld_from_shell(polar)
    f.set_solver("sor64_fast", tol=1e-10)
    assert o.call("coupled_energy_eqs", 1) == 0
    st = f.coupled_energy_eqs(True)
    assert st.energy_iter == int(o.get("energy_iter"))
    for n in ("ER", "T"):
        assert rel_l2(f.download(n), o.f(n)) <= TOL, n
    f.close()


def test_poles_pcg_solve_and_step(polar):
    """PCG on SOLVE_WITH_SOR's system with poles (rows 1 and NZ-1 take their
    mirror coupling into the diagonal, row NZ is decoupled and then
    pole-shifted; the weighted rows stay symmetric): the system from zero,
    solved to 1e-11, meets the oracle's 1e-12 SOR solution to 1e-9, and a
    full step at 1e-10 matches the oracle's with the same outer-iteration
    count."""
    o = oracle_from_shell(polar, eps=1e-12)
    assert o.call("coupled_energy_eqs", 1) == 0
    f = fld_from_shell(polar)
    _same_system(f, o)
    for n in ("EVAL1", "EVAL2", "EVAL3", "EVAL4", "EVAL5", "EVAL6", "EVAL7", "EVAL8", "EVAL_1_6"):
        f.upload(n, o.f(n))           # the symmetrising weight reads EVAL8
    o.f("DELTA_ER")[...] = 0.0
    assert o.call("solve_with_sor", 0, 0) == 0
    f.set_solver("pcg", tol=1e-11)   # the error is ~10x the residual on this system
    f.begin_step(new_run=True)
    st = f.solve_system()
    assert st.status == 0
    r, b = f.true_residual()
    assert r / b <= 1e-11
    assert rel_l2(f.download("DELTA_ER"), o.f("DELTA_ER")) <= TOL
    f.close()
    o = oracle_from_shell(polar, eps=1e-12)
    f = fld_from_shell(polar)
    f.set_solver("pcg", guess="previous", tol=1e-10)
    assert o.call("coupled_energy_eqs", 1) == 0
    st = f.coupled_energy_eqs(True)
    assert st.status == 0 and st.energy_iter == int(o.get("energy_iter"))
    for n in ("ER", "T"):
        assert rel_l2(f.download(n), o.f(n)) <= TOL, n
    f.close()


def test_poles_hypre_refuses(polar):
    """SOLVE_WITH_HYPRE's pole graph (pphypre.f:458-540) goes through
    hypre's neighbour boxes, which are not restated: status -3."""
    from ttcode_gb300._ffi import TTFLDError
    f = fld_from_shell(polar)
    with pytest.raises(TTFLDError) as e:
        f.solve_with_hypre()
    assert e.value.status == -3
    f.close()


def test_poles_run_directory_step(tmp_path):
    """A run directory whose ipp keeps inc_poles = 1 (the shipped value,
    ipp:20) opens without poles_off and starts a context with the pole
    shifts; its exact step is the oracle's."""
    from test_ipp import _ipp
    from ttcode_gb300 import akttd as A
    from ttcode_gb300.fld import start_run
    from ttcode_gb300.grid import RJUP
    from ttcode_gb300.ipp import open_run_directory
    from ttcode_gb300.synthetic import make_shell
    ipp = _ipp(l24=f"24 {RJUP!r} {1.1 * RJUP!r} 0.0", l25="32 0.0 1.0 0.0", l26="16 -0.95 0.95 0.0")
    (tmp_path / "ipp").write_text("\n".join(ipp) + "\n")
    s0 = make_shell(24, 32, 16, seed=5, delt=100.0)
    A.write_restart(str(tmp_path / "AKTTD"), A.combine([A.snapshot_of(s0, zeit=10.0, num_iter=4)]))
    sh, _, d, _ = open_run_directory(str(tmp_path), kappa_model=0, adjust_sor=0)
    assert d["inc_poles"] == 1 and sh.params["poles"] == 1
    o = oracle_from_shell(sh, eps=sh.params["epsmat"], itmax=sh.params["itmax"])
    f = start_run(sh)
    f.set_solver("sor64_exact")
    assert o.call("coupled_energy_eqs", 1) == 0
    st = f.coupled_energy_eqs(True)
    assert st.energy_iter == int(o.get("energy_iter"))
    assert st.sor_total == int(o.get("sor_total"))
    for n in ("ER", "T"):
        assert rel_l2(f.download(n), o.f(n)) <= TOL, n
    f.close()
