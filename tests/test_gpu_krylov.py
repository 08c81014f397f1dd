"""GPU tests of the conjugate-gradient solvers (through the C ABI).

* TTFLD_SOLVER_PCG on SOLVE_WITH_SOR's system: against the exact FP64 SOR
  converged to 1e-12, relative L2 <= 1e-9 and a true FP64 residual
  ||b-Ax||_1/||b||_1 <= 1e-10 (the mixed solver's bars); a full implicit
  step against the oracle's.
* ttfld_solve_with_hypre (SOLVE_WITH_HYPRE, the IRAD=2 path) on the system
  of FILLHYPREMATRIX / FILLHYPREVECTORS: against a sparse direct solve of the
  oracle's restatement of that system.  hypre itself is not available, so
  this pins the system and the solution, not hypre's iterates.
"""
import numpy as np
import pytest
import scipy.sparse.linalg as spla

from conftest import fld_from_shell, oracle_from_shell, rel_l2
from test_oracle import hypre_matrix

pytestmark = pytest.mark.gpu

TOL = 1e-9
EVALS = ("EVAL1", "EVAL2", "EVAL3", "EVAL4", "EVAL5", "EVAL6", "EVAL7", "EVAL8", "EVAL_1_6")


@pytest.fixture(scope="module")
def small():
    from ttcode_gb300.synthetic import make_shell
    return make_shell(40, 64, 32, seed=3, delt=100.0)


def _device_system(sh):
    """A device context holding a step's system: SOR_A..G refilled from the
    EVAL arrays it leaves (as SOLVE_WITH_SOR does at ppsor.f:24-26)."""
    f = fld_from_shell(sh)
    f.set_solver("mixed", tol=1e-10)
    f.coupled_energy_eqs(True)
    f.fill_sor_matrix()
    return f


@pytest.mark.parametrize("dims", [(40, 64, 32), (100, 128, 64)])
def test_pcg_matches_exact_sor(dims):
    from ttcode_gb300.synthetic import make_shell
    sh = make_shell(*dims, seed=5, delt=100.0)
    f = _device_system(sh)
    f.set_params(epsmat=1e-12)
    f.set_solver("sor64_exact")
    ref_st = f.solve_system()
    ref = f.download("DELTA_ER")
    f.set_params(epsmat=1e-10)
    f.set_solver("pcg", tol=1e-10)
    st = f.solve_system()
    x = f.download("DELTA_ER")
    r, b = f.true_residual()
    assert st.status == 0 and r / b <= 1e-10, (st.status, r / b)
    assert rel_l2(x, ref) <= TOL
    # the radial line preconditioner: far fewer iterations than SOR sweeps
    assert 0 < st.sor_iter < ref_st.sor_iter // 3, (st.sor_iter, ref_st.sor_iter)


def test_full_step_pcg_matches_oracle(small):
    o = oracle_from_shell(small, eps=1e-12)
    f = fld_from_shell(small)
    f.set_solver("pcg", guess="previous", tol=1e-10)
    assert o.call("coupled_energy_eqs", 1) == 0
    st = f.coupled_energy_eqs(True)
    assert st.energy_iter == int(o.get("energy_iter"))
    for n in ("ER", "T"):
        assert rel_l2(f.download(n), o.f(n)) <= TOL, n


def test_pcg_rejects_rows_without_weight(small):
    """EVAL8 >= 0 on a coupled row leaves no symmetrising weight: the PCG
    solver refuses the system (status -3) instead of iterating on it."""
    f = _device_system(small)
    e8 = f.download("EVAL8")
    e8[5, 5, 5] = 1.0
    f.upload("EVAL8", e8)
    f.set_solver("pcg", tol=1e-10)
    from ttcode_gb300._ffi import TTFLDError
    with pytest.raises(TTFLDError) as e:
        f.solve_system()
    assert e.value.status == -3


def _hypre_case(sh):
    o = oracle_from_shell(sh)
    assert o.call("coupled_energy_eqs", 1) == 0
    assert o.call("fill_hypre_system") == 0
    f = fld_from_shell(sh)
    for n in EVALS + ("RHS_ER",):
        f.upload(n, o.f(n))
    f.upload("UPPERBND", o.f("UPPERBND"))
    x_ref = spla.spsolve(hypre_matrix(o).tocsc(), o.f("HYP_RHS").ravel(order="F"))
    return o, f, x_ref.reshape(sh.dims, order="F")


def test_hypre_solve_against_direct(small):
    o, f, x_ref = _hypre_case(small)
    nx, ny, nz = small.dims
    rhs = f.download("RHS_ER")
    st = f.solve_with_hypre(tol=1e-12, maxit=10000)
    x = f.download("DELTA_ER")[2:nx + 2, 2:ny + 2, 2:nz + 2]
    assert st.status == 0
    assert rel_l2(x, x_ref) <= 1e-8
    assert np.array_equal(f.download("RHS_ER"), rhs)       # b is formed, RHS_ER is not changed
    assert np.max(np.abs(x[0])) <= 1e-9 * np.max(np.abs(x_ref))    # the Dirichlet rows i = 1
    # the reference's settings: tol 1e-6, at most 50 iterations
    st6 = f.solve_with_hypre()
    x6 = f.download("DELTA_ER")[2:nx + 2, 2:ny + 2, 2:nz + 2]
    assert st6.status == 0 and 0 < st6.sor_iter <= 50
    assert rel_l2(x6, x_ref) <= 1e-4


def test_hypre_iteration_limit_reports_status(small):
    """One iteration cannot reach 1e-14 however strong the preconditioner:
    the sweep count is raised to its limit (32), and the last attempt ends at
    the iteration limit with status 1."""
    o, f, x_ref = _hypre_case(small)
    st = f.solve_with_hypre(tol=1e-14, maxit=1)
    assert st.status == 1 and st.sor_iter == 1 and st.gs_sweeps == 32


def test_hypre_strengthens_its_preconditioner_to_meet_the_cap():
    """On a 160x256x128 shell (opacity contrast 1e4, dt 300 s) one symmetric
    line Gauss-Seidel sweep per preconditioner application needs more than
    20 PCG iterations for tol 1e-6; with a cap of 20 SOLVE_WITH_HYPRE runs
    the solve again with more sweeps and ends with status 0 within the cap,
    its answer within 1e-4 of the same system's 1e-12 solution, and the
    context keeps the sweep count for its next solve."""
    from ttcode_gb300.fld import start_run
    from ttcode_gb300.synthetic import make_shell
    sh = make_shell(160, 256, 128, seed=1, delt=300.0, contrast=1e4)
    f = start_run(sh)
    f.set_solver("mixed", tol=1e-10)
    f.coupled_energy_eqs(True)                  # leaves the EVAL arrays of a real step
    st_ref = f.solve_with_hypre(tol=1e-12, maxit=5000)
    assert st_ref.status == 0 and st_ref.gs_sweeps == 1
    ref = f.download("DELTA_ER")[2:-2, 2:-2, 2:-2]
    st = f.solve_with_hypre(tol=1e-6, maxit=20)
    assert st.status == 0 and st.sor_iter <= 20 and st.gs_sweeps > 1, (st.status, st.sor_iter, st.gs_sweeps)
    assert rel_l2(f.download("DELTA_ER")[2:-2, 2:-2, 2:-2], ref) <= 1e-4
    st2 = f.solve_with_hypre(tol=1e-6, maxit=20)
    assert st2.status == 0 and st2.gs_sweeps == st.gs_sweeps and st2.sor_iter <= 20
    f.close()
