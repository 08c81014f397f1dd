"""The CPU oracle against known answers (no GPU).

The reference ships no tests or golden vectors, so the oracle is pinned by:
the reference's own commented-out Laplacian toggle (ppenergy.f:1017-1025)
solved independently by a sparse direct solver; a manufactured solution of
the assembled FLD operator; the volume-weighted symmetry of FILL_EVALUES
(ppenergy.f:999-1002); formulas re-evaluated independently in numpy; the
red-black ordering; and the committed golden fixtures of tests/golden/.
"""
import math
import os

import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from conftest import ROOT, oracle_from_shell, rel_l2


@pytest.fixture(scope="module")
def shell():
    from ttcode_gb300.synthetic import make_shell
    return make_shell(24, 16, 12, seed=11, delt=100.0)


def sor_matrix(o):
    """The 7-point SOR system of the oracle state as a scipy matrix over the
    interior, with the periodic phi wrap of the one-rank PLANETSHIFT."""
    nx, ny, nz = o.nx, o.ny, o.nz
    idx = lambda i, j, k: (i - 1) + nx * ((j - 1) + ny * (k - 1))
    A, B, C, D, E, F, G = (o.f(n) for n in ("SOR_A", "SOR_B", "SOR_C", "SOR_D", "SOR_E", "SOR_F", "SOR_G"))
    rows, cols, vals = [], [], []
    for k in range(1, nz + 1):
        for j in range(1, ny + 1):
            for i in range(1, nx + 1):
                r = idx(i, j, k)
                c0 = (i - 1, j - 1, k - 1)
                ent = [((i, j, k), A[c0]), ((i - 1, j, k), B[c0]), ((i + 1, j, k), C[c0]),
                       ((i, ((j - 2) % ny) + 1, k), D[c0]), ((i, (j % ny) + 1, k), E[c0]),
                       ((i, j, k - 1), F[c0]), ((i, j, k + 1), G[c0])]
                for (ii, jj, kk), v in ent:
                    if 1 <= ii <= nx and 1 <= kk <= nz and v != 0.0:
                        rows.append(r); cols.append(idx(ii, jj, kk)); vals.append(v)
    n = nx * ny * nz
    return sp.csr_matrix((vals, (rows, cols)), shape=(n, n))


def test_laplacian_toggle_known_answer():
    """ppenergy.f:1017-1025 (EVAL1..6=1, EVAL7=6, EVAL8=1, EVAL_1_6=0) makes
    FILL_SOR_MATRIX produce the 6/-1 Laplacian; with b=1 (the hypre test
    vector, pphypre.f:136-137) SOLVE_WITH_SOR must reproduce a sparse direct
    solve of the same system."""
    from oracle import Oracle
    nx, ny, nz = 12, 8, 10
    o = Oracle(nx, ny, nz)
    for n in ("EVAL1", "EVAL2", "EVAL3", "EVAL4", "EVAL5", "EVAL6", "EVAL8"):
        o.f(n)[...] = 1.0
    o.f("EVAL7")[...] = 6.0
    o.f("EVAL_1_6")[...] = 0.0
    o.f("UPPERBND")[...] = nx - 1
    o.f("RHS_ER")[...] = 1.0
    o.set("sorparam", 1.7)
    o.set("epsmat", 1e-14)
    o.set("itmax", 100000)
    assert o.call("fill_sor_matrix") == 0 and o.call("b_vector_boundaries") == 0
    A = o.f("SOR_A")
    assert A[0, 0, 1] == 6.0
    assert np.all(A[:, :, 0] == 1.0) and np.all(A[nx - 2:, :, :] == 1.0)
    assert np.all(o.f("SOR_B")[1:nx - 2, :, 1:nz - 1] == -1.0)
    b = o.f("RHS_ER").ravel(order="F").copy()
    x_ref = spla.spsolve(sor_matrix(o).tocsc(), b)
    assert o.call("solve_with_sor", 0, 0) == 0
    x = o.f("DELTA_ER")[2:nx + 2, 2:ny + 2, 2:nz + 2].ravel(order="F")
    assert np.max(np.abs(x - x_ref)) <= 1e-11 * np.max(np.abs(x_ref))


def test_manufactured_solution_fld_operator(shell):
    """b = A x* for the assembled FLD matrix of a real step; the SOR solve
    returns x* (A is the oracle's own FILL_SOR_MATRIX output)."""
    o = oracle_from_shell(shell, eps=1e-14, itmax=200000)
    assert o.call("coupled_energy_eqs", 1) == 0
    A = sor_matrix(o)
    nx, ny, nz = o.nx, o.ny, o.nz
    rng = np.random.default_rng(5)
    xs = rng.random(nx * ny * nz)
    # identity rows keep x = b; make x* zero there so ghosts stay consistent
    ident = (o.f("SOR_A").ravel(order="F") == 1.0) & (o.f("SOR_B").ravel(order="F") == 0.0)
    xs[ident] = 0.0
    b = A @ xs
    o.f("RHS_ER")[...] = b.reshape((nx, ny, nz), order="F")
    assert o.call("solve_with_sor", 0, 0) == 0
    x = o.f("DELTA_ER")[2:nx + 2, 2:ny + 2, 2:nz + 2].ravel(order="F")
    assert rel_l2(x, xs) < 1e-10


def test_fill_evalues_volume_symmetry(shell):
    """EVAL1(i)*r_i^2*dr_i = EVAL2(i+1)*r_{i+1}^2*dr_{i+1} (ppenergy.f:999-1002)
    and the same for phi (EVAL3/EVAL4) and theta (EVAL5/EVAL6) faces."""
    o = oracle_from_shell(shell)
    o.set("energy_iter", 0)
    assert o.call("calculateflux") == 0
    o.call("fill_evalues", 1.0)
    g = shell.grid
    nx, ny, nz = shell.dims
    i = np.arange(1, nx)
    vol = (g.at("surxb", i) * g.at("dxa", i))[:, None, None]
    vol1 = (g.at("surxb", i + 1) * g.at("dxa", i + 1))[:, None, None]
    l = o.f("EVAL1")[:-1] * vol
    r = o.f("EVAL2")[1:] * vol1
    assert np.max(np.abs(l - r)) <= 1e-14 * np.max(np.abs(l))
    k = np.arange(1, nz)
    vz = (g.at("surzb", k) * g.at("dza", k))[None, None, :]
    vz1 = (g.at("surzb", k + 1) * g.at("dza", k + 1))[None, None, :]
    l = o.f("EVAL5")[:, :, :-1] * vz
    r = o.f("EVAL6")[:, :, 1:] * vz1
    assert np.max(np.abs(l - r)) <= 1e-13 * np.max(np.abs(l))


def test_flim_formula_independent(shell):
    """Levermore-Pomraning lambda = (2+R)/(6+3R+R^2) with R = 2|grad E| /
    (rho_face (kappa_i+kappa_{i-1})/2 (E_i+E_{i-1})) (pprphy.f:422-446),
    recomputed in numpy on the interior x faces."""
    o = oracle_from_shell(shell)
    o.set("energy_iter", 0)
    assert o.call("diff") == 0
    g = shell.grid
    nx, ny, nz = shell.dims
    ER, K, RQ = o.f("ER"), o.f("XKAPR"), o.f("RHQX")
    H = lambda a, i, j, k: a[i + 1, j + 1, k + 1]
    for (i, j, k) in [(3, 4, 5), (10, 1, 2), (nx - 3, ny, nz - 1), (1, 7, 6)]:
        gx = (H(ER, i, j, k) - H(ER, i - 1, j, k)) / g.at("dxb", i)
        gy = (0.5 * (H(ER, i, j + 1, k) - H(ER, i, j - 1, k)) + 0.5 * (H(ER, i - 1, j + 1, k) - H(ER, i - 1, j - 1, k))) / \
             (g.at("geoxga", i) * g.at("geozg", k) * (g.at("xyb", j + 1) - g.at("xyb", j - 1)))
        gz = (0.5 * (H(ER, i, j, k + 1) - H(ER, i, j, k - 1)) + 0.5 * (H(ER, i - 1, j, k + 1) - H(ER, i - 1, j, k - 1))) / \
             (g.at("geoxha", i) * (g.at("xzb", k + 1) - g.at("xzb", k - 1)))
        R = 2 * (math.sqrt(gx * gx + gy * gy + gz * gz) + 1e-50) / (
            H(RQ, i, j, k) * (0.5 * H(K, i, j, k) + 0.5 * H(K, i - 1, j, k)) * (H(ER, i, j, k) + H(ER, i - 1, j, k)))
        lam = (2 + R) / (6 + 3 * R + R * R)
        assert abs(o.f("FLIMX")[i - 1, j - 1, k - 1] - lam) <= 1e-15 * lam
        fd = float(np.float32(2.99792458e10))
        difr = fd * lam / (g.at("dxb", i) * H(RQ, i, j, k) * (0.5 * H(K, i, j, k) + 0.5 * H(K, i - 1, j, k)))
        assert abs(o.f("DIFRX")[i - 1, j - 1, k - 1] - difr) <= 1e-14 * difr


def test_flim_limits():
    """lambda -> 1/3 in the diffusion limit (R -> 0) and -> 1/R when R >> 1."""
    lam = lambda R: (2 + R) / (6 + 3 * R + R * R)
    assert abs(lam(0.0) - 1.0 / 3.0) < 1e-16
    assert abs(lam(1e8) * 1e8 - 1.0) < 1e-7


def test_red_black_order_is_colour_jacobi(shell):
    """Within a colour no cell reads another cell of that colour, so one
    serial red-black sweep equals a vectorised two-colour Jacobi update."""
    o = oracle_from_shell(shell)
    assert o.call("coupled_energy_eqs", 1) == 0
    nx, ny, nz = shell.dims
    A = sor_matrix(o)
    b = o.f("RHS_ER").ravel(order="F").copy()
    diag = o.f("SOR_A").ravel(order="F")
    I, J, K = np.meshgrid(np.arange(1, nx + 1), np.arange(1, ny + 1), np.arange(1, nz + 1), indexing="ij")
    colour = ((I + J + K) % 2).ravel(order="F")
    x = np.zeros(nx * ny * nz)
    w = o.get("sorparam")
    for col in (0, 1):
        r = A @ x - b
        m = colour == col
        x[m] = x[m] - w * r[m] / diag[m]
    o.f("DELTA_ER")[...] = 0.0
    assert o.call("sor_sweeps", 1) == 0
    xo = o.f("DELTA_ER")[2:nx + 2, 2:ny + 2, 2:nz + 2].ravel(order="F")
    assert np.max(np.abs(xo - x)) <= 1e-13 * max(np.max(np.abs(x)), 1e-300)


def test_sweep_count_reproducible(shell):
    a = oracle_from_shell(shell)
    b = oracle_from_shell(shell)
    assert a.call("coupled_energy_eqs", 1) == 0 and b.call("coupled_energy_eqs", 1) == 0
    assert a.get("sor_total") == b.get("sor_total")
    assert np.array_equal(a.f("ER"), b.f("ER"))


def test_itmax_stops_with_status(shell):
    """ITMAX ends the SOR loop after exactly ITMAX sweeps (ppsor.f:161-174)
    and, shared with the outer loop, ends COUPLED_ENERGY_EQS with the
    iteration-limit status (ppenergy.f:750-775)."""
    o = oracle_from_shell(shell, itmax=1)
    rc = o.call("coupled_energy_eqs", 1)
    assert rc == 1 and o.get("sor_total") == 1 and o.get("energy_iter") == 1
    o = oracle_from_shell(shell, itmax=3)
    o.call("coupled_energy_eqs", 1)
    o.f("DELTA_ER")[...] = 0.0
    assert o.call("solve_with_sor", 0, 0) == 1 and o.get("sor_iter") == 3


def test_nonpositive_q_is_clean_stop(shell):
    """A planted mistake (an unstable over-relaxation factor, omega = 2.5, that
    makes the SOR iterate blow up within ITMAX sweeps) drives Q + 0.1 dQ <= 0
    somewhere, and the step returns the CLEAN_STOP status
    (ppenergy.f:411-521)."""
    o = oracle_from_shell(shell, itmax=60)
    o.set("sorparam", 2.5)
    rc = o.call("coupled_energy_eqs", 1)
    assert rc == -7


def test_nan_rhs_stops_after_one_sweep():
    """A NaN in the right-hand side makes RNORM/RHSNORM NaN; the reference's
    test `ratio > EPSMAT` is then false and the loop exits (ppsor.f:176)."""
    from oracle import Oracle
    o = Oracle(8, 6, 6)
    for n in ("EVAL1", "EVAL2", "EVAL3", "EVAL4", "EVAL5", "EVAL6", "EVAL8"):
        o.f(n)[...] = 1.0
    o.f("EVAL7")[...] = 6.0
    o.f("UPPERBND")[...] = 7
    o.f("RHS_ER")[...] = 1.0
    o.call("fill_sor_matrix")
    o.call("b_vector_boundaries")
    o.f("RHS_ER")[3, 3, 3] = np.nan
    o.call("solve_with_sor", 0, 0)
    assert o.get("sor_iter") == 1


def test_grid_matches_oracle_gitter(shell):
    from oracle import Oracle
    from ttcode_gb300.grid import full_1d
    g = shell.grid
    o = Oracle(*shell.dims)
    o.set("xmin", g.xmin)
    o.set("xmax", g.xmax)
    o.call("gitter")
    for n in g.m:
        a = full_1d(g, n)
        lo = g.lo[n]
        sl = slice(lo + 1, lo + 1 + g.m[n].size)
        assert np.array_equal(a[sl], o.f(n)[:a.size][sl]), n


def test_mustar_tincident_match_oracle(shell):
    from oracle import Oracle
    from ttcode_gb300.grid import full_1d
    o = Oracle(*shell.dims)
    for n in shell.grid.m:
        a = full_1d(shell.grid, n)
        o.f(n)[:a.size] = a
    o.set("tirr", 2048.0)
    o.set("f_incident", 2)
    o.call("calcmustar")
    assert np.array_equal(o.f("MU_STAR"), shell.fields["MU_STAR"])
    assert np.array_equal(o.f("TINCIDENT"), shell.fields["TINCIDENT"])


GOLDEN = os.path.join(ROOT, "tests", "golden")


@pytest.mark.parametrize("name", ["shell_step", "poles_step"])
def test_golden_step_fixture(name):
    """The committed fixtures (made by tests/golden/make_golden.py, with the
    theta boundary rows and with the one-rank pole shifts) reproduce:
    inputs -> one COUPLED_ENERGY_EQS step -> E_R, T and the counts."""
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    from ttcode_gb300.synthetic import make_shell
    sh = make_shell(int(z["nx"]), int(z["ny"]), int(z["nz"]), seed=int(z["seed"]), delt=float(z["delt"]),
                    poles="poles" in z.files)
    o = oracle_from_shell(sh, eps=float(z["eps"]))
    assert o.call("coupled_energy_eqs", 1) == 0
    assert int(o.get("sor_total")) == int(z["sor_total"])
    assert int(o.get("energy_iter")) == int(z["energy_iter"])
    nx, ny, nz = sh.dims
    for n in ("ER", "T"):
        got = o.f(n)[2:nx + 2, 2:ny + 2, 2:nz + 2]
        assert rel_l2(got, z[n]) <= 1e-12, n


def hypre_matrix(o):
    """The oracle's FILLHYPREMATRIX system (HYP_A..HYP_G) as a scipy matrix;
    no entry may reach outside the grid (hypre's grid has no periodicity)."""
    nx, ny, nz = o.nx, o.ny, o.nz
    n = nx * ny * nz
    I, J, K = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    rows, cols, vals = [], [], []
    for name, (di, dj, dk) in zip(("HYP_A", "HYP_B", "HYP_C", "HYP_D", "HYP_E", "HYP_F", "HYP_G"),
                                  ((0, 0, 0), (-1, 0, 0), (1, 0, 0), (0, -1, 0), (0, 1, 0), (0, 0, -1), (0, 0, 1))):
        v = o.f(name)
        ii, jj, kk = I + di, J + dj, K + dk
        inside = (ii >= 0) & (ii < nx) & (jj >= 0) & (jj < ny) & (kk >= 0) & (kk < nz)
        assert np.all(v[~inside] == 0.0), name
        m = inside & (v != 0.0)
        rows.append((I + nx * (J + ny * K))[m]); cols.append((ii + nx * (jj + ny * kk))[m]); vals.append(v[m])
    return sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(n, n))


def test_hypre_system_is_sor_system_with_dirichlet_bottom(shell):
    """FILLHYPREMATRIX / FILLHYPREVECTORS (pphypre.f:115-334) against
    FILL_SOR_MATRIX / B_VECTOR_BOUNDARIES (ppsor.f:189-329) on the same EVAL
    arrays: equal except the i = 1 rows (identity, b = 0), the i-1 coupling
    of the i = 2 rows and the phi couplings that leave hypre's grid (j-1 of
    j = 1, j+1 of j = NY); the system is non-singular."""
    o = oracle_from_shell(shell)
    assert o.call("coupled_energy_eqs", 1) == 0
    assert o.call("fill_sor_matrix") == 0 and o.call("b_vector_boundaries") == 0
    assert o.call("fill_hypre_system") == 0
    nx, ny, nz = o.nx, o.ny, o.nz
    for s, h in zip("ABCDEFG", ("HYP_A", "HYP_B", "HYP_C", "HYP_D", "HYP_E", "HYP_F", "HYP_G")):
        a, b = o.f("SOR_" + s).copy(), o.f(h)
        a[0] = 1.0 if s == "A" else 0.0
        if s == "B":
            a[1] = 0.0
        if s == "D":
            a[:, 0] = 0.0
        if s == "E":
            a[:, ny - 1] = 0.0
        assert np.array_equal(a, b), s
    rhs = o.f("RHS_ER").copy()
    rhs[0] = 0.0
    assert np.array_equal(rhs, o.f("HYP_RHS"))
    A = hypre_matrix(o)
    x = spla.spsolve(A.tocsc(), o.f("HYP_RHS").ravel(order="F"))
    assert np.all(np.isfinite(x)) and np.all(x.reshape((nx, ny, nz), order="F")[0] == 0.0)


def test_weighted_rows_are_symmetric(shell):
    """The symmetrising weight of the PCG solvers: W = V / |EVAL8| with
    V = surxb dxa dya surzb dza makes W_n A_nm = W_m A_mn for every radial
    and theta pair and every phi pair away from the periodic seam (whose two
    face coefficients come from different halo cells)."""
    o = oracle_from_shell(shell)
    assert o.call("coupled_energy_eqs", 1) == 0
    o.call("fill_evalues", 1.0)
    assert o.call("fill_sor_matrix") == 0
    g = shell.grid
    nx, ny, nz = shell.dims
    I, J, K = np.meshgrid(np.arange(1, nx + 1), np.arange(1, ny + 1), np.arange(1, nz + 1), indexing="ij")
    V = g.at("surxb", I) * g.at("dxa", I) * g.at("dya", J) * g.at("surzb", K) * g.at("dza", K)
    W = V / np.abs(o.f("EVAL8"))
    S = {c: o.f("SOR_" + c) for c in "ABCDEFG"}
    for fwd, bwd, ax in (("C", "B", 0), ("E", "D", 1), ("G", "F", 2)):
        lhs = (W * S[fwd])
        rhs = np.roll(W * S[bwd], -1, axis=ax)
        sl = [slice(None)] * 3
        sl[ax] = slice(0, -1)           # the pair (n, n+1) inside the grid
        l, r = lhs[tuple(sl)], rhs[tuple(sl)]
        scale = np.max(np.abs(l))
        assert np.max(np.abs(l - r)) <= 1e-12 * scale, fwd


def rad_oracle(sh, ibdrad, eps, itmax):
    """An oracle state for RADDIF: the shell, GITTER's volumes, IBDRAD,
    III = 2 and the stellar heating the IBDRAD = 9 top reads."""
    from ttcode_gb300.grid import volumes
    o = oracle_from_shell(sh, eps=eps, itmax=itmax)
    nx, ny, nz = sh.dims
    vx, vy, vz = volumes(sh.grid)
    o.f("volxb")[2:nx + 2] = vx
    o.f("volyb")[2:ny + 2] = vy
    o.f("volzb")[2:nz + 2] = vz
    o.set("ibdrad", ibdrad)
    o.set("iii", 2)
    assert o.call("stellarinput_heating") == 0
    return o


def test_volumes_match_oracle_gitter(shell):
    """grid.volumes (the VOLXB/VOLYB/VOLZB the RADDIF caller passes) equal
    the oracle's restatement of GITTER (ppinit.f:1346-1375)."""
    from oracle import Oracle
    from ttcode_gb300.grid import volumes
    nx, ny, nz = shell.dims
    o = Oracle(nx, ny, nz)
    g = shell.grid
    for k, v in (("xmin", g.xmin), ("xmax", g.xmax)):
        o.set(k, v)
    assert o.call("gitter") == 0
    vx, vy, vz = volumes(g)
    assert np.array_equal(o.f("volxb")[2:nx + 2], vx)
    assert np.array_equal(o.f("volyb")[2:ny + 2], vy)
    assert np.array_equal(o.f("volzb")[2:nz + 2], vz)


def test_raddif_solves_its_system(shell):
    """RADDIF with a fixed top (IBDRAD = 4) and ITMAX iterations: the
    interior ER it leaves satisfies B ER + couplings = RHS up to the
    residual norm SOLVMAT reports; DIFFEL's rows are diagonally dominant."""
    o = rad_oracle(shell, 4, 1e-10, 400)
    assert o.call("raddif", 0.0, 0.0, 1, 0) == 1          # ITMAX: the boundary rows keep a residual
    assert int(o.get("sor_iter")) == 400
    B = o.f("RAD_B")
    off = sum(np.abs(o.f(n)) for n in ("RAD_AX", "RAD_CX", "RAD_AY", "RAD_CY", "RAD_AZ", "RAD_CZ"))
    assert np.all(B > off)
    T = o.f("T")
    assert np.all(np.isfinite(T)) and np.all(T[2:-2, 2:-2, 2:-2] > 0)


def test_raddif_converges_with_gradient_top(shell):
    """IBDRAD = 7 (zero gradient at the top): SOLVMAT reaches EPSMAT = 1e-6
    (the L2 rule, ppmat.f:152-178) and stops; ITMIN = 5 holds."""
    o = rad_oracle(shell, 7, 1e-6, 3000)
    assert o.call("raddif", 0.0, 0.0, 1, 0) == 0
    assert 5 <= int(o.get("sor_iter")) < 3000
    assert o.get("global_rnorm") / o.get("global_rhsnorm") <= 1e-6


def test_raddif_rejects_unimplemented_boundaries(shell):
    for ib in (1, 3, 5, 6, 8):
        o = rad_oracle(shell, ib, 1e-6, 10)
        assert o.call("raddif", 0.0, 0.0, 1, 0) == -3
    o = rad_oracle(shell, 9, 1e-6, 10)
    assert o.call("raddif", 0.0, 0.0, 6, 0) == -3       # MODVER > 5


def test_slab_threads_give_the_serial_sweeps(shell):
    """The CPU baseline's slab-parallel sweeps (one thread per theta slab, a
    barrier per colour) leave the serial loop's iterate bit for bit."""
    o = oracle_from_shell(shell)
    assert o.call("coupled_energy_eqs", 1) == 0
    o.f("DELTA_ER")[...] = 0.0
    assert o.call("sor_sweeps", 7) == 0
    x1, r1 = o.f("DELTA_ER").copy(), o.get("global_rnorm")
    o.f("DELTA_ER")[...] = 0.0
    assert o.call("sor_sweeps_mt", 7, 5) == 0
    assert np.array_equal(o.f("DELTA_ER"), x1)
    assert abs(o.get("global_rnorm") - r1) <= 1e-12 * r1


def test_slab_threads_complete_solve(shell):
    """The CPU baseline's complete threaded solve (slab norms added in slab
    order, the ppsor.f:161-177 stopping rule) stops at the serial loop's
    sweep with its iterate: a different summation order can only move the
    stop by one sweep where the ratio ties EPSMAT in the last bits."""
    o = oracle_from_shell(shell)
    assert o.call("coupled_energy_eqs", 1) == 0
    o.f("DELTA_ER")[...] = 0.0
    assert o.call("solve_with_sor", 0, 0) == 0
    x1, n1 = o.f("DELTA_ER").copy(), int(o.get("sor_iter"))
    assert o.call("solve_with_sor_mt", 5) == 0
    n2 = int(o.get("sor_iter"))
    assert abs(n2 - n1) <= 1
    if n2 == n1:
        assert np.array_equal(o.f("DELTA_ER"), x1)
    assert o.get("global_rnorm") / o.get("global_rhsnorm") <= o.get("epsmat")


def test_opacity_table_interpolation(shell):
    """BurrowsOPC's interpolation (ttor_set_opacity_table + KAPPA) on a table
    of the analytic model reproduces the model (log kappa is linear in log T
    and log rho), with the T-derivative stand-ins of pprphy.f:1180-1185."""
    from ttcode_gb300.synthetic import analytic_opacity_table
    o = oracle_from_shell(shell, start=False)
    o.f("KMUL")[...] = 1.0
    o.set("iii", 0)
    assert o.call("bounds") == 0 and o.call("kappa") == 0
    ref = {n: o.f(n).copy() for n in ("XKAPR", "XKAPP", "XKAPA")}
    lt, lr, kr, kp, ka = analytic_opacity_table(1e-2)
    keep = [np.ascontiguousarray(a) for a in (lt, lr)] + [np.asfortranarray(a) for a in (kr, kp, ka)]
    lib = __import__("oracle")._load()
    assert lib.ttor_set_opacity_table(o.h, lt.size, lr.size, *[a.ctypes.data for a in keep]) == 0
    assert o.call("kappa") == 0
    # inside the table's range (the ghosts below the shell, rho > 1e-2, are
    # clamped to its edge as the reference clamps them)
    rho = o.f("RH")
    inside = (np.log10(rho) < -1.99994) & (np.log10(rho) > -11.9995)
    for n, a in ref.items():
        assert rel_l2(o.f(n)[inside], a[inside]) <= 1e-12, n
    assert not np.all(inside)
    # dkappa_P/dT: the table's finite difference at the bracketing T nodes
    assert np.all(o.f("DXKAPP_DT")[2:-2, 2:-2, 2:-2] > 0)
    # T <= 0 stops (pprphy.f:1037-1043)
    o.f("T")[5, 5, 5] = -1.0
    assert o.call("kappa") == -10


def test_pcg_design_restated_on_the_cpu(shell):
    """The PCG solvers' construction in numpy on an oracle system: W = V/|EVAL8|
    symmetrises the rows; CG in float32 on Sigma sym(W A) Sigma with the exact
    radial line solve as preconditioner, inside float64 defect correction on
    the rows as they are, reaches ||b - A x||_1 / ||b||_1 <= 1e-10 and the
    sparse direct solution, with far fewer iterations than SOR sweeps."""
    from scipy.linalg import solve_banded
    o = oracle_from_shell(shell, eps=1e-10)
    assert o.call("coupled_energy_eqs", 1) == 0
    o.call("fill_evalues", 1.0)
    assert o.call("fill_sor_matrix") == 0 and o.call("b_vector_boundaries") == 0
    nx, ny, nz = shell.dims
    A = sor_matrix(o)
    b = o.f("RHS_ER").ravel(order="F").copy()
    g = shell.grid
    I, J, K = np.meshgrid(np.arange(1, nx + 1), np.arange(1, ny + 1), np.arange(1, nz + 1), indexing="ij")
    V = (g.at("surxb", I) * g.at("dxa", I) * g.at("dya", J) * g.at("surzb", K) * g.at("dza", K)).ravel(order="F")
    offd = (A - sp.diags(A.diagonal())).tocsr()
    decoupled = np.asarray(abs(offd).sum(axis=1)).ravel() == 0
    W = np.where(decoupled, V, V / np.abs(o.f("EVAL8").ravel(order="F")))
    M = (sp.diags(W) @ A).tocsr()
    Ms = ((M + M.T) * 0.5).tocsr()
    sig = 1.0 / np.sqrt(Ms.diagonal())
    S = (sp.diags(sig) @ Ms @ sp.diags(sig)).astype(np.float32).tocsr()
    n = S.shape[0]
    ar = np.arange(n)
    up = np.zeros(n, np.float32)
    up[:-1] = np.asarray(S[ar[:-1], ar[1:]]).ravel()
    up[(ar % nx) == nx - 1] = 0.0
    ab = np.vstack([np.concatenate([[0], up[:-1]]), np.ones(n, np.float32), np.concatenate([up[:-1], [0]])])

    def line(r):
        return solve_banded((1, 1), ab, r).astype(np.float32)

    def inner(r, reduce=1e-4, maxit=500):
        e = np.zeros_like(r); z = line(r); p = z.copy(); gam = np.float32(r @ z); g0 = gam
        for it in range(1, maxit + 1):
            s = S @ p; al = gam / np.float32(p @ s)
            e += al * p; r = r - al * s; z = line(r); gn = np.float32(r @ z)
            if gn <= reduce * reduce * g0:
                return e, it
            p = z + (gn / gam) * p; gam = gn
        return e, maxit

    x = np.zeros(n)
    its = 0
    for anchor in range(20):
        res = b - A @ x
        if np.abs(res).sum() <= 1e-10 * np.abs(b).sum():
            break
        e, k = inner((sig * W * res).astype(np.float32))
        its += k
        x += sig * e.astype(np.float64)
    assert np.abs(b - A @ x).sum() <= 1e-10 * np.abs(b).sum()
    xd = spla.spsolve(A.tocsc(), b)
    assert rel_l2(x, xd) <= 1e-9
    o.f("DELTA_ER")[...] = 0.0
    o.set("epsmat", 1e-10)
    assert o.call("solve_with_sor", 0, 0) == 0
    assert its < int(o.get("sor_iter")) // 2, (its, int(o.get("sor_iter")))


def test_hypre_laplacian_toggle_known_answer():
    """pphypre.f:251-258 (and ppenergy.f:1017-1025) turn the system into the
    6/-1 Laplacian; with b = 1 (pphypre.f:136-137) FILLHYPREMATRIX /
    FILLHYPREVECTORS must give the Laplacian whose boundary cells (i = 1,
    i = NX, i >= upperbnd, k = 1, k = NZ) are identity rows with b = 0 and
    whose phi direction ends at the grid (no periodic coupling), built here
    independently."""
    from oracle import Oracle
    nx, ny, nz = 12, 8, 10
    o = Oracle(nx, ny, nz)
    for n in ("EVAL1", "EVAL2", "EVAL3", "EVAL4", "EVAL5", "EVAL6", "EVAL8"):
        o.f(n)[...] = 1.0
    o.f("EVAL7")[...] = 6.0
    o.f("EVAL_1_6")[...] = 0.0
    o.f("UPPERBND")[...] = nx - 1
    o.f("RHS_ER")[...] = 1.0
    assert o.call("fill_hypre_system") == 0
    A = hypre_matrix(o).toarray()
    b = o.f("HYP_RHS").ravel(order="F")
    idx = lambda i, j, k: (i - 1) + nx * ((j - 1) + ny * (k - 1))
    n = nx * ny * nz
    R = np.zeros((n, n))
    rb = np.ones(n)
    ub = nx - 1
    for k in range(1, nz + 1):
        for j in range(1, ny + 1):
            for i in range(1, nx + 1):
                r = idx(i, j, k)
                if i == 1 or i >= ub or k == 1 or k == nz:
                    R[r, r] = 1.0
                    rb[r] = 0.0
                    continue
                R[r, r] = 6.0
                for (ii, jj, kk) in ((i - 1, j, k), (i + 1, j, k), (i, j - 1, k), (i, j + 1, k), (i, j, k - 1),
                                     (i, j, k + 1)):
                    if not (1 <= jj <= ny):
                        continue                       # outside hypre's grid
                    if ii == 1 or ii >= ub or kk == 1 or kk == nz:
                        continue                       # a boundary cell: its coupling is zeroed
                    R[r, idx(ii, jj, kk)] = -1.0
    assert np.array_equal(A, R)
    assert np.array_equal(b, rb)


def test_raddif_uniform_state_is_a_fixed_point():
    """RADDIF on an isothermal shell with a flat bottom (D_T = 0) and the top
    held at the same temperature (IBDRAD = 4, Tirr = T): every row of SOLVMAT
    is satisfied by the uniform E_R = arad T^4 (B E - RHS + sum of the
    couplings times E = 0), so the solve stops at ITMIN = 5 iterations and
    T comes back unchanged."""
    from ttcode_gb300.synthetic import make_shell
    sh = make_shell(16, 12, 10, seed=2, delt=100.0)
    sh.fields["T"][...] = 1500.0
    sh.fields["ER"][...] = 7.56596e-15 * 1500.0 ** 4
    o = rad_oracle(sh, 4, 1e-10, 100)
    o.set("tirr", 1500.0)
    assert o.call("raddif", 0.0, 0.0, 1, 0) == 0
    assert int(o.get("sor_iter")) == 5
    assert o.get("global_rnorm") / o.get("global_rhsnorm") <= 1e-14
    assert np.max(np.abs(o.f("T")[2:-2, 2:-2, 2:-2] - 1500.0)) <= 1e-9


def _mirrored(a, nz):
    """Whether halo array a (index k+1 for k = -1..NZ+2) holds the one-rank
    pole shifts: planes NZ-1, NZ-2, NZ-3 on NZ, NZ+1, NZ+2 and planes 1, 2 on
    0, -1."""
    return (np.array_equal(a[:, :, nz + 1], a[:, :, nz]) and np.array_equal(a[:, :, nz + 2], a[:, :, nz - 1])
            and np.array_equal(a[:, :, nz + 3], a[:, :, nz - 2]) and np.array_equal(a[:, :, 1], a[:, :, 2])
            and np.array_equal(a[:, :, 0], a[:, :, 3]))


def test_poles_mirror_rows_and_manufactured_solution():
    """inc_poles with one rank (the partner across each pole is the rank
    itself, ppshift.f:820-833): BOUNDS leaves T and RH mirrored at the theta
    edges (NORTH/SOUTH_POLE_SHIFT,
    ppshift.f:2217-2453), the theta edges are ordinary rows of the SOR system
    (ppsor.f:228-272), and SOLVE_WITH_SOR solves the rows k = 1..NZ-1
    (ppsor.f:39-43): a manufactured solution of those rows, with the mirrored
    ghosts as the closure, is recovered."""
    from ttcode_gb300.synthetic import make_shell
    nx, ny, nz = 16, 24, 12
    sh = make_shell(nx, ny, nz, seed=7, delt=100.0, poles=True)
    o = oracle_from_shell(sh, eps=1e-10)
    assert _mirrored(o.f("T"), nz) and _mirrored(o.f("RH"), nz)
    assert o.call("coupled_energy_eqs", 1) == 0
    assert np.isfinite(o.f("ER")).all()   # E_R is shifted at the next iteration's start
    A = {n: o.f(n) for n in ("SOR_A", "SOR_B", "SOR_C", "SOR_D", "SOR_E", "SOR_F", "SOR_G")}
    assert np.all(A["SOR_F"][:nx - 3, :, 0] != 0.0) and np.all(A["SOR_G"][:nx - 3, :, nz - 2] != 0.0)
    # x* on k = 1..NZ-1, mirrored ghosts, zero radial ghosts; b = A x* on those rows
    rng = np.random.default_rng(3)
    xs = np.zeros((nx + 4, ny + 4, nz + 4))
    xs[2:nx + 2, 2:ny + 2, 2:nz + 1] = rng.uniform(-1.0, 1.0, (nx, ny, nz - 1))
    xs[:, 0:2, :] = xs[:, ny:ny + 2, :]
    xs[:, ny + 2:ny + 4, :] = xs[:, 2:4, :]
    for m in range(3):
        xs[:, :, nz + 1 + m] = xs[:, :, nz - m]
    xs[:, :, 1], xs[:, :, 0] = xs[:, :, 2], xs[:, :, 3]
    c = np.s_[2:nx + 2, 2:ny + 2, 2:nz + 2]
    sh3 = lambda di, dj, dk: xs[2 + di:nx + 2 + di, 2 + dj:ny + 2 + dj, 2 + dk:nz + 2 + dk]
    ax = (A["SOR_A"] * xs[c] + A["SOR_B"] * sh3(-1, 0, 0) + A["SOR_C"] * sh3(1, 0, 0) + A["SOR_D"] * sh3(0, -1, 0)
          + A["SOR_E"] * sh3(0, 1, 0) + A["SOR_F"] * sh3(0, 0, -1) + A["SOR_G"] * sh3(0, 0, 1))
    b = ax.copy()
    b[:, :, nz - 1] = 0.0                                  # row NZ is not solved
    o.f("RHS_ER")[...] = b
    o.set("epsmat", 1e-14)
    assert o.call("solve_with_sor", 0, 0) == 0
    x = o.f("DELTA_ER")
    assert rel_l2(x[2:nx + 2, 2:ny + 2, 2:nz + 1], xs[2:nx + 2, 2:ny + 2, 2:nz + 1]) <= 1e-9
    assert _mirrored(x, nz)


@pytest.mark.parametrize("ibdrad,eps,itmax,rc", [(7, 1e-6, 3000, 0), (4, 1e-10, 60, 1)])
def test_poles_raddif(ibdrad, eps, itmax, rc):
    """RADDIF with poles: SOLVMAT sweeps k = 1..NZ, RADIATIVEBOUND leaves the
    theta ghosts to the pole shifts that follow every PLANETSHIFT(6)
    (ppmat.f:39-136, ppbou.f:2256-2290).  With the zero-gradient top it
    still reaches EPSMAT; E_R and T come out mirrored at the theta edges."""
    from ttcode_gb300.synthetic import make_shell
    nx, ny, nz = 24, 16, 12
    sh = make_shell(nx, ny, nz, seed=11, delt=100.0, poles=True)
    o = rad_oracle(sh, ibdrad, eps, itmax)
    assert o.call("raddif", 0.0, 0.0, 1, 0) == rc
    assert 5 <= int(o.get("sor_iter")) <= itmax
    assert _mirrored(o.f("ER"), nz) and _mirrored(o.f("T"), nz)
    assert np.all(np.isfinite(o.f("T")))


def test_poles_diffusion_sweeps_every_row():
    """DIFFUSION with poles (ppdif.f:45-135): every theta row k = 1..NZ is
    swept (DIFFUSION has no zmax_sor_index) and the scalar is pole-shifted
    after each colour, which overwrites row NZ with row NZ-1.  Row NZ's
    residual therefore stays in RNORM, the ratio levels off, and the loop
    runs to SORITMAX = 500 (status 1, the reference's message) with the
    scalar mirrored."""
    from ttcode_gb300.synthetic import make_shell
    nx, ny, nz = 16, 24, 12
    sh = make_shell(nx, ny, nz, seed=9, delt=100.0, poles=True)
    o = oracle_from_shell(sh)
    rng = np.random.default_rng(5)
    o.f("SCALAR")[...] = 1.0 + rng.random((nx + 4, ny + 4, nz + 4))
    assert o.call("planetshift", "SCALAR") == 0
    assert _mirrored(o.f("SCALAR"), nz)
    o.set("pr_num", 1.0)
    o.set("xnue", 1.0e15)
    assert o.call("diffusion") == 1
    assert int(o.get("sor_iter")) == 500
    assert 1e-4 < o.get("global_rnorm") / o.get("global_rhsnorm") < 1e-1
    assert _mirrored(o.f("SCALAR"), nz)
