/*
 * ttfld_oracle.h -- CPU oracle for the implicit FLD radiation/gas energy step.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of ttcode's
 * COUPLED_ENERGY_EQS (ppenergy.f), DIFF (pprad.f), FLIM (pprphy.f),
 * QDENS (ppphy.f), the grey STELLARINPUT_HEATING (pprad.f), BOUNDS for the
 * planet set-up (ppbou.f), the one-rank PLANETSHIFT (ppshift.f) and
 * SOLVE_WITH_SOR / FILL_SOR_MATRIX / B_VECTOR_BOUNDARIES / ADJUST_SOR_PARAM
 * (ppsor.f), plus DIFFUSION (ppdif.f).  Only tests, the smoke check and the
 * CPU-baseline leg of bench.py may load it; the product library never does.
 *
 * Parity status: the reference ships no tests or golden vectors and cannot
 * be compiled here (no Fortran compiler, no MPI/bHYPRE), so this oracle is
 * pinned by known-answer tests (the reference's own Laplacian toggle,
 * manufactured solutions, hand-evaluated formulas), not by reference output.
 *
 * All arrays use the reference's Fortran column-major layout (i fastest).
 * Bounds (Fortran) of the storage classes used below:
 *   halo   (-1:NX+2, -1:NY+2, -1:NZ+2)   T RH CV ER ER_OLD Q Q_OLD DELTA_ER
 *                                        XKAPR XKAPP XKAPA DXKAPP_DT DXKAPA_DT
 *                                        KMUL RHQX RHQY RHQZ STELLARTAU DTAUS
 *                                        STELLARINPUT (only i in 1..NX used)
 *   cell   (1:NX, 1:NY, 1:NZ)            EVAL1..8 EVAL_1_6 JACOB_ETA FQ FR
 *                                        RHS_ER SOR_A..SOR_G DIVF DIVF_OLD
 *                                        DFQ_DQ DFR_DQ DELTA_Q
 *   face   (1:NX+1, 1:NY+1, 1:NZ+1)      FLIMX/Y/Z DIFRX/Y/Z FLUX_X/Y/Z
 *   plane  (-1:NY+2, -1:NZ+2)            UPPERBND (int) MU_STAR TINCIDENT
 *   1-D    (-1:N+2)                      grid metrics (entries outside the
 *                                        reference's own bounds are unused)
 */
#ifndef TTFLD_ORACLE_H
#define TTFLD_ORACLE_H
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif

typedef struct ttor_state ttor_state;

ttor_state* ttor_create(int nx, int ny, int nz);
void ttor_destroy(ttor_state* s);

/* Field access by reference name (upper case, e.g. "ER", "SOR_A", "XXB").
 * Returns a pointer to the storage and its element count in *n, or NULL. */
double* ttor_field(ttor_state* s, const char* name, size_t* n);
int* ttor_ifield(ttor_state* s, const char* name, size_t* n);

/* Scalar parameters / results by name ("DELT", "SORPARAM", "ITMAX", ...). */
int ttor_set(ttor_state* s, const char* name, double v);
double ttor_get(ttor_state* s, const char* name);

/* Reference subroutines (return 0 on success, <0 on error). */
int ttor_gitter(ttor_state* s);               /* GITTER ncosys=2, linear   */
int ttor_calcmustar(ttor_state* s);           /* CALCMUSTAR + CALC_TINCIDENT */
int ttor_planetshift(ttor_state* s, const char* field); /* one-rank halo (+ pole shifts) */
int ttor_bounds(ttor_state* s);               /* BOUNDS (T, RH, UPPERBND)  */
int ttor_kappa(ttor_state* s);                /* synthetic analytic KAPPA  */
int ttor_qdens(ttor_state* s);
int ttor_flim(ttor_state* s);
int ttor_diff(ttor_state* s);
int ttor_calculateflux(ttor_state* s);
int ttor_flux_bc(ttor_state* s);
int ttor_fill_evalues(ttor_state* s, double theta);
int ttor_calculatedivf_withf(ttor_state* s, int which /*0 DIVF, 1 DIVF_OLD*/, double theta);
int ttor_stellarinput_heating(ttor_state* s);
int ttor_fill_sor_matrix(ttor_state* s);
int ttor_b_vector_boundaries(ttor_state* s);
/* FILLHYPREMATRIX + FILLHYPREVECTORS (pphypre.f:115-334) into HYP_A..HYP_G,
 * HYP_RHS from the EVAL arrays, RHS_ER and UPPERBND. */
int ttor_fill_hypre_system(ttor_state* s);
/* The opacity table KAPPA interpolates (BurrowsOPC) once set: log10 T (nt),
 * log10 rho (nrh), log10 Rosseland / Planck / absorption means (nt x nrh, T
 * index fastest).  KAPPA then returns -10 where the reference stops. */
int ttor_set_opacity_table(ttor_state* s, int nt, int nrh, const double* lt, const double* lrh,
                           const double* ross, const double* plnk, const double* absk);
/* RADDIF (pprad.f:1-38, IRAD=1): ER = arad T^4, DIFFEL, SOLVMAT (ppmat.f,
 * red-black SOR on ER with the L2 stop and ITMIN = 5) with RADIATIVEBOUND
 * (ppbou.f:2049-2299; IBDRAD 4, 7, 9, MODVER <= 5) after each colour,
 * T = (ER/arad)^(1/4).  d_t is the bottom temperature gradient D_T,
 * tinit_bottom TinitBottom (read with BCXMIN = 6); returns 0, 1 at ITMAX,
 * -3 for a configuration outside that set. */
int ttor_raddif(ttor_state* s, double d_t, double tinit_bottom, int modver, int energy_iter);
/* SOLVE_WITH_SOR.  use_guess=0 starts from zero (ppsor.f:29); use_guess=1
 * keeps the interior of DELTA_ER as the initial iterate (ghosts zeroed). */
int ttor_solve_with_sor(ttor_state* s, int fill, int use_guess);
/* Plain red-black SOR on the current SOR_A..G / RHS_ER with no refill. */
int ttor_sor_sweeps(ttor_state* s, int nsweeps);
/* The same sweeps on nthreads theta slabs (the reference's rank
 * decomposition on the host cores, for the CPU baseline). */
int ttor_sor_sweeps_mt(ttor_state* s, int nsweeps, int nthreads);
int ttor_solve_with_sor_mt(ttor_state* s, int nthreads);
/* FreedmanXKAP_ross/plnk/abs (42 x 18 log10 means, T index fastest) and
 * mu_gas: KAPPA then takes the IKAPTYP 4:5 branch (FreedmanOPC). */
int ttor_set_freedman_table(ttor_state* s, const double* ross, const double* plnk, const double* absk,
                            double mu_gas);
/* After ttor_set_opacity_table: the per-bin log10 opacities (nt x nrh x nb,
 * T fastest, bin slowest), BSTAR_BIN (nb), RSTAR (solar radii) and semi
 * (cm): KAPPA also forms the per-bin opacities and STELLARINPUT_HEATING
 * takes the wavelength-binned branch of IKAPTYP 20-24. */
int ttor_set_wave_table(ttor_state* s, int nb, const double* waveopac, const double* bstar, double rstar,
                        double semi);
int ttor_adjust_sor_param(ttor_state* s);
int ttor_coupled_energy_eqs(ttor_state* s, int do_bounds);
/* DIFFUSION (ppdif.f) of the field "SCALAR" with constant xnue/Pr. */
int ttor_diffusion(ttor_state* s);
/* L1 norm of b - A x for the current SOR system (x = DELTA_ER). */
double ttor_true_residual_l1(ttor_state* s);

#ifdef __cplusplus
}
#endif
#endif
