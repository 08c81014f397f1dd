/*
 * ttfld_oracle.c -- CPU oracle (test infrastructure only) for ttcode's
 * implicit FLD step.  Every routine restates the reference subroutine named
 * in its comment, with the same loop order, the same operand order in each
 * expression (compile with -O2 -ffp-contract=off so no FMA is formed), and
 * the reference's REAL*4 literal constants converted to double.
 *
 * Parity status: unpinned by reference output (the reference has no tests
 * and cannot be built here); pinned by the known-answer tests under tests/.
 *
 * Where the reference reads an array outside its declared bounds (noted at
 * each site) the restatement uses a clamped, defined value instead; the
 * cells affected are ghost cells that the step never reads back.
 */
#define _POSIX_C_SOURCE 200809L  /* pthread barriers under -std=c11 */
#include "ttfld_oracle.h"
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

/* global_constants, ppmod.f:1074-1092: REAL*4 literals stored as double. */
#define PI_D 3.141592653589793
#define FD_C ((double)2.99792458e10f)
#define ARAD_C ((double)7.56596e-15f)
#define SBCONST_C ((double)5.6705e-5f)
#define RGAS_C ((double)8.315e7f)
#define RSOL_C ((double)6.9598e10f)

struct ttor_state {
  int nx, ny, nz;
  /* input_init / fluid_var_init scalars */
  double delt, sorparam, epsmat, fbottom, tirr, xnue, pr_num, sigval;
  double kap0, theta_last;
  int itmax, bcxmin, ibdrad, iflimtyp, f_incident, ieta, isigtyp, iii;
  int adjust_sor, poles, ikaptyp;
  /* opacity table (BurrowsOPC's arrays), used by KAPPA when opac_nt > 0 */
  int opac_nt, opac_nrh;
  double *opac_lt, *opac_lrh, *opac_ross, *opac_plnk, *opac_abs;
  /* per-wavelength-bin opacities of the same table (BurrowsXKAP_waveopac),
   * the star's flux per bin (BSTAR_BIN) and RSTAR, semi: with wave_nb > 0
   * KAPPA also forms XKAPW and STELLARINPUT_HEATING takes the binned branch
   * of IKAPTYP 20-24 */
  int wave_nb;
  double *wave_opac, *wave_bstar, *XKAPW, *STAU_W;
  double wave_rstar, wave_semi;
  /* FreedmanXKAP_ross/plnk/abs (42 x 18, T fastest) and mu_gas: with
   * freed_set KAPPA takes the IKAPTYP 4:5 branch */
  int freed_set;
  double freed_ross[42 * 18], freed_plnk[42 * 18], freed_abs[42 * 18], freed_mu;
  /* results */
  int sor_iter, energy_iter, status, sor_total, solves;
  double global_rnorm, global_rhsnorm, global_deltaq, global_deltaer;
  /* 1-D grid (stored on -1:N+2) */
  double *xxa, *xxb, *dxa, *dxb, *xya, *xyb, *dya, *dyb, *xza, *xzb, *dza, *dzb;
  double *ddx0, *ddx1, *ddy0, *ddy1, *ddz0, *ddz1;
  double *surxa, *surxb, *surza, *surzb, *geoxg, *geoxh, *geoxga, *geoxha,
      *geozg, *geozga, *volxb, *volyb, *volzb;
  double xmin, xmax, ymin, ymax, zmin, zmax;
  /* halo fields */
  double *T, *RH, *CV, *ER, *ER_OLD, *Q, *Q_OLD, *DELTA_ER, *XKAPR, *XKAPP,
      *XKAPA, *DXKAPP_DT, *DXKAPA_DT, *KMUL, *RHQX, *RHQY, *RHQZ,
      *STELLARTAU, *DTAUS, *STELLARINPUT, *SCALAR;
  /* cell fields */
  double *EVAL1, *EVAL2, *EVAL3, *EVAL4, *EVAL5, *EVAL6, *EVAL7, *EVAL8,
      *EVAL_1_6, *JACOB_ETA, *FQ, *FR, *RHS_ER, *SOR_A, *SOR_B, *SOR_C,
      *SOR_D, *SOR_E, *SOR_F, *SOR_G, *DIVF, *DIVF_OLD, *DFQ_DQ, *DFR_DQ,
      *DELTA_Q, *RHS_DIF;
  /* the IRAD=2 system of FILLHYPREMATRIX / FILLHYPREVECTORS */
  double *HYP_A, *HYP_B, *HYP_C, *HYP_D, *HYP_E, *HYP_F, *HYP_G, *HYP_RHS;
  /* the IRAD=1 system of RADDIF / DIFFEL (rad_var_init AX..CZ, B, RHS) */
  double *RAD_AX, *RAD_CX, *RAD_AY, *RAD_CY, *RAD_AZ, *RAD_CZ, *RAD_B, *RAD_RHS;
  /* face fields */
  double *FLIMX, *FLIMY, *FLIMZ, *DIFRX, *DIFRY, *DIFRZ, *FLUX_X, *FLUX_Y,
      *FLUX_Z;
  /* plane fields */
  int* UPPERBND;
  double *MU_STAR, *TINCIDENT;
};

/* ---- indexing (Fortran bounds documented in the header) ---------------- */
#define NXH (s->nx + 4)
#define NYH (s->ny + 4)
#define H(a, i, j, k) \
  (s->a[(size_t)((i) + 1) + (size_t)NXH * ((size_t)((j) + 1) + (size_t)NYH * (size_t)((k) + 1))])
#define C(a, i, j, k) \
  (s->a[(size_t)((i)-1) + (size_t)s->nx * ((size_t)((j)-1) + (size_t)s->ny * (size_t)((k)-1))])
#define F(a, i, j, k)                                                      \
  (s->a[(size_t)((i)-1) + (size_t)(s->nx + 1) *                            \
                              ((size_t)((j)-1) + (size_t)(s->ny + 1) * (size_t)((k)-1))])
#define P(a, j, k) (s->a[(size_t)((j) + 1) + (size_t)NYH * (size_t)((k) + 1)])
#define G1(a, i) (s->a[(i) + 1])

static size_t nhalo(const ttor_state* s) {
  return (size_t)(s->nx + 4) * (s->ny + 4) * (s->nz + 4);
}
static size_t ncell(const ttor_state* s) { return (size_t)s->nx * s->ny * s->nz; }
static size_t hidx(const ttor_state* s, int i, int j, int k) {
  return (size_t)(i + 1) + (size_t)NXH * ((size_t)(j + 1) + (size_t)NYH * (size_t)(k + 1));
}
static size_t nface(const ttor_state* s) {
  return (size_t)(s->nx + 1) * (s->ny + 1) * (s->nz + 1);
}
static size_t nplane(const ttor_state* s) { return (size_t)(s->ny + 4) * (s->nz + 4); }

static double p4(double x) { double x2 = x * x; return x2 * x2; }  /* x**4.d0 */
static double p3(double x) { return (x * x) * x; }                 /* x**3.d0 */

typedef struct { const char* name; size_t off; int kind; } fdesc;
enum { K_HALO, K_CELL, K_FACE, K_PLANE, K_1D };
#define FD_ENTRY(nm, kind) {#nm, offsetof(ttor_state, nm), kind}
static const fdesc FIELDS[] = {
    FD_ENTRY(T, K_HALO), FD_ENTRY(RH, K_HALO), FD_ENTRY(CV, K_HALO),
    FD_ENTRY(ER, K_HALO), FD_ENTRY(ER_OLD, K_HALO), FD_ENTRY(Q, K_HALO),
    FD_ENTRY(Q_OLD, K_HALO), FD_ENTRY(DELTA_ER, K_HALO), FD_ENTRY(XKAPR, K_HALO),
    FD_ENTRY(XKAPP, K_HALO), FD_ENTRY(XKAPA, K_HALO), FD_ENTRY(DXKAPP_DT, K_HALO),
    FD_ENTRY(DXKAPA_DT, K_HALO), FD_ENTRY(KMUL, K_HALO), FD_ENTRY(RHQX, K_HALO),
    FD_ENTRY(RHQY, K_HALO), FD_ENTRY(RHQZ, K_HALO), FD_ENTRY(STELLARTAU, K_HALO),
    FD_ENTRY(DTAUS, K_HALO), FD_ENTRY(STELLARINPUT, K_HALO), FD_ENTRY(SCALAR, K_HALO),
    FD_ENTRY(EVAL1, K_CELL), FD_ENTRY(EVAL2, K_CELL), FD_ENTRY(EVAL3, K_CELL),
    FD_ENTRY(EVAL4, K_CELL), FD_ENTRY(EVAL5, K_CELL), FD_ENTRY(EVAL6, K_CELL),
    FD_ENTRY(EVAL7, K_CELL), FD_ENTRY(EVAL8, K_CELL), FD_ENTRY(EVAL_1_6, K_CELL),
    FD_ENTRY(JACOB_ETA, K_CELL), FD_ENTRY(FQ, K_CELL), FD_ENTRY(FR, K_CELL),
    FD_ENTRY(RHS_ER, K_CELL), FD_ENTRY(SOR_A, K_CELL), FD_ENTRY(SOR_B, K_CELL),
    FD_ENTRY(SOR_C, K_CELL), FD_ENTRY(SOR_D, K_CELL), FD_ENTRY(SOR_E, K_CELL),
    FD_ENTRY(SOR_F, K_CELL), FD_ENTRY(SOR_G, K_CELL), FD_ENTRY(DIVF, K_CELL),
    FD_ENTRY(DIVF_OLD, K_CELL), FD_ENTRY(DFQ_DQ, K_CELL), FD_ENTRY(DFR_DQ, K_CELL),
    FD_ENTRY(DELTA_Q, K_CELL), FD_ENTRY(RHS_DIF, K_CELL),
    FD_ENTRY(HYP_A, K_CELL), FD_ENTRY(HYP_B, K_CELL), FD_ENTRY(HYP_C, K_CELL),
    FD_ENTRY(HYP_D, K_CELL), FD_ENTRY(HYP_E, K_CELL), FD_ENTRY(HYP_F, K_CELL),
    FD_ENTRY(HYP_G, K_CELL), FD_ENTRY(HYP_RHS, K_CELL),
    FD_ENTRY(RAD_AX, K_CELL), FD_ENTRY(RAD_CX, K_CELL), FD_ENTRY(RAD_AY, K_CELL),
    FD_ENTRY(RAD_CY, K_CELL), FD_ENTRY(RAD_AZ, K_CELL), FD_ENTRY(RAD_CZ, K_CELL),
    FD_ENTRY(RAD_B, K_CELL), FD_ENTRY(RAD_RHS, K_CELL),
    FD_ENTRY(FLIMX, K_FACE), FD_ENTRY(FLIMY, K_FACE), FD_ENTRY(FLIMZ, K_FACE),
    FD_ENTRY(DIFRX, K_FACE), FD_ENTRY(DIFRY, K_FACE), FD_ENTRY(DIFRZ, K_FACE),
    FD_ENTRY(FLUX_X, K_FACE), FD_ENTRY(FLUX_Y, K_FACE), FD_ENTRY(FLUX_Z, K_FACE),
    FD_ENTRY(MU_STAR, K_PLANE), FD_ENTRY(TINCIDENT, K_PLANE),
    FD_ENTRY(xxa, K_1D), FD_ENTRY(xxb, K_1D), FD_ENTRY(dxa, K_1D), FD_ENTRY(dxb, K_1D),
    FD_ENTRY(xya, K_1D), FD_ENTRY(xyb, K_1D), FD_ENTRY(dya, K_1D), FD_ENTRY(dyb, K_1D),
    FD_ENTRY(xza, K_1D), FD_ENTRY(xzb, K_1D), FD_ENTRY(dza, K_1D), FD_ENTRY(dzb, K_1D),
    FD_ENTRY(ddx0, K_1D), FD_ENTRY(ddx1, K_1D), FD_ENTRY(ddy0, K_1D), FD_ENTRY(ddy1, K_1D),
    FD_ENTRY(ddz0, K_1D), FD_ENTRY(ddz1, K_1D), FD_ENTRY(surxa, K_1D), FD_ENTRY(surxb, K_1D),
    FD_ENTRY(surza, K_1D), FD_ENTRY(surzb, K_1D), FD_ENTRY(geoxg, K_1D), FD_ENTRY(geoxh, K_1D),
    FD_ENTRY(geoxga, K_1D), FD_ENTRY(geoxha, K_1D), FD_ENTRY(geozg, K_1D),
    FD_ENTRY(geozga, K_1D), FD_ENTRY(volxb, K_1D), FD_ENTRY(volyb, K_1D), FD_ENTRY(volzb, K_1D),
};
#define NFIELDS (sizeof(FIELDS) / sizeof(FIELDS[0]))

static size_t field_count(const ttor_state* s, const fdesc* d, int n1d) {
  switch (d->kind) {
    case K_HALO: return nhalo(s);
    case K_CELL: return ncell(s);
    case K_FACE: return nface(s);
    case K_PLANE: return nplane(s);
    default: return (size_t)n1d;
  }
}

ttor_state* ttor_create(int nx, int ny, int nz) {
  if (nx < 4 || ny < 4 || nz < 4) return NULL;
  ttor_state* s = (ttor_state*)calloc(1, sizeof(ttor_state));
  if (!s) return NULL;
  s->nx = nx; s->ny = ny; s->nz = nz;
  int n1d = (nx > ny ? (nx > nz ? nx : nz) : (ny > nz ? ny : nz)) + 4;
  for (size_t f = 0; f < NFIELDS; ++f) {
    size_t n = field_count(s, &FIELDS[f], n1d);
    double** slot = (double**)((char*)s + FIELDS[f].off);
    *slot = (double*)calloc(n, sizeof(double));
    if (!*slot) { ttor_destroy(s); return NULL; }
  }
  s->UPPERBND = (int*)calloc(nplane(s), sizeof(int));
  /* ipp defaults (ipp:12-13, 20) and the compile-time constants. */
  s->delt = 100.0; s->sorparam = 1.71; s->epsmat = 1.0e-7; s->itmax = 500;
  s->fbottom = 15844.23; s->tirr = 2048.0; s->bcxmin = 9; s->ibdrad = 9;
  s->iflimtyp = 2; s->f_incident = 2; s->ieta = 4; s->isigtyp = 0;
  s->xnue = 1.0e9; s->pr_num = 0.0; s->sigval = 0.0; s->kap0 = 1.0e-2;
  s->iii = 2; s->adjust_sor = 0; s->poles = 0; s->ikaptyp = 0;
  s->xmin = 7149199872.0; s->xmax = 1.1 * 7149199872.0;
  s->ymin = 0.0; s->ymax = 1.0; s->zmin = -0.95; s->zmax = 0.95;
  return s;
}

void ttor_destroy(ttor_state* s) {
  if (!s) return;
  for (size_t f = 0; f < NFIELDS; ++f) free(*(double**)((char*)s + FIELDS[f].off));
  free(s->UPPERBND);
  free(s->opac_lt); free(s->opac_lrh); free(s->opac_ross); free(s->opac_plnk); free(s->opac_abs);
  free(s->wave_opac); free(s->wave_bstar); free(s->XKAPW); free(s->STAU_W);
  free(s);
}

double* ttor_field(ttor_state* s, const char* name, size_t* n) {
  int n1d = (s->nx > s->ny ? (s->nx > s->nz ? s->nx : s->nz) : (s->ny > s->nz ? s->ny : s->nz)) + 4;
  for (size_t f = 0; f < NFIELDS; ++f)
    if (strcmp(FIELDS[f].name, name) == 0) {
      if (n) *n = field_count(s, &FIELDS[f], n1d);
      return *(double**)((char*)s + FIELDS[f].off);
    }
  return NULL;
}

int* ttor_ifield(ttor_state* s, const char* name, size_t* n) {
  if (strcmp(name, "UPPERBND") == 0) { if (n) *n = nplane(s); return s->UPPERBND; }
  return NULL;
}

typedef struct { const char* name; size_t off; int isint; } pdesc;
#define PD(nm, isint) {#nm, offsetof(ttor_state, nm), isint}
static const pdesc PARAMS[] = {
    PD(delt, 0), PD(sorparam, 0), PD(epsmat, 0), PD(fbottom, 0), PD(tirr, 0),
    PD(xnue, 0), PD(pr_num, 0), PD(sigval, 0), PD(kap0, 0), PD(global_rnorm, 0),
    PD(global_rhsnorm, 0), PD(global_deltaq, 0), PD(global_deltaer, 0),
    PD(xmin, 0), PD(xmax, 0), PD(ymin, 0), PD(ymax, 0), PD(zmin, 0), PD(zmax, 0),
    PD(itmax, 1), PD(bcxmin, 1), PD(ibdrad, 1), PD(iflimtyp, 1), PD(f_incident, 1),
    PD(ieta, 1), PD(isigtyp, 1), PD(iii, 1), PD(adjust_sor, 1), PD(poles, 1),
    PD(sor_iter, 1), PD(energy_iter, 1), PD(status, 1), PD(sor_total, 1),
    PD(solves, 1), PD(ikaptyp, 1),
};
int ttor_set(ttor_state* s, const char* name, double v) {
  for (size_t p = 0; p < sizeof(PARAMS) / sizeof(PARAMS[0]); ++p)
    if (strcmp(PARAMS[p].name, name) == 0) {
      if (PARAMS[p].isint) *(int*)((char*)s + PARAMS[p].off) = (int)v;
      else *(double*)((char*)s + PARAMS[p].off) = v;
      return 0;
    }
  return -1;
}
double ttor_get(ttor_state* s, const char* name) {
  for (size_t p = 0; p < sizeof(PARAMS) / sizeof(PARAMS[0]); ++p)
    if (strcmp(PARAMS[p].name, name) == 0)
      return PARAMS[p].isint ? (double)*(int*)((char*)s + PARAMS[p].off)
                             : *(double*)((char*)s + PARAMS[p].off);
  return NAN;
}

/* ---- GITTER, ppinit.f:1028-1406 (NCOSYS=2, linear grids, one rank) ---- */
int ttor_gitter(ttor_state* s) {
  const int nx = s->nx, ny = s->ny, nz = s->nz;
  double ymax1 = s->ymax * 2.0 * PI_D, ymin1 = s->ymin * 2.0 * PI_D;   /* :1064-1065 */
  double zmax1 = (s->zmax / 2.0) * PI_D, zmin1 = (s->zmin / 2.0) * PI_D; /* :1066-1067 */
  /* x grid, :1075-1093 */
  double delx = (s->xmax - s->xmin) / nx;
  for (int i = 1; i <= nx + 2; ++i) G1(dxa, i) = delx;
  G1(xxa, 1) = s->xmin + (0 * (s->xmax - s->xmin) / 1);
  G1(xxa, 0) = G1(xxa, 1) - G1(dxa, 1);
  for (int i = 2; i <= nx + 2; ++i) G1(xxa, i) = G1(xxa, i - 1) + G1(dxa, i);
  for (int i = 0; i <= nx + 1; ++i) G1(xxb, i) = (G1(xxa, i) + G1(xxa, i + 1)) / 2.0;
  {
    double dran3 = G1(dxa, nx + 2) * 1.0, xxan3 = G1(xxa, nx + 2) + dran3;
    G1(xxb, nx + 2) = (G1(xxa, nx + 2) + xxan3) / 2.0;
    dran3 = G1(dxa, 1) / 1.0; xxan3 = G1(xxa, 0) - dran3;
    G1(xxb, -1) = (G1(xxa, 0) + xxan3) / 2.0;
  }
  /* y grid, :1134-1157 */
  double dely = (ymax1 - ymin1) / ny;
  for (int j = 1; j <= ny + 2; ++j) G1(dya, j) = dely;
  G1(xya, 1) = ymin1 + (0 * (ymax1 - ymin1) / 1);
  G1(xya, 0) = G1(xya, 1) - G1(dya, 1);
  for (int j = 2; j <= ny + 2; ++j) G1(xya, j) = G1(xya, j - 1) + G1(dya, j);
  for (int j = 0; j <= ny + 1; ++j) G1(xyb, j) = (G1(xya, j) + G1(xya, j + 1)) / 2.0;
  {
    double d3 = G1(dya, ny + 2) * 1.0, x3 = G1(xya, ny + 2) + d3;
    G1(xyb, ny + 2) = (G1(xya, ny + 2) + x3) / 2.0;
    d3 = G1(dya, 1) / 1.0; x3 = G1(xya, 0) - d3;
    G1(xyb, -1) = (G1(xya, 0) + x3) / 2.0;
  }
  /* z grid, :1160-1178 */
  double delz = (zmax1 - zmin1) / nz;
  for (int k = 1; k <= nz + 2; ++k) G1(dza, k) = delz;
  G1(xza, 1) = zmin1 + (0 * (zmax1 - zmin1) / 1);
  G1(xza, 0) = G1(xza, 1) - G1(dza, 1);
  for (int k = 2; k <= nz + 2; ++k) G1(xza, k) = G1(xza, k - 1) + G1(dza, k);
  for (int k = 0; k <= nz + 1; ++k) G1(xzb, k) = (G1(xza, k) + G1(xza, k + 1)) / 2.0;
  {
    double d3 = G1(dza, nz + 2) * 1.0, x3 = G1(xza, nz + 2) + d3;
    G1(xzb, nz + 2) = (G1(xza, nz + 2) + x3) / 2.0;
    d3 = G1(dza, 1) / 1.0; x3 = G1(xza, 0) - d3;
    G1(xzb, -1) = (G1(xza, 0) + x3) / 2.0;
  }
  /* B-grid deltas, :1181-1189 */
  for (int i = 0; i <= nx + 2; ++i) G1(dxb, i) = G1(xxb, i) - G1(xxb, i - 1);
  for (int j = 0; j <= ny + 2; ++j) G1(dyb, j) = G1(xyb, j) - G1(xyb, j - 1);
  for (int k = 0; k <= nz + 2; ++k) G1(dzb, k) = G1(xzb, k) - G1(xzb, k - 1);
  /* interpolation weights, :1198-1241 (DXMIN=DYMIN=DZMIN=0) */
  for (int i = 0; i <= nx + 2; ++i) { G1(ddx0, i) = 0.5; G1(ddx1, i) = 0.5; }
  for (int j = 0; j <= ny + 2; ++j) { G1(ddy0, j) = 0.5; G1(ddy1, j) = 0.5; }
  for (int k = 0; k <= nz + 2; ++k) { G1(ddz0, k) = 0.5; G1(ddz1, k) = 0.5; }
  /* spherical metric, :1342-1400 */
  double xxa1 = G1(xxa, 1);
  if (xxa1 == 0.0) xxa1 = (double)1.e-20f;
  for (int i = 0; i <= nx + 1; ++i)
    G1(volxb, i) = (G1(xxa, i + 1) * G1(xxa, i + 1) * G1(xxa, i + 1) -
                    G1(xxa, i) * G1(xxa, i) * G1(xxa, i)) / 3.0;
  for (int i = 0; i <= nx + 2; ++i) {
    G1(surxa, i) = G1(xxa, i) * G1(xxa, i);
    G1(surxb, i) = G1(xxb, i) * G1(xxb, i);
    G1(geoxga, i) = G1(xxa, i);
    G1(geoxha, i) = G1(xxa, i);
  }
  G1(geoxga, 1) = xxa1; G1(geoxha, 1) = xxa1;
  for (int i = -1; i <= nx + 2; ++i) { G1(geoxg, i) = G1(xxb, i); G1(geoxh, i) = G1(xxb, i); }
  for (int j = 0; j <= ny + 1; ++j) G1(volyb, j) = G1(xya, j + 1) - G1(xya, j);   /* :1364 */
  for (int k = 0; k <= nz + 1; ++k) G1(volzb, k) = sin(G1(xza, k + 1)) - sin(G1(xza, k));
  for (int k = 0; k <= nz + 2; ++k) {
    G1(surza, k) = cos(G1(xza, k));
    G1(surzb, k) = cos(G1(xzb, k));
    G1(geozga, k) = cos(G1(xza, k));
  }
  for (int k = -1; k <= nz + 2; ++k) G1(geozg, k) = cos(G1(xzb, k));
  if (G1(geozga, nz + 1) == 0.0) G1(geozga, nz + 1) = (double)1.e-10f;
  if (G1(geozga, 1) == 0.0) G1(geozga, 1) = (double)1.e-10f;
  return 0;
}

/* ---- CALCMUSTAR ppsub.f:156-179 and CALC_TINCIDENT pprad.f:296-405 ----- */
int ttor_calcmustar(ttor_state* s) {
  for (int k = -1; k <= s->nz + 2; ++k)
    for (int j = -1; j <= s->ny + 2; ++j) {
      double cyz = cos(G1(xyb, j)) * cos(G1(xzb, k));
      if (s->f_incident == 2 || s->f_incident == 3 || s->f_incident == 8)
        P(MU_STAR, j, k) = fmax(cyz, (double)1.0e-7f);
      else
        P(MU_STAR, j, k) = 1.0;
      double tinc = 0.0;
      if (s->f_incident == 2 || s->f_incident == 3) {
        if (cyz >= 0) { tinc = s->tirr * pow(cyz, 0.25); tinc = fmax(tinc, 0.0); }
      } else if (s->f_incident == 4 || s->f_incident == 5) {
        tinc = s->tirr;
      }
      P(TINCIDENT, j, k) = tinc;
    }
  return 0;
}

/* ---- PLANETSHIFT ppshift.f:1009-1214 with one rank --------------------
 * With one rank MPIupper = MPIlower = self and every z or corner partner is
 * MPI_PROC_NULL (SETUP3DMPIGRID ppshift.f:795-819), so only the "from
 * lower" (:1096-1107) and "from upper" (:1164-1173) copies act. */
static void shift_halo(ttor_state* s, double* a) {
  const int nx = s->nx, ny = s->ny, nz = s->nz;
#define A(i, j, k) a[(size_t)((i) + 1) + (size_t)NXH * ((size_t)((j) + 1) + (size_t)NYH * (size_t)((k) + 1))]
  for (int k = 1; k <= nz; ++k)
    for (int i = -1; i <= nx + 2; ++i) A(i, 0, k) = A(i, ny, k);
  for (int k = 1; k <= nz; ++k)
    for (int i = -1; i <= nx + 2; ++i) A(i, -1, k) = A(i, ny - 1, k);
  for (int k = 1; k <= nz; ++k)
    for (int i = -1; i <= nx + 2; ++i) A(i, ny + 1, k) = A(i, 1, k);
  for (int k = 1; k <= nz; ++k)
    for (int i = -1; i <= nx + 2; ++i) A(i, ny + 2, k) = A(i, 2, k);
#undef A
}

/* NORTH_POLE_SHIFT and SOUTH_POLE_SHIFT (ppshift.f:2217-2453) with one
 * rank: the partner across each pole (myid -/+ numprocs/2, ppshift.f:
 * 820-833) is the rank itself, so the exchanges copy planes NZ-1, NZ-2,
 * NZ-3 onto NZ, NZ+1, NZ+2 and planes 1, 2 onto 0, -1, over the whole
 * (i, j) extent including the ghosts; nothing without poles. */
static void pole_shift(ttor_state* s, double* a) {
  if (!s->poles) return;
  const int nx = s->nx, ny = s->ny, nz = s->nz;
#define A(i, j, k) a[(size_t)((i) + 1) + (size_t)NXH * ((size_t)((j) + 1) + (size_t)NYH * (size_t)((k) + 1))]
  for (int m = 0; m < 3; ++m)
    for (int j = -1; j <= ny + 2; ++j)
      for (int i = -1; i <= nx + 2; ++i) A(i, j, nz + m) = A(i, j, nz - 1 - m);
  for (int m = 0; m < 2; ++m)
    for (int j = -1; j <= ny + 2; ++j)
      for (int i = -1; i <= nx + 2; ++i) A(i, j, -m) = A(i, j, 1 + m);
#undef A
}

/* PLANETSHIFT followed by the pole shifts, as every caller in the
 * reference pairs them when poles are on (e.g. ppenergy.f:230-245). */
int ttor_planetshift(ttor_state* s, const char* field) {
  size_t n;
  double* a = ttor_field(s, field, &n);
  if (!a || n != nhalo(s)) return -1;
  shift_halo(s, a);
  pole_shift(s, a);
  return 0;
}

/* PASSUPPERBND ppbou.f:522-682 with one rank. */
static void passupperbnd(ttor_state* s) {
  const int ny = s->ny, nz = s->nz;
  for (int k = 1; k <= nz; ++k) {
    P(UPPERBND, 0, k) = P(UPPERBND, ny, k);
    P(UPPERBND, -1, k) = P(UPPERBND, ny - 1, k);
  }
  for (int k = 1; k <= nz; ++k) {
    P(UPPERBND, ny + 1, k) = P(UPPERBND, 1, k);
    P(UPPERBND, ny + 2, k) = P(UPPERBND, 2, k);
  }
  /* processor boundaries, :619-674 */
  P(UPPERBND, 0, 0) = P(UPPERBND, 0, 1); P(UPPERBND, 0, -1) = P(UPPERBND, 0, 1);
  P(UPPERBND, -1, 0) = P(UPPERBND, -1, 1); P(UPPERBND, -1, -1) = P(UPPERBND, -1, 1);
  P(UPPERBND, 0, nz + 1) = P(UPPERBND, 0, nz); P(UPPERBND, 0, nz + 2) = P(UPPERBND, 0, nz);
  P(UPPERBND, -1, nz + 1) = P(UPPERBND, -1, nz); P(UPPERBND, -1, nz + 2) = P(UPPERBND, -1, nz);
  for (int j = 1; j <= ny; ++j) {
    P(UPPERBND, j, nz + 1) = P(UPPERBND, j, nz);
    P(UPPERBND, j, nz + 2) = P(UPPERBND, j, nz);
  }
  P(UPPERBND, ny + 1, nz + 1) = P(UPPERBND, ny + 1, nz);
  P(UPPERBND, ny + 1, nz + 2) = P(UPPERBND, ny + 1, nz);
  P(UPPERBND, ny + 2, nz + 1) = P(UPPERBND, ny + 2, nz);
  P(UPPERBND, ny + 2, nz + 2) = P(UPPERBND, ny + 2, nz);
  P(UPPERBND, ny + 1, 0) = P(UPPERBND, ny + 1, 1); P(UPPERBND, ny + 1, -1) = P(UPPERBND, ny + 1, 1);
  P(UPPERBND, ny + 2, 0) = P(UPPERBND, ny + 2, 1); P(UPPERBND, ny + 2, -1) = P(UPPERBND, ny + 2, 1);
  for (int j = 1; j <= ny; ++j) {
    P(UPPERBND, j, 0) = P(UPPERBND, j, 1);
    P(UPPERBND, j, -1) = P(UPPERBND, j, 1);
  }
}

/* Synthetic analytic opacity standing in for BurrowsOPC in KAPPA's
 * IKAPTYP 20:25 branch (pprphy.f:321-351): same extents, kappa_R =
 * kap0 * sqrt(rho) * (T/1000)^1.5 * KMUL, kappa_P = kappa_A = kappa_R and
 * zero temperature derivatives (the IKAPTYP=3 convention, pprphy.f:84-87). */
static double kap_formula(const ttor_state* s, double t, double rh, double kmul) {
  double th = t / 1000.0;
  return ((s->kap0 * sqrt(rh)) * (th * sqrt(th))) * kmul;
}

/* BurrowsOPC pprphy.f:1005-1229 (Rosseland, Planck, absorption means and
 * the T-derivative stand-ins of :1180-1185).  Returns 0, or 1 T <= 0, 2
 * above the table, 3 below it, 4 a non-positive opacity. */
static int burrows_opc(const ttor_state* s, double t, double rh, double* kp, double* kr, double* ka, double* dkp,
                       double* dka) {
  if (!(t > 0.0)) return 1;
  double rh1 = log10(rh), tm1 = log10(t);
  if (tm1 < (double)1.69896f) tm1 = (double)1.69897f;
  if (tm1 > (double)3.69889f) tm1 = (double)3.69888f;
  if (rh1 < (double)-11.9996f) rh1 = (double)-11.9995f;
  if (rh1 > (double)-1.99993f) rh1 = (double)-1.99994f;
  const int nt = s->opac_nt, nr = s->opac_nrh;
  int K;
  for (K = 1; K <= nt; ++K)
    if (s->opac_lt[K - 1] > tm1) break;
  if (K == nt + 1) return 2;
  const int it = K, it1 = K - 1;
  if (it1 == 0) return 3;
  double ws1 = s->opac_lt[it1 - 1] - tm1;
  double ws = s->opac_lt[it1 - 1] - s->opac_lt[it - 1];
  ws1 = ws1 / ws;
  ws = 1.0 - ws1;
  for (K = 1; K <= nr; ++K)
    if (s->opac_lrh[K - 1] > rh1) break;
  if (K == nr + 1) return 2;
  const int iw = K, iw1 = K - 1;
  if (iw1 == 0) return 3;
  double ws2 = rh1 - s->opac_lrh[iw1 - 1];
  double ws3 = s->opac_lrh[iw - 1] - s->opac_lrh[iw1 - 1];
  ws2 = ws2 / ws3;
  ws3 = 1.0 - ws2;
#define TB(a, p, q) a[(size_t)((p) - 1) + (size_t)nt * (size_t)((q) - 1)]
  const double* tabs[3] = {s->opac_ross, s->opac_plnk, s->opac_abs};
  double out[3];
  for (int m = 0; m < 3; ++m) {
    const double* a = tabs[m];
    const double w4 = ws2 * (ws1 * TB(a, it, iw) + ws * TB(a, it1, iw));
    const double w5 = ws3 * (ws1 * TB(a, it, iw1) + ws * TB(a, it1, iw1));
    out[m] = pow(10.0, w4 + w5);
  }
  *kr = out[0]; *kp = out[1]; *ka = out[2];
  const double dt = pow(10.0, s->opac_lt[it - 1]) - pow(10.0, s->opac_lt[it1 - 1]);
  *dkp = (pow(10.0, TB(s->opac_plnk, it, iw)) - pow(10.0, TB(s->opac_plnk, it1, iw))) / dt;
  *dka = (pow(10.0, TB(s->opac_abs, it, iw)) - pow(10.0, TB(s->opac_abs, it1, iw))) / dt;
#undef TB
  if (*kr <= 0.0 || *kp <= 0.0 || *ka <= 0.0) return 4;
  return 0;
}

int ttor_set_opacity_table(ttor_state* s, int nt, int nrh, const double* lt, const double* lrh,
                           const double* ross, const double* plnk, const double* absk) {
  if (nt < 2 || nrh < 2) return -1;
  free(s->opac_lt); free(s->opac_lrh); free(s->opac_ross); free(s->opac_plnk); free(s->opac_abs);
  const size_t nn = (size_t)nt * nrh;
  s->opac_lt = (double*)malloc(nt * sizeof(double));
  s->opac_lrh = (double*)malloc(nrh * sizeof(double));
  s->opac_ross = (double*)malloc(nn * sizeof(double));
  s->opac_plnk = (double*)malloc(nn * sizeof(double));
  s->opac_abs = (double*)malloc(nn * sizeof(double));
  if (!s->opac_lt || !s->opac_lrh || !s->opac_ross || !s->opac_plnk || !s->opac_abs) return -2;
  memcpy(s->opac_lt, lt, nt * sizeof(double));
  memcpy(s->opac_lrh, lrh, nrh * sizeof(double));
  memcpy(s->opac_ross, ross, nn * sizeof(double));
  memcpy(s->opac_plnk, plnk, nn * sizeof(double));
  memcpy(s->opac_abs, absk, nn * sizeof(double));
  s->opac_nt = nt;
  s->opac_nrh = nrh;
  return 0;
}

/* BurrowsOPC's per-bin opacities (pprphy.f:1138-1151) at the bracketing of
 * (T, rho) burrows_opc uses: 10**(bilinear of log BurrowsXKAP_waveopac). */
static int burrows_wave(const ttor_state* s, double t, double rh, double* kw) {
  double rh1 = log10(rh), tm1 = log10(t);
  if (tm1 < (double)1.69896f) tm1 = (double)1.69897f;
  if (tm1 > (double)3.69889f) tm1 = (double)3.69888f;
  if (rh1 < (double)-11.9996f) rh1 = (double)-11.9995f;
  if (rh1 > (double)-1.99993f) rh1 = (double)-1.99994f;
  const int nt = s->opac_nt, nr = s->opac_nrh;
  int K;
  for (K = 1; K <= nt; ++K)
    if (s->opac_lt[K - 1] > tm1) break;
  if (K == nt + 1 || K == 1) return 2;
  const int it = K, it1 = K - 1;
  double ws1 = s->opac_lt[it1 - 1] - tm1;
  double ws = s->opac_lt[it1 - 1] - s->opac_lt[it - 1];
  ws1 = ws1 / ws;
  ws = 1.0 - ws1;
  for (K = 1; K <= nr; ++K)
    if (s->opac_lrh[K - 1] > rh1) break;
  if (K == nr + 1 || K == 1) return 2;
  const int iw = K, iw1 = K - 1;
  double ws2 = rh1 - s->opac_lrh[iw1 - 1];
  double ws3 = s->opac_lrh[iw - 1] - s->opac_lrh[iw1 - 1];
  ws2 = ws2 / ws3;
  ws3 = 1.0 - ws2;
  const size_t nn = (size_t)nt * nr;
#define TW(p, q, l) s->wave_opac[(size_t)((p) - 1) + (size_t)nt * (size_t)((q) - 1) + nn * (size_t)(l)]
  for (int l = 0; l < s->wave_nb; ++l) {
    const double w4 = ws2 * (ws1 * TW(it, iw, l) + ws * TW(it1, iw, l));
    const double w5 = ws3 * (ws1 * TW(it, iw1, l) + ws * TW(it1, iw1, l));
    kw[l] = pow(10.0, w4 + w5);
  }
#undef TW
  return 0;
}

int ttor_set_wave_table(ttor_state* s, int nb, const double* waveopac, const double* bstar, double rstar,
                        double semi) {
  if (nb < 1 || s->opac_nt < 2 || !waveopac || !bstar || !(semi > 0.0)) return -1;
  free(s->wave_opac); free(s->wave_bstar); free(s->XKAPW); free(s->STAU_W);
  const size_t nn = (size_t)s->opac_nt * s->opac_nrh * nb;
  s->wave_opac = (double*)malloc(nn * sizeof(double));
  s->wave_bstar = (double*)malloc(nb * sizeof(double));
  s->XKAPW = (double*)calloc(nhalo(s) * nb, sizeof(double));
  s->STAU_W = (double*)calloc(nhalo(s) * nb, sizeof(double));
  if (!s->wave_opac || !s->wave_bstar || !s->XKAPW || !s->STAU_W) return -2;
  memcpy(s->wave_opac, waveopac, nn * sizeof(double));
  memcpy(s->wave_bstar, bstar, nb * sizeof(double));
  s->wave_nb = nb;
  s->wave_rstar = rstar;
  s->wave_semi = semi;
  return 0;
}

/* The node values of FreedmanTVAL / FreedmanPVAL (ppmod.f:690-700; P in mbar). */
static const double FREED_T[42] = {
    75.0, 100.0, 110.0, 120.0, 130.0, 140.0, 150.0, 160.0, 170.0, 180.0, 190.0, 200.0, 210.0, 220.0,
    230.0, 240.0, 250.0, 275.0, 300.0, 400.0, 500.0, 575.0, 650.0, 725.0, 800.0, 900.0, 1000.0, 1100.0,
    1200.0, 1300.0, 1400.0, 1500.0, 1600.0, 1700.0, 1800.0, 1900.0, 2000.0, 2300.0, 2600.0, 3000.0,
    3500.0, 4000.0};
static const double FREED_P[18] = {0.001, 0.003, 0.01, 0.03, 0.1, 0.3, 1.0, 3.0, 10.0,
                                   30.0, 100.0, 300.0, 1000.0, 3000.0, 10000.0, 30000.0, 100000.0, 300000.0};

/* FreedmanOPC pprphy.f:800-942 at (T, P_gas in dyn/cm^2): P in mbar, the
 * clamps of :830-833, the first node above T and above P, weights linear
 * in T and P (WS3 = 1. - WS2 with a REAL*4 1., exactly 1), 10** of the
 * bilinear log means, the T-derivative stand-ins of :895-899.  Returns 0,
 * or 1 T <= 0, 2 above / 3 below the nodes, 4 a non-positive opacity. */
static int freedman_opc(const ttor_state* s, double t, double pg, double* kp, double* kr, double* ka, double* dkp,
                        double* dka) {
  if (t <= 0.0) return 1;
  double pg1 = pg * (0.001);
  double tm1 = t;
  if (tm1 < 75.0) tm1 = 75.001;
  if (tm1 > 4000.0) tm1 = 3999.9;
  if (pg1 < 0.001) pg1 = 0.001001;
  if (pg1 > 300000.0) pg1 = 299999.9;
  int K;
  for (K = 1; K <= 42; ++K)
    if (FREED_T[K - 1] > tm1) break;
  if (K == 43) return 2;
  const int it = K, it1 = K - 1;
  if (it1 == 0) return 3;
  double ws1 = FREED_T[it1 - 1] - tm1;
  double ws = FREED_T[it1 - 1] - FREED_T[it - 1];
  ws1 = ws1 / ws;
  ws = 1.0 - ws1;
  for (K = 1; K <= 18; ++K)
    if (FREED_P[K - 1] > pg1) break;
  if (K == 19) return 2;
  const int iw = K, iw1 = K - 1;
  if (iw1 == 0) return 3;
  double ws2 = pg1 - FREED_P[iw1 - 1];
  double ws3 = FREED_P[iw - 1] - FREED_P[iw1 - 1];
  ws2 = ws2 / ws3;
  ws3 = 1.0 - ws2;
#define TF(a, p, q) a[(size_t)((p) - 1) + (size_t)42 * (size_t)((q) - 1)]
  const double* tabs[3] = {s->freed_ross, s->freed_plnk, s->freed_abs};
  double out[3];
  for (int m = 0; m < 3; ++m) {
    const double* a = tabs[m];
    const double w4 = ws2 * (ws1 * TF(a, it, iw) + ws * TF(a, it1, iw));
    const double w5 = ws3 * (ws1 * TF(a, it, iw1) + ws * TF(a, it1, iw1));
    out[m] = pow(10.0, w4 + w5);
  }
  *kr = out[0]; *kp = out[1]; *ka = out[2];
  *dkp = ((pow(10.0, TF(s->freed_plnk, it, iw))) - (pow(10.0, TF(s->freed_plnk, it1, iw)))) /
         (FREED_T[it - 1] - FREED_T[it1 - 1]);
  *dka = ((pow(10.0, TF(s->freed_abs, it, iw))) - (pow(10.0, TF(s->freed_abs, it1, iw)))) /
         (FREED_T[it - 1] - FREED_T[it1 - 1]);
#undef TF
  if (*kr <= 0.0 || *kp <= 0.0 || *ka <= 0.0) return 4;
  return 0;
}

int ttor_set_freedman_table(ttor_state* s, const double* ross, const double* plnk, const double* absk,
                            double mu_gas) {
  if (!ross || !plnk || !absk || !(mu_gas > 0.0)) return -1;
  memcpy(s->freed_ross, ross, sizeof(s->freed_ross));
  memcpy(s->freed_plnk, plnk, sizeof(s->freed_plnk));
  memcpy(s->freed_abs, absk, sizeof(s->freed_abs));
  s->freed_mu = mu_gas;
  s->freed_set = 1;
  return 0;
}

int ttor_kappa(ttor_state* s) {
  const int nx = s->nx, ny = s->ny, nz = s->nz;
  if (s->freed_set) {   /* the IKAPTYP 4:5 branch, MODTYP 2, pprphy.f:88-110 */
    for (int k = -1; k <= nz + 2; ++k)
      for (int j = -1; j <= ny + 2; ++j) {
        int ub = P(UPPERBND, j, k);
        if (ub < -1 || ub > nx + 2) return -2;
        for (int i = -1; i <= ub; ++i) {
          /* PRESSG, ideal gas (ppphy.f:17-20): PG = Rgas*T*RH/mu_gas */
          const double pg = RGAS_C * H(T, i, j, k) * H(RH, i, j, k) / s->freed_mu;
          double kp, kr, ka, dkp, dka;
          if (freedman_opc(s, H(T, i, j, k), pg, &kp, &kr, &ka, &dkp, &dka)) return -10;
          H(XKAPP, i, j, k) = kp; H(XKAPR, i, j, k) = kr; H(XKAPA, i, j, k) = ka;
          H(DXKAPP_DT, i, j, k) = dkp; H(DXKAPA_DT, i, j, k) = dka;
        }
        for (int i = ub + 1; i <= nx + 2; ++i) {
          H(XKAPR, i, j, k) = H(XKAPR, ub, j, k);
          H(XKAPP, i, j, k) = H(XKAPP, ub, j, k);
          H(XKAPA, i, j, k) = H(XKAPA, ub, j, k);
          H(DXKAPP_DT, i, j, k) = H(DXKAPP_DT, ub, j, k);
          H(DXKAPA_DT, i, j, k) = H(DXKAPA_DT, ub, j, k);
        }
      }
    return 0;
  }
  if (s->opac_nt > 0) {   /* the IKAPTYP 20:25 branch with BurrowsOPC, pprphy.f:321-351 */
    for (int k = -1; k <= nz + 2; ++k)
      for (int j = -1; j <= ny + 2; ++j) {
        int ub = P(UPPERBND, j, k);
        if (ub < 1 || ub > nx + 1) return -2;
        for (int i = -1; i <= ub; ++i) {
          double kp, kr, ka, dkp, dka;
          if (burrows_opc(s, H(T, i, j, k), H(RH, i, j, k), &kp, &kr, &ka, &dkp, &dka)) return -10;
          H(XKAPP, i, j, k) = kp; H(XKAPR, i, j, k) = kr; H(XKAPA, i, j, k) = ka;
          H(DXKAPP_DT, i, j, k) = dkp; H(DXKAPA_DT, i, j, k) = dka;
          if (s->wave_nb > 0) {
            double kw[64];
            if (s->wave_nb > 64 || burrows_wave(s, H(T, i, j, k), H(RH, i, j, k), kw)) return -10;
            for (int l = 0; l < s->wave_nb; ++l) s->XKAPW[hidx(s, i, j, k) + nhalo(s) * (size_t)l] = kw[l];
          }
        }
        for (int i = ub; i <= nx + 2; ++i) {
          H(XKAPR, i, j, k) = H(XKAPR, ub - 1, j, k);
          H(XKAPP, i, j, k) = H(XKAPP, ub - 1, j, k);
          H(XKAPA, i, j, k) = H(XKAPA, ub - 1, j, k);
          H(DXKAPP_DT, i, j, k) = H(DXKAPP_DT, ub - 1, j, k);
          H(DXKAPA_DT, i, j, k) = H(DXKAPA_DT, ub - 1, j, k);
          for (int l = 0; l < s->wave_nb; ++l)
            s->XKAPW[hidx(s, i, j, k) + nhalo(s) * (size_t)l] = s->XKAPW[hidx(s, ub - 1, j, k) + nhalo(s) * (size_t)l];
        }
      }
    return 0;
  }
  for (int k = -1; k <= nz + 2; ++k)
    for (int j = -1; j <= ny + 2; ++j) {
      int ub = P(UPPERBND, j, k);
      if (ub < 1 || ub > nx + 1) return -2;
      for (int i = -1; i <= ub; ++i) {
        double kr = kap_formula(s, H(T, i, j, k), H(RH, i, j, k), H(KMUL, i, j, k));
        H(XKAPR, i, j, k) = kr; H(XKAPP, i, j, k) = kr; H(XKAPA, i, j, k) = kr;
        H(DXKAPP_DT, i, j, k) = 0.0; H(DXKAPA_DT, i, j, k) = 0.0;
      }
      for (int i = ub; i <= nx + 2; ++i) {
        H(XKAPR, i, j, k) = H(XKAPR, ub - 1, j, k);
        H(XKAPP, i, j, k) = H(XKAPP, ub - 1, j, k);
        H(XKAPA, i, j, k) = H(XKAPA, ub - 1, j, k);
        H(DXKAPP_DT, i, j, k) = H(DXKAPP_DT, ub - 1, j, k);
        H(DXKAPA_DT, i, j, k) = H(DXKAPA_DT, ub - 1, j, k);
      }
    }
  return 0;
}

/* SUBSIG pprphy.f:567-583: sig is uniform, kept as a scalar. */
static void subsig(ttor_state* s) { s->sigval = (s->isigtyp == 1) ? 0.4 : 0.0; }

/* QDENS ppphy.f:47-76 */
int ttor_qdens(ttor_state* s) {
  const int nx = s->nx, ny = s->ny, nz = s->nz;
  for (int k = -1; k <= nz + 2; ++k)
    for (int j = -1; j <= ny + 2; ++j)
      for (int i = 0; i <= nx + 2; ++i)
        H(RHQX, i, j, k) = G1(ddx1, i) * H(RH, i, j, k) + G1(ddx0, i) * H(RH, i - 1, j, k);
  for (int k = -1; k <= nz + 2; ++k)
    for (int j = 0; j <= ny + 2; ++j)
      for (int i = -1; i <= nx + 2; ++i)
        H(RHQY, i, j, k) = G1(ddy1, j) * H(RH, i, j, k) + G1(ddy0, j) * H(RH, i, j - 1, k);
  for (int k = 0; k <= nz + 2; ++k)
    for (int j = -1; j <= ny + 2; ++j)
      for (int i = -1; i <= nx + 2; ++i)
        H(RHQZ, i, j, k) = G1(ddz1, k) * H(RH, i, j, k) + G1(ddz0, k) * H(RH, i, j, k - 1);
  return 0;
}

/* FLIM pprphy.f:362-565 (IFLIMTYP 1 and 2; irad=3). */
int ttor_flim(ttor_state* s) {
  const int nx = s->nx, ny = s->ny, nz = s->nz;
  const double xdmin = 1.0e-50;
  if (s->energy_iter <= 1) {            /* :396-402 */
    int rc = ttor_kappa(s);
    if (rc) return rc;
    subsig(s);
    ttor_qdens(s);
  }
  const double sg = s->sigval;
  if (s->iflimtyp == 1) {               /* :405-409 */
    for (size_t q = 0; q < nface(s); ++q) s->FLIMX[q] = s->FLIMY[q] = s->FLIMZ[q] = 1.0 / 3.0;
    return 0;
  }
  if (s->iflimtyp != 2) return -3;
  int xmax_index = 0;
  for (int k = 1; k <= nz; ++k)         /* x-direction :414-456 */
    for (int j = 1; j <= ny; ++j) {
      xmax_index = P(UPPERBND, j, k) - 1;
      for (int i = 1; i <= xmax_index; ++i) {
        double gradx = (H(ER, i, j, k) - H(ER, i - 1, j, k)) / G1(dxb, i);
        double grady = (G1(ddx1, i) * (H(ER, i, j + 1, k) - H(ER, i, j - 1, k)) +
                        G1(ddx0, i) * (H(ER, i - 1, j + 1, k) - H(ER, i - 1, j - 1, k))) /
                       (G1(geoxga, i) * G1(geozg, k) * (G1(xyb, j + 1) - G1(xyb, j - 1)));
        double gradz = (G1(ddx1, i) * (H(ER, i, j, k + 1) - H(ER, i, j, k - 1)) +
                        G1(ddx0, i) * (H(ER, i - 1, j, k + 1) - H(ER, i - 1, j, k - 1))) /
                       (G1(geoxha, i) * (G1(xzb, k + 1) - G1(xzb, k - 1)));
        double grad = sqrt(gradx * gradx + grady * grady + gradz * gradz) + xdmin;
        double rrx = 2.0 * grad /
                     (H(RHQX, i, j, k) *
                      (G1(ddx1, i) * (H(XKAPR, i, j, k) + sg) + G1(ddx0, i) * (H(XKAPR, i - 1, j, k) + sg)) *
                      (H(ER, i, j, k) + H(ER, i - 1, j, k)));
        F(FLIMX, i, j, k) = (2.0 + rrx) / (6.0 + 3.0 * rrx + rrx * rrx);
      }
      int ub = P(UPPERBND, j, k);
      for (int i = ub; i <= nx + 1; ++i) F(FLIMX, i, j, k) = F(FLIMX, ub - 1, j, k);
    }
  /* y-direction :462-491 -- reuses the last x-loop xmax_index (:464) */
  for (int k = 1; k <= nz; ++k)
    for (int j = 1; j <= ny + 1; ++j) {
      for (int i = 1; i <= xmax_index; ++i) {
        double gradx = (G1(ddy1, j) * (H(ER, i + 1, j, k) - H(ER, i - 1, j, k)) +
                        G1(ddy0, j) * (H(ER, i + 1, j - 1, k) - H(ER, i - 1, j - 1, k))) /
                       (G1(xxb, i + 1) - G1(xxb, i - 1));
        double grady = (H(ER, i, j, k) - H(ER, i, j - 1, k)) / (G1(geoxg, i) * G1(geozg, k) * G1(dyb, j));
        double gradz = (G1(ddy1, j) * (H(ER, i, j, k + 1) - H(ER, i, j, k - 1)) +
                        G1(ddy0, j) * (H(ER, i, j - 1, k + 1) - H(ER, i, j - 1, k - 1))) /
                       ((G1(xzb, k + 1) - G1(xzb, k - 1)) * G1(geoxh, i));
        double grad = sqrt(gradx * gradx + grady * grady + gradz * gradz) + xdmin;
        double rry = 2.0 * grad /
                     (H(RHQY, i, j, k) *
                      (G1(ddy1, j) * (H(XKAPR, i, j, k) + sg) + G1(ddy0, j) * (H(XKAPR, i, j - 1, k) + sg)) *
                      (H(ER, i, j, k) + H(ER, i, j - 1, k)));
        F(FLIMY, i, j, k) = (2.0 + rry) / (6.0 + 3.0 * rry + rry * rry);
      }
      int ub = P(UPPERBND, j, k);
      for (int i = ub; i <= nx; ++i) F(FLIMY, i, j, k) = F(FLIMY, ub - 1, j, k);
    }
  /* z-direction :493-522 */
  for (int k = 1; k <= nz + 1; ++k)
    for (int j = 1; j <= ny; ++j) {
      for (int i = 1; i <= xmax_index; ++i) {
        double gradx = (G1(ddz1, k) * (H(ER, i + 1, j, k) - H(ER, i - 1, j, k)) +
                        G1(ddz0, k) * (H(ER, i + 1, j, k - 1) - H(ER, i - 1, j, k - 1))) /
                       (G1(xxb, i + 1) - G1(xxb, i - 1));
        double grady = (G1(ddz1, k) * (H(ER, i, j + 1, k) - H(ER, i, j - 1, k)) +
                        G1(ddz0, k) * (H(ER, i, j + 1, k - 1) - H(ER, i, j - 1, k - 1))) /
                       ((G1(xyb, j + 1) - G1(xyb, j - 1)) * G1(geoxg, i) * G1(geozga, k));
        double gradz = (H(ER, i, j, k) - H(ER, i, j, k - 1)) / (G1(geoxh, i) * G1(dzb, k));
        double grad = sqrt(gradx * gradx + grady * grady + gradz * gradz) + xdmin;
        double rrz = 2.0 * grad /
                     (H(RHQZ, i, j, k) *
                      (G1(ddz1, k) * (H(XKAPR, i, j, k) + sg) + G1(ddz0, k) * (H(XKAPR, i, j, k - 1) + sg)) *
                      (H(ER, i, j, k) + H(ER, i, j, k - 1)));
        F(FLIMZ, i, j, k) = (2.0 + rrz) / (6.0 + 3.0 * rrz + rrz * rrz);
      }
      int ub = P(UPPERBND, j, k);
      for (int i = ub; i <= nx; ++i) F(FLIMZ, i, j, k) = F(FLIMZ, ub - 1, j, k);
    }
  return 0;
}

/* DIFF pprad.f:74-156 */
int ttor_diff(ttor_state* s) {
  const int nx = s->nx, ny = s->ny, nz = s->nz;
  int rc = ttor_flim(s);
  if (rc) return rc;
  const double sg = s->sigval;
  for (int k = 1; k <= nz; ++k)
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx + 1; ++i) {
        F(DIFRX, i, j, k) = FD_C * F(FLIMX, i, j, k) /
                            (G1(dxb, i) * H(RHQX, i, j, k) *
                             (G1(ddx1, i) * (H(XKAPR, i, j, k) + sg) + G1(ddx0, i) * (H(XKAPR, i - 1, j, k) + sg)));
        if (s->ieta == 5) {
          double difr_min = H(RHQX, i, j, k) * H(CV, i, j, k) * s->xnue /
                            (G1(dxb, i) * 4.0 * ARAD_C *
                             p3(G1(ddx1, i) * H(T, i, j, k) + G1(ddx0, i) * H(T, i - 1, j, k)) * s->pr_num);
          F(DIFRX, i, j, k) = fmax(F(DIFRX, i, j, k), difr_min);
        }
      }
  for (int k = 1; k <= nz; ++k)
    for (int j = 1; j <= ny + 1; ++j)
      for (int i = 1; i <= nx; ++i) {
        F(DIFRY, i, j, k) = FD_C * F(FLIMY, i, j, k) /
                            (G1(dyb, j) * G1(geoxg, i) * G1(geozg, k) * H(RHQY, i, j, k) *
                             (G1(ddy1, j) * (H(XKAPR, i, j, k) + sg) + G1(ddy0, j) * (H(XKAPR, i, j - 1, k) + sg)));
        if (s->ieta == 5) {
          double difr_min = H(RHQY, i, j, k) * H(CV, i, j, k) * s->xnue /
                            (G1(dyb, j) * G1(geoxg, i) * G1(geozg, k) * 4.0 * ARAD_C *
                             p3(G1(ddy1, j) * H(T, i, j, k) + G1(ddy0, j) * H(T, i, j - 1, k)) * s->pr_num);
          F(DIFRY, i, j, k) = fmax(F(DIFRY, i, j, k), difr_min);
        }
      }
  for (int k = 1; k <= nz + 1; ++k)
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i) {
        F(DIFRZ, i, j, k) = FD_C * F(FLIMZ, i, j, k) /
                            (G1(dzb, k) * G1(geoxh, i) * H(RHQZ, i, j, k) *
                             (G1(ddz1, k) * (H(XKAPR, i, j, k) + sg) + G1(ddz0, k) * (H(XKAPR, i, j, k - 1) + sg)));
        if (s->ieta == 5) {
          double difr_min = H(RHQZ, i, j, k) * H(CV, i, j, k) * s->xnue /
                            (G1(dzb, k) * G1(geoxh, i) * 4.0 * ARAD_C *
                             p3(G1(ddz1, k) * H(T, i, j, k) + G1(ddz0, k) * H(T, i, j, k - 1)) * s->pr_num);
          F(DIFRZ, i, j, k) = fmax(F(DIFRZ, i, j, k), difr_min);
        }
      }
  return 0;
}

/* CALCULATEFLUX ppenergy.f:880-920 */
int ttor_calculateflux(ttor_state* s) {
  const int nx = s->nx, ny = s->ny, nz = s->nz;
  int rc = ttor_diff(s);
  if (rc) return rc;
  for (int k = 1; k <= nz; ++k)
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx + 1; ++i)
        F(FLUX_X, i, j, k) = -F(DIFRX, i, j, k) * (H(ER, i, j, k) - H(ER, i - 1, j, k));
  for (int k = 1; k <= nz; ++k)
    for (int j = 1; j <= ny + 1; ++j)
      for (int i = 1; i <= nx; ++i)
        F(FLUX_Y, i, j, k) = -F(DIFRY, i, j, k) * (H(ER, i, j, k) - H(ER, i, j - 1, k));
  for (int k = 1; k <= nz + 1; ++k)
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i)
        F(FLUX_Z, i, j, k) = -F(DIFRZ, i, j, k) * (H(ER, i, j, k) - H(ER, i, j, k - 1));
  return 0;
}

/* FLUX_BC ppenergy.f:922-982 */
int ttor_flux_bc(ttor_state* s) {
  const int nx = s->nx, ny = s->ny, nz = s->nz;
  for (int k = 1; k <= nz; ++k)
    for (int j = 1; j <= ny; ++j) {
      int ub = P(UPPERBND, j, k);
      for (int i = ub; i <= nx + 1; ++i) {
        F(FLUX_X, i, j, k) = FD_C * H(ER, ub - 1, j, k) / 2.0;
        if (i != nx + 1) { F(FLUX_Y, i, j, k) = 0.0; F(FLUX_Z, i, j, k) = 0.0; }
      }
      F(FLUX_X, 1, j, k) = s->fbottom;
    }
  return 0;
}

/* FILL_EVALUES ppenergy.f:984-1030 */
int ttor_fill_evalues(ttor_state* s, double theta) {
  const int nx = s->nx, ny = s->ny, nz = s->nz;
  for (int k = 1; k <= nz; ++k)
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i) {
        C(EVAL1, i, j, k) = -G1(surxa, i + 1) * F(DIFRX, i + 1, j, k) / (G1(surxb, i) * G1(dxa, i));
        C(EVAL2, i, j, k) = -G1(surxa, i) * F(DIFRX, i, j, k) / (G1(surxb, i) * G1(dxa, i));
        C(EVAL3, i, j, k) = -F(DIFRY, i, j + 1, k) / (G1(xxb, i) * G1(surzb, k) * G1(dya, j));
        C(EVAL4, i, j, k) = -F(DIFRY, i, j, k) / (G1(xxb, i) * G1(surzb, k) * G1(dya, j));
        C(EVAL5, i, j, k) = -F(DIFRZ, i, j, k + 1) * G1(surza, k + 1) / (G1(xxb, i) * G1(surzb, k) * G1(dza, k));
        C(EVAL6, i, j, k) = -F(DIFRZ, i, j, k) * G1(surza, k) / (G1(xxb, i) * G1(surzb, k) * G1(dza, k));
        C(EVAL7, i, j, k) = 1.0 + (1.0 - C(JACOB_ETA, i, j, k)) * s->delt * H(RH, i, j, k) *
                                      H(XKAPP, i, j, k) * FD_C;
        C(EVAL8, i, j, k) = (C(JACOB_ETA, i, j, k) * (1.0 - theta) - 1.0) * s->delt;
        C(EVAL_1_6, i, j, k) = C(EVAL1, i, j, k) + C(EVAL2, i, j, k) + C(EVAL3, i, j, k) +
                               C(EVAL4, i, j, k) + C(EVAL5, i, j, k) + C(EVAL6, i, j, k);
      }
  return 0;
}

/* CALCULATEDIVF_WITHF ppenergy.f:825-878, NCOSYS=2 branch (:853-867). */
int ttor_calculatedivf_withf(ttor_state* s, int which, double theta) {
  const int nx = s->nx, ny = s->ny, nz = s->nz;
  double* out = which ? s->DIVF_OLD : s->DIVF;
  for (int k = 1; k <= nz; ++k)
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i) {
        double xb = G1(xxb, i), szb = G1(surzb, k);
        double v = ((G1(surxa, i + 1) / (G1(surxb, i) * G1(dxa, i))) * F(FLUX_X, i + 1, j, k) -
                    (G1(surxa, i) / (G1(surxb, i) * G1(dxa, i))) * F(FLUX_X, i, j, k)) +
                   ((1.0 / (xb * szb * G1(dya, j))) * F(FLUX_Y, i, j + 1, k) -
                    (1.0 / (xb * szb * G1(dya, j))) * F(FLUX_Y, i, j, k)) +
                   ((G1(surza, k + 1) / (xb * szb * G1(dza, k))) * F(FLUX_Z, i, j, k + 1) -
                    (G1(surza, k) / (xb * szb * G1(dza, k))) * F(FLUX_Z, i, j, k));
        out[(size_t)(i - 1) + (size_t)nx * ((size_t)(j - 1) + (size_t)ny * (size_t)(k - 1))] = v;
      }
  return ttor_fill_evalues(s, theta);
}

/* CALCSTELLARTAU pprad.f:191-221, STELLAR_DTAU pprad.f:223-242 and the grey
 * branch of STELLARINPUT_HEATING pprad.f:490-502.  STELLARINPUT is declared
 * (1:NX, -1:NY+2, -1:NZ+2) (ppmod.f:341); the reference loop runs i to
 * NX+2 and its last two writes land in the next column, which the loop
 * then overwrites, so only i = 1..NX is kept here. */
/* The wavelength-binned branch of STELLARINPUT_HEATING for IKAPTYP 20-24
 * (pprad.f:433-448): WAVELENGTH_CALCSTELLARTAU (pprad.f:519-547: per bin,
 * the optical depth summed from UPPERBND inward, zero elsewhere),
 * WAVELENGTH_STELLAR_DTAU (:549-568: central differences for i = 2..NX,
 * dtaus(1) = dtaus(2), dtaus(NX+1) = 0), then the bins summed in order,
 * times (RSTAR*RSOL/semi)**2 / dxb(i).  STELLARINPUT is formed for
 * i = 1..NX, its declared extent. */
static int stellar_binned(ttor_state* s) {
  const int nx = s->nx, ny = s->ny, nz = s->nz, nb = s->wave_nb;
  const size_t nh = nhalo(s);
  double dr = G1(xxb, 2) - G1(xxb, 1);
  for (size_t q = 0; q < nh * (size_t)nb; ++q) s->STAU_W[q] = 0.0;
  for (int k = -1; k <= nz + 2; ++k)
    for (int j = -1; j <= ny + 2; ++j) {
      double tot[64];
      for (int l = 0; l < nb; ++l) tot[l] = 0.0;
      int ub = P(UPPERBND, j, k);
      if (ub > nx + 1) ub = nx + 1;
      for (int i = ub; i >= 1; --i)
        for (int l = 0; l < nb; ++l) {
          tot[l] = tot[l] + (s->XKAPW[hidx(s, i, j, k) + nh * (size_t)l] * H(RH, i, j, k) * dr);
          s->STAU_W[hidx(s, i, j, k) + nh * (size_t)l] = tot[l];
        }
    }
  const double f = s->wave_rstar * RSOL_C / s->wave_semi;
  const double geo = f * f;
  for (int k = -1; k <= nz + 2; ++k)
    for (int j = -1; j <= ny + 2; ++j) {
      const double mu = P(MU_STAR, j, k);
      for (int i = 1; i <= nx; ++i) {
        const int is = i < 2 ? 2 : i;   /* dtaus(1) = dtaus(2); i <= NX here */
        double si = 0.0;
        for (int l = 0; l < nb; ++l) {
          const double* tw = s->STAU_W + nh * (size_t)l;
          const double dtaus = (tw[hidx(s, is - 1, j, k)] - tw[hidx(s, is + 1, j, k)]) / 2.0;
          si = si + s->wave_bstar[l] * (exp(-tw[hidx(s, i, j, k)] / mu)) * dtaus;
        }
        H(STELLARINPUT, i, j, k) = si * geo / G1(dxb, i);
      }
    }
  return 0;
}

int ttor_stellarinput_heating(ttor_state* s) {
  const int nx = s->nx, ny = s->ny, nz = s->nz;
  if (s->f_incident == 0) {
    for (size_t q = 0; q < nhalo(s); ++q) s->STELLARINPUT[q] = 0.0;
    return 0;
  }
  if (s->wave_nb > 0) return stellar_binned(s);
  double dr = G1(xxb, 2) - G1(xxb, 1);
  for (int k = -1; k <= nz + 2; ++k)
    for (int j = -1; j <= ny + 2; ++j) {
      int ub = P(UPPERBND, j, k);
      if (ub < nx)
        for (int i = ub + 1; i <= nx + 1; ++i) H(STELLARTAU, i, j, k) = 0.0;
      double tot = 0.0;
      for (int i = ub; i >= 1; --i) {
        tot = tot + (H(XKAPA, i, j, k) * H(RH, i, j, k) * dr);
        H(STELLARTAU, i, j, k) = tot;
      }
    }
  for (int k = -1; k <= nz + 2; ++k)
    for (int j = -1; j <= ny + 2; ++j) {
      for (int i = 2; i <= nx; ++i)
        H(DTAUS, i, j, k) = (H(STELLARTAU, i - 1, j, k) - H(STELLARTAU, i + 1, j, k)) / 2.0;
      H(DTAUS, 1, j, k) = H(DTAUS, 2, j, k);
      H(DTAUS, nx + 1, j, k) = H(DTAUS, nx, j, k);
    }
  for (int k = -1; k <= nz + 2; ++k)
    for (int j = -1; j <= ny + 2; ++j) {
      double tinc = P(TINCIDENT, j, k), mu = P(MU_STAR, j, k);
      for (int i = 1; i <= nx; ++i)
        H(STELLARINPUT, i, j, k) = SBCONST_C * (p4(tinc) / mu) *
                                   (exp(-H(STELLARTAU, i, j, k) / mu)) * H(DTAUS, i, j, k) / G1(dxb, i);
    }
  return 0;
}

/* BOUNDS ppbou.f:1-92 for MODTYP=2, MODVER in {0,2,3,4,5}, restricted to
 * the fields the energy step reads (T, RH, UPPERBND): BOUNDPLANET's
 * density-based UPPERBND (ppbou.f:124-144), BOUNDXMIN(9) (ppbou.f:1029-1049),
 * BOUNDXMAX(2) (ppbou.f:1269-1384), BOUNDZMIN(0)/BOUNDZMAX(0)
 * (ppbou.f:1833-1846, 1946-1958), and the PLANETSHIFT calls around them. */
int ttor_bounds(ttor_state* s) {
  const int nx = s->nx, ny = s->ny, nz = s->nz;
  if (s->bcxmin != 9) return -4;
  shift_halo(s, s->T); shift_halo(s, s->RH);
  pole_shift(s, s->T); pole_shift(s, s->RH);
  for (int k = 1; k <= nz; ++k)
    for (int j = 1; j <= ny; ++j) {
      int ub = nx + 1, found = 0;
      for (int i = 1; i <= nx; ++i)
        if (H(RH, i, j, k) < (double)1.0e-9f) { ub = i; found = 1; break; }
      if (!found) ub = nx - 1;
      P(UPPERBND, j, k) = ub;
    }
  passupperbnd(s);
  /* BOUNDXMIN(9) */
  double kapT111 = 0.0;
  if (s->iii <= 0) kapT111 = kap_formula(s, H(T, 1, 1, 1), H(RH, 1, 1, 1), H(KMUL, 1, 1, 1));
  if (s->iii <= 0 && s->opac_nt > 0) {   /* ppbou.f:1040-1044 */
    double kp, ka, dkp, dka;
    if (burrows_opc(s, H(T, 1, 1, 1), H(RH, 1, 1, 1), &kp, &kapT111, &ka, &dkp, &dka)) return -10;
  }
  for (int k = -1; k <= nz + 2; ++k)
    for (int j = -1; j <= ny + 2; ++j) {
      double dtdr;
      if (s->ieta == 5) {
        dtdr = -s->fbottom / (H(RH, 1, j, k) * H(CV, 1, j, k) * (s->xnue / s->pr_num));
      } else if (s->iii > 0) {
        dtdr = -(3.0 * s->fbottom * H(XKAPR, 1, j, k) * H(RH, 1, j, k) /
                 (4.0 * ARAD_C * FD_C * p3(H(T, 1, j, k))));
      } else {
        dtdr = -(3.0 * s->fbottom * kapT111 * H(RH, 1, 1, 1) /
                 (4.0 * ARAD_C * FD_C * p3(H(T, 1, 1, 1))));
      }
      H(T, 0, j, k) = H(T, 1, j, k) - dtdr * (G1(xxb, 1) - G1(xxb, 0));
      H(T, -1, j, k) = H(T, 1, j, k) - dtdr * (G1(xxb, 1) - G1(xxb, -1));
    }
  /* BOUNDXMAX(2) with IBDRAD */
  for (int k = 1; k <= nz; ++k)
    for (int j = 1; j <= ny; ++j) {
      int ub = P(UPPERBND, j, k);
      if (!(ub < nx + 1)) return -5;
      double tj;
      if (s->ibdrad == 9) {
        if (s->iii <= 1) {
          tj = H(T, ub - 1, j, k);
        } else {
          tj = pow((H(ER, ub - 1, j, k) / ARAD_C) +
                       (H(STELLARINPUT, ub - 1, j, k) /
                        (4.0 * SBCONST_C * H(RH, ub - 1, j, k) * H(XKAPP, ub - 1, j, k))),
                   0.25);
        }
      } else if (s->ibdrad == 7) {
        tj = H(T, ub - 1, j, k);
      } else if (s->ibdrad == 4) {
        tj = s->tirr;
      } else {
        return -6;
      }
      H(T, ub, j, k) = tj;
      for (int i = ub + 1; i <= nx + 2; ++i) {
        H(T, i, j, k) = tj;
        H(RH, i, j, k) = (double)1.0e-10f;
      }
      if (ub == nx) { H(RH, nx, j, k) = (double)1.0e-10f; H(T, nx, j, k) = tj; }
    }
  /* BOUNDZMIN(0) / BOUNDZMAX(0), without poles only (ppbou.f:188-193) */
  if (!s->poles) {
  for (int j = -1; j <= ny + 2; ++j)
    for (int i = -1; i <= nx + 2; ++i) {
      H(RH, i, j, 1) = H(RH, i, j, 2);
      H(RH, i, j, 0) = H(RH, i, j, 1);
      H(RH, i, j, -1) = H(RH, i, j, 1);
      H(T, i, j, 1) = H(T, i, j, 2);
      H(T, i, j, 0) = H(T, i, j, 1);
      H(T, i, j, -1) = H(T, i, j, 1);
    }
  for (int j = -1; j <= ny + 2; ++j)
    for (int i = -1; i <= nx + 2; ++i) {
      H(RH, i, j, nz) = H(RH, i, j, nz - 1);
      H(RH, i, j, nz + 1) = H(RH, i, j, nz);
      H(RH, i, j, nz + 2) = H(RH, i, j, nz);
      H(T, i, j, nz) = H(T, i, j, nz - 1);
      H(T, i, j, nz + 1) = H(T, i, j, nz);
      H(T, i, j, nz + 2) = H(T, i, j, nz);
    }
  }
  shift_halo(s, s->T); shift_halo(s, s->RH);
  pole_shift(s, s->T); pole_shift(s, s->RH);
  return 0;
}

/* FILL_SOR_MATRIX ppsor.f:189-277 (one rank: MPIright, MPIbelow and
 * MPIabove are MPI_PROC_NULL; MPIlower/MPIupper are self, so the j rows are
 * never boundaries). */
int ttor_fill_sor_matrix(ttor_state* s) {
  const int nx = s->nx, ny = s->ny, nz = s->nz;
  for (int k = 1; k <= nz; ++k)
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i) {
        double e8 = C(EVAL8, i, j, k);
        C(SOR_A, i, j, k) = C(EVAL7, i, j, k) + e8 * C(EVAL_1_6, i, j, k);
        C(SOR_B, i, j, k) = -e8 * C(EVAL2, i, j, k);
        C(SOR_C, i, j, k) = -e8 * C(EVAL1, i, j, k);
        C(SOR_D, i, j, k) = -e8 * C(EVAL4, i, j, k);
        C(SOR_E, i, j, k) = -e8 * C(EVAL3, i, j, k);
        C(SOR_F, i, j, k) = -e8 * C(EVAL6, i, j, k);
        C(SOR_G, i, j, k) = -e8 * C(EVAL5, i, j, k);
        int ub = P(UPPERBND, j, k);
        int ident = (i >= ub) || (i == nx) || (!s->poles && (k == 1 || k == nz));
        if (ident) {
          C(SOR_A, i, j, k) = 1.0; C(SOR_B, i, j, k) = 0.0; C(SOR_C, i, j, k) = 0.0;
          C(SOR_D, i, j, k) = 0.0; C(SOR_E, i, j, k) = 0.0; C(SOR_F, i, j, k) = 0.0;
          C(SOR_G, i, j, k) = 0.0;
        }
        if (i == ub - 1) C(SOR_C, i, j, k) = 0.0;
        if (i == nx - 1) C(SOR_C, i, j, k) = 0.0;
        if (!s->poles && k == 2) C(SOR_F, i, j, k) = 0.0;
        if (!s->poles && k == nz - 1) C(SOR_G, i, j, k) = 0.0;
      }
  return 0;
}

/* FILLHYPREMATRIX pphypre.f:221-334 and the b of FILLHYPREVECTORS
 * pphypre.f:115-219 (one rank: MPIleft, MPIright, MPIbelow and MPIabove
 * are MPI_PROC_NULL; MPIlower/MPIupper are the rank itself, so no j row is
 * a boundary row).  Stencil entries 1..7 are (i,j,k), i-1, i+1, j-1, j+1,
 * k-1, k+1 (pphypre.f:553-581) -> HYP_A..HYP_G.  The grid is given only its
 * extents (pphypre.f:404-413, no periodicity), so hypre drops the entries
 * of rows j = 1 (j-1) and j = NY (j+1) that reach outside it; they are
 * zeroed here.  The initial x of pphypre.f:136 is 1 everywhere. */
int ttor_fill_hypre_system(ttor_state* s) {
  const int nx = s->nx, ny = s->ny, nz = s->nz;
  for (int k = 1; k <= nz; ++k)
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i) {
        double h[7];
        const double e8 = C(EVAL8, i, j, k);
        h[0] = C(EVAL7, i, j, k) + e8 * C(EVAL_1_6, i, j, k);
        h[1] = -e8 * C(EVAL2, i, j, k);
        h[2] = -e8 * C(EVAL1, i, j, k);
        h[3] = -e8 * C(EVAL4, i, j, k);
        h[4] = -e8 * C(EVAL3, i, j, k);
        h[5] = -e8 * C(EVAL6, i, j, k);
        h[6] = -e8 * C(EVAL5, i, j, k);
        const int ub = P(UPPERBND, j, k);
        if (i >= ub) { h[0] = 1.0; for (int m = 1; m < 7; ++m) h[m] = 0.0; }
        if (i == ub - 1) h[2] = 0.0;
        if (i == 1 || i == nx || (!s->poles && (k == 1 || k == nz))) {
          h[0] = 1.0;
          for (int m = 1; m < 7; ++m) h[m] = 0.0;
        }
        if (i == 2) h[1] = 0.0;
        if (i == nx - 1) h[2] = 0.0;
        if (!s->poles && k == 2) h[5] = 0.0;
        if (!s->poles && k == nz - 1) h[6] = 0.0;
        if (j == 1) h[3] = 0.0;   /* outside the hypre grid */
        if (j == ny) h[4] = 0.0;
        C(HYP_A, i, j, k) = h[0]; C(HYP_B, i, j, k) = h[1]; C(HYP_C, i, j, k) = h[2];
        C(HYP_D, i, j, k) = h[3]; C(HYP_E, i, j, k) = h[4]; C(HYP_F, i, j, k) = h[5];
        C(HYP_G, i, j, k) = h[6];
        double b = C(RHS_ER, i, j, k);
        if (i >= ub || i == 1 || i == nx || (!s->poles && (k == 1 || k == nz))) b = 0.0;
        C(HYP_RHS, i, j, k) = b;
      }
  return 0;
}

/* B_VECTOR_BOUNDARIES ppsor.f:280-329 */
int ttor_b_vector_boundaries(ttor_state* s) {
  const int nx = s->nx, ny = s->ny, nz = s->nz;
  for (int k = 1; k <= nz; ++k)
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i) {
        int ub = P(UPPERBND, j, k);
        if (i >= ub || i == nx || (!s->poles && (k == 1 || k == nz))) C(RHS_ER, i, j, k) = 0.0;
      }
  return 0;
}

/* One colour pass of the red-black loop, ppsor.f:59-88 / 107-136. */
static double sor_colour_k(ttor_state* s, double* x, const double* b, int colour, int k0, int k1) {
  const int nx = s->nx, ny = s->ny;
  double rnorm = 0.0;
#define X(i, j, k) x[(size_t)((i) + 1) + (size_t)NXH * ((size_t)((j) + 1) + (size_t)NYH * (size_t)((k) + 1))]
  for (int k = k0; k <= k1; ++k)
    for (int j = 1; j <= ny; ++j) {
      int imin = 2 - ((j + k + colour) % 2);
      for (int i = imin; i <= nx; i += 2) {
        size_t c = (size_t)(i - 1) + (size_t)nx * ((size_t)(j - 1) + (size_t)ny * (size_t)(k - 1));
        double resid = s->SOR_A[c] * X(i, j, k) + s->SOR_B[c] * X(i - 1, j, k) +
                       s->SOR_C[c] * X(i + 1, j, k) + s->SOR_D[c] * X(i, j - 1, k) +
                       s->SOR_E[c] * X(i, j + 1, k) + s->SOR_F[c] * X(i, j, k - 1) +
                       s->SOR_G[c] * X(i, j, k + 1) - b[c];
        rnorm = rnorm + fabs(resid);
        X(i, j, k) = X(i, j, k) - s->sorparam * resid / s->SOR_A[c];
      }
    }
#undef X
  return rnorm;
}

static double sor_colour(ttor_state* s, double* x, const double* b, int colour, int zmax) {
  return sor_colour_k(s, x, b, colour, 1, zmax);
}

/* The red-black iteration with the ppsor.f:161-177 stopping rule over the
 * rows k = 1..zmax, the halo and pole shifts after each colour. */
static int sor_loop_rows(ttor_state* s, double* x, const double* b, int itmin, int itmax, int zmax) {
  double rhsnorm = 0.0;
  for (size_t c = 0; c < ncell(s); ++c) rhsnorm = rhsnorm + fabs(b[c]);
  s->global_rhsnorm = rhsnorm;
  int it = 0;
  for (;;) {
    ++it;
    double rnorm = sor_colour(s, x, b, 0, zmax);
    shift_halo(s, x);
    pole_shift(s, x);
    rnorm = rnorm + sor_colour(s, x, b, 1, zmax);
    shift_halo(s, x);
    pole_shift(s, x);
    s->global_rnorm = rnorm;
    if (it == itmax) { s->sor_iter = it; return 1; }
    if (rnorm / rhsnorm > s->epsmat || it < itmin) continue;
    break;
  }
  s->sor_iter = it;
  return 0;
}

/* SOLVE_WITH_SOR's loop: with poles the rows stop at zmax_sor_index = NZ-1
 * (ppsor.f:39-43). */
static int sor_loop(ttor_state* s, double* x, const double* b, int itmin, int itmax) {
  return sor_loop_rows(s, x, b, itmin, itmax, s->poles ? s->nz - 1 : s->nz);
}

/* SOLVE_WITH_SOR ppsor.f:2-187 */
int ttor_solve_with_sor(ttor_state* s, int fill, int use_guess) {
  if (fill) { ttor_fill_sor_matrix(s); ttor_b_vector_boundaries(s); }
  if (!use_guess) {
    for (size_t q = 0; q < nhalo(s); ++q) s->DELTA_ER[q] = 0.0;
  } else {
    /* keep the interior as the initial iterate, zero ghosts, refresh halo */
    for (int k = -1; k <= s->nz + 2; ++k)
      for (int j = -1; j <= s->ny + 2; ++j)
        for (int i = -1; i <= s->nx + 2; ++i)
          if (i < 1 || i > s->nx || j < 1 || j > s->ny || k < 1 || k > s->nz) H(DELTA_ER, i, j, k) = 0.0;
    shift_halo(s, s->DELTA_ER);
    pole_shift(s, s->DELTA_ER);
  }
  int rc = sor_loop(s, s->DELTA_ER, s->RHS_ER, 1, s->itmax);
  s->sor_total += s->sor_iter;
  s->solves += 1;
  return rc;
}

/* The phi halo copies of shift_halo for the theta rows k0..k1. */
static void shift_halo_k(ttor_state* s, double* a, int k0, int k1) {
  const int nx = s->nx, ny = s->ny;
#define A(i, j, k) a[(size_t)((i) + 1) + (size_t)NXH * ((size_t)((j) + 1) + (size_t)NYH * (size_t)((k) + 1))]
  for (int k = k0; k <= k1; ++k)
    for (int i = -1; i <= nx + 2; ++i) {
      A(i, 0, k) = A(i, ny, k);
      A(i, -1, k) = A(i, ny - 1, k);
      A(i, ny + 1, k) = A(i, 1, k);
      A(i, ny + 2, k) = A(i, 2, k);
    }
#undef A
}

/* The reference decomposes the grid over MPI ranks, one serial rank per
 * core; its CPU baseline is the same red-black sweeps on theta slabs, one
 * thread per slab, a barrier after each colour (where the ranks exchange
 * halos), the slab norms added in slab order. */
typedef struct {
  ttor_state* s;
  int k0, k1, nsweeps;
  pthread_barrier_t* bar;
  double* part;  /* per slab */
} mt_arg;

static void* mt_worker(void* p) {
  mt_arg* a = (mt_arg*)p;
  ttor_state* s = a->s;
  for (int it = 0; it < a->nsweeps; ++it) {
    double r = sor_colour_k(s, s->DELTA_ER, s->RHS_ER, 0, a->k0, a->k1);
    shift_halo_k(s, s->DELTA_ER, a->k0, a->k1);
    pthread_barrier_wait(a->bar);
    r = r + sor_colour_k(s, s->DELTA_ER, s->RHS_ER, 1, a->k0, a->k1);
    shift_halo_k(s, s->DELTA_ER, a->k0, a->k1);
    *a->part = r;
    pthread_barrier_wait(a->bar);
  }
  return NULL;
}

int ttor_sor_sweeps_mt(ttor_state* s, int nsweeps, int nthreads) {
  if (nthreads < 1) nthreads = 1;
  if (nthreads > s->nz) nthreads = s->nz;
  if (nthreads > 256) nthreads = 256;
  double rhsnorm = 0.0;
  for (size_t c = 0; c < ncell(s); ++c) rhsnorm = rhsnorm + fabs(s->RHS_ER[c]);
  s->global_rhsnorm = rhsnorm;
  pthread_barrier_t bar;
  if (pthread_barrier_init(&bar, NULL, (unsigned)nthreads)) return -2;
  pthread_t th[256];
  mt_arg args[256];
  double part[256];
  int rc = 0, started = 0;
  for (int t = 0; t < nthreads; ++t) {
    args[t].s = s;
    args[t].k0 = 1 + (int)((long long)s->nz * t / nthreads);
    args[t].k1 = (int)((long long)s->nz * (t + 1) / nthreads);
    args[t].nsweeps = nsweeps;
    args[t].bar = &bar;
    args[t].part = &part[t];
  }
  for (int t = 1; t < nthreads; ++t) {
    if (pthread_create(&th[t], NULL, mt_worker, &args[t])) { rc = -2; break; }
    ++started;
  }
  if (rc == 0) mt_worker(&args[0]);
  for (int t = 1; t <= started; ++t) pthread_join(th[t], NULL);
  pthread_barrier_destroy(&bar);
  if (rc) return rc;
  double r = 0.0;
  for (int t = 0; t < nthreads; ++t) r = r + part[t];
  s->global_rnorm = r;
  s->sor_iter = nsweeps;
  return 0;
}

/* SOLVE_WITH_SOR (ppsor.f:2-187) from zero on theta slabs, one thread per
 * slab as the reference runs one rank per slab: after each sweep thread 0
 * adds the slab norms in slab order (the ranks' allreduce, ppsor.f:155-160)
 * and applies the stopping rule (ppsor.f:161-177); the others wait for its
 * decision at a third barrier. */
typedef struct {
  int stop, it, itmin, itmax, maxit;
  double eps, rhsnorm, rnorm;
  double* parts;
  int nthreads;
} mt_ctl;

typedef struct {
  ttor_state* s;
  int k0, k1, t;
  pthread_barrier_t* bar;
  mt_ctl* ctl;
} mt_solve_arg;

static void* mt_solve_worker(void* p) {
  mt_solve_arg* a = (mt_solve_arg*)p;
  ttor_state* s = a->s;
  mt_ctl* c = a->ctl;
  for (;;) {
    double r = sor_colour_k(s, s->DELTA_ER, s->RHS_ER, 0, a->k0, a->k1);
    shift_halo_k(s, s->DELTA_ER, a->k0, a->k1);
    pthread_barrier_wait(a->bar);
    r = r + sor_colour_k(s, s->DELTA_ER, s->RHS_ER, 1, a->k0, a->k1);
    shift_halo_k(s, s->DELTA_ER, a->k0, a->k1);
    c->parts[a->t] = r;
    pthread_barrier_wait(a->bar);
    if (a->t == 0) {
      double rn = 0.0;
      for (int t = 0; t < c->nthreads; ++t) rn = rn + c->parts[t];
      c->rnorm = rn;
      c->it += 1;
      if (c->it == c->itmax) { c->maxit = 1; c->stop = 1; }
      else if (!(rn / c->rhsnorm > c->eps) && c->it >= c->itmin) c->stop = 1;
    }
    pthread_barrier_wait(a->bar);
    if (c->stop) break;
  }
  return NULL;
}

int ttor_solve_with_sor_mt(ttor_state* s, int nthreads) {
  if (s->poles) return -4;
  if (nthreads < 1) nthreads = 1;
  if (nthreads > s->nz) nthreads = s->nz;
  if (nthreads > 256) nthreads = 256;
  for (size_t q = 0; q < nhalo(s); ++q) s->DELTA_ER[q] = 0.0;  /* ppsor.f:29 */
  double rhsnorm = 0.0;
  for (size_t c = 0; c < ncell(s); ++c) rhsnorm = rhsnorm + fabs(s->RHS_ER[c]);
  s->global_rhsnorm = rhsnorm;
  pthread_barrier_t bar;
  if (pthread_barrier_init(&bar, NULL, (unsigned)nthreads)) return -2;
  double parts[256];
  mt_ctl ctl = {0, 0, 1, s->itmax, 0, s->epsmat, rhsnorm, 0.0, parts, nthreads};
  pthread_t th[256];
  mt_solve_arg args[256];
  int rc = 0, started = 0;
  for (int t = 0; t < nthreads; ++t) {
    args[t].s = s;
    args[t].k0 = 1 + (int)((long long)s->nz * t / nthreads);
    args[t].k1 = (int)((long long)s->nz * (t + 1) / nthreads);
    args[t].t = t;
    args[t].bar = &bar;
    args[t].ctl = &ctl;
  }
  for (int t = 1; t < nthreads; ++t) {
    if (pthread_create(&th[t], NULL, mt_solve_worker, &args[t])) { rc = -2; break; }
    ++started;
  }
  if (rc == 0) mt_solve_worker(&args[0]);
  for (int t = 1; t <= started; ++t) pthread_join(th[t], NULL);
  pthread_barrier_destroy(&bar);
  if (rc) return rc;
  s->global_rnorm = ctl.rnorm;
  s->sor_iter = ctl.it;
  return ctl.maxit ? 1 : 0;
}

int ttor_sor_sweeps(ttor_state* s, int nsweeps) {
  double rhsnorm = 0.0;
  for (size_t c = 0; c < ncell(s); ++c) rhsnorm = rhsnorm + fabs(s->RHS_ER[c]);
  s->global_rhsnorm = rhsnorm;
  const int zmax = s->poles ? s->nz - 1 : s->nz;
  for (int it = 0; it < nsweeps; ++it) {
    double r = sor_colour(s, s->DELTA_ER, s->RHS_ER, 0, zmax);
    shift_halo(s, s->DELTA_ER);
    pole_shift(s, s->DELTA_ER);
    r = r + sor_colour(s, s->DELTA_ER, s->RHS_ER, 1, zmax);
    shift_halo(s, s->DELTA_ER);
    pole_shift(s, s->DELTA_ER);
    s->global_rnorm = r;
  }
  s->sor_iter = nsweeps;
  return 0;
}

double ttor_true_residual_l1(ttor_state* s) {
  const int nx = s->nx, ny = s->ny, nz = s->nz;
  double acc = 0.0;
  for (int k = 1; k <= nz; ++k)
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i) {
        double r = C(SOR_A, i, j, k) * H(DELTA_ER, i, j, k) + C(SOR_B, i, j, k) * H(DELTA_ER, i - 1, j, k) +
                   C(SOR_C, i, j, k) * H(DELTA_ER, i + 1, j, k) + C(SOR_D, i, j, k) * H(DELTA_ER, i, j - 1, k) +
                   C(SOR_E, i, j, k) * H(DELTA_ER, i, j + 1, k) + C(SOR_F, i, j, k) * H(DELTA_ER, i, j, k - 1) +
                   C(SOR_G, i, j, k) * H(DELTA_ER, i, j, k + 1) - C(RHS_ER, i, j, k);
        acc = acc + fabs(r);
      }
  return acc;
}

/* ADJUST_SOR_PARAM ppsor.f:332-354 */
int ttor_adjust_sor_param(ttor_state* s) {
  int save_it[50];
  double save_p[50];
  s->sorparam = (double)1.01f;
  for (int n = 0; n < 50; ++n) {
    ttor_solve_with_sor(s, 1, 0);
    save_it[n] = s->sor_iter;
    save_p[n] = s->sorparam;
    s->sorparam = s->sorparam + (double)0.02f;
  }
  int best = 0;
  for (int n = 1; n < 50; ++n)
    if (save_it[n] < save_it[best]) best = n;
  s->sorparam = save_p[best];
  return 0;
}

/* Q/E_R boundary blocks of COUPLED_ENERGY_EQS. */
static void upper_bc(ttor_state* s) {           /* ppenergy.f:80-105, 678-702 */
  const int nx = s->nx, ny = s->ny, nz = s->nz;
  for (int k = -1; k <= nz + 2; ++k)
    for (int j = -1; j <= ny + 2; ++j) {
      int ub = P(UPPERBND, j, k);
      double qupper = H(RH, ub - 1, j, k) * H(CV, ub - 1, j, k) * H(T, ub, j, k);
      /* FLUX_X is declared (1:NX+1,1:NY,1:NZ) (ppmod.f:513); the loop
       * reads it up to i=NX+2 and at ghost j,k.  Clamp those reads. */
      int jc = j < 1 ? 1 : (j > ny ? ny : j);
      int kc = k < 1 ? 1 : (k > nz ? nz : k);
      for (int i = ub; i <= nx + 2; ++i) {
        int ic = i > nx + 1 ? nx + 1 : i;
        H(Q, i, j, k) = qupper;
        H(ER, i, j, k) = fabs(2.0 * F(FLUX_X, ic, jc, kc) / FD_C);
      }
    }
}

static int left_bc(ttor_state* s) {             /* ppenergy.f:108-201, 578-671 */
  const int ny = s->ny, nz = s->nz;
  if (s->bcxmin != 9) return -4;
  for (int k = -1; k <= nz + 2; ++k)
    for (int j = -1; j <= ny + 2; ++j) {
      double dqdr;
      if (s->ieta == 5)
        dqdr = -H(RH, 1, j, k) * H(CV, 1, j, k) * s->fbottom /
               (H(RH, 1, j, k) * H(CV, 1, j, k) * (s->xnue / s->pr_num));
      else
        dqdr = -(H(RH, 1, j, k) * H(CV, 1, j, k) * 3.0 * s->fbottom * H(XKAPR, 1, j, k) * H(RH, 1, j, k) /
                 (4.0 * ARAD_C * FD_C * p3(H(T, 1, j, k))));
      H(Q, 0, j, k) = H(Q, 1, j, k) - dqdr * (G1(xxb, 1) - G1(xxb, 0));
      H(Q, -1, j, k) = H(Q, 1, j, k) - dqdr * (G1(xxb, 1) - G1(xxb, -1));
      H(ER, 1, j, k) = ARAD_C * p4(H(Q, 1, j, k) / (H(RH, 1, j, k) * H(CV, 1, j, k)));
      H(ER, 0, j, k) = ARAD_C * p4(H(Q, 0, j, k) / (H(RH, 0, j, k) * H(CV, 0, j, k)));
      H(ER, -1, j, k) = ARAD_C * p4(H(Q, -1, j, k) / (H(RH, -1, j, k) * H(CV, -1, j, k)));
    }
  return 0;
}

static void z_bc(ttor_state* s) {               /* ppenergy.f:204-227, 706-733 */
  const int nx = s->nx, ny = s->ny, nz = s->nz;
  if (s->poles) return;
  for (int j = -1; j <= ny + 2; ++j)
    for (int i = -1; i <= nx + 2; ++i) {
      H(Q, i, j, 1) = H(Q, i, j, 2);
      H(ER, i, j, 1) = H(ER, i, j, 2);
      H(Q, i, j, 0) = H(Q, i, j, 1);
      H(Q, i, j, -1) = H(Q, i, j, 1);
      H(ER, i, j, 0) = H(ER, i, j, 1);
      H(ER, i, j, -1) = H(ER, i, j, 1);
    }
  for (int j = -1; j <= ny + 2; ++j)
    for (int i = -1; i <= nx + 2; ++i) {
      H(Q, i, j, nz) = H(Q, i, j, nz - 1);
      H(ER, i, j, nz) = H(ER, i, j, nz - 1);
      H(Q, i, j, nz + 1) = H(Q, i, j, nz);
      H(Q, i, j, nz + 2) = H(Q, i, j, nz);
      H(ER, i, j, nz + 1) = H(ER, i, j, nz);
      H(ER, i, j, nz + 2) = H(ER, i, j, nz);
    }
}

/* COUPLED_ENERGY_EQS ppenergy.f:2-791 (IRAD=3). */
int ttor_coupled_energy_eqs(ttor_state* s, int do_bounds) {
  const int nx = s->nx, ny = s->ny, nz = s->nz;
  const double delta_max = 0.005, conv_parm = 0.1, theta = 1.0;   /* :42, :49, :60 */
  int rc;
  s->status = 0;
  s->sor_total = 0; s->solves = 0;
  for (size_t q = 0; q < nhalo(s); ++q) s->DELTA_ER[q] = 0.0;     /* :52-53 */
  for (size_t q = 0; q < ncell(s); ++q) s->DELTA_Q[q] = 0.0;
  s->energy_iter = 0;
  if (do_bounds && (rc = ttor_bounds(s))) return rc;              /* :63 */
  for (size_t q = 0; q < nhalo(s); ++q) s->Q[q] = s->RH[q] * s->CV[q] * s->T[q];  /* :65 */
  if (s->f_incident > 1) {                                        /* :68-71 */
    if ((rc = ttor_kappa(s))) return rc;
    ttor_stellarinput_heating(s);
  }
  if ((rc = ttor_calculateflux(s))) return rc;                    /* :74-75 */
  ttor_flux_bc(s);
  upper_bc(s);
  if ((rc = left_bc(s))) return rc;
  z_bc(s);
  shift_halo(s, s->ER);                                           /* :230-245 */
  pole_shift(s, s->ER);
  memcpy(s->Q_OLD, s->Q, nhalo(s) * sizeof(double));             /* :248-249 */
  memcpy(s->ER_OLD, s->ER, nhalo(s) * sizeof(double));
  if ((rc = ttor_calculateflux(s))) return rc;                    /* :253-255 */
  ttor_flux_bc(s);
  ttor_calculatedivf_withf(s, 1, theta);
  for (;;) {
    s->energy_iter += 1;                                          /* :260 */
    shift_halo(s, s->ER);                                         /* :264-279 */
    pole_shift(s, s->ER);
    if ((rc = ttor_calculateflux(s))) return rc;                  /* :283-285 */
    ttor_flux_bc(s);
    ttor_calculatedivf_withf(s, 0, theta);
    for (int k = 1; k <= nz; ++k)                                 /* :287-345 */
      for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) {
          double q = H(Q, i, j, k), rh = H(RH, i, j, k), cv = H(CV, i, j, k), er = H(ER, i, j, k);
          double kp = H(XKAPP, i, j, k);
          double qr = q / (rh * cv);
          double bb = ARAD_C * p4(qr);
          double fq, dfq;
          double dfr = -((s->delt / cv) * (kp * 4.0 * ARAD_C * FD_C * p3(qr) +
                                           FD_C * (bb - er) * H(DXKAPP_DT, i, j, k)));
          if (s->f_incident > 1) {
            double si = H(STELLARINPUT, i, j, k);
            double heat = si / (rh * H(XKAPA, i, j, k));
            fq = q - H(Q_OLD, i, j, k) +
                 s->delt * ((1 - theta) * (C(DIVF_OLD, i, j, k) - C(DIVF, i, j, k)) +
                            (rh * kp * FD_C * (bb - er)) - si);
            dfq = 1.0 + (s->delt / cv) * (kp * 4.0 * ARAD_C * FD_C * p3(qr) +
                                          (FD_C * (bb - er) * H(DXKAPP_DT, i, j, k)) -
                                          heat * H(DXKAPA_DT, i, j, k));
          } else {
            fq = q - H(Q_OLD, i, j, k) +
                 s->delt * ((1 - theta) * (C(DIVF_OLD, i, j, k) - C(DIVF, i, j, k)) +
                            rh * kp * FD_C * (bb - er));
            dfq = 1.0 + (s->delt / cv) * (kp * 4.0 * ARAD_C * FD_C * p3(qr) +
                                          FD_C * (bb - er) * H(DXKAPP_DT, i, j, k));
          }
          double fr = er - H(ER_OLD, i, j, k) +
                      s->delt * (C(DIVF, i, j, k) - rh * kp * FD_C * (bb - er));
          C(FQ, i, j, k) = fq; C(FR, i, j, k) = fr;
          C(DFQ_DQ, i, j, k) = dfq; C(DFR_DQ, i, j, k) = dfr;
          double eta = (dfq != 0.0) ? -dfr / dfq : 0.0;
          C(JACOB_ETA, i, j, k) = eta;
          C(RHS_ER, i, j, k) = -fr - eta * fq;
        }
    ttor_fill_evalues(s, theta);                                  /* :348 */
    if (s->adjust_sor && s->energy_iter == 1 && (s->iii % 10000 == 0 || s->iii == 1))
      ttor_adjust_sor_param(s);                                   /* :372-374 */
    rc = ttor_solve_with_sor(s, 1, 0);                            /* :375 */
    if (rc < 0) return rc;
    double locmax_q = 0.0, locmax_er = 0.0;                       /* :379-541 */
    for (int k = 1; k <= nz; ++k)
      for (int j = 1; j <= ny; ++j) {
        int xmax_index = P(UPPERBND, j, k) - 1;
        int xmin_index = 2;
        for (int i = xmin_index; i <= xmax_index; ++i) {
          double q1 = -s->delt * (1.0 - theta);
          double q2 = s->delt * H(RH, i, j, k) * H(XKAPP, i, j, k) * FD_C;
          double dq = (1.0 / C(DFQ_DQ, i, j, k)) *
                      (q1 * C(EVAL_1_6, i, j, k) * H(DELTA_ER, i, j, k) -
                       q1 * C(EVAL1, i, j, k) * H(DELTA_ER, i + 1, j, k) -
                       q1 * C(EVAL2, i, j, k) * H(DELTA_ER, i - 1, j, k) -
                       q1 * C(EVAL3, i, j, k) * H(DELTA_ER, i, j + 1, k) -
                       q1 * C(EVAL4, i, j, k) * H(DELTA_ER, i, j - 1, k) -
                       q1 * C(EVAL5, i, j, k) * H(DELTA_ER, i, j, k + 1) -
                       q1 * C(EVAL6, i, j, k) * H(DELTA_ER, i, j, k - 1) +
                       q2 * H(DELTA_ER, i, j, k) - C(FQ, i, j, k));
          C(DELTA_Q, i, j, k) = dq;
          if ((H(Q, i, j, k) + conv_parm * dq) <= 0.0) { s->status = -7; return -7; }  /* :411-521 */
          locmax_q = fmax(locmax_q, fabs(dq / H(Q, i, j, k)));
          locmax_er = fmax(locmax_er, fabs(H(DELTA_ER, i, j, k) / H(ER, i, j, k)));
        }
      }
    for (int k = 1; k <= nz; ++k)                                 /* :551-573 */
      for (int j = 1; j <= ny; ++j) {
        int xmax_index = P(UPPERBND, j, k) - 1;
        for (int i = 2; i <= xmax_index; ++i) {
          H(ER, i, j, k) = H(ER, i, j, k) + conv_parm * H(DELTA_ER, i, j, k);
          H(Q, i, j, k) = H(Q, i, j, k) + conv_parm * C(DELTA_Q, i, j, k);
        }
      }
    if ((rc = left_bc(s))) return rc;                             /* :578-671 */
    upper_bc(s);                                                  /* :678-702 */
    z_bc(s);                                                      /* :706-733 */
    s->global_deltaq = locmax_q;                                  /* :736-739 */
    s->global_deltaer = locmax_er;
    if (s->energy_iter == s->itmax) { s->status = 1; break; }     /* :750-775 */
    if (!(s->global_deltaq > delta_max)) break;                   /* :778 */
  }
  for (size_t q = 0; q < nhalo(s); ++q) {                         /* :787-789 */
    s->DELTA_ER[q] = s->ER[q] - s->ER_OLD[q];
    s->T[q] = s->Q[q] / (s->RH[q] * s->CV[q]);
  }
  return s->status;
}

/* DIFFUSION ppdif.f:1-167 with DIFFUSION_MAT_ELEM (:169-223),
 * DIFFUSION_COEF (:226-275) and FILL_DVALUES (:278-308).  The scalar is the
 * halo field SCALAR; the SOR system is stored in SOR_A..G / RHS_DIF. */
int ttor_diffusion(ttor_state* s) {
  const int nx = s->nx, ny = s->ny, nz = s->nz;
  const double dconst = s->xnue / s->pr_num;
  for (int k = 1; k <= nz; ++k)
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i) C(RHS_DIF, i, j, k) = H(SCALAR, i, j, k);
  for (int k = 1; k <= nz; ++k)
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i) {
        double dx1 = dconst / G1(dxb, i + 1), dx2 = dconst / G1(dxb, i);
        double dy1 = dconst / (G1(dyb, j + 1) * G1(geoxg, i) * G1(geozg, k));
        double dy2 = dconst / (G1(dyb, j) * G1(geoxg, i) * G1(geozg, k));
        double dz1 = dconst / (G1(dzb, k + 1) * G1(geoxh, i));
        double dz2 = dconst / (G1(dzb, k) * G1(geoxh, i));
        double d1 = s->delt * G1(surxa, i + 1) * dx1 / (G1(surxb, i) * G1(dxa, i));
        double d2 = s->delt * G1(surxa, i) * dx2 / (G1(surxb, i) * G1(dxa, i));
        double d3 = s->delt * dy1 / (G1(geoxg, i) * G1(surzb, k) * G1(dya, j));
        double d4 = s->delt * dy2 / (G1(geoxg, i) * G1(surzb, k) * G1(dya, j));
        double d5 = s->delt * dz1 * G1(surza, k + 1) / (G1(geoxg, i) * G1(surzb, k) * G1(dza, k));
        double d6 = s->delt * dz2 * G1(surza, k) / (G1(geoxg, i) * G1(surzb, k) * G1(dza, k));
        double d16 = d1 + d2 + d3 + d4 + d5 + d6;
        C(SOR_A, i, j, k) = 1.0 + d16;
        C(SOR_B, i, j, k) = -d2; C(SOR_C, i, j, k) = -d1;
        C(SOR_D, i, j, k) = -d4; C(SOR_E, i, j, k) = -d3;
        C(SOR_F, i, j, k) = -d6; C(SOR_G, i, j, k) = -d5;
        if (i == nx) {
          C(SOR_A, i, j, k) = 1.0 + d2; C(SOR_B, i, j, k) = -d2;
          C(SOR_C, i, j, k) = 0.0; C(SOR_D, i, j, k) = 0.0; C(SOR_E, i, j, k) = 0.0;
          C(SOR_F, i, j, k) = 0.0; C(SOR_G, i, j, k) = 0.0;
        }
      }
  /* every theta row (ppdif.f:45-46, 93-94), with the pole shifts of the
   * scalar after each colour when poles are on (ppdif.f:80-89, 123-132) */
  int rc = sor_loop_rows(s, s->SCALAR, s->RHS_DIF, 5, 500, nz);
  return rc;
}

/* ---- IRAD=1: RADDIF pprad.f:1-38, DIFFEL :40-72, SOLVMAT ppmat.f:1-186,
 * RADIATIVEBOUND ppbou.f:2049-2299 (RADBOUNDVER = IBDRAD 4, 7 or 9, the
 * top boundaries the rest of this library implements, with MODVER <= 5; one
 * rank, periodic phi; with poles the theta ghosts come from the pole shifts
 * after every PLANETSHIFT(6)) --------------------------------------------- */

/* RADIATIVEBOUND: bottom T and ER (:2127-2139), top ER at i >= upperbnd
 * (:2145-2236), theta ghost copies (:2256-2271), PLANETSHIFT(6) (:2280). */
static int radiativebound(ttor_state* s, double d_t, double tinit_bottom, int modver) {
  const int nx = s->nx, ny = s->ny, nz = s->nz;
  if (s->ibdrad != 4 && s->ibdrad != 7 && s->ibdrad != 9) return -3;
  if (modver > 5) return -3;
  for (int k = -1; k <= nz + 2; ++k)
    for (int j = -1; j <= ny + 2; ++j) {
      if (s->bcxmin == 6) H(T, 1, j, k) = tinit_bottom;
      H(T, 0, j, k) = H(T, 1, j, k) - d_t * (G1(xxb, 1) - G1(xxb, 0));
      H(T, -1, j, k) = H(T, 1, j, k) - d_t * (G1(xxb, 1) - G1(xxb, -1));
      H(ER, 1, j, k) = ARAD_C * p4(H(T, 1, j, k));
      H(ER, 0, j, k) = ARAD_C * p4(H(T, 0, j, k));
      H(ER, -1, j, k) = ARAD_C * p4(H(T, -1, j, k));
    }
  for (int k = 1; k <= nz; ++k)
    for (int j = 1; j <= ny; ++j) {
      const int ub = P(UPPERBND, j, k);
      if (!(ub < nx + 1)) return -3;
      double tj = 0.0;
      switch (s->ibdrad) {
        case 4: tj = s->tirr; break;
        case 7: tj = H(T, ub - 1, j, k); break;
        case 9:
          if (s->iii <= 1) tj = H(T, ub - 1, j, k);
          else
            tj = pow(H(ER, ub, j, k) / ARAD_C +
                         H(STELLARINPUT, ub - 1, j, k) /
                             (4.0 * SBCONST_C * H(RH, ub - 1, j, k) * H(XKAPP, ub - 1, j, k)),
                     0.25);
          break;
      }
      for (int i = ub; i <= nx + 2; ++i) H(ER, i, j, k) = ARAD_C * p4(tj);
    }
  if (!s->poles) {
    for (int j = -1; j <= ny + 2; ++j)
      for (int i = -1; i <= nx + 2; ++i) {
        H(ER, i, j, -1) = H(ER, i, j, 1);
        H(ER, i, j, 0) = H(ER, i, j, 1);
      }
    for (int j = -1; j <= ny + 2; ++j)
      for (int i = -1; i <= nx + 2; ++i) {
        H(ER, i, j, nz + 1) = H(ER, i, j, nz);
        H(ER, i, j, nz + 2) = H(ER, i, j, nz);
      }
  }
  shift_halo(s, s->ER);  /* PLANETSHIFT(6) and the pole shifts (:2280-2290) */
  pole_shift(s, s->ER);
  return 0;
}

/* One colour of SOLVMAT (ppmat.f:66-82 / 110-121); returns nothing, XS
 * (the residual of each updated cell) goes to xs. */
static void solvmat_colour(ttor_state* s, double* xs, int parity, double om) {
  const int nx = s->nx, ny = s->ny, nz = s->nz;
  for (int k = 1; k <= nz; ++k)
    for (int j = 1; j <= ny; ++j) {
      const int imin = 2 - ((j + k + parity) % 2);
      for (int i = imin; i <= nx; i += 2) {
        const size_t c = (size_t)(i - 1) + (size_t)nx * ((size_t)(j - 1) + (size_t)ny * (size_t)(k - 1));
        const double x = s->RAD_B[c] * H(ER, i, j, k) - s->RAD_RHS[c] + s->RAD_AX[c] * H(ER, i - 1, j, k) +
                         s->RAD_CX[c] * H(ER, i + 1, j, k) + s->RAD_AY[c] * H(ER, i, j - 1, k) +
                         s->RAD_CY[c] * H(ER, i, j + 1, k) + s->RAD_AZ[c] * H(ER, i, j, k - 1) +
                         s->RAD_CZ[c] * H(ER, i, j, k + 1);
        xs[c] = x;
        H(ER, i, j, k) = H(ER, i, j, k) - om * x / s->RAD_B[c];
      }
    }
}

int ttor_raddif(ttor_state* s, double d_t, double tinit_bottom, int modver, int energy_iter) {
  const int nx = s->nx, ny = s->ny, nz = s->nz;
  if (nz == 1) return -3;
  /* ER = arad T^4 on the whole array (pprad.f:12) */
  for (size_t q = 0; q < nhalo(s); ++q) s->ER[q] = ARAD_C * p4(s->T[q]);
  /* DIFFEL (pprad.f:40-72): DIFF, then the couplings */
  s->energy_iter = energy_iter;
  int rc = ttor_diff(s);
  if (rc) return rc;
  for (int k = 1; k <= nz; ++k)
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i) {
        const size_t c = (size_t)(i - 1) + (size_t)nx * ((size_t)(j - 1) + (size_t)ny * (size_t)(k - 1));
        s->RAD_AX[c] = -F(DIFRX, i, j, k) * G1(surxa, i) / G1(volxb, i);
        s->RAD_CX[c] = -F(DIFRX, i + 1, j, k) * G1(surxa, i + 1) / G1(volxb, i);
        s->RAD_AY[c] = -F(DIFRY, i, j, k) * 1.0 / G1(volyb, j) / G1(geoxg, i) / G1(geozg, k);
        s->RAD_CY[c] = -F(DIFRY, i, j + 1, k) * 1.0 / G1(volyb, j) / G1(geoxg, i) / G1(geozg, k);
        s->RAD_AZ[c] = -F(DIFRZ, i, j, k) * G1(surza, k) / G1(volzb, k) / G1(geoxh, i);
        s->RAD_CZ[c] = -F(DIFRZ, i, j, k + 1) * G1(surza, k + 1) / G1(volzb, k) / G1(geoxh, i);
        /* B and RHS, pprad.f:21-29 */
        const double t = H(T, i, j, k);
        const double w = 1.0 / s->delt * H(CV, i, j, k) * H(RH, i, j, k) / (4.0 * ARAD_C * t * t * t);
        s->RAD_B[c] = w - s->RAD_AX[c] - s->RAD_CX[c] - s->RAD_AY[c] - s->RAD_CY[c] - s->RAD_AZ[c] -
                      s->RAD_CZ[c];
        s->RAD_RHS[c] = H(ER, i, j, k) / s->delt * H(CV, i, j, k) * H(RH, i, j, k) / (4.0 * ARAD_C * t * t * t);
      }
  /* SOLVMAT */
  double rhsnorm = 0.0;
  for (size_t c = 0; c < ncell(s); ++c) rhsnorm = rhsnorm + s->RAD_RHS[c] * s->RAD_RHS[c];
  rhsnorm = sqrt(rhsnorm);
  s->global_rhsnorm = rhsnorm;
  shift_halo(s, s->ER);  /* ppmat.f:39-49 */
  pole_shift(s, s->ER);
  double* xs = (double*)calloc(ncell(s), sizeof(double));
  if (!xs) return -2;
  const double om = s->sorparam;
  int it = 0;
  for (;;) {
    ++it;
    solvmat_colour(s, xs, 0, om);
    if ((rc = radiativebound(s, d_t, tinit_bottom, modver))) break;
    shift_halo(s, s->ER);  /* ppmat.f:87-97 */
    pole_shift(s, s->ER);
    solvmat_colour(s, xs, 1, om);
    if ((rc = radiativebound(s, d_t, tinit_bottom, modver))) break;
    shift_halo(s, s->ER);  /* ppmat.f:126-136 */
    pole_shift(s, s->ER);
    double rnorm = 0.0;
    for (size_t c = 0; c < ncell(s); ++c) rnorm = rnorm + xs[c] * xs[c];
    rnorm = sqrt(rnorm);
    s->global_rnorm = rnorm;
    if (it == s->itmax) { rc = 1; break; }
    if (rnorm / rhsnorm > s->epsmat || it < 5) continue;
    break;
  }
  free(xs);
  s->sor_iter = it;
  if (rc < 0) return rc;
  /* T = (ER/arad)**0.25 (pprad.f:35) */
  for (size_t q = 0; q < nhalo(s); ++q) s->T[q] = pow(s->ER[q] / ARAD_C, 0.25);
  return rc;
}
