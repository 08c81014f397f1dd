/*
 * ttfld.h -- C ABI of libttfld, the GB300 (sm_103a) implementation of
 * ttcode's implicit flux-limited-diffusion radiation/gas energy step.
 *
 * The library holds the reference's module arrays on the device for the
 * whole run; the host copies fields in and out only where the Fortran side
 * reads or writes them.  One context = one device, one stream, one host
 * thread (the reference is one serial MPI rank per core; the calls are not
 * re-entrant).  Every entry point returns an int status:
 *     0   success
 *     1   an iteration limit (ITMAX) was reached; the reference prints and
 *         continues (ppsor.f:161-174, ppenergy.f:750-775), so do the callers
 *     2   the learned initial guess was rejected and the zero guess used
 *    <0   error (see TTFLD_E_*); the reference's CLEAN_STOP cases map here
 *
 * Arrays cross the boundary in the reference's own Fortran layout
 * (column-major, i = radius fastest) with the reference's bounds:
 *     halo  (-1:NX+2,-1:NY+2,-1:NZ+2)  T RH CV ER ER_OLD DELTA_ER XKAP* KMUL ...
 *     cell  (1:NX,1:NY,1:NZ)           EVAL1..8 EVAL_1_6 JACOB_ETA RHS_ER SOR_A..G
 *     facex (1:NX+1,1:NY,1:NZ)         FLIMX DIFRX FLUX_X
 *     facey (1:NX,1:NY+1,1:NZ)         FLIMY DIFRY FLUX_Y
 *     facez (1:NX,1:NY,1:NZ+1)         FLIMZ DIFRZ FLUX_Z
 *     plane (-1:NY+2,-1:NZ+2)          UPPERBND (int32) MU_STAR TINCIDENT
 *     sinp  (1:NX,-1:NY+2,-1:NZ+2)     STELLARINPUT
 *     stau  (1:NX+1,-1:NY+2,-1:NZ+2)   STELLARTAU DTAUS
 * i.e. exactly what a Fortran caller passes with arr(lbound(arr,1),...).
 */
#ifndef TTFLD_H
#define TTFLD_H
#include <stddef.h>
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

#define TTFLD_ABI_VERSION 2

enum ttfld_status {
  TTFLD_OK = 0,
  TTFLD_MAXITER = 1,
  TTFLD_FALLBACK = 2,
  TTFLD_E_ARGS = -1,        /* bad argument / unknown field id            */
  TTFLD_E_CUDA = -2,        /* CUDA runtime error                         */
  TTFLD_E_UNSUPPORTED = -3, /* configuration outside the implemented set  */
  TTFLD_E_NONPOSITIVE_Q = -7, /* Q+conv*dQ <= 0, ppenergy.f:411-521       */
  TTFLD_E_NONFINITE = -8,   /* NaN/Inf found in a solver norm             */
  TTFLD_E_NOMODEL = -9,     /* learned guess requested without a model    */
  TTFLD_E_OPACITY = -10,    /* KAPPA from a table: T <= 0, (T, rho) outside
                               the table, or a non-positive interpolated
                               opacity, where the reference stops          */
  TTFLD_E_INTERNAL = -11    /* a loop of the library broke its own
                               invariant (e.g. ran past ITMAX without its
                               stopping flag); a bug, please report it     */
};

/* Fields addressable through ttfld_upload / ttfld_download. */
enum ttfld_field {
  /* halo (-1:NX+2,-1:NY+2,-1:NZ+2) */
  TTFLD_T = 0, TTFLD_RH, TTFLD_CV, TTFLD_ER, TTFLD_ER_OLD, TTFLD_DELTA_ER,
  TTFLD_XKAPR, TTFLD_XKAPP, TTFLD_XKAPA, TTFLD_DXKAPP_DT, TTFLD_DXKAPA_DT,
  TTFLD_KMUL, TTFLD_Q, TTFLD_SCALAR,
  /* cell (1:NX,1:NY,1:NZ) */
  TTFLD_EVAL1 = 32, TTFLD_EVAL2, TTFLD_EVAL3, TTFLD_EVAL4, TTFLD_EVAL5,
  TTFLD_EVAL6, TTFLD_EVAL7, TTFLD_EVAL8, TTFLD_EVAL_1_6, TTFLD_JACOB_ETA,
  TTFLD_RHS_ER, TTFLD_SOR_A, TTFLD_SOR_B, TTFLD_SOR_C, TTFLD_SOR_D,
  TTFLD_SOR_E, TTFLD_SOR_F, TTFLD_SOR_G, TTFLD_FQ, TTFLD_FR, TTFLD_DIVF,
  TTFLD_DELTA_Q,
  /* faces */
  TTFLD_FLIMX = 64, TTFLD_FLIMY, TTFLD_FLIMZ, TTFLD_DIFRX, TTFLD_DIFRY,
  TTFLD_DIFRZ, TTFLD_FLUX_X, TTFLD_FLUX_Y, TTFLD_FLUX_Z,
  /* planes (-1:NY+2,-1:NZ+2) */
  TTFLD_UPPERBND = 96, /* int32 */
  TTFLD_MU_STAR, TTFLD_TINCIDENT,
  /* stellar heating arrays */
  TTFLD_STELLARINPUT = 112, TTFLD_STELLARTAU, TTFLD_DTAUS
};

/* Grid sizes of the one subdomain (the reference's locNX/locNY/locNZ). */
typedef struct {
  int32_t nx, ny, nz;
  int32_t poles;  /* inc_poles (ipp:20).  1: the one-rank pole shifts
                     (ppshift.f:2217-2453) -- planes NZ-1..NZ-3 mirrored
                     onto NZ..NZ+2 and planes 1, 2 onto 0, -1 after every
                     phi exchange, no theta boundary rows, the SOR stopping
                     at NZ-1 (ppsor.f:39-43).  The SOR solvers of
                     COUPLED_ENERGY_EQS (exact, scaled and FP32/FP64) take
                     it, and so do DIFFUSION and RADDIF (every theta row,
                     the pole shifts after each colour, ppdif.f:45-135,
                     ppmat.f:39-136), and PCG (the mirror coupling of
                     rows 1 and NZ-1 in their diagonal, row NZ decoupled);
                     SOLVE_WITH_HYPRE returns TTFLD_E_UNSUPPORTED */
} ttfld_dims;

/* 1-D metric arrays of GITTER (ppinit.f:1028-1406), each passed with the
 * reference's bounds: xxa(0:NX+2) xxb(-1:NX+2) dxa(1:NX+2) dxb(0:NX+2),
 * the same pattern for y and z, ddx0/ddx1 (0:NX+2) ..., surxa/surxb,
 * surza/surzb, geoxga/geoxha, geozga (0:N+2), geoxg/geoxh, geozg (-1:N+2). */
typedef struct {
  const double *xxa, *xxb, *dxa, *dxb;
  const double *xya, *xyb, *dya, *dyb;
  const double *xza, *xzb, *dza, *dzb;
  const double *ddx0, *ddx1, *ddy0, *ddy1, *ddz0, *ddz1;
  const double *surxa, *surxb, *surza, *surzb;
  const double *geoxg, *geoxh, *geoxga, *geoxha, *geozg, *geozga;
} ttfld_metrics;

/* The input_init switches and constants the step reads (ppmod.f:2-33) plus
 * the opacity model. */
typedef struct {
  double delt;      /* DELT                                               */
  double sorparam;  /* SORPARAM (omega), ipp:13                           */
  double epsmat;    /* EPSMAT, ipp:13                                     */
  double fbottom;   /* Fbottom, ipp:12                                    */
  double tirr;      /* TIRR, ipp:22                                       */
  double xnue;      /* XNUE, ipp:8 (ieta=5 floor and DIFFUSION)           */
  double pr_num;    /* PR_NUM, ipp:8                                      */
  double kap0;      /* synthetic opacity scale, kappa_R = kap0*sqrt(rho)*(T/1000)^1.5*KMUL */
  int32_t itmax;    /* ITMAX (shared by SOR and the outer loop), ipp:13   */
  int32_t bcxmin;   /* BCXMIN, ipp:12 (9 implemented)                     */
  int32_t ibdrad;   /* IBDRAD, ipp:12 (4, 7, 9 implemented)               */
  int32_t iflimtyp; /* IFLIMTYP, ipp:12 (1, 2)                            */
  int32_t f_incident; /* F_INCIDENT, ipp:12 (0..5)                        */
  int32_t ieta;     /* IETA, ipp:8                                        */
  int32_t isigtyp;  /* ISIGTYP, ipp:10 (0, 1)                             */
  int32_t iii;      /* the main program's step counter III                */
  int32_t adjust_sor; /* call ADJUST_SOR_PARAM where the reference would  */
  int32_t kappa_model; /* 0 = synthetic analytic (stand-in for the tables) */
                       /* 1 = prescribed: XKAP* are uploaded, KAPPA no-op  */
                       /* 2 = a (T, rho) table, BurrowsOPC's interpolation
                              (ttfld_set_opacity_table)                    */
                       /* 3 = Freedman's (T, P) table, FreedmanOPC's
                              interpolation (ttfld_set_freedman_table)     */
} ttfld_params;

/* How SOLVE_WITH_SOR's linear system is solved on the device. */
enum ttfld_solver {
  TTFLD_SOLVER_SOR64_EXACT = 0, /* red-black SOR in FP64, same rounding as the
                                   reference loop (bitwise per sweep)      */
  TTFLD_SOLVER_SOR64_FAST = 1,  /* red-black SOR in FP64 on Jacobi-scaled
                                   coefficients with FMA (same iteration,
                                   different rounding)                     */
  TTFLD_SOLVER_MIXED = 2,       /* FP32 red-black sweeps inside FP64 defect
                                   correction, stopped on the true FP64
                                   residual ||b-Ax||_1/||b||_1            */
  TTFLD_SOLVER_PCG = 3          /* FP32 conjugate gradients (radial line
                                   preconditioner) on the symmetrised system
                                   inside FP64 defect correction, same stop
                                   rule as MIXED; a guess is kept if its
                                   preconditioned residual r.z is below the
                                   zero guess's (fallback rules 0 and 3)  */
};

enum ttfld_guess {
  TTFLD_GUESS_ZERO = 0,     /* delta_ER = 0 (ppsor.f:29)                   */
  TTFLD_GUESS_PREVIOUS = 1, /* the previous solve's solution: times
                               (1-conv_parm) inside a step, as is from one
                               step to the next                           */
  TTFLD_GUESS_LEARNED = 2   /* 3-D conv net prediction, zero-guess fallback  */
};

typedef struct {
  int32_t solver;      /* enum ttfld_solver                                */
  int32_t guess;       /* enum ttfld_guess                                 */
  double tol;          /* mixed solver: stop at ||b-Ax||_1/||b||_1 <= tol  */
  int32_t inner_digits; /* mixed solver: an FP32 inner run on A e = r stops
                          once its in-sweep norm is 10^-inner_digits of the
                          FP64 anchor's (or at tol, or at the FP32 rounding
                          floor); 0 = the default, 4: on the stiff
                          160x512x256 systems 5 reaches the FP32 rounding
                          floor before the target (8208 sweeps against
                          the FP64 loop's 7858), 3 and 4 do not (7864,
                          7872)                                           */
  int32_t reserved;    /* set to 0                                         */
  int32_t max_sweeps;  /* mixed solver sweep budget (0 = ITMAX)            */
  int32_t fallback_rule; /* when a previous/learned guess is replaced by 0:
                            0 = the residual its first red-black sweep
                                leaves (the in-sweep norm RNORM of the
                                second sweep) is not below the one the
                                first sweep from zero leaves;
                            1 = never;
                            2 = ||b - A x0||_1 >= ||b||_1;
                            3 = (default) as 0 after four sweeps (RNORM of
                                the fifth): robust to the cell-scale error
                                of a good guess, which the first sweep has
                                not yet removed.
                            The mixed solver runs tests 0 and 3 with its own
                            FP32 sweeps and keeps the winner's sweeps.   */
  int32_t sweep_form;  /* mixed solver's FP32 sweep kernel, every form
                          the same iterate: 0 = (default) one persistent
                          cooperative launch per FP64 anchor in which each
                          block waits between the colours only for the
                          blocks within one theta plane of its items
                          (per-block flags; a grid barrier after norm
                          sweeps only; two launches per sweep where
                          cooperative launch is unavailable), 1 = a
                          persistent launch with TMA-staged coefficients
                          (slower here), 2 = two launches per sweep, 3 = the
                          sweeps in pairs, each pair one wavefront over
                          windows of theta planes with a grid barrier per
                          phase (temporal blocking through L2), 4 = one
                          persistent launch with a grid barrier after each
                          colour */
} ttfld_solve_opts;

typedef struct {
  int32_t sor_iter;        /* sweeps of the last solve (SOR_ITER)          */
  int32_t corrections;     /* FP64 defect-correction passes (mixed)        */
  int32_t fallback;        /* 1 if the learned guess was rejected          */
  int32_t status;
  double rnorm;            /* global_RNORM of the last sweep               */
  double rhsnorm;          /* global_RHSNORM                               */
  double true_resid_l1;    /* ||b - A x||_1 at exit (mixed solver)         */
  double guess_resid_l1;   /* ||b - A x0||_1 of the initial guess          */
  double solve_ms;         /* device time of the solve (CUDA events on the
                              library's stream, guess included)           */
  double guess_ms;         /* of which: making and checking the initial
                              guess (network inference, fallback test)    */
  int32_t stalls;          /* FP32 inner runs ended at their rounding floor
                              and re-anchored in FP64 (mixed, PCG)        */
  int32_t gs_sweeps;       /* SOLVE_WITH_HYPRE: symmetric line Gauss-Seidel
                              sweeps per preconditioner application       */
} ttfld_solve_stats;

typedef struct {
  int32_t energy_iter;     /* outer Newton iterations (energy_ITER)        */
  int32_t sor_total;       /* sweeps summed over the step's solves         */
  int32_t solves;          /* linear solves in the step                    */
  int32_t fallbacks;       /* learned-guess rejections                     */
  int32_t status;
  int32_t stalls;          /* FP32 rounding-floor re-anchors, all solves   */
  double global_deltaq;    /* max |dQ/Q| of the last outer iteration       */
  double global_deltaer;   /* max |dER/ER| of the last outer iteration     */
  double solve_ms;         /* device time in the linear solves             */
  double step_ms;          /* device time of the whole step                */
} ttfld_step_stats;

typedef struct ttfld_ctx ttfld_ctx;

#if defined(__GNUC__)
#pragma GCC visibility push(default)
#endif

/* ---- lifetime (replaces the allocate* routines of ppmod.f for the
 *      arrays the step touches, and MPI_INIT's one-rank decomposition) ---- */
int ttfld_create(ttfld_ctx** out, const ttfld_dims* dims,
                 const ttfld_metrics* metrics, const ttfld_params* params,
                 int device);
int ttfld_destroy(ttfld_ctx* ctx);
int ttfld_set_params(ttfld_ctx* ctx, const ttfld_params* params);
int ttfld_get_params(const ttfld_ctx* ctx, ttfld_params* params);
int ttfld_set_solver(ttfld_ctx* ctx, const ttfld_solve_opts* opts);
const char* ttfld_status_string(int status);
int ttfld_abi_version(void);

/* ---- field transfer (module array <-> device) ------------------------- */
int ttfld_upload(ttfld_ctx* ctx, int field, const void* host);
int ttfld_download(ttfld_ctx* ctx, int field, void* host);
/* Element count of a field in its reference bounds (0 if unknown). */
size_t ttfld_field_size(const ttfld_ctx* ctx, int field);
/* Device pointer of a field (for callers that keep data on the GPU). */
void* ttfld_device_ptr(ttfld_ctx* ctx, int field);
/* Device copies inside the context: dst <- src (same storage class). */
int ttfld_copy_field(ttfld_ctx* ctx, int dst_field, int src_field);
int ttfld_synchronize(ttfld_ctx* ctx);
/* The cudaStream_t every call of this context is issued on (for callers
 * that order their own work or CUDA events against the library's). */
void* ttfld_stream(ttfld_ctx* ctx);

/* ---- the reference subroutines, device-resident ------------------------ */
/* BOUNDS, ppbou.f:1-92 (MODTYP=2) restricted to T, RH and UPPERBND. */
int ttfld_bounds(ttfld_ctx* ctx);
/* KAPPA, pprphy.f:1-360, and SUBSIG, pprphy.f:567-583, by kappa_model:
 * 0 the synthetic analytic opacity on the extents of the IKAPTYP 20:25
 * branch (pprphy.f:321-351); 1 nothing (XKAP* are the caller's); 2 that
 * branch with BurrowsOPC on the table of ttfld_set_opacity_table (and,
 * after ttfld_set_wave_table, the per-bin opacities xkapW); 3 the IKAPTYP
 * 4:5 branch (pprphy.f:88-110, MODTYP 2) with FreedmanOPC on the table of
 * ttfld_set_freedman_table and PRESSG's ideal-gas pressure (TTFLD_E_OPACITY
 * where the reference stops). */
int ttfld_kappa(ttfld_ctx* ctx);
/* CALCMUSTAR ppsub.f:156-179 and CALC_TINCIDENT pprad.f:296-405 are
 * evaluated by the caller and uploaded as MU_STAR / TINCIDENT. */
/* STELLARINPUT_HEATING, pprad.f:408-516: the grey branch (:490-502), or
 * after ttfld_set_wave_table the wavelength-binned branch of IKAPTYP 20-24
 * (:433-448, WAVELENGTH_CALCSTELLARTAU :519-547 and
 * WAVELENGTH_STELLAR_DTAU :549-568) on KAPPA's per-bin opacities. */
int ttfld_stellarinput_heating(ttfld_ctx* ctx);
/* DIFF, pprad.f:74-156, including FLIM pprphy.f:362-565; energy_iter <= 1
 * also re-evaluates KAPPA, SUBSIG and QDENS (pprphy.f:396-402). */
int ttfld_diff(ttfld_ctx* ctx, int energy_iter);
/* CALCULATEFLUX + FLUX_BC, ppenergy.f:880-982. */
int ttfld_calculateflux(ttfld_ctx* ctx, int energy_iter);
/* FILL_EVALUES(theta_param), ppenergy.f:984-1030. */
int ttfld_fill_evalues(ttfld_ctx* ctx, double theta);
/* FILL_SOR_MATRIX + B_VECTOR_BOUNDARIES, ppsor.f:189-329. */
int ttfld_fill_sor_matrix(ttfld_ctx* ctx);
/* SOLVE_WITH_SOR(print_max_values), ppsor.f:2-187: fills the matrix from the
 * device EVAL arrays and RHS_ER, solves for DELTA_ER with the configured
 * solver and guess.  stats may be NULL. */
int ttfld_solve_with_sor(ttfld_ctx* ctx, int print_max_values,
                         ttfld_solve_stats* stats);
/* As above on SOR_A..G / RHS_ER already on the device (no refill). */
int ttfld_solve_system(ttfld_ctx* ctx, ttfld_solve_stats* stats);
/* SOLVE_WITH_HYPRE, pphypre.f:1-111 (the IRAD=2 path): the system of
 * FILLHYPREMATRIX / FILLHYPREVECTORS (pphypre.f:115-334; SOLVE_WITH_SOR's
 * rows from the device EVAL arrays with the i=1 rows made identity rows and
 * b zero on the boundary rows; RHS_ER itself is not changed, SOR_A..G are
 * refilled) solved for DELTA_ER by PCG from x = 1 (pphypre.f:136) until
 * ||Sigma W (b-Ax)||_2 / ||Sigma W b||_2 <= tol on the symmetrised system,
 * or maxit iterations (then status 1).  tol <= 0 and maxit <= 0 select the
 * reference's 1e-6 and 50 (pphypre.f:45-55).  hypre's SMG preconditioner is
 * replaced by m symmetric red-black Gauss-Seidel sweeps over the radial
 * lines (each line solved exactly): m starts at 1 and, when a solve reaches
 * maxit before tol, the solve is run again from x = 1 with a larger m
 * (predicted from the rate it showed); the context keeps m for its next
 * solves (stats->gs_sweeps).  stats may be NULL. */
int ttfld_solve_with_hypre(ttfld_ctx* ctx, double tol, int maxit,
                           ttfld_solve_stats* stats);
/* The IRAD=1 radiation step, RADDIF (pprad.f:1-38): ER = arad T^4, DIFFEL
 * (DIFF's face coefficients into AX..CZ, pprad.f:40-72), B and RHS
 * (pprad.f:21-29), SOLVMAT (ppmat.f:1-186: red-black SOR on ER, stop at
 * ||XS||_2/||RHS||_2 <= EPSMAT after at least 5 iterations, or ITMAX, then
 * status 1) with RADIATIVEBOUND (ppbou.f:2049-2299) after each colour, and
 * T = (ER/arad)^(1/4).  RADIATIVEBOUND is implemented for the IBDRAD values
 * the context accepts (4, 7, 9) with MODVER <= 5 (MODVER > 5: status -3). */
typedef struct {
  double d_t;           /* D_T, the bottom temperature gradient of the model
                           (LOCALINIT, ppinit.f:149-245)                    */
  double tinit_bottom;  /* TinitBottom (the bottom T when BCXMIN = 6)      */
  int32_t modver;       /* MODVER                                           */
  int32_t energy_iter;  /* energy_iter as DIFF/FLIM read it (<= 1: KAPPA,
                           SUBSIG and QDENS are evaluated first)            */
  const double* volxb;  /* VOLXB(1:NX), VOLYB(1:NY), VOLZB(1:NZ) of GITTER
                           (ppinit.f:1342-1376), host memory               */
  const double* volyb;
  const double* volzb;
} ttfld_raddif_params;
int ttfld_raddif(ttfld_ctx* ctx, const ttfld_raddif_params* params,
                 ttfld_solve_stats* stats);
/* Exactly n red-black sweeps on the current system from the current
 * DELTA_ER, FP64, reference rounding (for sweep-by-sweep parity tests). */
int ttfld_sor_sweeps(ttfld_ctx* ctx, int n, double* rnorm, double* rhsnorm);
/* ||b - A x||_1 (FP64) of the current system with x = DELTA_ER. */
int ttfld_true_residual(ttfld_ctx* ctx, double* l1, double* rhs_l1);
/* ADJUST_SOR_PARAM, ppsor.f:332-354 (50 solves, omega = 1.01 + 0.02 n). */
int ttfld_adjust_sor_param(ttfld_ctx* ctx, double* sorparam);
/* COUPLED_ENERGY_EQS, ppenergy.f:2-791 (IRAD=3).  do_bounds=1 runs the
 * device BOUNDS first, as ppenergy.f:63 does; a Fortran caller that keeps
 * BOUNDS on the host passes 0 after uploading T, RH and UPPERBND. */
int ttfld_coupled_energy_eqs(ttfld_ctx* ctx, int do_bounds,
                             ttfld_step_stats* stats);
/* DIFFUSION(scalar), ppdif.f:1-167, on the SCALAR field (the pass_sc
 * module array) with diffusion constant xnue/pr_num.  As at the reference's
 * call sites, SCALAR's phi halo must be current (PLANETSHIFT(10)) on entry. */
int ttfld_diffusion(ttfld_ctx* ctx, ttfld_solve_stats* stats);

/* Marks the next solve as the first of an implicit step: it starts from the
 * previous solution unscaled (TTFLD_GUESS_PREVIOUS, and TTFLD_GUESS_LEARNED
 * once the run has one).  ttfld_coupled_energy_eqs does this itself; a
 * caller that runs its own step loop around ttfld_solve_with_sor calls it at
 * the top of each step.  new_run = 1 also forgets the previous solution (a
 * new run, or a state it does not belong to): the next solve then starts
 * from the learned guess or zero.  No reference counterpart. */
int ttfld_begin_step(ttfld_ctx* ctx, int new_run);

/* FP64 energy sums over the active cells (below UPPERBND, not an identity
 * row of FILL_SOR_MATRIX: i < min(UPPERBND, NX), 1 < k < NZ), each cell
 * weighted by V = surxb(i) dxa(i) dya(j) surzb(k) dza(k), the weight under
 * which the discrete divergence of CALCULATEDIVF_WITHF telescopes (V is
 * proportional to the cell volume).  Summed in a fixed order, so the
 * results are reproducible.  No reference counterpart. */
typedef struct {
  double volume;       /* sum of V                                         */
  double e_rad;        /* sum of V E_R                                     */
  double e_gas;        /* sum of V Q                                       */
  double heating;      /* sum of V STELLARINPUT (per unit time)            */
  double flux_bottom;  /* FLUX_X through the faces i = 1, into the region  */
  double flux_top;     /* FLUX_X through the upper faces of the last active
                          cells, out of the region                        */
  double flux_theta;   /* FLUX_Z through the faces k = 2 and k = NZ, out  */
} ttfld_energy;
/* The sums of the current state (E_R, Q, STELLARINPUT, FLUX_X/Z). */
int ttfld_energy_sums(ttfld_ctx* ctx, ttfld_energy* out);

/* The opacity table of kappa_model 2 (BurrowsOPC, pprphy.f:1005-1229, as
 * KAPPA's IKAPTYP 20:25 branch calls it, pprphy.f:321-351): log10 T and
 * log10 rho nodes (increasing) and log10 of the Rosseland, Planck and
 * absorption means on them, T index fastest (the layout of
 * BurrowsXKAP_ross(IT,IW)).  The reference reads them from files
 * (READBURROWSOPCTABLE, pprphy.f:1231-1541) that are not in its tree; the
 * caller passes the arrays.  Host memory, copied. */
typedef struct {
  int32_t nt, nrh;
  const double* log_t;     /* (nt)  */
  const double* log_rho;   /* (nrh) */
  const double* log_ross;  /* (nt, nrh) */
  const double* log_plnk;
  const double* log_abs;
} ttfld_opacity_table;
int ttfld_set_opacity_table(ttfld_ctx* ctx, const ttfld_opacity_table* table);

/* The per-wavelength-bin part of the same Burrows table for IKAPTYP 20-24:
 * log10 BurrowsXKAP_waveopac on the kappa_model 2 table's nodes (nt x nrh x
 * nbins, T fastest, bin slowest; pprphy.f:1138-1151), the star's flux per
 * bin BSTAR_BIN (READBURROWSOPCTABLE's BSTAR_WAVEBINS file,
 * pprphy.f:1525-1539), RSTAR in solar radii (ipp) and the orbit's semi-major
 * axis semi in cm (pp.f:205).  Needs ttfld_set_opacity_table first; the
 * per-bin opacities and optical depths take 2 x nbins halo arrays on the
 * device.  nbins = 0 drops the table (grey heating again).  Host memory,
 * copied. */
typedef struct {
  int32_t nbins;
  const double* log_waveopac;  /* (nt, nrh, nbins) */
  const double* bstar_bin;     /* (nbins) */
  double rstar;                /* RSTAR, solar radii */
  double semi;                 /* semi-major axis, cm */
} ttfld_wave_table;
int ttfld_set_wave_table(ttfld_ctx* ctx, const ttfld_wave_table* table);

/* FreedmanOPC's table for kappa_model 3 (pprphy.f:800-942; read by
 * READFREEDMANOPCTABLE, pprphy.f:944-1002, from files not in the
 * reference's tree): log10 Rosseland, Planck and absorption means on the
 * 42 FreedmanTVAL x 18 FreedmanPVAL nodes (ppmod.f:690-700; T index
 * fastest), and the gas's mu_gas for PRESSG's ideal-gas pressure
 * PG = Rgas T RH / mu_gas (ppphy.f:17-20).  Host memory, copied. */
typedef struct {
  const double* log_ross;  /* (42, 18) */
  const double* log_plnk;
  const double* log_abs;
  double mu_gas;
} ttfld_freedman_table;
int ttfld_set_freedman_table(ttfld_ctx* ctx, const ttfld_freedman_table* table);

/* ---- measurement (no reference counterpart) --------------------------- */
/* Runs n back-to-back sweeps of a solver's sweep kernels on the current
 * system (TTFLD_SOLVER_SOR64_EXACT: DELTA_ER is iterated in place;
 * SOR64_FAST / MIXED: only their private iterate is touched) and returns
 * the mean device time of one full sweep (both colours), CUDA events on the
 * library's stream.  MIXED times the solver's own kernel (all n sweeps in
 * one launch of sweep_form 0, the in-sweep norm every 8th); for comparison,
 * solver = 3 times the same FP32 sweeps issued as two launches per sweep,
 * solver = 4 as one launch of the TMA-staged persistent kernel, solver = 5
 * as one launch of the wavefront form (sweep_form 3) with its own window
 * size, solver = 16 + P with windows of P theta planes (P = 1..256) and
 * solver = 6 as one launch of the grid-barrier kernel (sweep_form 4). */
int ttfld_time_sweeps(ttfld_ctx* ctx, int solver, int n, double* ms_per_sweep);
/* Number of kernels this process has launched through libttfld. */
uint64_t ttfld_kernel_launches(void);

/* ---- learned initial guess (no reference counterpart) ----------------- */
/* A 3-D U-Net (4 levels, 16-32-64-64 channels, 3x3x3 kernels, BF16 weights
 * and activations, FP32 accumulation on the tensor cores, run at half the
 * grid's resolution) maps the state of a solve -- log E, log kappa_R,
 * log rho, log dt and the heating -- to delta_ER / E, SOLVE_WITH_SOR's
 * initial iterate where the run has no previous solution yet (its first
 * solve, or after ttfld_begin_step(ctx, 1)); with TTFLD_GUESS_LEARNED the
 * solves after that start from the previous solution, which over a run is
 * the better guess.  It is trained on the GPU on pairs captured from this
 * context's own solves. */
/* Random (seeded, He-normal) weights for this context's grid. */
int ttfld_guess_init(ttfld_ctx* ctx, uint64_t seed);
/* Device storage for up to `capacity` training pairs (16 BF16 inputs per
 * 2x2x2 cells, a BF16 target and a mask per cell; about 7 B per cell and
 * pair). */
int ttfld_guess_dataset(ttfld_ctx* ctx, int capacity);
/* Store the next solve of this context (its starting state and its answer)
 * as a training pair. */
int ttfld_guess_capture_next(ttfld_ctx* ctx);
int ttfld_guess_dataset_count(ttfld_ctx* ctx);
/* Adam (lr, beta 0.9/0.999) over the stored pairs, `epochs` seeded passes;
 * mean masked MSE of the normalised target over the steps in *mean_loss. */
int ttfld_guess_train(ttfld_ctx* ctx, int epochs, double lr, uint64_t seed, double* mean_loss);
/* Loss and gradient of every parameter for one input (NX*NY*NZ cells x 5
 * features, r fastest), target and mask -- the hook gradient checks use. */
int ttfld_guess_gradients(ttfld_ctx* ctx, const float* feat, const float* target,
                          const unsigned char* mask, double* loss, float* grads);
/* Network output (normalised target units) for one input. */
int ttfld_guess_predict(ttfld_ctx* ctx, const float* feat, float* pred);
size_t ttfld_guess_num_params(void);
/* Kernel form of the network's large-level convolutions, for the process:
 * 0 mma.sync on shared-memory tiles everywhere, 1 tcgen05 (5th-generation
 * tensor cores, accumulators in tensor memory, operands by TMA) on every
 * layer it takes, 2 (default) tcgen05 on the layers with 16 output channels,
 * where it is the faster form, mma.sync elsewhere.  Same results up to FP32
 * summation order. */
int ttfld_guess_set_conv(int use_tcgen05);
/* Weights blob: "TTFLDNN2", uint64 parameter count, FP32 parameters. */
int ttfld_guess_load(ttfld_ctx* ctx, const void* blob, size_t bytes);
int ttfld_guess_save(ttfld_ctx* ctx, void* blob, size_t bytes, size_t* needed);

/* ---- solve without any allocation ------------------------------------- */
/* No counterpart in the reference.  The FP64 red-black SOR solve of
 * SOLVE_WITH_SOR (the same iterate, bit for bit, and the same stopping rule
 * as ttfld_solve_with_sor with TTFLD_SOLVER_SOR64_EXACT) on arrays the caller
 * already holds on the device, with no context and no device allocation.
 * It is for callers that cannot let a library call cudaMalloc: hosts whose
 * device memory is all managed by their own pool or offload data region,
 * jobs held to a fixed memory budget beside other work on the GPU, and codes
 * that must not have a hidden allocation or free synchronise the device
 * under their running kernels.
 *   sor_a..sor_g, rhs : device pointers, cell layout (1:NX,1:NY,1:NZ)
 *   x                 : device pointer, halo layout (-1:NX+2,-1:NY+2,-1:NZ+2);
 *                       holds the initial iterate and the fixed ghost
 *                       values, returns the solution with its phi halo
 *                       refreshed as PLANETSHIFT(8) does
 *   stream            : the cudaStream_t to run on (NULL = default stream)
 * Its only working memory is one fixed __device__ array of 2 MiB + 256 B
 * that every GPU loading the library keeps until the process exits; grids
 * with NY*NZ > 131072 are rejected with TTFLD_E_ARGS.  All calls on a device
 * share that array (each clears what it needs at its start), so calls whose
 * GPU work overlaps race and must be serialised by the caller.  The first
 * call on a device (in each CUDA context: a caller's own context on the
 * device counts as a new one) looks up the array's device address in that
 * context.  Every call returns only after its solve has finished on the
 * GPU (it blocks the calling host thread): it waits on `stream` to read
 * the stopping flag between chunks of sweeps.  NY must be
 * even. */
int ttfld_sor_solve_noalloc(const double* sor_a, const double* sor_b, const double* sor_c,
                            const double* sor_d, const double* sor_e, const double* sor_f,
                            const double* sor_g, const double* rhs, double* x, int nx, int ny,
                            int nz, double omega, double epsmat, int itmin, int itmax,
                            void* stream, int* sor_iter, double* rnorm, double* rhsnorm);

#if defined(__GNUC__)
#pragma GCC visibility pop
#endif

#ifdef __cplusplus
}
#endif
#endif /* TTFLD_H */
