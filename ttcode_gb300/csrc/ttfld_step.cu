// ttfld_step.cu -- COUPLED_ENERGY_EQS (ppenergy.f:2-791, IRAD=3) on the
// device: the damped Newton loop over (Q = rho c_v T, E_R) with one linear
// solve for delta E_R per outer iteration.  Every array stays in HBM for
// the whole step; the host reads back one small struct per outer iteration
// (the two max-norms that decide convergence).
#include <string.h>

#include "ttfld_internal.cuh"

namespace ttfld {
int asm_kappa(ttfld_ctx* c);
int asm_calculateflux(ttfld_ctx* c, int energy_iter, bool skip_kappa = false, bool skip_qdens = false);
int asm_fill_evalues(ttfld_ctx* c, double theta);
int asm_divf(ttfld_ctx* c, double* out, double theta, bool fill = true);
int asm_stellar(ttfld_ctx* c);
int asm_bounds(ttfld_ctx* c);
int asm_top_fluxes(ttfld_ctx* c, bool kappa_done);
int asm_prepare(ttfld_ctx* c);
int solve_delta_er(ttfld_ctx* c, ttfld_solve_stats* st);

// Q/E_R upper boundary, ppenergy.f:80-105 and :678-702.  FLUX_X is declared
// (1:NX+1,1:NY,1:NZ) (ppmod.f:513) but the loop runs i to NX+2 and over the
// j,k ghosts; those reads are clamped into the array here.  The cells they
// feed (ghost corners and the i=NX+2 plane of E_R) are never read by the
// step.
static int upper_bc(ttfld_ctx* c) {
  Dev d = c->d;
  launch_box(c->stream, box(1, d.nx + 2, -1, d.ny + 2, -1, d.nz + 2), [=] __device__(int i, int j, int k) {
    int ub = PA(UB, j, k);
    if (i < ub || ub < 1) return;
    double qupper = HA(RH, ub - 1, j, k) * HA(CV, ub - 1, j, k) * HA(T, ub, j, k);
    int ic = i > d.nx + 1 ? d.nx + 1 : i;
    int jc = j < 1 ? 1 : (j > d.ny ? d.ny : j);
    int kc = k < 1 ? 1 : (k > d.nz ? d.nz : k);
    HA(Q, i, j, k) = qupper;
    HA(ER, i, j, k) = fabs(2.0 * FA(FLUXX, ic, jc, kc) / TT_FD);
  });
  TT_CHECK_LAUNCH();
  return 0;
}

// Left (XMIN) boundary for BCXMIN=9, ppenergy.f:150-167 and :620-637.
static int left_bc(ttfld_ctx* c) {
  Dev d = c->d;
  if (d.bcxmin != 9) return TTFLD_E_UNSUPPORTED;
  launch_box(c->stream, box(0, 0, -1, d.ny + 2, -1, d.nz + 2), [=] __device__(int, int j, int k) {
    double dqdr;
    if (d.ieta == 5)
      dqdr = -HA(RH, 1, j, k) * HA(CV, 1, j, k) * d.fbottom /
             (HA(RH, 1, j, k) * HA(CV, 1, j, k) * (d.xnue / d.pr_num));
    else
      dqdr = -(HA(RH, 1, j, k) * HA(CV, 1, j, k) * 3.0 * d.fbottom * HA(XKAPR, 1, j, k) * HA(RH, 1, j, k) /
               (4.0 * TT_ARAD * TT_FD * p3(HA(T, 1, j, k))));
    HA(Q, 0, j, k) = HA(Q, 1, j, k) - dqdr * (G(xxb, 1) - G(xxb, 0));
    HA(Q, -1, j, k) = HA(Q, 1, j, k) - dqdr * (G(xxb, 1) - G(xxb, -1));
    HA(ER, 1, j, k) = TT_ARAD * p4(HA(Q, 1, j, k) / (HA(RH, 1, j, k) * HA(CV, 1, j, k)));
    HA(ER, 0, j, k) = TT_ARAD * p4(HA(Q, 0, j, k) / (HA(RH, 0, j, k) * HA(CV, 0, j, k)));
    HA(ER, -1, j, k) = TT_ARAD * p4(HA(Q, -1, j, k) / (HA(RH, -1, j, k) * HA(CV, -1, j, k)));
  });
  TT_CHECK_LAUNCH();
  return 0;
}

// theta boundaries without poles, ppenergy.f:204-227 and :706-733.
static int z_bc(ttfld_ctx* c) {
  Dev d = c->d;
  if (d.poles) return 0;  // the pole shifts of ER take their place
  launch_box(c->stream, box(-1, d.nx + 2, -1, d.ny + 2, 0, 0), [=] __device__(int i, int j, int) {
    const int nz = d.nz;
    HA(Q, i, j, 1) = HA(Q, i, j, 2);
    HA(ER, i, j, 1) = HA(ER, i, j, 2);
    HA(Q, i, j, 0) = HA(Q, i, j, 1);
    HA(Q, i, j, -1) = HA(Q, i, j, 1);
    HA(ER, i, j, 0) = HA(ER, i, j, 1);
    HA(ER, i, j, -1) = HA(ER, i, j, 1);
    HA(Q, i, j, nz) = HA(Q, i, j, nz - 1);
    HA(ER, i, j, nz) = HA(ER, i, j, nz - 1);
    HA(Q, i, j, nz + 1) = HA(Q, i, j, nz);
    HA(Q, i, j, nz + 2) = HA(Q, i, j, nz);
    HA(ER, i, j, nz + 1) = HA(ER, i, j, nz);
    HA(ER, i, j, nz + 2) = HA(ER, i, j, nz);
  });
  TT_CHECK_LAUNCH();
  return 0;
}

// One pass over the cells for an outer iteration's linear system:
// CALCULATEDIVF_WITHF's divergence (ppenergy.f:285, from the metric-quotient
// table; in the first iteration the fluxes are those DIVF_OLD was formed
// from, so DIVF is DIVF_OLD), the per-cell FQ, FR, Jacobian, eta and RHS_ER
// (:287-345), FILL_EVALUES (:348), and FILL_SOR_MATRIX with
// B_VECTOR_BOUNDARIES (ppsor.f:24-26).  Each cell reads only its own cell
// values and its faces, so fusing the loops keeps every value bit for bit.
static int rows(ttfld_ctx* c, double theta, bool divf_is_old) {
  Dev d = c->d;
  const DivfTab t = divf_tab(c);
  launch_box(c->stream, box(1, d.nx, 1, d.ny, 1, d.nz), [=] __device__(int i, int j, int k) {
    size_t h = hidx(d, i, j, k), q = cidx(d, i, j, k);
    const double divf = divf_is_old ? d.DIVF_OLD[q] : divf_cell(d, t, i, j, k);
    d.DIVF[q] = divf;
    double qq = d.Q[h], rh = d.RH[h], cv = d.CV[h], er = d.ER[h], kp = d.XKAPP[h];
    double qr = qq / (rh * cv);
    double bb = TT_ARAD * p4(qr);
    double fq, dfq;
    double dfr = -((d.delt / cv) * (kp * 4.0 * TT_ARAD * TT_FD * p3(qr) + TT_FD * (bb - er) * d.DXKAPP[h]));
    if (d.f_incident > 1) {
      double si = d.SI[h];
      double heat = si / (rh * d.XKAPA[h]);
      fq = qq - d.Q_OLD[h] + d.delt * ((1 - theta) * (d.DIVF_OLD[q] - divf) + (rh * kp * TT_FD * (bb - er)) - si);
      dfq = 1.0 + (d.delt / cv) * (kp * 4.0 * TT_ARAD * TT_FD * p3(qr) + (TT_FD * (bb - er) * d.DXKAPP[h]) -
                                   heat * d.DXKAPA[h]);
    } else {
      fq = qq - d.Q_OLD[h] + d.delt * ((1 - theta) * (d.DIVF_OLD[q] - divf) + rh * kp * TT_FD * (bb - er));
      dfq = 1.0 + (d.delt / cv) * (kp * 4.0 * TT_ARAD * TT_FD * p3(qr) + TT_FD * (bb - er) * d.DXKAPP[h]);
    }
    double fr = er - d.ER_OLD[h] + d.delt * (divf - rh * kp * TT_FD * (bb - er));
    d.FQ[q] = fq; d.FR[q] = fr; d.DFQ[q] = dfq; d.DFR[q] = dfr;
    double eta;
    if (dfq != 0.0) eta = -dfr / dfq;
    else { eta = 0.0; d.stp->dfq_zero = 1; }
    d.ETA[q] = eta;
    const EvalRow e = evalues_cell(d, i, j, k, theta, eta);
    store_evalues(d, q, e);
    const bool ident = sor_row(d, i, j, k, q, e);
    d.RHS[q] = ident ? 0.0 : -fr - eta * fq;
  });
  TT_CHECK_LAUNCH();
  return 0;
}

// Algebraic delta Q with the positivity guard and the two max-norms
// (ppenergy.f:379-541), fused with the damped update of :551-573 (each cell
// reads only its own Q and E_R, which only it updates).
__global__ void __launch_bounds__(kThreads) delta_q_kernel(Dev d, double theta, double conv) {
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  const long long n = (long long)(nx - 1) * ny * nz;  // i = 2..NX
  const size_t sj = (size_t)(nx + 4), sk = (size_t)(nx + 4) * (ny + 4);
  const double* x = d.DELTA_ER;
  double mq = 0.0, me = 0.0;
  int bad = 0;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    int i = 2 + (int)(t % (nx - 1));
    long long r = t / (nx - 1);
    int j = (int)(r % ny) + 1, k = (int)(r / ny) + 1;
    int xmax_index = PA(UB, j, k) - 1;
    if (i > xmax_index || xmax_index > nx) continue;
    size_t h = hidx(d, i, j, k), q = cidx(d, i, j, k);
    double q1 = -d.delt * (1.0 - theta);
    double q2 = d.delt * d.RH[h] * d.XKAPP[h] * TT_FD;
    double dq = (1.0 / d.DFQ[q]) *
                (q1 * d.E16[q] * x[h] - q1 * d.E1[q] * x[h + 1] - q1 * d.E2[q] * x[h - 1] -
                 q1 * d.E3[q] * x[h + sj] - q1 * d.E4[q] * x[h - sj] - q1 * d.E5[q] * x[h + sk] -
                 q1 * d.E6[q] * x[h - sk] + q2 * x[h] - d.FQ[q]);
    d.DQ[q] = dq;
    double qv = d.Q[h], erv = d.ER[h];
    if ((qv + conv * dq) <= 0.0) bad = 1;
    mq = fmax(mq, fabs(dq / qv));
    me = fmax(me, fabs(x[h] / erv));
    d.ER[h] = erv + conv * x[h];
    d.Q[h] = qv + conv * dq;
  }
  // max is exact in any order: reduce in the warp, one atomic per warp
  for (int o = 16; o > 0; o >>= 1) {
    mq = fmax(mq, __shfl_xor_sync(0xffffffffu, mq, o));
    me = fmax(me, __shfl_xor_sync(0xffffffffu, me, o));
    bad |= __shfl_xor_sync(0xffffffffu, bad, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomic_max_nonneg(&d.stp->maxq_bits, mq);
    atomic_max_nonneg(&d.stp->maxer_bits, me);
    if (bad) d.stp->nonpositive_q = 1;
  }
}

static int delta_q_update(ttfld_ctx* c, double theta, double conv) {
  const Dev& d = c->d;
  delta_q_kernel<<<grid_for((long long)(d.nx - 1) * d.ny * d.nz), kThreads, 0, c->stream>>>(d, theta, conv);
  count_launches(1);
  TT_CHECK_LAUNCH();
  return 0;
}

static int finish_step(ttfld_ctx* c) {  // ppenergy.f:787-789
  Dev d = c->d;
  launch_box(c->stream, box(-1, d.nx + 2, -1, d.ny + 2, -1, d.nz + 2), [=] __device__(int i, int j, int k) {
    size_t h = hidx(d, i, j, k);
    d.DELTA_ER[h] = d.ER[h] - d.ER_OLD[h];
    d.T[h] = d.Q[h] / (d.RH[h] * d.CV[h]);
  });
  TT_CHECK_LAUNCH();
  return 0;
}

int coupled_energy_eqs(ttfld_ctx* c, int do_bounds, ttfld_step_stats* out) {
  const double delta_max = 0.005, conv_parm = 0.1, theta = 1.0;  // ppenergy.f:42, 49, 60
  Dev d = c->d;
  ttfld_step_stats st{};
  int rc;
  cudaEvent_t t0, t1;
  TT_CHECK(cudaEventCreate(&t0));
  TT_CHECK(cudaEventCreate(&t1));
  TT_CHECK(cudaEventRecord(t0, c->stream));
  TT_CHECK(cudaMemsetAsync(d.DELTA_ER, 0, nhalo(d) * 8, c->stream));  // :52-53
  TT_CHECK(cudaMemsetAsync(d.DQ, 0, ncell(d) * 8, c->stream));
  c->prev_scale = 1.0;  // the last step's solution guesses this step's first solve as is
  c->solve_idx = 0;
  if (do_bounds && (rc = asm_bounds(c))) return rc;                     // :63
  launch_box(c->stream, box(-1, d.nx + 2, -1, d.ny + 2, -1, d.nz + 2), [=] __device__(int i, int j, int k) {
    size_t h = hidx(d, i, j, k);
    d.Q[h] = d.RH[h] * d.CV[h] * d.T[h];                                 // :65
  });
  TT_CHECK_LAUNCH();
  // Recomputations that reproduce their inputs bit for bit are left out:
  // KAPPA and QDENS inside FLIM (energy_iter <= 1, pprphy.f:396-402) see the
  // T and rho of the first call of this step, and the FILL_EVALUES that
  // CALCULATEDIVF_WITHF ends with (ppenergy.f:876) is overwritten by the one
  // at :348 before anything reads the EVAL arrays.
  bool kappa_done = false;
  if (d.f_incident > 1) {                                               // :68-71
    if ((rc = asm_kappa(c)) || (rc = asm_stellar(c))) return rc;
    kappa_done = true;
  }
  if ((rc = asm_prepare(c))) return rc;
  // :74-75: only the top faces' fluxes are read (by :80-105) before :253-255
  // forms every face again
  if ((rc = asm_top_fluxes(c, kappa_done))) return rc;
  if ((rc = upper_bc(c)) || (rc = left_bc(c)) || (rc = z_bc(c))) return rc;
  if ((rc = halo_shift(c, d.ER)) || (rc = pole_shift(c, d.ER))) return rc;   // :230-245
  TT_CHECK(cudaMemcpyAsync(d.Q_OLD, d.Q, nhalo(d) * 8, cudaMemcpyDeviceToDevice, c->stream));
  TT_CHECK(cudaMemcpyAsync(d.ER_OLD, d.ER, nhalo(d) * 8, cudaMemcpyDeviceToDevice, c->stream));
  if ((rc = asm_calculateflux(c, 0, true, true))) return rc;            // :253-255
  if ((rc = asm_divf(c, d.DIVF_OLD, theta, false))) return rc;
  int energy_iter = 0;
  int status = TTFLD_OK;
  double solve_ms = 0.0;
  for (;;) {
    ++energy_iter;                                                      // :260
    if ((rc = halo_shift(c, d.ER)) || (rc = pole_shift(c, d.ER))) return rc; // :264-279
    // :283-285.  In the first iteration the fluxes are those of :253-255
    // already in FLUX_X/Y/Z: E_R, T and rho are unchanged since, the halo
    // shift just done repeats the one of :230-245, and FLIM at energy_iter
    // 0 and 1 takes the same branch (:396-402) -- so they are not formed again.
    if (energy_iter > 1 && (rc = asm_calculateflux(c, energy_iter))) return rc;
    if ((rc = rows(c, theta, energy_iter == 1))) return rc;             // :285-348, ppsor.f:24-26
    if (c->params.adjust_sor && energy_iter == 1 && (c->params.iii % 10000 == 0 || c->params.iii == 1)) {
      if ((rc = ttfld_adjust_sor_param(c, nullptr))) return rc;         // :372-374
      d = c->d;
      if ((rc = fill_sor_matrix(c))) return rc;
    }
    ttfld_solve_stats ss{};
    rc = solve_delta_er(c, &ss);                                        // :375
    if (rc < 0) return rc;
    solve_ms += c->last_solve_ms;
    st.sor_total += ss.sor_iter;
    st.solves += 1;
    st.fallbacks += ss.fallback;
    st.stalls += ss.stalls;
    if (rc == TTFLD_MAXITER)
      printf("MAX COUPLED SOR ITERATION %8d %8d %12.6e\n", c->params.iii, energy_iter, ss.rnorm / ss.rhsnorm);
    TT_CHECK(cudaMemsetAsync(c->stp, 0, sizeof(StepDev), c->stream));
    if ((rc = delta_q_update(c, theta, conv_parm))) return rc;          // :379-573
    if ((rc = left_bc(c)) || (rc = upper_bc(c)) || (rc = z_bc(c))) return rc;  // :578-733
    StepDev hs;
    TT_CHECK(cudaMemcpyAsync(&hs, c->stp, sizeof(StepDev), cudaMemcpyDeviceToHost, c->stream));
    TT_CHECK(cudaStreamSynchronize(c->stream));
    if (hs.nonpositive_q) { status = TTFLD_E_NONPOSITIVE_Q; break; }   // CLEAN_STOP, :519
    memcpy(&st.global_deltaq, &hs.maxq_bits, 8);
    memcpy(&st.global_deltaer, &hs.maxer_bits, 8);
    if (energy_iter == c->params.itmax) {                               // :750-775
      printf("Max iteration reached in coupled_energy_eqs %8d %12.6e %12.6e\n", energy_iter,
             st.global_deltaq, st.global_deltaer);
      status = TTFLD_MAXITER;
      break;
    }
    if (!(st.global_deltaq > delta_max)) break;                         // :778
  }
  if (status >= 0 && (rc = finish_step(c))) return rc;
  TT_CHECK(cudaEventRecord(t1, c->stream));
  TT_CHECK(cudaEventSynchronize(t1));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, t0, t1);
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  st.energy_iter = energy_iter;
  st.solve_ms = solve_ms;
  st.step_ms = ms;
  st.status = status;
  if (out) *out = st;
  return status;
}

}  // namespace ttfld

extern "C" int ttfld_coupled_energy_eqs(ttfld_ctx* c, int do_bounds, ttfld_step_stats* st) {
  if (!c) return TTFLD_E_ARGS;
  TT_CHECK(cudaSetDevice(c->device));
  return ttfld::coupled_energy_eqs(c, do_bounds, st);
}
