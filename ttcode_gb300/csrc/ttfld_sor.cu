// ttfld_sor.cu -- FILL_SOR_MATRIX / B_VECTOR_BOUNDARIES and the FP64
// red-black SOR of SOLVE_WITH_SOR (ppsor.f:2-329) on the device.
//
// The exact kernel evaluates each cell update with the reference's operand
// order and no fused multiply-add, so every sweep leaves DELTA_ER bitwise
// equal to the serial Fortran loop: within one colour no cell reads another
// cell of the same colour, so the order of the updates inside a colour does
// not change any value.  The periodic phi direction is read by wrapping the
// j index, which equals the reference's halo copy (PLANETSHIFT(8)) after
// each colour because NY is even (the two wrapped neighbours have the
// other colour).  The L1 norm of the in-sweep residuals is reduced in a
// fixed order (block partials, then one block), so the sweep count is
// reproducible run to run.
#include "ttfld_internal.cuh"

namespace ttfld {

// FILL_SOR_MATRIX ppsor.f:189-277 and B_VECTOR_BOUNDARIES ppsor.f:280-329,
// one rank; with poles the theta-edge rows stay ordinary rows (sor_row).
// zero_rhs = false leaves RHS_ER as it is (B_VECTOR_BOUNDARIES not applied).
int fill_sor_matrix(ttfld_ctx* c, bool zero_rhs) {
  Dev d = c->d;
  launch_box(c->stream, box(1, d.nx, 1, d.ny, 1, d.nz), [=] __device__(int i, int j, int k) {
    const size_t q = cidx(d, i, j, k);
    EvalRow r;
    r.e1 = d.E1[q]; r.e2 = d.E2[q]; r.e3 = d.E3[q]; r.e4 = d.E4[q]; r.e5 = d.E5[q]; r.e6 = d.E6[q];
    r.e7 = d.E7[q]; r.e8 = d.E8[q]; r.e16 = d.E16[q];
    if (sor_row(d, i, j, k, q, r) && zero_rhs) d.RHS[q] = 0.0;
  });
  TT_CHECK_LAUNCH();
  return 0;
}

// Sum |b| over the interior (RHSNORM, ppsor.f:33) and reset the solver state.
__global__ void __launch_bounds__(kThreads) rhsnorm_kernel(Dev d, const double* b, double* partials) {
  __shared__ double sh[32];
  __shared__ bool last;
  const long long n = (long long)ncell(d);
  double acc = 0.0;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x)
    acc += fabs(b[t]);
  double s = block_sum(acc, sh);
  if (threadIdx.x == 0) {
    partials[blockIdx.x] = s;
    __threadfence();
    last = (atomicAdd(&d.sol->ticket2, 1u) == gridDim.x - 1);
  }
  __syncthreads();
  if (last) {
    __threadfence();
    double tot = block_sum_array(partials, gridDim.x, sh);
    if (threadIdx.x == 0) {
      d.sol->rhsnorm = tot;
      d.sol->ticket2 = 0;
    }
  }
}

// One colour of the red-black loop, ppsor.f:59-88 (COLOUR 0) and :107-136
// (COLOUR 1), reference rounding.  x is a halo array.
template <int COLOUR>
__global__ void __launch_bounds__(kThreads) sor_exact_kernel(Dev d, double* __restrict__ x,
                                                             const double* __restrict__ b, double omega,
                                                             double* partials, int itmin, int itmax, double eps) {
  __shared__ double sh[32];
  __shared__ bool last;
  if (solver_done(d)) return;
  const int nx = d.nx, ny = d.ny;
  const int nxh = (nx + 1) >> 1;
  const long long n = (long long)nxh * ny * sor_zmax(d);  // rows k = 1..zmax_sor_index
  const size_t sj = (size_t)(nx + 4), sk = (size_t)(nx + 4) * (ny + 4);
  double acc = 0.0;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    int h = (int)(t % nxh);
    long long r = t / nxh;
    int j = (int)(r % ny) + 1, k = (int)(r / ny) + 1;
    int i = 2 - ((j + k + COLOUR) & 1) + 2 * h;
    if (i > nx) continue;
    size_t c = cidx(d, i, j, k);
    size_t q = hidx(d, i, j, k);
    size_t qjm = (j == 1) ? hidx(d, i, ny, k) : q - sj;
    size_t qjp = (j == ny) ? hidx(d, i, 1, k) : q + sj;
    double xc = x[q];
    double resid = d.SA[c] * xc + d.SB[c] * x[q - 1] + d.SC[c] * x[q + 1] + d.SD[c] * x[qjm] +
                   d.SE[c] * x[qjp] + d.SF[c] * x_km(d, x, q, k, sk) + d.SG[c] * x_kp(d, x, q, k, sk) - b[c];
    acc = acc + fabs(resid);
    x[q] = xc - omega * resid / d.SA[c];
  }
  double s = block_sum(acc, sh);
  if (threadIdx.x == 0) {
    partials[COLOUR * kMaxPartials + blockIdx.x] = s;
    if (COLOUR == 1) {
      __threadfence();
      last = (atomicAdd(&d.sol->ticket, 1u) == gridDim.x - 1);
    }
  }
  if (COLOUR == 1) {
    __syncthreads();
    if (last) {
      __threadfence();
      finalize_sweep(d, partials, gridDim.x, itmin, itmax, eps, sh);
    }
  }
}

// ||b - A x||_1 (FP64, reference operand order) into sol->true_l1.
__global__ void __launch_bounds__(kThreads) resid_l1_kernel(Dev d, const double* __restrict__ x,
                                                            const double* __restrict__ b, double* partials) {
  __shared__ double sh[32];
  __shared__ bool last;
  const int nx = d.nx, ny = d.ny;
  const long long n = (long long)nx * ny * sor_zmax(d);  // the rows the SOR solves
  const size_t sj = (size_t)(nx + 4), sk = (size_t)(nx + 4) * (ny + 4);
  double acc = 0.0;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    int i = (int)(t % nx) + 1;
    long long r = t / nx;
    int j = (int)(r % ny) + 1, k = (int)(r / ny) + 1;
    size_t q = hidx(d, i, j, k);
    size_t qjm = (j == 1) ? hidx(d, i, ny, k) : q - sj;
    size_t qjp = (j == ny) ? hidx(d, i, 1, k) : q + sj;
    double rr = d.SA[t] * x[q] + d.SB[t] * x[q - 1] + d.SC[t] * x[q + 1] + d.SD[t] * x[qjm] +
                d.SE[t] * x[qjp] + d.SF[t] * x_km(d, x, q, k, sk) + d.SG[t] * x_kp(d, x, q, k, sk) - b[t];
    acc = acc + fabs(rr);
  }
  double s = block_sum(acc, sh);
  if (threadIdx.x == 0) {
    partials[blockIdx.x] = s;
    __threadfence();
    last = (atomicAdd(&d.sol->ticket2, 1u) == gridDim.x - 1);
  }
  __syncthreads();
  if (last) {
    __threadfence();
    double tot = block_sum_array(partials, gridDim.x, sh);
    if (threadIdx.x == 0) {
      d.sol->true_l1 = tot;
      d.sol->ticket2 = 0;
    }
  }
}

// The seven sums of ttfld_energy_sums: per-block partials in a fixed order,
// then the last block adds them (fixed order) into part[7 * nbmax + q].
__global__ void __launch_bounds__(kThreads) energy_sums_kernel(Dev d, double* part, int nbmax) {
  __shared__ double sh[32];
  __shared__ bool last;
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  const long long n = (long long)nx * ny * nz;
  double s[7] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(t % nx) + 1;
    const long long r = t / nx;
    const int j = (int)(r % ny) + 1, k = (int)(r / ny) + 1;
    const int ub = PA(UB, j, k);
    const int itop = (ub < nx ? ub : nx) - 1;  // last active cell of the column
    if (i > itop || k < 2 || k > nz - 1) continue;
    const size_t h = hidx(d, i, j, k);
    const double vol = G(surxb, i) * G(dxa, i) * G(dya, j) * G(surzb, k) * G(dza, k);
    s[0] += vol;
    s[1] += vol * d.ER[h];
    s[2] += vol * d.Q[h];
    s[3] += vol * d.SI[h];
    const double ax = G(dya, j) * G(surzb, k) * G(dza, k);
    if (i == 1) s[4] += G(surxa, 1) * ax * FA(FLUXX, 1, j, k);
    if (i == itop) s[5] += G(surxa, i + 1) * ax * FA(FLUXX, i + 1, j, k);
    const double az = G(surxb, i) * G(dxa, i) * G(dya, j) / G(xxb, i);
    if (k == 2) s[6] -= G(surza, 2) * az * FA(FLUXZ, i, j, 2);
    if (k == nz - 1) s[6] += G(surza, nz) * az * FA(FLUXZ, i, j, nz);
  }
  for (int q = 0; q < 7; ++q) {
    const double b = block_sum(s[q], sh);
    if (threadIdx.x == 0) part[q * nbmax + blockIdx.x] = b;
  }
  if (threadIdx.x == 0) {
    __threadfence();
    last = (atomicAdd(&d.sol->ticket2, 1u) == gridDim.x - 1);
  }
  __syncthreads();
  if (last) {
    __threadfence();
    for (int q = 0; q < 7; ++q) {
      const double tot = block_sum_array(part + q * nbmax, gridDim.x, sh);
      if (threadIdx.x == 0) part[7 * nbmax + q] = tot;
    }
    if (threadIdx.x == 0) d.sol->ticket2 = 0;
  }
}

int rhs_norm(ttfld_ctx* c, const double* b, double* out_host) {
  int nb = grid_for((long long)ncell(c->d));
  if (nb > kMaxPartials) nb = kMaxPartials;
  rhsnorm_kernel<<<nb, kThreads, 0, c->stream>>>(c->d, b, c->partials);
  count_launches(1);
  TT_CHECK_LAUNCH();
  if (out_host) {
    TT_CHECK(cudaMemcpyAsync(c->host_sol, c->sol, sizeof(SolverDev), cudaMemcpyDeviceToHost, c->stream));
    TT_CHECK(cudaStreamSynchronize(c->stream));
    *out_host = c->host_sol->rhsnorm;
  }
  return 0;
}

int true_residual(ttfld_ctx* c, const double* x, const double* b, double* l1) {
  int nb = grid_for((long long)ncell(c->d));
  if (nb > kMaxPartials) nb = kMaxPartials;
  resid_l1_kernel<<<nb, kThreads, 0, c->stream>>>(c->d, x, b, c->partials + kMaxPartials);
  count_launches(1);
  TT_CHECK_LAUNCH();
  if (l1) {
    TT_CHECK(cudaMemcpyAsync(c->host_sol, c->sol, sizeof(SolverDev), cudaMemcpyDeviceToHost, c->stream));
    TT_CHECK(cudaStreamSynchronize(c->stream));
    *l1 = c->host_sol->true_l1;
  }
  return 0;
}

static int sweep_blocks(const Dev& d) {
  long long n = (long long)((d.nx + 1) / 2) * d.ny * d.nz;
  int nb = grid_for(n);
  return nb > kMaxPartials ? kMaxPartials : nb;
}

int launch_exact_sweeps(ttfld_ctx* c, double* x, const double* b, int nsweeps, int itmin, int itmax,
                               double eps) {
  const int nb = sweep_blocks(c->d);
  const double omega = c->d.sorparam;
  for (int s = 0; s < nsweeps; ++s) {
    sor_exact_kernel<0><<<nb, kThreads, 0, c->stream>>>(c->d, x, b, omega, c->partials, itmin, itmax, eps);
    sor_exact_kernel<1><<<nb, kThreads, 0, c->stream>>>(c->d, x, b, omega, c->partials, itmin, itmax, eps);
  }
  count_launches(2 * nsweeps);
  TT_CHECK_LAUNCH();
  return 0;
}

static void fill_stats(ttfld_ctx* c, ttfld_solve_stats* st, int status) {
  if (!st) return;
  const SolverDev* h = c->host_sol;
  st->sor_iter = h->iter;
  st->rnorm = h->rnorm;
  st->rhsnorm = h->rhsnorm;
  st->status = status;
}

// Red-black SOR to the ppsor.f:161-177 rule.  The host checks the device
// flag after chunks of sweeps; sweeps queued after the rule fired return at
// once, so the iteration count is exactly the reference's.
// DIFFUSION's sweeps on a context with poles: every theta row k = 1..NZ
// (ppdif.f:45-46, 93-94; no zmax_sor_index), the theta ghosts read as they
// are, and the pole shifts of the scalar after each colour (ppdif.f:80-89,
// 123-132), which row NZ needs: its k+1 ghost holds row NZ-2 from before
// the half-sweep.
static int launch_exact_sweeps_all_rows(ttfld_ctx* c, double* x, const double* b, int nsweeps, int itmin,
                                        int itmax, double eps) {
  const int nb = sweep_blocks(c->d);
  const double omega = c->d.sorparam;
  Dev d = c->d;
  d.poles = 0;  // sor_zmax = NZ and x_km / x_kp read the ghosts
  int rc;
  for (int s = 0; s < nsweeps; ++s) {
    sor_exact_kernel<0><<<nb, kThreads, 0, c->stream>>>(d, x, b, omega, c->partials, itmin, itmax, eps);
    if ((rc = pole_shift(c, x))) return rc;
    sor_exact_kernel<1><<<nb, kThreads, 0, c->stream>>>(d, x, b, omega, c->partials, itmin, itmax, eps);
    if ((rc = pole_shift(c, x))) return rc;
  }
  count_launches(2 * nsweeps);
  TT_CHECK_LAUNCH();
  return 0;
}

// all_rows: DIFFUSION's row range and pole shifts (above) instead of
// SOLVE_WITH_SOR's.
static int solve_exact_rows(ttfld_ctx* c, double* x, const double* b, int itmin, int itmax, ttfld_solve_stats* st,
                            bool all_rows) {
  all_rows = all_rows && c->d.poles;
  TT_CHECK(cudaMemsetAsync(c->sol, 0, sizeof(SolverDev), c->stream));
  int rc = rhs_norm(c, b, nullptr);
  if (rc) return rc;
  int chunk = 4, launched = 0;
  for (;;) {
    rc = all_rows ? launch_exact_sweeps_all_rows(c, x, b, chunk, itmin, itmax, c->d.epsmat)
                  : launch_exact_sweeps(c, x, b, chunk, itmin, itmax, c->d.epsmat);
    if (rc) return rc;
    launched += chunk;
    TT_CHECK(cudaMemcpyAsync(c->host_sol, c->sol, sizeof(SolverDev), cudaMemcpyDeviceToHost, c->stream));
    TT_CHECK(cudaStreamSynchronize(c->stream));
    if (c->host_sol->done) break;
    if (launched >= itmax + 2) return TTFLD_E_CUDA;  // the rule must have fired by ITMAX
    chunk = chunk < 128 ? chunk * 2 : 256;
  }
  // PLANETSHIFT(8) and the pole shifts after the last colour
  if ((rc = halo_shift(c, x)) || (rc = pole_shift(c, x))) return rc;
  int status = c->host_sol->nonfinite ? TTFLD_E_NONFINITE : (c->host_sol->maxit ? TTFLD_MAXITER : TTFLD_OK);
  fill_stats(c, st, status);
  return status;
}

int solve_exact64(ttfld_ctx* c, double* x, const double* b, int itmin, int itmax, ttfld_solve_stats* st) {
  return solve_exact_rows(c, x, b, itmin, itmax, st, false);
}

}  // namespace ttfld

using namespace ttfld;

namespace {

int solve_current(ttfld_ctx* c, double* x, const double* b, int itmin, int itmax, ttfld_solve_stats* st) {
  switch (c->opts.solver) {
    case TTFLD_SOLVER_SOR64_EXACT: return solve_exact64(c, x, b, itmin, itmax, st);
    case TTFLD_SOLVER_SOR64_FAST: return solve_fast64(c, x, b, itmin, itmax, st);
    case TTFLD_SOLVER_MIXED: return solve_mixed(c, x, b, st);
    case TTFLD_SOLVER_PCG: return solve_pcg(c, x, b, st);
  }
  return TTFLD_E_ARGS;
}

}  // namespace

namespace ttfld {
// Solve A x = RHS_ER for DELTA_ER with the context's solver and guess.
int solve_delta_er(ttfld_ctx* c, ttfld_solve_stats* st) {
  Dev d = c->d;
  ttfld_solve_stats local{};
  if (!st) st = &local;
  int fallback = 0;
  bool race = false;
  // the network makes the guess where the run has no previous solution (its
  // first solve, or after ttfld_begin_step(ctx, 1)); once there is one, the
  // previous solution is the better guess (it beats the network's
  // two-to-three-digit prediction over a run), so it is used instead
  int guess = c->opts.guess;
  if (guess == TTFLD_GUESS_LEARNED && !c->have_model) return TTFLD_E_NOMODEL;
  if (guess == TTFLD_GUESS_LEARNED && (c->solve_idx > 0 || c->have_prev)) guess = TTFLD_GUESS_PREVIOUS;
  TT_CHECK(cudaEventRecord(c->ev0, c->stream));
  if (guess == TTFLD_GUESS_ZERO || (guess == TTFLD_GUESS_PREVIOUS && !c->have_prev)) {
    TT_CHECK(cudaMemsetAsync(d.DELTA_ER, 0, nhalo(d) * 8, c->stream));  // ppsor.f:29
  } else {
    // initial iterate in the interior; ghosts zero as in ppsor.f:29
    double* x = d.DELTA_ER;
    TT_CHECK(cudaMemsetAsync(x, 0, nhalo(d) * 8, c->stream));
    double gl1 = 0.0, bl1 = 0.0;
    if (guess == TTFLD_GUESS_PREVIOUS) {
      const double* px = c->prev_x;
      const double sc = c->prev_scale;
      launch_box(c->stream, box(1, d.nx, 1, d.ny, 1, d.nz), [=] __device__(int i, int j, int k) {
        size_t q = hidx(d, i, j, k);
        x[q] = sc * px[q];
      });
      TT_CHECK_LAUNCH();
    } else {
      int rc = unet_guess(c, x, nullptr);
      if (rc) return rc;
    }
    int rc;
    bool reject = false;
    // rule 0: the residual the first sweep leaves (RNORM of sweep 2); rule 3:
    // the residual four sweeps leave (RNORM of sweep 5)
    const int race_sweeps = c->opts.fallback_rule == 0 ? 2 : (c->opts.fallback_rule == 3 ? 5 : 0);
    if (c->opts.fallback_rule == 2) {
      // no better than the zero guess's residual ||b||_1
      if ((rc = rhs_norm(c, d.RHS, &bl1)) || (rc = true_residual(c, x, d.RHS, &gl1))) return rc;
      st->guess_resid_l1 = gl1;
      reject = !(gl1 < bl1);
    } else if (race_sweeps > 0 && (c->opts.solver == TTFLD_SOLVER_MIXED || c->opts.solver == TTFLD_SOLVER_PCG)) {
      race = true;  // the mixed solver races the guess against zero itself, PCG compares r.z
    } else if (race_sweeps > 0) {
      // race_sweeps FP64 red-black sweeps from the guess and as many from
      // zero, on a scratch copy: keep the guess if the in-sweep residual
      // norm (RNORM) of its last sweep -- the residual the sweeps before it
      // left -- is the smaller.  (With over-relaxation the first sweep from
      // zero itself leaves a residual above ||b||_1, so the comparison is
      // made sweep for sweep rather than against ||b||_1.)
      if (!c->guess_tmp) TT_CHECK(cudaMalloc((void**)&c->guess_tmp, nhalo(d) * 8));
      double r2[2];
      for (int q = 0; q < 2; ++q) {
        if (q == 0) TT_CHECK(cudaMemcpyAsync(c->guess_tmp, x, nhalo(d) * 8, cudaMemcpyDeviceToDevice, c->stream));
        else TT_CHECK(cudaMemsetAsync(c->guess_tmp, 0, nhalo(d) * 8, c->stream));
        TT_CHECK(cudaMemsetAsync(c->sol, 0, sizeof(SolverDev), c->stream));
        if ((rc = rhs_norm(c, d.RHS, nullptr))) return rc;
        if ((rc = launch_exact_sweeps(c, c->guess_tmp, d.RHS, race_sweeps, race_sweeps + 1, race_sweeps + 1, -1.0)))
          return rc;
        TT_CHECK(cudaMemcpyAsync(c->host_sol, c->sol, sizeof(SolverDev), cudaMemcpyDeviceToHost, c->stream));
        TT_CHECK(cudaStreamSynchronize(c->stream));
        r2[q] = c->host_sol->rnorm;
      }
      reject = !(r2[0] < r2[1]);
    }
    if (reject) {
      TT_CHECK(cudaMemsetAsync(x, 0, nhalo(d) * 8, c->stream));
      fallback = 1;
    }
  }
  TT_CHECK(cudaEventRecord(c->evg, c->stream));
  int rc;
  if (race && c->opts.solver == TTFLD_SOLVER_PCG) rc = solve_pcg(c, d.DELTA_ER, d.RHS, st, 1, &fallback);
  else if (race) rc = solve_mixed(c, d.DELTA_ER, d.RHS, st, c->opts.fallback_rule == 3 ? 5 : 2, &fallback);
  else rc = solve_current(c, d.DELTA_ER, d.RHS, 1, d.itmax, st);
  TT_CHECK(cudaEventRecord(c->ev1, c->stream));
  TT_CHECK(cudaEventSynchronize(c->ev1));
  float ms = 0.f, gms = 0.f;
  cudaEventElapsedTime(&ms, c->ev0, c->ev1);
  cudaEventElapsedTime(&gms, c->ev0, c->evg);
  c->last_solve_ms = ms;
  st->solve_ms = ms;
  st->guess_ms = gms;
  st->fallback = fallback;
  if (rc < 0) return rc;
  // a requested training pair: the state this solve started from and its answer
  if (c->unet) {
    int rc2 = unet_capture(c);
    if (rc2) return rc2;
  }
  // keep this solution for the previous-solution guess of the next solve:
  // scaled by (1 - conv_parm) inside a step (ER moved by conv_parm * delta_ER),
  // as is from one step to the next
  if (!c->prev_x) TT_CHECK(cudaMalloc((void**)&c->prev_x, nhalo(d) * 8));
  TT_CHECK(cudaMemcpyAsync(c->prev_x, d.DELTA_ER, nhalo(d) * 8, cudaMemcpyDeviceToDevice, c->stream));
  c->have_prev = 1;
  c->prev_scale = 0.9;
  c->solve_idx += 1;
  if (fallback && rc == TTFLD_OK) rc = TTFLD_FALLBACK;
  return rc;
}
}  // namespace ttfld

extern "C" {

int ttfld_fill_sor_matrix(ttfld_ctx* c) {
  if (!c) return TTFLD_E_ARGS;
  int rc = fill_sor_matrix(c);
  if (rc) return rc;
  TT_CHECK(cudaStreamSynchronize(c->stream));
  return 0;
}

int ttfld_sor_sweeps(ttfld_ctx* c, int n, double* rnorm, double* rhsnorm) {
  if (!c || n < 0) return TTFLD_E_ARGS;
  TT_CHECK(cudaMemsetAsync(c->sol, 0, sizeof(SolverDev), c->stream));
  int rc = rhs_norm(c, c->d.RHS, nullptr);
  if (rc) return rc;
  // itmax beyond n so the rule never stops the requested sweeps
  if ((rc = launch_exact_sweeps(c, c->d.DELTA_ER, c->d.RHS, n, n + 1, n + 2, -1.0))) return rc;
  if ((rc = halo_shift(c, c->d.DELTA_ER)) || (rc = pole_shift(c, c->d.DELTA_ER))) return rc;
  TT_CHECK(cudaMemcpyAsync(c->host_sol, c->sol, sizeof(SolverDev), cudaMemcpyDeviceToHost, c->stream));
  TT_CHECK(cudaStreamSynchronize(c->stream));
  if (rnorm) *rnorm = c->host_sol->rnorm;
  if (rhsnorm) *rhsnorm = c->host_sol->rhsnorm;
  return c->host_sol->iter == n ? 0 : TTFLD_E_CUDA;
}

int ttfld_true_residual(ttfld_ctx* c, double* l1, double* rhs_l1) {
  if (!c) return TTFLD_E_ARGS;
  int rc = rhs_norm(c, c->d.RHS, rhs_l1);
  if (rc) return rc;
  double v = 0.0;
  if ((rc = true_residual(c, c->d.DELTA_ER, c->d.RHS, &v))) return rc;
  if (l1) *l1 = v;
  return 0;
}

int ttfld_energy_sums(ttfld_ctx* c, ttfld_energy* out) {
  if (!c || !out) return TTFLD_E_ARGS;
  constexpr int kNb = 1024;  // blocks; partials [7][kNb] then 7 totals
  int nb = grid_for((long long)ncell(c->d));
  if (nb > kNb) nb = kNb;
  energy_sums_kernel<<<nb, kThreads, 0, c->stream>>>(c->d, c->partials, kNb);
  count_launches(1);
  TT_CHECK_LAUNCH();
  double t[7];
  TT_CHECK(cudaMemcpyAsync(t, c->partials + 7 * kNb, sizeof(t), cudaMemcpyDeviceToHost, c->stream));
  TT_CHECK(cudaStreamSynchronize(c->stream));
  out->volume = t[0]; out->e_rad = t[1]; out->e_gas = t[2]; out->heating = t[3];
  out->flux_bottom = t[4]; out->flux_top = t[5]; out->flux_theta = t[6];
  return 0;
}

int ttfld_begin_step(ttfld_ctx* c, int new_run) {
  if (!c) return TTFLD_E_ARGS;
  c->solve_idx = 0;
  c->prev_scale = 1.0;
  if (new_run) c->have_prev = 0;
  return 0;
}

int ttfld_solve_system(ttfld_ctx* c, ttfld_solve_stats* st) {
  if (!c) return TTFLD_E_ARGS;
  c->solve_idx = 0;  // a system solved on its own counts as a step's first solve
  return solve_delta_er(c, st);
}

int ttfld_solve_with_sor(ttfld_ctx* c, int print_max_values, ttfld_solve_stats* st) {
  if (!c) return TTFLD_E_ARGS;
  int rc = fill_sor_matrix(c);
  if (rc) return rc;
  rc = solve_delta_er(c, st);
  if (rc == TTFLD_MAXITER && print_max_values) {
    const SolverDev* h = c->host_sol;
    printf("MAX COUPLED SOR ITERATION %8d %12.6e %12.6e %12.6e %12.6e\n", h->iter, h->ratio, h->rnorm,
           h->rhsnorm, c->d.epsmat);
  }
  return rc;
}

int ttfld_adjust_sor_param(ttfld_ctx* c, double* out) {
  if (!c) return TTFLD_E_ARGS;
  int save_it[50];
  double save_p[50];
  double omega = (double)1.01f;  // ppsor.f:341, REAL*4 literal
  int rc = fill_sor_matrix(c);
  if (rc) return rc;
  for (int n = 0; n < 50; ++n) {
    c->d.sorparam = omega;
    TT_CHECK(cudaMemsetAsync(c->d.DELTA_ER, 0, nhalo(c->d) * 8, c->stream));
    rc = solve_exact64(c, c->d.DELTA_ER, c->d.RHS, 1, c->d.itmax, nullptr);
    if (rc < 0) return rc;
    save_it[n] = c->host_sol->iter;
    save_p[n] = omega;
    omega = omega + (double)0.02f;  // ppsor.f:346
  }
  int best = 0;
  for (int n = 1; n < 50; ++n)
    if (save_it[n] < save_it[best]) best = n;
  c->d.sorparam = save_p[best];
  c->params.sorparam = save_p[best];
  if (out) *out = save_p[best];
  return 0;
}

}  // extern "C"

namespace ttfld {
// DIFFUSION ppdif.f:1-167 with DIFFUSION_MAT_ELEM (:169-223),
// DIFFUSION_COEF (:226-275) and FILL_DVALUES (:278-308): implicit diffusion
// of the SCALAR field with the constant xnue/Pr_num, the same red-black
// SOR with ITMIN=5 and SORITMAX=500 (ppdif.f:14-15), in place on SCALAR.
static int diffusion(ttfld_ctx* c, ttfld_solve_stats* st) {
  Dev d = c->d;
  if (!(d.pr_num != 0.0)) return TTFLD_E_ARGS;
  const double dconst = d.xnue / d.pr_num;
  launch_box(c->stream, box(1, d.nx, 1, d.ny, 1, d.nz), [=] __device__(int i, int j, int k) {
    size_t q = cidx(d, i, j, k);
    d.RHS_DIF[q] = HA(SCALAR, i, j, k);
    double dx1 = dconst / G(dxb, i + 1), dx2 = dconst / G(dxb, i);
    double dy1 = dconst / (G(dyb, j + 1) * G(geoxg, i) * G(geozg, k));
    double dy2 = dconst / (G(dyb, j) * G(geoxg, i) * G(geozg, k));
    double dz1 = dconst / (G(dzb, k + 1) * G(geoxh, i));
    double dz2 = dconst / (G(dzb, k) * G(geoxh, i));
    double d1 = d.delt * G(surxa, i + 1) * dx1 / (G(surxb, i) * G(dxa, i));
    double d2 = d.delt * G(surxa, i) * dx2 / (G(surxb, i) * G(dxa, i));
    double d3 = d.delt * dy1 / (G(geoxg, i) * G(surzb, k) * G(dya, j));
    double d4 = d.delt * dy2 / (G(geoxg, i) * G(surzb, k) * G(dya, j));
    double d5 = d.delt * dz1 * G(surza, k + 1) / (G(geoxg, i) * G(surzb, k) * G(dza, k));
    double d6 = d.delt * dz2 * G(surza, k) / (G(geoxg, i) * G(surzb, k) * G(dza, k));
    double d16 = d1 + d2 + d3 + d4 + d5 + d6;
    if (i == d.nx) {  // XMAX zero-gradient row, ppdif.f:212-220
      d.SA[q] = 1.0 + d2; d.SB[q] = -d2; d.SC[q] = 0.0; d.SD[q] = 0.0;
      d.SE[q] = 0.0; d.SF[q] = 0.0; d.SG[q] = 0.0;
    } else {
      d.SA[q] = 1.0 + d16; d.SB[q] = -d2; d.SC[q] = -d1; d.SD[q] = -d4;
      d.SE[q] = -d3; d.SF[q] = -d6; d.SG[q] = -d5;
    }
  });
  TT_CHECK_LAUNCH();
  return solve_exact_rows(c, d.SCALAR, d.RHS_DIF, 5, 500, st, true);
}
}  // namespace ttfld

extern "C" int ttfld_diffusion(ttfld_ctx* c, ttfld_solve_stats* st) {
  if (!c) return TTFLD_E_ARGS;
  return ttfld::diffusion(c, st);
}
