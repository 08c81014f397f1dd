// ttfld_raddif.cu -- the IRAD=1 radiation step: RADDIF (pprad.f:1-38) with
// DIFFEL (pprad.f:40-72), SOLVMAT (ppmat.f:1-186) and RADIATIVEBOUND
// (ppbou.f:2049-2299).
//
// RADDIF sets ER = arad T^4, forms the diffusion couplings AX..CZ from DIFF's
// face coefficients, B = c_v rho / (dt 4 arad T^3) - sum of the couplings and
// RHS = ER c_v rho / (dt 4 arad T^3), solves B ER + sum(couplings * ER_nb) =
// RHS for ER by red-black SOR on ER itself, and returns T = (ER/arad)^(1/4).
// SOLVMAT's stopping rule is the L2 ratio ||XS|| / ||RHS|| <= EPSMAT after at
// least ITMIN = 5 iterations (ppmat.f:152-178); after each colour
// RADIATIVEBOUND resets the bottom (T and ER at i <= 1 from the gradient D_T)
// and the top (ER at i >= upperbnd), copies the theta ghosts and shifts the
// phi halo.  Every kernel keeps the reference's operation order (the library
// is built with --fmad=false), so the iterates equal the reference loop's
// except where pow() enters (the IBDRAD = 9 top and the final T).
#include <math.h>

#include "ttfld_internal.cuh"

namespace ttfld {
int asm_diff(ttfld_ctx* c, int energy_iter);

namespace {

struct RadWork {
  double *ax, *cx, *ay, *cy, *az, *cz, *b, *rhs, *xs;
  double *volxb, *volyb, *volzb;  // (1:NX), (1:NY), (1:NZ)
  void* mem;
};

__global__ void __launch_bounds__(kThreads) er_from_t_kernel(Dev d) {
  const long long n = (long long)nhalo(d);
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x)
    d.ER[q] = TT_ARAD * p4(d.T[q]);
}

__global__ void __launch_bounds__(kThreads) t_from_er_kernel(Dev d) {
  const long long n = (long long)nhalo(d);
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x)
    d.T[q] = pow(d.ER[q] / TT_ARAD, 0.25);
}

// DIFFEL (pprad.f:56-66) and B, RHS (pprad.f:21-29); SURYA = 1 (ppinit.f:1367).
__global__ void __launch_bounds__(kThreads) diffel_kernel(Dev d, RadWork w) {
  const long long n = (long long)ncell(d);
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(t % d.nx) + 1;
    const long long r = t / d.nx;
    const int j = (int)(r % d.ny) + 1, k = (int)(r / d.ny) + 1;
    const double vx = w.volxb[i - 1], vy = w.volyb[j - 1], vz = w.volzb[k - 1];
    const double ax = -FA(DIFRX, i, j, k) * G(surxa, i) / vx;
    const double cx = -FA(DIFRX, i + 1, j, k) * G(surxa, i + 1) / vx;
    const double ay = -FA(DIFRY, i, j, k) * 1.0 / vy / G(geoxg, i) / G(geozg, k);
    const double cy = -FA(DIFRY, i, j + 1, k) * 1.0 / vy / G(geoxg, i) / G(geozg, k);
    const double az = -FA(DIFRZ, i, j, k) * G(surza, k) / vz / G(geoxh, i);
    const double cz = -FA(DIFRZ, i, j, k + 1) * G(surza, k + 1) / vz / G(geoxh, i);
    const double tt = HA(T, i, j, k);
    const double wt = 1.0 / d.delt * HA(CV, i, j, k) * HA(RH, i, j, k) / (4.0 * TT_ARAD * tt * tt * tt);
    w.ax[t] = ax; w.cx[t] = cx; w.ay[t] = ay; w.cy[t] = cy; w.az[t] = az; w.cz[t] = cz;
    w.b[t] = wt - ax - cx - ay - cy - az - cz;
    w.rhs[t] = HA(ER, i, j, k) / d.delt * HA(CV, i, j, k) * HA(RH, i, j, k) / (4.0 * TT_ARAD * tt * tt * tt);
  }
}

// One colour of SOLVMAT (ppmat.f:66-82, 110-121): XS = B ER - RHS + the
// couplings (left to right), ER -= OM * XS / B.
template <int PARITY>
__global__ void __launch_bounds__(kThreads) solvmat_colour_kernel(Dev d, RadWork w, double om) {
  if (solver_done(d)) return;
  const int nx = d.nx, ny = d.ny;
  const int nxh = (nx + 1) >> 1;
  const long long n = (long long)nxh * ny * d.nz;
  const size_t sj = (size_t)(nx + 4), sk = (size_t)(nx + 4) * (ny + 4);
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    const int h = (int)(t % nxh);
    const long long r = t / nxh;
    const int j = (int)(r % ny) + 1, k = (int)(r / ny) + 1;
    const int imin = 2 - ((j + k + PARITY) % 2);
    const int i = imin + 2 * h;
    if (i > nx) continue;
    const size_t c = cidx(d, i, j, k);
    const size_t q = hidx(d, i, j, k);
    double* er = d.ER;
    const double x = w.b[c] * er[q] - w.rhs[c] + w.ax[c] * er[q - 1] + w.cx[c] * er[q + 1] + w.ay[c] * er[q - sj] +
                     w.cy[c] * er[q + sj] + w.az[c] * er[q - sk] + w.cz[c] * er[q + sk];
    w.xs[c] = x;
    er[q] = er[q] - om * x / w.b[c];
  }
}

// RADIATIVEBOUND, part 1 (ppbou.f:2127-2139 and 2145-2236): bottom T and ER
// on (j,k) in -1..N+2, top ER on the interior columns.  Sets
// sol->nonfinite = 2 (read as an error) if a column has upperbnd >= NX+1,
// where the reference stops (:2238-2240).
__global__ void __launch_bounds__(kThreads) radbound_xkernel(Dev d, double d_t, double tinit_bottom) {
  if (solver_done(d)) return;  // applied once more after the stop it would move the IBDRAD = 9 top
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  const long long n = (long long)(ny + 4) * (nz + 4);
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    const int j = (int)(t % (ny + 4)) - 1, k = (int)(t / (ny + 4)) - 1;
    if (d.bcxmin == 6) HA(T, 1, j, k) = tinit_bottom;
    HA(T, 0, j, k) = HA(T, 1, j, k) - d_t * (G(xxb, 1) - G(xxb, 0));
    HA(T, -1, j, k) = HA(T, 1, j, k) - d_t * (G(xxb, 1) - G(xxb, -1));
    HA(ER, 1, j, k) = TT_ARAD * p4(HA(T, 1, j, k));
    HA(ER, 0, j, k) = TT_ARAD * p4(HA(T, 0, j, k));
    HA(ER, -1, j, k) = TT_ARAD * p4(HA(T, -1, j, k));
    if (j < 1 || j > ny || k < 1 || k > nz) continue;
    const int ub = PA(UB, j, k);
    if (!(ub < nx + 1)) {
      atomicExch(&d.sol->nonfinite, 2);
      continue;
    }
    double tj = 0.0;
    switch (d.ibdrad) {
      case 4: tj = d.tirr; break;
      case 7: tj = HA(T, ub - 1, j, k); break;
      default:  // 9
        if (d.iii <= 1) tj = HA(T, ub - 1, j, k);
        else
          tj = pow(HA(ER, ub, j, k) / TT_ARAD +
                       HA(SI, ub - 1, j, k) / (4.0 * TT_SBCONST * HA(RH, ub - 1, j, k) * HA(XKAPP, ub - 1, j, k)),
                   0.25);
    }
    const double e = TT_ARAD * p4(tj);
    for (int i = ub; i <= nx + 2; ++i) HA(ER, i, j, k) = e;
  }
}

// PLANETSHIFT(6) and, with poles, the pole shifts of E_R that follow it
// everywhere in RADDIF (ppmat.f:39-49, 87-97, 126-136; ppbou.f:2280-2290).
static int er_shift(ttfld_ctx* c) {
  int rc = halo_shift(c, c->d.ER);
  return rc ? rc : pole_shift(c, c->d.ER);
}

// RADIATIVEBOUND, part 2 (ppbou.f:2256-2271): theta ghosts from k = 1, NZ.
__global__ void __launch_bounds__(kThreads) radbound_zkernel(Dev d) {
  if (solver_done(d)) return;
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  const long long n = (long long)(nx + 4) * (ny + 4);
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(t % (nx + 4)) - 1, j = (int)(t / (nx + 4)) - 1;
    HA(ER, i, j, -1) = HA(ER, i, j, 1);
    HA(ER, i, j, 0) = HA(ER, i, j, 1);
    HA(ER, i, j, nz + 1) = HA(ER, i, j, nz);
    HA(ER, i, j, nz + 2) = HA(ER, i, j, nz);
  }
}

// sqrt(sum a^2) over the cells, fixed order; the last block applies the
// stopping rule when `stop` (ratio against sol->rhsnorm, ITMIN = 5).
__global__ void __launch_bounds__(kThreads) l2_kernel(Dev d, const double* a, double* partials, int stop, int itmax,
                                                      double eps) {
  __shared__ double sh[32];
  __shared__ bool last;
  if (stop && solver_done(d)) return;
  const long long n = (long long)ncell(d);
  double acc = 0.0;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x)
    acc += a[t] * a[t];
  const double s = block_sum(acc, sh);
  if (threadIdx.x == 0) {
    partials[blockIdx.x] = s;
    __threadfence();
    last = (atomicAdd(&d.sol->ticket2, 1u) == gridDim.x - 1);
  }
  __syncthreads();
  if (last) {
    __threadfence();
    const double tot = block_sum_array(partials, gridDim.x, sh);
    if (threadIdx.x == 0) {
      const double nrm = sqrt(tot);
      SolverDev* sol = d.sol;
      if (!stop) {
        sol->rhsnorm = nrm;
      } else {
        const int it = sol->iter + 1;
        sol->iter = it;
        sol->rnorm = nrm;
        sol->ratio = nrm / sol->rhsnorm;
        if (!isfinite(nrm)) { sol->nonfinite = 1; sol->done = 1; }
        else if (it == itmax) { sol->maxit = 1; sol->done = 1; }
        else if (!(sol->ratio > eps) && it >= 5) sol->done = 1;
      }
      sol->ticket2 = 0;
    }
  }
}

int cell_blocks(const Dev& d) {
  const int nb = grid_for((long long)ncell(d));
  return nb > kMaxPartials ? kMaxPartials : nb;
}

// With poles the theta ghosts come from the pole shifts instead
// (ppbou.f:2256-2271 run only without poles; :2280-2290).
int radiativebound(ttfld_ctx* c, double d_t, double tinit_bottom) {
  const Dev& d = c->d;
  radbound_xkernel<<<grid_for((long long)(d.ny + 4) * (d.nz + 4)), kThreads, 0, c->stream>>>(d, d_t, tinit_bottom);
  count_launches(1);
  if (!d.poles) {
    radbound_zkernel<<<grid_for((long long)(d.nx + 4) * (d.ny + 4)), kThreads, 0, c->stream>>>(d);
    count_launches(1);
  }
  TT_CHECK_LAUNCH();
  return er_shift(c);
}

}  // namespace
}  // namespace ttfld

extern "C" int ttfld_raddif(ttfld_ctx* c, const ttfld_raddif_params* p, ttfld_solve_stats* st) {
  using namespace ttfld;
  if (!c || !p || !p->volxb || !p->volyb || !p->volzb) return TTFLD_E_ARGS;
  const Dev& d = c->d;
  if (d.nz == 1) return TTFLD_E_UNSUPPORTED;
  if (!(d.ibdrad == 4 || d.ibdrad == 7 || d.ibdrad == 9) || p->modver > 5)
    return TTFLD_E_UNSUPPORTED;
  TT_CHECK(cudaSetDevice(c->device));
  ttfld_solve_stats local{};
  if (!st) st = &local;
  RadWork w{};
  const size_t n = ncell(d);
  const size_t bytes = (9 * n + (size_t)d.nx + d.ny + d.nz) * sizeof(double);
  TT_CHECK(cudaMallocAsync(&w.mem, bytes, c->stream));
  double* q = (double*)w.mem;
  double** arrs[] = {&w.ax, &w.cx, &w.ay, &w.cy, &w.az, &w.cz, &w.b, &w.rhs, &w.xs};
  for (double** a : arrs) { *a = q; q += n; }
  w.volxb = q; q += d.nx;
  w.volyb = q; q += d.ny;
  w.volzb = q;
  int rc = 0;
  TT_CHECK(cudaMemcpyAsync(w.volxb, p->volxb, d.nx * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  TT_CHECK(cudaMemcpyAsync(w.volyb, p->volyb, d.ny * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  TT_CHECK(cudaMemcpyAsync(w.volzb, p->volzb, d.nz * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  TT_CHECK(cudaEventRecord(c->ev0, c->stream));
  er_from_t_kernel<<<grid_for((long long)nhalo(d)), kThreads, 0, c->stream>>>(d);
  count_launches(1);
  TT_CHECK_LAUNCH();
  rc = asm_diff(c, p->energy_iter);
  if (!rc) {
    diffel_kernel<<<grid_for((long long)n), kThreads, 0, c->stream>>>(d, w);
    count_launches(1);
    TT_CHECK_LAUNCH();
    TT_CHECK(cudaMemsetAsync(c->sol, 0, sizeof(SolverDev), c->stream));
    const int nb = cell_blocks(d);
    l2_kernel<<<nb, kThreads, 0, c->stream>>>(d, w.rhs, c->partials, 0, d.itmax, d.epsmat);
    count_launches(1);
    rc = er_shift(c);
  }
  // iterations in chunks between polls of the stopping flag
  const int sweeps_nb = grid_for((long long)((d.nx + 1) / 2) * d.ny * d.nz);
  int chunk = 8;
  while (!rc) {
    for (int s = 0; s < chunk && !rc; ++s) {
      solvmat_colour_kernel<0><<<sweeps_nb, kThreads, 0, c->stream>>>(d, w, d.sorparam);
      count_launches(1);
      if ((rc = radiativebound(c, p->d_t, p->tinit_bottom)) || (rc = er_shift(c))) break;
      solvmat_colour_kernel<1><<<sweeps_nb, kThreads, 0, c->stream>>>(d, w, d.sorparam);
      count_launches(1);
      if ((rc = radiativebound(c, p->d_t, p->tinit_bottom)) || (rc = er_shift(c))) break;
      l2_kernel<<<cell_blocks(d), kThreads, 0, c->stream>>>(d, w.xs, c->partials, 1, d.itmax, d.epsmat);
      count_launches(1);
      TT_CHECK_LAUNCH();
    }
    if (rc) break;
    TT_CHECK(cudaMemcpyAsync(c->host_sol, c->sol, sizeof(SolverDev), cudaMemcpyDeviceToHost, c->stream));
    TT_CHECK(cudaStreamSynchronize(c->stream));
    if (c->host_sol->nonfinite == 2) { rc = TTFLD_E_UNSUPPORTED; break; }
    if (c->host_sol->done) break;
    if (chunk < 64) chunk *= 2;
  }
  // the colour kernels, bounds and norms queued after the stop return at
  // once or leave ER unchanged (the bounds re-apply the same values)
  if (!rc) {
    t_from_er_kernel<<<grid_for((long long)nhalo(d)), kThreads, 0, c->stream>>>(d);
    count_launches(1);
    TT_CHECK_LAUNCH();
  }
  TT_CHECK(cudaEventRecord(c->ev1, c->stream));
  TT_CHECK(cudaFreeAsync(w.mem, c->stream));
  TT_CHECK(cudaStreamSynchronize(c->stream));
  if (rc) return rc;
  float ms = 0.f;
  cudaEventElapsedTime(&ms, c->ev0, c->ev1);
  const SolverDev& h = *c->host_sol;
  st->sor_iter = h.iter;
  st->rnorm = h.rnorm;
  st->rhsnorm = h.rhsnorm;
  st->solve_ms = ms;
  st->status = h.nonfinite ? TTFLD_E_NONFINITE : (h.maxit ? TTFLD_MAXITER : TTFLD_OK);
  if (h.maxit) printf("Max iteration reached in SOR matrix solver %8d %8d %12.6e %12.6e %12.6e %12.6e %12.6e\n", d.iii,
                      h.iter, h.ratio, h.rnorm, h.rhsnorm, d.epsmat, d.sorparam);
  return st->status;
}
